"""Exactness of the FP32 emulation of the reference's double-precision dequantization
x = (float)((double)s * 2eb): every integer s in [-2^24, 2^24] and a spread of non-integer, tiny,
huge and special values, for several error bounds, against numpy's IEEE double multiply."""
import numpy as np
import pytest

from vecsz_gb300 import api

pytestmark = pytest.mark.gpu

EBS = [1e-4, 1e-3, 1e-6, 2.0 ** -14, 1e-4 * 7.3712345, 0.5, 3.3e-9, 12.5]


def _dequant_on_device(cuda, s: np.ndarray, eb: float) -> np.ndarray:
    n = s.size
    x = cuda.zeros(1, dtype=cuda.float32, device="cuda")
    consts, info, st = api.eb_setup(x, eb, "abs")
    assert st == 0
    code = cuda.zeros(n, dtype=cuda.int16, device="cuda")  # all outliers: xhat = dequant(outlier)
    outl = cuda.from_numpy(s.astype(np.float32)).cuda()
    out = api.dualquant_decompress((n,), 8, 1024, code, outl, consts)
    return out.cpu().numpy()


@pytest.mark.parametrize("eb", EBS)
def test_dequant_all_integers(cuda, eb):
    s = np.arange(-(1 << 24), (1 << 24) + 1, dtype=np.float64).astype(np.float32)
    got = _dequant_on_device(cuda, s, eb)
    want = (s.astype(np.float64) * (2.0 * eb)).astype(np.float32)
    bad = np.nonzero(got.view(np.uint32) != want.view(np.uint32))[0]
    assert bad.size == 0, f"eb={eb}: {bad.size} mismatches, e.g. s={s[bad[:5]]}"


@pytest.mark.parametrize("eb", EBS)
def test_dequant_special_values(cuda, eb):
    rng = np.random.default_rng(7)
    parts = [
        rng.standard_normal(200000).astype(np.float32) * 1e3,
        (rng.standard_normal(200000) * 1e30).astype(np.float32),
        (rng.standard_normal(200000) * 1e-30).astype(np.float32),
        rng.integers(-(1 << 31), 1 << 31, 200000).astype(np.float32),
        np.array([0.0, -0.0, np.inf, -np.inf, 3.4e38, -3.4e38, 1e-45, -1e-45, 2.0 ** 24, 2.0 ** 25 + 2,
                  1.1754944e-38], np.float32),
    ]
    s = np.concatenate(parts)
    got = _dequant_on_device(cuda, s, eb)
    with np.errstate(over="ignore", invalid="ignore"):
        want = (s.astype(np.float64) * (2.0 * eb)).astype(np.float32)
    same = (got.view(np.uint32) == want.view(np.uint32)) | (np.isnan(got) & np.isnan(want))
    assert same.all(), f"eb={eb}: {np.count_nonzero(~same)} mismatches, e.g. {s[~same][:5]}"


# Error bounds whose c_d = 2 eb makes the separable pass's two-operation dequantization,
# RN32(s c_hi + RN32(s c_lo)), differ from the reference's (float)((double)s c_d) at exactly one
# pair +-s with 0 < s < 2^21 (kept as the check's exception), and one where it differs at several
# (the check falls back to the checked FP32 path).  Found by an exhaustive C loop over s with a
# correctly rounded fmaf.
ONE_PAIR = [(0.00013056223589487476, 1698755), (0.00019158748290109797, 1478839)]
MANY = [0.00011538630910934243]


@pytest.mark.parametrize("eb,s_exc", ONE_PAIR + [(e, None) for e in MANY])
def test_separable_dequant_exception_and_fallback(cuda, eb, s_exc, monkeypatch):
    """A 2^22-element 3D field (the size from which decompress checks the two-operation form)
    whose prequantized values pass through the exception value +-s_exc (or, for the fallback bound,
    a comparable range): archive and reconstruction bit-identical to the oracle's."""
    import oracle as O
    import vecsz_gb300 as V
    monkeypatch.setenv("VSZ_DQ_NO_WAVEFRONT", "1")  # a field this small else takes the wavefront pass
    nz, ny, nx = 128, 128, 256
    z, y, xx = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    g = (np.sin(xx / 9.0) * np.cos(y / 7.0) + 0.3 * np.sin(z / 5.0 + xx / 13.0)).ravel() / 1.3  # [-1, 1]
    centre = (s_exc if s_exc else 1500000) * 2.0 * eb
    half = g.size // 2
    x = np.empty(g.size, np.float64)
    x[:half] = centre + g[:half] * 1000 * 2.0 * eb   # about +-1000 quanta around +s
    x[half:] = -centre + g[half:] * 1000 * 2.0 * eb  # and around -s
    x = x.astype(np.float32)
    if s_exc:
        s = np.rint(x * np.float32(1.0 / (2.0 * eb)))  # the AVX prequantization, float32
        assert (s == s_exc).any() and (s == -s_exc).any()
    dims = (nx, ny, nz)
    c = V.compress(x, dims, eb=eb, mode="abs", dict_size=1024, block_size=8)
    oa, meta = O.compress(x, dims, 8, 1024, eb, False)
    assert c.data[: c.data_size] == oa
    assert meta["n_outlier"] * 64 < x.size  # the separable pass is taken
    np.testing.assert_array_equal(V.decompress(c).view(np.uint32), O.decompress(oa, 8, 1024).view(np.uint32))
