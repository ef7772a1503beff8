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
