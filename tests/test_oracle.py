"""Pins the C oracle (oracle/vsz_oracle.c) to the reference: golden fixtures produced by the
reference itself (tests/golden/make_golden.py), and -- where the reference can be compiled here
(x86-64 with its sources) -- the reference directly on seeded random shapes.  CPU only."""
import os
import tempfile

import numpy as np
import pytest

import oracle as O
from conftest import golden_cases, load_golden

CASES = golden_cases()


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_golden_stages(name):
    g = load_golden(name)
    code, outl = O.dualquant(g["x"], g["dims"], g["bs"], g["dict_size"], g["eb_final"])
    np.testing.assert_array_equal(code.astype(np.uint16), g["code"])
    outliers = O.gather_outliers(code, outl)
    np.testing.assert_array_equal(outliers.view(np.uint32), g["outliers"].view(np.uint32))
    huff = O.huffman_encode(code, g["dict_size"])
    assert huff == g["huff"].tobytes()
    np.testing.assert_array_equal(O.huffman_decode(huff, code.size), code)


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_golden_archive(name):
    g = load_golden(name)
    archive, meta = O.compress(g["x"], g["dims"], g["bs"], g["dict_size"], g["eb"], bool(g["r2r"]))
    assert archive == g["archive"].tobytes()
    assert meta["n_outlier"] == g["n_outlier"]
    vr = O.value_range(g["x"]) if g["r2r"] else 0.0
    xhat = O.decompress(archive, g["bs"], g["dict_size"], vr)
    np.testing.assert_array_equal(xhat.view(np.uint32), g["xhat"].view(np.uint32))


def test_oracle_value_range_rules():
    x = np.array([1.5, -2.0, 7.25, 0.0], np.float32)
    assert O.value_range(x) == float(np.float32(7.25) - np.float32(-2.0))
    # std::max_element keeps a leading NaN; later NaNs are ignored
    y = np.array([1.0, np.nan, 3.0], np.float32)
    assert O.value_range(y) == 2.0


def test_oracle_error_bound_on_smooth_field():
    from vecsz_gb300 import fields
    x = fields.bump_field_2d(60, 96, seed=11).ravel()  # d0 % 8 == 0: no zeroed tail columns
    for eb in (1e-2, 1e-3, 1e-4):
        archive, meta = O.compress(x, (96, 60), 8, 1024, eb, False)
        xhat = O.decompress(archive, 8, 1024)
        err = np.abs(x.astype(np.float64) - xhat.astype(np.float64))
        # documented reference overshoot: at most eb plus two ulps of the value
        ulp = np.spacing(np.abs(x)).astype(np.float64)
        assert np.all(err <= eb + 2 * ulp + 1e-12)


def test_oracle_b1_tail_columns_zeroed():
    """2D fields with d0 % 8 != 0: the last d0 % 8 columns decode to 0 (reference quirk)."""
    from vecsz_gb300 import fields
    x = fields.bump_field_2d(20, 21, seed=2).ravel() + 1.0
    archive, _ = O.compress(x, (21, 20), 8, 1024, 1e-3, False)
    xhat = O.decompress(archive, 8, 1024).reshape(20, 21)
    assert np.all(xhat[:, 16:] == 0.0)
    assert np.all(xhat[:, :16] != 0.0)


ref_only = pytest.mark.skipif(not (O.ref_available() or os.path.isdir("/root/reference/src")),
                              reason="reference sources not available (pinned by the golden fixtures instead)")


@ref_only
@pytest.mark.parametrize("seed", range(6))
def test_oracle_matches_reference_random_shapes(seed):
    if not O.ref_available():
        if O.build_ref() is None:
            pytest.skip("reference cannot be built on this machine")
    rng = np.random.default_rng(100 + seed)
    ndim = 1 + seed % 3
    if ndim == 1:
        dims = (int(rng.integers(50, 4000)),)
    elif ndim == 2:
        dims = (int(rng.integers(5, 140)), int(rng.integers(5, 90)))
    else:
        dims = tuple(int(rng.integers(3, 40)) for _ in range(3))
    n = int(np.prod(dims))
    bs = int(rng.choice([8, 16, 32, 64]))
    dct = int(rng.choice([256, 1024, 4096]))
    eb = float(10 ** rng.uniform(-6, -1))
    x = (np.cumsum(rng.standard_normal(n)) * 10 ** rng.uniform(-2, 3)).astype(np.float32)
    r2r = bool(seed % 2)
    tmp = tempfile.mkdtemp()
    f = os.path.join(tmp, "f.f32")
    a_ref, dsz, _, nout = O.ref_compress(x, dims, bs, dct, eb, r2r, 0, f)
    a_or, meta = O.compress(x, dims, bs, dct, eb, r2r)
    assert a_or == a_ref
    if ndim > 1:
        y_ref = O.ref_decompress(a_ref, dsz, 0, n, bs, dct, r2r, f)
        y_or = O.decompress(a_or, bs, dct, O.value_range(x) if r2r else 0.0)
        np.testing.assert_array_equal(y_or.view(np.uint32), y_ref.view(np.uint32))
