"""Pins the C oracle (oracle/vsz_oracle.c) to the reference: golden fixtures produced by the
reference itself (tests/golden/make_golden.py), and -- where the reference can be compiled here
(x86-64 with its sources) -- the reference directly on seeded random shapes.  CPU only."""
import os
import tempfile

import numpy as np
import pytest

import oracle as O
from conftest import golden_cases, load_golden, pad_golden_cases

CASES = golden_cases()
PAD_CASES = pad_golden_cases()


def pad_section(archive: bytes, ndim: int, npad: int) -> np.ndarray:
    hdr = 4 * (ndim + 1) + 8 + 24
    return np.frombuffer(archive[hdr:hdr + 4 * npad], np.uint32)


def assert_same_padded_archive(got: bytes, want: bytes, ndim: int, pinned: np.ndarray):
    """Byte-equal packed blocks, except pad values the reference leaves unpinned."""
    assert len(got) == len(want)
    npad = pinned.size
    hdr = 4 * (ndim + 1) + 8 + 24
    assert got[:hdr] == want[:hdr]
    np.testing.assert_array_equal(pad_section(got, ndim, npad)[pinned], pad_section(want, ndim, npad)[pinned])
    assert got[hdr + 4 * npad:] == want[hdr + 4 * npad:]


@pytest.mark.parametrize("name", PAD_CASES)
def test_oracle_matches_golden_padded(name):
    g = load_golden(name)
    archive, meta = O.compress(g["x"], g["dims"], g["bs"], g["dict_size"], g["eb"], bool(g["r2r"]),
                               pad_mode=g["pad_mode"], pad_type=g["pad_type"], pad_const=g["pad_const"])
    assert_same_padded_archive(archive, g["archive"].tobytes(), len(g["dims"]), g["pad_pinned"])
    assert meta["n_outlier"] == g["n_outlier"]
    vr = O.value_range(g["x"]) if g["r2r"] else 0.0
    # the reference's own archive decodes to the reference's reconstruction
    xhat = O.decompress(g["archive"].tobytes(), g["bs"], g["dict_size"], vr)
    np.testing.assert_array_equal(xhat.view(np.uint32), g["xhat"].view(np.uint32))


def test_oracle_padding_corner_codes():
    """1D raw block pads: code 2R (one past the dictionary) and a quantizable code 0."""
    g = load_golden("p1_block_min_corner")
    code, outl, pads = O.dualquant_pad(g["x"], g["dims"], g["bs"], g["dict_size"], g["eb"], O.PAD_BLOCK,
                                       O.PADV_MIN)
    assert code[0] == g["dict_size"]               # residual 513 - 1.3 = 511.7 -> rint(1023.7) = 1024
    assert np.float32(pads[0]) == np.float32(1.3)  # raw block minimum, not prequantized
    code, outl, pads = O.dualquant_pad(g["x"], g["dims"], g["bs"], g["dict_size"], g["eb"], O.PAD_BLOCK,
                                       O.PADV_MAX)
    assert code[8] == 0 and outl[8] == 0.0         # residual -510 - 1.7 = -511.7 -> rint(0.3) = 0, quantizable


def test_oracle_pad_counts():
    # get_nblk = (d + bs + 1) // bs per axis; edge mode stores ndim values per block (1 in 1D)
    assert O.pad_count((16,), 8, O.PAD_BLOCK) == 3
    assert O.pad_count((14,), 8, O.PAD_BLOCK) == 2
    assert O.pad_count((16,), 8, O.PAD_EDGE) == 3
    assert O.pad_count((16, 17), 8, O.PAD_EDGE) == 2 * 3 * 3
    assert O.pad_count((8, 8, 8), 8, O.PAD_EDGE) == 3 * 8
    assert O.pad_count((100, 7, 3), 16, O.PAD_GLOBAL) == 1
    assert O.pad_count((100,), 16, O.PAD_NONE) == 0


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


ref_only = pytest.mark.skipif(not (O.ref_available() or
                                   os.path.isdir(os.path.join(os.environ.get("VSZ_REFERENCE_SRC", ""), "src"))),
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


@ref_only
@pytest.mark.parametrize("seed", range(8))
def test_oracle_matches_reference_padding(seed):
    """Padded archives and reconstructions against the reference itself (one OpenMP thread)."""
    if not O.ref_available():
        if O.build_ref() is None:
            pytest.skip("reference cannot be built on this machine")
    rng = np.random.default_rng(300 + seed)
    ndim = 1 + seed % 3
    bs = int(rng.choice([8, 16]))
    mode = 1 + seed % 3 if seed < 6 else int(rng.integers(1, 4))
    ptype = int(rng.integers(0, 4))
    whole = mode == 1 or ptype == 3 or ndim == 1
    if ndim == 1:
        dims = (int(rng.integers(50, 3000)),)
    elif ndim == 2:
        dims = (int(rng.integers(5, 120)), int(rng.integers(5, 90))) if whole else \
            (bs * int(rng.integers(1, 8)), bs * int(rng.integers(1, 6)))
    else:
        dims = tuple(int(rng.integers(3, 30)) for _ in range(3)) if whole else \
            tuple(bs * int(rng.integers(1, 4)) for _ in range(3))
    n = int(np.prod(dims))
    x = (np.cumsum(rng.standard_normal(n)) * 10 ** rng.uniform(-2, 1)).astype(np.float32)
    eb = float(10 ** rng.uniform(-5, -2))
    cst = float(rng.choice([0.0, 0.37, 12.5, -3.25]))
    r2r = bool(seed % 2)
    tmp = tempfile.mkdtemp()
    f = os.path.join(tmp, "f.f32")
    a_ref, nout = O.ref_compress_pad(x, dims, bs, 1024, eb, r2r, mode, ptype, cst, f)
    a_or, meta = O.compress(x, dims, bs, 1024, eb, r2r, pad_mode=mode, pad_type=ptype, pad_const=cst)
    assert_same_padded_archive(a_or, a_ref, ndim, O.ref_pinned_pads(dims, bs, mode, ptype))
    y_ref = O.ref_decompress(a_ref, len(a_ref), 0, n, bs, 1024, r2r, f)
    y_or = O.decompress(a_ref, bs, 1024, O.value_range(x) if r2r else 0.0)
    np.testing.assert_array_equal(y_or.view(np.uint32), y_ref.view(np.uint32))
