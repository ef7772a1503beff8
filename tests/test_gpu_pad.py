"""Padding (-p) on the GPU, through the C ABI: packed blocks byte-identical to the reference's
(golden fixtures; pad values the reference leaves undefined excepted) and to the oracle's (all
bytes), reconstructions bit-identical, over every mode, value type, dimensionality and block size."""
import numpy as np
import pytest

import oracle as O
import vecsz_gb300 as V
from vecsz_gb300 import api, fields
from conftest import load_golden, pad_golden_cases

pytestmark = pytest.mark.gpu
PAD_CASES = pad_golden_cases()
MODES = {O.PAD_GLOBAL: "global", O.PAD_BLOCK: "block", O.PAD_EDGE: "edge"}
TYPES = {O.PADV_MAX: "max", O.PADV_MIN: "min", O.PADV_AVG: "avg", O.PADV_CONST: "constant"}


def padding_of(mode, ptype, cst):
    return (MODES[mode], TYPES[ptype], cst)


def masked_equal(got: bytes, want: bytes, ndim: int, pinned: np.ndarray):
    assert len(got) == len(want)
    hdr = 4 * (ndim + 1) + 8 + 24
    npad = pinned.size
    assert got[:hdr] == want[:hdr]
    pg = np.frombuffer(got[hdr:hdr + 4 * npad], np.uint32)
    pw = np.frombuffer(want[hdr:hdr + 4 * npad], np.uint32)
    np.testing.assert_array_equal(pg[pinned], pw[pinned])
    assert got[hdr + 4 * npad:] == want[hdr + 4 * npad:]


def gpu_compress(x, dims, bs, dct, eb, r2r, padding):
    c = V.compress(x, dims, eb=eb, mode="r2r" if r2r else "abs", dict_size=dct, block_size=bs, padding=padding)
    return c, c.data[:c.data_size]


@pytest.mark.parametrize("name", PAD_CASES)
def test_padded_archive_matches_reference(cuda, name):
    g = load_golden(name)
    pad = padding_of(g["pad_mode"], g["pad_type"], g["pad_const"])
    c, block = gpu_compress(g["x"], g["dims"], g["bs"], g["dict_size"], g["eb"], bool(g["r2r"]), pad)
    masked_equal(block, g["archive"].tobytes(), len(g["dims"]), g["pad_pinned"])
    assert c.n_outlier == g["n_outlier"]
    # every byte, the undefined pad values included, equals the oracle's (zero outside the field)
    oa, _ = O.compress(g["x"], g["dims"], g["bs"], g["dict_size"], g["eb"], bool(g["r2r"]), pad_mode=g["pad_mode"],
                       pad_type=g["pad_type"], pad_const=g["pad_const"])
    assert block == oa
    vr = O.value_range(g["x"]) if g["r2r"] else 0.0
    mode = "r2r" if g["r2r"] else "abs"
    # our archive (trailer: indexed decode) and the reference's (no trailer: self-synchronising)
    y = V.decompress(c)
    np.testing.assert_array_equal(y.view(np.uint32), g["xhat"].view(np.uint32))
    y = V.decompress(g["archive"].tobytes(), g["archive"].size, 0, g["dict_size"], g["bs"], mode, vr)
    np.testing.assert_array_equal(y.view(np.uint32), g["xhat"].view(np.uint32))


def random_field(rng, dims):
    n = int(np.prod(dims))
    if len(dims) == 1 or rng.random() < 0.4:
        return (np.cumsum(rng.standard_normal(n)) * 10 ** rng.uniform(-2, 1)).astype(np.float32)
    if len(dims) == 2:
        return fields.bump_field_2d(dims[1], dims[0], seed=int(rng.integers(1 << 30))).ravel()
    return fields.grf_3d(dims[2], dims[1], dims[0], seed=int(rng.integers(1 << 30))).ravel()


@pytest.mark.parametrize("ndim", [1, 2, 3])
@pytest.mark.parametrize("mode", [O.PAD_GLOBAL, O.PAD_BLOCK, O.PAD_EDGE])
def test_padded_random_against_oracle(cuda, ndim, mode):
    rng = np.random.default_rng(1000 * ndim + mode)
    for trial in range(8):
        ptype = trial % 4
        bs = (8, 16, 32, 64)[(trial // 2) % 4] if trial < 6 else 8
        if ndim == 1:
            dims = (int(rng.integers(100, 20000)),)
        elif ndim == 2:
            dims = (int(rng.integers(5, 300)), int(rng.integers(5, 200)))
        else:
            dims = tuple(int(rng.integers(3, 48)) for _ in range(3))
        x = random_field(rng, dims)
        eb = float(10 ** rng.uniform(-5, -2))
        cst = float(rng.choice([0.0, 0.37, 12.5, -3.25]))
        r2r = bool(trial % 3 == 1)
        dct = 1024 if ndim > 1 or trial % 2 else 4096
        pad = padding_of(mode, ptype, cst)
        c, block = gpu_compress(x, dims, bs, dct, eb, r2r, pad)
        oa, meta = O.compress(x, dims, bs, dct, eb, r2r, pad_mode=mode, pad_type=ptype, pad_const=cst)
        assert block == oa, (dims, bs, mode, ptype, eb, r2r)
        vr = O.value_range(x) if r2r else 0.0
        want = O.decompress(oa, bs, dct, vr)
        y = V.decompress(c)
        np.testing.assert_array_equal(y.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("mode", [O.PAD_BLOCK, O.PAD_EDGE, O.PAD_GLOBAL])
def test_padded_general_decompress_kernel(cuda, mode, monkeypatch):
    """Block size 8 through the general reverse-Lorenzo kernel as well."""
    monkeypatch.setenv("VSZ_FORCE_GENERAL_DECOMPRESS", "1")
    rng = np.random.default_rng(77 + mode)
    for dims in [(777,), (130, 70), (40, 33, 21)]:
        x = random_field(rng, dims)
        pad = padding_of(mode, O.PADV_AVG, 0.0)
        c, block = gpu_compress(x, dims, 8, 1024, 1e-3, False, pad)
        oa, _ = O.compress(x, dims, 8, 1024, 1e-3, False, pad_mode=mode, pad_type=O.PADV_AVG)
        assert block == oa
        y = V.decompress(c)
        np.testing.assert_array_equal(y.view(np.uint32), O.decompress(oa, 8, 1024).view(np.uint32))


def test_padded_device_tree_builder(cuda):
    """1D raw block pads give the extra symbol 2R; the device tree builder takes it too."""
    from vecsz_gb300 import _lib as L
    g = load_golden("p1_block_min_corner")
    prev = L.lib().vsz_set_tree_builder(L.TREE_DEVICE)
    try:
        c, block = gpu_compress(g["x"], g["dims"], g["bs"], g["dict_size"], g["eb"], False,
                                padding_of(g["pad_mode"], g["pad_type"], 0.0))
    finally:
        L.lib().vsz_set_tree_builder(prev)
    assert block == g["archive"].tobytes()
    np.testing.assert_array_equal(V.decompress(c).view(np.uint32), g["xhat"].view(np.uint32))


@pytest.mark.parametrize("padding", ["global,avg", "global,max", "block,min", "edge,avg"])
def test_padded_large_3d_roundtrip(cuda, padding):
    """A 192^3 field (bigger than L2) against the oracle."""
    x = fields.grf_3d(192, 192, 192, seed=5).ravel()
    dims = (192, 192, 192)
    p = api.make_params(block_size=8, padding=padding)
    c, block = gpu_compress(x, dims, 8, 1024, 1e-4, False, padding)
    oa, _ = O.compress(x, dims, 8, 1024, 1e-4, False, pad_mode=p.pad_mode, pad_type=p.pad_type,
                       pad_const=p.pad_constant)
    assert block == oa
    y = V.decompress(c)
    np.testing.assert_array_equal(y.view(np.uint32), O.decompress(oa, 8, 1024).view(np.uint32))


def test_padded_global_extremes_first_zero_and_nan(cuda):
    """Global max/min follow the reference's first-wins scan: the sign of the first zero, a
    leading NaN."""
    for x0, mode_type in [(-0.0, "global,max"), (0.0, "global,min")]:
        x = np.full(5000, -1.0 if mode_type.endswith("max") else 1.0, np.float32)
        x[17] = x0
        x[900] = -x0
        c, block = gpu_compress(x, (5000,), 8, 1024, 1e-3, False, mode_type)
        p = api.make_params(padding=mode_type)
        oa, _ = O.compress(x, (5000,), 8, 1024, 1e-3, False, pad_mode=p.pad_mode, pad_type=p.pad_type)
        assert block == oa
    x = fields.bump_field_2d(40, 64, seed=3).ravel().copy()
    x[0] = np.nan
    c, block = gpu_compress(x, (64, 40), 8, 1024, 1e-3, False, "global,max")
    oa, _ = O.compress(x, (64, 40), 8, 1024, 1e-3, False, pad_mode=O.PAD_GLOBAL, pad_type=O.PADV_MAX)
    assert block == oa
