"""The f64 path (vsz_compress_f64 / vsz_decompress_f64, the command line's -t f64).

The reference parses -t f64 but reads its input as float and has no double-precision dual-quant
code, so there is no reference arithmetic to pin.  What the path promises is checked instead, in
double precision: every reconstructed value lies within the absolute error bound of its input
(eb, or eb times the value range in r2r mode), outliers -- NaN, infinities and values too large to
quantize included -- come back bit for bit, the archive is deterministic, and the f32 and f64
entry points refuse each other's archives."""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import vecsz_gb300 as V
from vecsz_gb300 import _lib as L
from vecsz_gb300 import fields

pytestmark = pytest.mark.gpu


def _bound(x, eb, mode):
    if mode == "abs":
        return eb
    fin = x[np.isfinite(x)]
    return eb * (float(fin.max()) - float(fin.min()))


def _check(x, y, ebf):
    assert y.dtype == np.float64 and y.shape == x.shape
    fin = np.isfinite(x)
    err = np.abs(x[fin] - y[fin])
    assert err.max() <= ebf, (float(err.max()), ebf)
    # non-finite inputs are outliers: stored and returned as they were
    assert np.array_equal(x[~fin].view(np.uint64), y[~fin].view(np.uint64))


def _smooth(dims, seed):
    if len(dims) == 1:
        rng = np.random.default_rng(seed)
        return np.cumsum(rng.standard_normal(dims[0])) * 0.37 + 1.0e3
    if len(dims) == 2:
        return fields.bump_field_2d(dims[1], dims[0], seed=seed).astype(np.float64).ravel() * 1.0e4
    g = fields.grf_3d(dims[2], dims[1], dims[0], seed=seed).astype(np.float64)
    return (g * np.pi + 1.0e-3 * g * g).ravel()  # full double mantissas: not representable in f32 as is


@pytest.mark.parametrize("dims", [(100003,), (257, 131), (70, 33, 21), (64, 64, 32)])
@pytest.mark.parametrize("bs", [8, 16, 32, 64])
@pytest.mark.parametrize("mode,eb", [("abs", 1e-3), ("r2r", 1e-6), ("r2r", 1e-11)])
def test_f64_roundtrip_within_bound(cuda, dims, bs, mode, eb):
    x = _smooth(dims, seed=sum(dims) + bs)
    c = V.compress(x, dims, eb=eb, mode=mode, dict_size=1024, block_size=bs, dtype="f64")
    d = V.parse_archive(c.data)
    assert d.has_trailer and d.f64 and d.n_outlier == c.n_outlier
    y = V.decompress(c)
    _check(x, y, _bound(x, eb, mode))
    # an error bound far below f32's resolution: the reconstruction is still within it
    if eb < 1e-9:
        assert np.abs(x - y).max() < np.abs(x - x.astype(np.float32)).max()
    c2 = V.compress(x, dims, eb=eb, mode=mode, dict_size=1024, block_size=bs, dtype="f64")
    assert c2.data == c.data


def test_f64_special_values_are_outliers(cuda):
    rng = np.random.default_rng(5)
    dims = (40, 30, 20)
    x = np.cumsum(rng.standard_normal(np.prod(dims))) * 0.01
    bits = x.view(np.uint64)
    idx = rng.choice(x.size, 40, replace=False)
    bits[idx[:8]] = 0x7ff8000000001234     # quiet NaN with a payload
    bits[idx[8:16]] = 0xfff0000000000000   # -inf
    bits[idx[16:24]] = 0x7ff0000000000000  # +inf
    x[idx[24:32]] = 1.0e300                # far beyond 2^59 quanta
    x[idx[32:40]] = 5e-324                 # subnormal: quantized to 0, within the bound
    c = V.compress(x, dims, eb=1e-4, mode="abs", dict_size=256, block_size=8, dtype="f64")
    assert c.n_outlier >= 32
    y = V.decompress(c)
    _check(x, y, 1e-4)
    assert np.array_equal(x[idx[:32]].view(np.uint64), y[idx[:32]].view(np.uint64))


def test_f64_lossless_and_dictionaries(cuda):
    x = _smooth((96, 80, 40), seed=7)
    for dct, lossless in ((256, "zstd"), (4096, "gzip"), (65536, None)):
        c = V.compress(x, (96, 80, 40), eb=1e-5, mode="r2r", dict_size=dct, block_size=8, lossless=lossless,
                       dtype="f64")
        if lossless:
            assert c.lossless_size > 0
        _check(x, V.decompress(c), _bound(x, 1e-5, "r2r"))


def test_f32_and_f64_refuse_each_others_archives(cuda):
    x = _smooth((64, 48), seed=3)
    c64 = V.compress(x, (64, 48), eb=1e-4, mode="abs", dict_size=1024, block_size=8, dtype="f64")
    c32 = V.compress(x.astype(np.float32), (64, 48), eb=1e-4, mode="abs", dict_size=1024, block_size=8)
    lib = L.lib()
    a = np.frombuffer(c64.data, np.uint8)
    out, n = C.c_void_p(0), C.c_size_t(0)
    o = L.DecompressOpts(1024, 8, 0, 0.0)
    assert lib.vsz_decompress_host(a.ctypes.data_as(C.c_void_p), a.size, c64.data_size, 0, C.byref(o), C.byref(out),
                                   C.byref(n)) == L.VSZ_ERR_UNSUPPORTED
    b = np.frombuffer(c32.data, np.uint8)
    assert lib.vsz_decompress_host_f64(b.ctypes.data_as(C.c_void_p), b.size, c32.data_size, 0, C.byref(out),
                                       C.byref(n)) == L.VSZ_ERR_UNSUPPORTED
    with pytest.raises(L.VszError) as e:
        V.BatchDecompressor([c64.data])
    assert e.value.status == L.VSZ_ERR_UNSUPPORTED
    # padding keeps the reference's f32 pad section: refused on the f64 path
    with pytest.raises(L.VszError) as e:
        V.compress(x, (64, 48), eb=1e-4, mode="abs", dict_size=1024, block_size=8, padding="block,avg", dtype="f64")
    assert e.value.status == L.VSZ_ERR_UNSUPPORTED


def test_cli_f64_roundtrip(cuda, tmp_path):
    from vecsz_gb300 import _build
    cli = _build.build_cli()
    x = _smooth((50, 40, 30), seed=9)
    src = tmp_path / "field.f64"
    x.tofile(src)
    r = subprocess.run([cli, "-z", "-i", str(src), "-t", "f64", "-m", "abs", "-e", "1e-7", "-l", "50,40,30",
                        "-d", "1024", "-b", "16", "-L", "zstd"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([cli, "-x", "-i", str(src) + ".sz", "-d", "1024", "-b", "16"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    y = np.fromfile(str(src) + ".sz.out" if os.path.exists(str(src) + ".sz.out") else str(src) + ".out", np.float64)
    _check(x, y, 1e-7)
