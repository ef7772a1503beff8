"""ctypes wrapper of the C oracle (oracle/vsz_oracle.c) and of the reference probe harness.

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as the checker and by
bench.py's CPU-baseline leg.  The product package (vecsz_gb300) never imports it.

Conventions follow the reference: ``dims = (d0, d1, d2)`` with d0 the fastest axis (x), arrays
flat in that order; ``dict_size`` is the reference's ``-d`` (radius = dict_size // 2);
``bs`` is the reference's ``-b`` block size.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libvszoracle.so")
REF_SO = os.path.join(HERE, "_ref", "libvszref.so")

_lib = None
_ref = None


def build(quiet: bool = True) -> str:
    """Compile the C oracle with its Makefile (gcc only; takes about a second)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return ORACLE_SO


def build_ref() -> str | None:
    """Compile the reference itself (x86-64 only) from the sources VSZ_REFERENCE_SRC points at."""
    ref_src = os.environ.get("VSZ_REFERENCE_SRC")
    if not ref_src or not os.path.isdir(os.path.join(ref_src, "src")):
        return None
    import platform

    if platform.machine() not in ("x86_64", "AMD64"):
        return None
    out = subprocess.run(["make", "-C", os.path.join(HERE, "ref"), f"REF={ref_src}", "-j8"],
                         capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference build failed:\n" + out.stdout[-4000:] + out.stderr[-4000:])
    return REF_SO


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(
                os.path.join(HERE, "vsz_oracle.c")):
            build()
        L = C.CDLL(ORACLE_SO)
        p, sz, d, i, u64p = C.c_void_p, C.c_size_t, C.c_double, C.c_int, C.POINTER(C.c_uint64)
        L.vso_value_range.argtypes = [p, sz]
        L.vso_value_range.restype = d
        L.vso_eb_family.argtypes = [d, p]
        L.vso_dualquant.argtypes = [p, i, sz, sz, sz, i, i, d, p, p]
        L.vso_gather_outliers.argtypes = [p, p, sz, p]
        L.vso_gather_outliers.restype = sz
        L.vso_scatter_outliers.argtypes = [p, p, sz, p]
        L.vso_scatter_outliers.restype = sz
        L.vso_xlorenzo.argtypes = [p, p, i, sz, sz, sz, i, i, d, p]
        L.vso_huffman_codebook.argtypes = [p, i, p, p, p, p]
        L.vso_huffman_bound.argtypes = [sz, i]
        L.vso_huffman_bound.restype = sz
        L.vso_huffman_encode.argtypes = [p, sz, i, p, sz, p]
        L.vso_huffman_decode.argtypes = [p, sz, sz, p]
        L.vso_compress_bound.argtypes = [i, sz, i]
        L.vso_compress_bound.restype = sz
        L.vso_compress.argtypes = [p, i, p, i, i, d, i, p, sz, p, p, p, p]
        L.vso_compress_pad.argtypes = [p, i, p, i, i, d, i, i, i, C.c_float, p, sz, p, p, p, p]
        L.vso_compress_bound_pad.argtypes = [i, p, i, i, i]
        L.vso_compress_bound_pad.restype = sz
        L.vso_pad_count.argtypes = [i, sz, sz, sz, i, i]
        L.vso_pad_count.restype = sz
        L.vso_pad_values.argtypes = [p, i, sz, sz, sz, i, i, i, C.c_float, d, p, p]
        L.vso_dualquant_pad.argtypes = [p, i, sz, sz, sz, i, i, d, i, i, C.c_float, p, p, p]
        L.vso_xlorenzo_pad.argtypes = [p, p, i, sz, sz, sz, i, i, d, p, sz, p]
        L.vso_decompress.argtypes = [p, sz, i, i, d, p, sz, p]
        L.vso_parse_header.argtypes = [p, sz, p, p, p, p]
        L.vso_tree_bytes_size.argtypes = [C.c_uint32]
        L.vso_tree_bytes_size.restype = sz
        L.vso_num_threads.restype = i
        _lib = L
    return _lib


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def _dims3(dims):
    d = list(dims) + [1] * (3 - len(dims))
    return int(d[0]), int(d[1]), int(d[2])


class OracleError(RuntimeError):
    pass


def _check(rc, what):
    if rc != 0:
        raise OracleError(f"{what} failed with status {rc}")


def value_range(x: np.ndarray) -> float:
    x = np.ascontiguousarray(x, dtype=np.float32).ravel()
    return lib().vso_value_range(_ptr(x), x.size)


def eb_family(eb_final: float) -> np.ndarray:
    out = np.zeros(4, np.float64)
    lib().vso_eb_family(eb_final, _ptr(out))
    return out


def dualquant(x: np.ndarray, dims, bs: int, dict_size: int, eb_final: float):
    """Dense int32 codes and dense outlier values, as c_lorenzo_*d1l leaves them."""
    x = np.ascontiguousarray(x, dtype=np.float32).ravel()
    d0, d1, d2 = _dims3(dims)
    n = d0 * d1 * d2
    code = np.zeros(n, np.int32)
    outl = np.zeros(n, np.float32)
    ebs = eb_family(eb_final)
    _check(lib().vso_dualquant(_ptr(x), len(dims), d0, d1, d2, bs, dict_size // 2, float(ebs[3]),
                               _ptr(code), _ptr(outl)), "dualquant")
    return code, outl


# Padding (-p): modes and value types as the reference numbers them (src/utils/padding.hh:9-12).
PAD_NONE, PAD_GLOBAL, PAD_BLOCK, PAD_EDGE = 0, 1, 2, 3
PADV_MAX, PADV_MIN, PADV_AVG, PADV_CONST = 0, 1, 2, 3


def pad_count(dims, bs: int, pad_mode: int) -> int:
    d0, d1, d2 = _dims3(dims)
    return lib().vso_pad_count(len(dims), d0, d1, d2, bs, pad_mode)


def pad_values(x: np.ndarray, dims, bs: int, eb_final: float, pad_mode: int, pad_type: int,
               pad_const: float = 0.0):
    """(archive pad values, value the compressor predicts from in global mode)."""
    x = np.ascontiguousarray(x, dtype=np.float32).ravel()
    d0, d1, d2 = _dims3(dims)
    out = np.zeros(max(1, pad_count(dims, bs, pad_mode)), np.float32)
    hg = C.c_float(0)
    ebs = eb_family(eb_final)
    _check(lib().vso_pad_values(_ptr(x), len(dims), d0, d1, d2, bs, pad_mode, pad_type, C.c_float(pad_const),
                                float(ebs[3]), _ptr(out), C.byref(hg)), "pad_values")
    return out[:pad_count(dims, bs, pad_mode)], hg.value


def dualquant_pad(x: np.ndarray, dims, bs: int, dict_size: int, eb_final: float, pad_mode: int, pad_type: int,
                  pad_const: float = 0.0):
    """Dense codes, dense outliers and the pad section, with -p padding."""
    x = np.ascontiguousarray(x, dtype=np.float32).ravel()
    d0, d1, d2 = _dims3(dims)
    n = d0 * d1 * d2
    code = np.zeros(n, np.int32)
    outl = np.zeros(n, np.float32)
    pads = np.zeros(max(1, pad_count(dims, bs, pad_mode)), np.float32)
    ebs = eb_family(eb_final)
    _check(lib().vso_dualquant_pad(_ptr(x), len(dims), d0, d1, d2, bs, dict_size // 2, float(ebs[3]), pad_mode,
                                   pad_type, C.c_float(pad_const), _ptr(code), _ptr(outl), _ptr(pads)),
           "dualquant_pad")
    return code, outl, pads[:pad_count(dims, bs, pad_mode)]


def ref_pinned_pads(dims, bs: int, pad_mode: int, pad_type: int) -> np.ndarray:
    """Which pad values of an archive the reference computes deterministically: all of them in 1D
    (its input is handed over zero-extended), for global mode and for constants; in 2D/3D
    block/edge max/min/avg only those of blocks wholly inside the field -- for the others it
    reads an uninitialised buffer (src/utils/padding.hh:18-36, fill_*_block)."""
    nd = len(dims)
    d = list(dims) + [1] * (3 - nd)
    nb = [(v + bs + 1) // bs for v in d]
    if pad_mode == PAD_GLOBAL:
        return np.ones(1, bool)
    per = nd if (pad_mode == PAD_EDGE and nd > 1) else 1
    out = []
    for b2 in range(nb[2]):
        for b1 in range(nb[1]):
            for b0 in range(nb[0]):
                inside = all((b + 1) * bs <= v for b, v in zip((b0, b1, b2)[:nd], d[:nd]))
                out += [nd == 1 or pad_type == PADV_CONST or inside] * per
    return np.array(out, bool)


def gather_outliers(code: np.ndarray, outlier_dense: np.ndarray) -> np.ndarray:
    code = np.ascontiguousarray(code, np.int32)
    outlier_dense = np.ascontiguousarray(outlier_dense, np.float32)
    out = np.zeros(max(1, int((code == 0).sum())), np.float32)
    k = lib().vso_gather_outliers(_ptr(code), _ptr(outlier_dense), code.size, _ptr(out))
    return out[:k]


def scatter_outliers(code: np.ndarray, outliers: np.ndarray) -> np.ndarray:
    code = np.ascontiguousarray(code, np.int32)
    outliers = np.ascontiguousarray(outliers, np.float32)
    dense = np.zeros(code.size, np.float32)
    lib().vso_scatter_outliers(_ptr(code), _ptr(outliers), code.size, _ptr(dense))
    return dense


def xlorenzo(code: np.ndarray, outlier_dense: np.ndarray, dims, bs: int, dict_size: int, eb_final: float,
             pads: np.ndarray | None = None):
    code = np.ascontiguousarray(code, np.int32).ravel()
    outlier_dense = np.ascontiguousarray(outlier_dense, np.float32).ravel()
    d0, d1, d2 = _dims3(dims)
    xhat = np.zeros(d0 * d1 * d2, np.float32)
    ebs = eb_family(eb_final)
    npad = 0 if pads is None else int(np.asarray(pads).size)
    pads = np.zeros(1, np.float32) if npad == 0 else np.ascontiguousarray(pads, np.float32).ravel()
    _check(lib().vso_xlorenzo_pad(_ptr(code), _ptr(outlier_dense), len(dims), d0, d1, d2, bs, dict_size // 2,
                                  float(ebs[2]), _ptr(pads), npad, _ptr(xhat)), "xlorenzo")
    return xhat


def histogram(code: np.ndarray, dict_size: int) -> np.ndarray:
    return np.bincount(np.asarray(code, np.int64).ravel(), minlength=dict_size).astype(np.uint64)[:dict_size]


def huffman_codebook(hist: np.ndarray, dict_size: int):
    """(lengths u8[dict], first word u64[dict], second word u64[dict], node_count)."""
    hist = np.ascontiguousarray(hist, np.uint64)
    lens = np.zeros(dict_size, np.uint8)
    w0 = np.zeros(dict_size, np.uint64)
    w1 = np.zeros(dict_size, np.uint64)
    nc = C.c_uint32(0)
    _check(lib().vso_huffman_codebook(_ptr(hist), dict_size, _ptr(lens), _ptr(w0), _ptr(w1), C.byref(nc)),
           "huffman_codebook")
    return lens, w0, w1, nc.value


def huffman_encode(code: np.ndarray, dict_size: int) -> bytes:
    code = np.ascontiguousarray(code, np.int32).ravel()
    cap = lib().vso_huffman_bound(code.size, dict_size)
    out = np.zeros(cap, np.uint8)
    sz = C.c_size_t(0)
    _check(lib().vso_huffman_encode(_ptr(code), code.size, dict_size, _ptr(out), cap, C.byref(sz)),
           "huffman_encode")
    return out[:sz.value].tobytes()


def huffman_decode(buf: bytes, n: int) -> np.ndarray:
    a = np.frombuffer(buf, np.uint8).copy()
    out = np.zeros(n, np.int32)
    _check(lib().vso_huffman_decode(_ptr(a), a.size, n, _ptr(out)), "huffman_decode")
    return out


def compress(x: np.ndarray, dims, bs: int = 8, dict_size: int = 1024, eb: float = 1e-4, r2r: bool = False,
             timings: np.ndarray | None = None, pad_mode: int = PAD_NONE, pad_type: int = PADV_CONST,
             pad_const: float = 0.0):
    """Packed block bytes (the reference's Compress output without -L), plus metadata dict."""
    x = np.ascontiguousarray(x, dtype=np.float32).ravel()
    ndim = len(dims)
    d = np.array(list(dims) + [1] * (3 - ndim), np.uint64)
    cap = lib().vso_compress_bound_pad(ndim, _ptr(d), bs, dict_size, pad_mode)
    out = np.zeros(cap, np.uint8)
    sz, nout, ebf = C.c_size_t(0), C.c_size_t(0), C.c_double(0)
    tp = _ptr(timings) if timings is not None else None
    _check(lib().vso_compress_pad(_ptr(x), ndim, _ptr(d), bs, dict_size, eb, int(r2r), pad_mode, pad_type,
                                  C.c_float(pad_const), _ptr(out), cap, C.byref(sz), C.byref(nout), C.byref(ebf),
                                  tp), "compress")
    return out[:sz.value].tobytes(), {"n_outlier": nout.value, "eb_final": ebf.value}


def decompress(buf: bytes, bs: int = 8, dict_size: int = 1024, value_range_: float = 0.0,
               timings: np.ndarray | None = None) -> np.ndarray:
    a = np.frombuffer(buf, np.uint8).copy()
    hdr = parse_header(buf)
    n = int(np.prod(hdr["dims"]))
    out = np.zeros(n, np.float32)
    tp = _ptr(timings) if timings is not None else None
    _check(lib().vso_decompress(_ptr(a), a.size, bs, dict_size, float(value_range_), _ptr(out), n, tp),
           "decompress")
    return out


def parse_header(buf: bytes) -> dict:
    a = np.frombuffer(buf, np.uint8).copy()
    nd = C.c_int(0)
    dims = np.zeros(3, np.uint64)
    eb = C.c_double(0)
    lens = np.zeros(3, np.uint64)
    _check(lib().vso_parse_header(_ptr(a), a.size, C.byref(nd), _ptr(dims), C.byref(eb), _ptr(lens)),
           "parse_header")
    return {"ndim": nd.value, "dims": tuple(int(v) for v in dims[:nd.value]), "eb": eb.value,
            "lens": tuple(int(v) for v in lens)}


def num_threads() -> int:
    return lib().vso_num_threads()


# ----------------------------------------------------------------------------------------------
# The reference itself (oracle/_ref/libvszref.so), where it could be built
# ----------------------------------------------------------------------------------------------

def ref_available() -> bool:
    return os.path.exists(REF_SO)


def ref():
    global _ref
    if _ref is None:
        L = C.CDLL(REF_SO)
        p, sz, d, i = C.c_void_p, C.c_size_t, C.c_double, C.c_int
        L.vszref_dualquant.argtypes = [p, i, i, i, i, i, i, d, p, p]
        L.vszref_huffman_encode.argtypes = [p, sz, i, p, p]
        L.vszref_huffman_codebook.argtypes = [p, sz, i, p, p, p]
        L.vszref_huffman_decode.argtypes = [p, sz, i, p]
        L.vszref_xlorenzo.argtypes = [p, p, i, i, i, i, i, i, d, p]
        L.vszref_compress.argtypes = [p, i, i, i, i, i, i, d, i, i, C.c_char_p, p, p, p, p]
        L.vszref_compress_pad.argtypes = [p, i, i, i, i, i, i, d, i, i, i, C.c_float, C.c_char_p, p, p, p]
        L.vszref_decompress.argtypes = [p, sz, sz, i, i, i, C.c_char_p, p, sz]
        L.vszref_free.argtypes = [p]
        _ref = L
    return _ref


def ref_dualquant(x, dims, bs, dict_size, eb_final):
    x = np.ascontiguousarray(x, dtype=np.float32).ravel()
    d0, d1, d2 = _dims3(dims)
    n = d0 * d1 * d2
    code = np.zeros(n, np.int32)
    outl = np.zeros(n, np.float32)
    ref().vszref_dualquant(_ptr(x), len(dims), d0, d1, d2, bs, dict_size, eb_final, _ptr(code), _ptr(outl))
    return code, outl


def ref_huffman_encode(code, dict_size) -> bytes:
    code = np.ascontiguousarray(code, np.int32).ravel()
    outp = C.c_void_p(0)
    sz = C.c_size_t(0)
    ref().vszref_huffman_encode(_ptr(code), code.size, dict_size, C.byref(outp), C.byref(sz))
    data = C.string_at(outp.value, sz.value)
    ref().vszref_free(outp)
    return data


def ref_huffman_codebook(code, dict_size):
    code = np.ascontiguousarray(code, np.int32).ravel()
    lens = np.zeros(dict_size, np.uint8)
    w0 = np.zeros(dict_size, np.uint64)
    w1 = np.zeros(dict_size, np.uint64)
    ref().vszref_huffman_codebook(_ptr(code), code.size, dict_size, _ptr(lens), _ptr(w0), _ptr(w1))
    return lens, w0, w1


def ref_huffman_decode(buf: bytes, n: int, dict_size: int) -> np.ndarray:
    a = np.frombuffer(buf, np.uint8).copy()
    out = np.zeros(n, np.int32)
    ref().vszref_huffman_decode(_ptr(a), n, dict_size, _ptr(out))
    return out


def ref_xlorenzo(code, outlier_dense, dims, bs, dict_size, eb_final):
    code = np.ascontiguousarray(code, np.int32).ravel()
    outlier_dense = np.ascontiguousarray(outlier_dense, np.float32).ravel()
    d0, d1, d2 = _dims3(dims)
    xhat = np.zeros(d0 * d1 * d2, np.float32)
    ref().vszref_xlorenzo(_ptr(code), _ptr(outlier_dense), len(dims), d0, d1, d2, bs, dict_size, eb_final,
                          _ptr(xhat))
    return xhat


def ref_compress(x, dims, bs, dict_size, eb, r2r, lossless, tmpfile):
    x = np.ascontiguousarray(x, dtype=np.float32).ravel()
    d0, d1, d2 = _dims3(dims)
    outp = C.c_void_p(0)
    dsz, lsz, nout = C.c_size_t(0), C.c_size_t(0), C.c_size_t(0)
    ref().vszref_compress(_ptr(x), len(dims), d0, d1, d2, bs, dict_size, eb, int(r2r), int(lossless),
                          tmpfile.encode(), C.byref(outp), C.byref(dsz), C.byref(lsz), C.byref(nout))
    nbytes = lsz.value if lossless else dsz.value
    data = C.string_at(outp.value, nbytes)
    ref().vszref_free(outp)
    return data, dsz.value, lsz.value, nout.value


def ref_compress_pad(x, dims, bs, dict_size, eb, r2r, pad_mode, pad_type, pad_const, tmpfile):
    """The reference's Compress with -p (one OpenMP thread); (packed block, n_outlier)."""
    x = np.ascontiguousarray(x, dtype=np.float32).ravel()
    d0, d1, d2 = _dims3(dims)
    outp = C.c_void_p(0)
    dsz, nout = C.c_size_t(0), C.c_size_t(0)
    ref().vszref_compress_pad(_ptr(x), len(dims), d0, d1, d2, bs, dict_size, eb, int(r2r), pad_mode, pad_type,
                              C.c_float(pad_const), tmpfile.encode(), C.byref(outp), C.byref(dsz), C.byref(nout))
    data = C.string_at(outp.value, dsz.value)
    ref().vszref_free(outp)
    return data, nout.value


def ref_decompress(buf: bytes, data_size: int, lossless_size: int, n: int, bs, dict_size, r2r=False,
                   orig_file=None):
    a = np.frombuffer(buf, np.uint8).copy()
    out = np.zeros(n, np.float32)
    ref().vszref_decompress(_ptr(a), data_size, lossless_size, bs, dict_size, int(r2r),
                            orig_file.encode() if orig_file else None, _ptr(out), n)
    return out
