"""ctypes binding of libvecsz_gb300.so (the C ABI in include/vecsz_gb300.h).

There is no fallback: if the shared library is missing or cannot load, every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import _build

VSZ_OK = 0
VSZ_ERR_INVALID = 1
VSZ_ERR_CUDA = 2
VSZ_ERR_CORRUPT = 3
VSZ_ERR_CAPACITY = 4
VSZ_ERR_TIMEOUT = 5
VSZ_ERR_UNSUPPORTED = 6
VSZ_ERR_RANGE = 7
VSZ_ERR_NOMEM = 8
VSZ_ERR_NO_DEVICE = 9
VSZ_ERR_CANCELLED = 10

MODE_ABS = 0
MODE_R2R = 1
FLAG_STRICT_EB = 1

# -p padding (include/vecsz_gb300.h VSZ_PAD_*, VSZ_PADV_*)
PAD_NONE, PAD_GLOBAL, PAD_BLOCK, PAD_EDGE = 0, 1, 2, 3
PADV_MAX, PADV_MIN, PADV_AVG, PADV_CONST = 0, 1, 2, 3

TREE_DEVICE = 1
TREE_HOST = 2
LOSSLESS_NONE = 0
LOSSLESS_ZSTD = 1
LOSSLESS_GZIP = 2
LOSSLESS_GZIP_DEVICE = 3
CONSTS_BYTES = 64


class VszError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = lib().vsz_status_string(status).decode() if _LIB is not None else str(status)
        super().__init__(f"{what}: {msg} (status {status})" if what else f"{msg} (status {status})")


class Params(C.Structure):
    _fields_ = [("eb", C.c_double), ("mode", C.c_int), ("dict_size", C.c_int), ("block_size", C.c_int),
                ("lossless", C.c_int), ("flags", C.c_int), ("pad_mode", C.c_int), ("pad_type", C.c_int),
                ("pad_constant", C.c_float)]


class BatchField(C.Structure):
    _fields_ = [("d_in", C.c_void_p), ("ndim", C.c_int), ("dims", C.c_size_t * 3), ("params", Params),
                ("d_archive", C.c_void_p), ("archive_capacity", C.c_size_t)]


class Result(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("data_size", "trailer_size", "n_outlier", "huff_bytes", "payload_bits",
                                          "status", "max_code_len", "node_count")]


class ArchiveDesc(C.Structure):
    _fields_ = [("ndim", C.c_int), ("dims", C.c_uint64 * 3), ("eb", C.c_double), ("n_pad", C.c_uint64),
                ("huff_bytes", C.c_uint64), ("n_outlier", C.c_uint64), ("header_bytes", C.c_uint64),
                ("huff_offset", C.c_uint64), ("node_count", C.c_uint32), ("tree_bytes", C.c_uint64),
                ("payload_offset", C.c_uint64), ("payload_bytes", C.c_uint64), ("outlier_offset", C.c_uint64),
                ("data_size", C.c_uint64), ("has_trailer", C.c_int), ("eb_final", C.c_double),
                ("value_range", C.c_double), ("mode", C.c_int), ("dict_size", C.c_int), ("block_size", C.c_int),
                ("chunk_syms", C.c_uint32), ("n_chunks", C.c_uint64), ("index_offset", C.c_uint64),
                ("trailer_size", C.c_uint64), ("strict", C.c_int), ("f64", C.c_int)]


class TuneResult(C.Structure):
    _fields_ = [("block_size", C.c_int), ("cached", C.c_int), ("sample_elements", C.c_uint64),
                ("compress_ms", C.c_double * 4), ("decompress_ms", C.c_double * 4),
                ("archive_bytes", C.c_uint64 * 4), ("score_ms", C.c_double * 4)]


class DBatchField(C.Structure):
    _fields_ = [("d_archive", C.c_void_p), ("desc", ArchiveDesc), ("d_out", C.c_void_p)]


class DecompressOpts(C.Structure):
    _fields_ = [("dict_size", C.c_int), ("block_size", C.c_int), ("mode", C.c_int), ("value_range", C.c_double)]


class Request(C.Structure):
    _fields_ = [("kind", C.c_int), ("d_in", C.c_void_p), ("ndim", C.c_int), ("dims", C.c_size_t * 3),
                ("params", Params), ("desc", ArchiveDesc), ("opts", DecompressOpts)]


class Completion(C.Structure):
    _fields_ = [("status", C.c_int), ("d_out", C.c_void_p), ("out_bytes", C.c_size_t), ("t_submit", C.c_double),
                ("t_start", C.c_double), ("t_done", C.c_double), ("result", C.c_uint64 * 8)]


REQ_COMPRESS = 0
REQ_DECOMPRESS = 1

_LIB = None

_p, _sz, _i, _d, _u64p, _u32p = C.c_void_p, C.c_size_t, C.c_int, C.c_double, C.c_void_p, C.c_void_p
_PROTOS = {
    "vsz_status_string": ([_i], C.c_char_p),
    "vsz_version": ([], C.c_char_p),
    "vsz_parse_padding": ([C.c_char_p, C.POINTER(Params)], _i),
    "vsz_pad_count": ([_i, C.POINTER(C.c_size_t), _i, _i], _sz),
    "vsz_eb_setup": ([C.POINTER(Params), _p, _sz, _p, _p, _p], _i),
    "vsz_consts_read": ([_p, C.POINTER(C.c_double), C.POINTER(C.c_int), _p], _i),
    "vsz_outlier_segments": ([_i, C.POINTER(C.c_size_t)], _sz),
    "vsz_dualquant": ([_i, C.POINTER(C.c_size_t), _i, _i, _p, _p, _p, _p, _p, _p, _p], _i),
    "vsz_outlier_gather_tmp_bytes": ([_i, C.POINTER(C.c_size_t)], _sz),
    "vsz_outlier_gather": ([_i, C.POINTER(C.c_size_t), _p, _p, _p, _p, _p, _sz, _p], _i),
    "vsz_outlier_gather_noalloc": ([_i, C.POINTER(C.c_size_t), _p, _p, _p, _p, _p], _i),
    "vsz_codebook_bytes": ([_i], _sz),
    "vsz_huff_head_max": ([_i], _sz),
    "vsz_huffman_build_tmp_bytes": ([_i], _sz),
    "vsz_huffman_build": ([_p, _i, _p, _p, _p, _p, _sz, _p], _i),
    "vsz_huffman_build_host": ([_p, _i, _p, _p, _p], _i),
    "vsz_set_tree_builder": ([_i], _i),
    "vsz_launch_count": ([], C.c_uint64),
    "vsz_debug_set_spin_limit": ([C.c_longlong], _i),
    "vsz_debug_scan_stalled_predecessor": ([_sz, C.POINTER(C.c_int)], _i),
    "vsz_debug_tree_hold": ([C.c_int], _i),
    "vsz_debug_set_tree_wait_ns": ([C.c_longlong], _i),
    "vsz_batch_workspace_bytes": ([_p, _i, C.POINTER(C.c_size_t)], _i),
    "vsz_batch_create": ([_p, _i, _p, _sz, _p, C.POINTER(C.c_void_p)], _i),
    "vsz_batch_compress": ([_p, _p], _i),
    "vsz_batch_destroy": ([_p], None),
    "vsz_batch_set_task_sizes": ([_p, _i, _i], _i),
    "vsz_batch_autotune": ([_p, _i, C.POINTER(C.c_int), C.POINTER(C.c_int), _p], _i),
    "vsz_autotune_bounds": ([_p, _i, C.POINTER(C.c_size_t), C.c_double, C.POINTER(C.c_size_t)], _i),
    "vsz_autotune": ([_p, _i, C.POINTER(C.c_size_t), _p, C.c_double, _i, C.c_double, _p, _sz, _p, _p], _i),
    "vsz_autotune_cache_clear": ([], None),
    "vsz_compress_f64_bounds": ([C.POINTER(Params), _i, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t),
                                 C.POINTER(C.c_size_t)], _i),
    "vsz_compress_f64": ([C.POINTER(Params), _i, C.POINTER(C.c_size_t), _p, _p, _sz, _p, _sz, _p, _p], _i),
    "vsz_decompress_f64_bounds": ([C.POINTER(ArchiveDesc), C.POINTER(C.c_size_t)], _i),
    "vsz_decompress_f64": ([C.POINTER(ArchiveDesc), _p, _p, _sz, _p, _p, _p], _i),
    "vsz_compress_host_f64": ([C.POINTER(Params), _i, C.POINTER(C.c_size_t), _p, C.POINTER(C.c_void_p),
                               C.POINTER(C.c_size_t),
                               C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)], _i),
    "vsz_decompress_host_f64": ([_p, _sz, _sz, _sz, C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)], _i),
    "vsz_dbatch_workspace_bytes": ([_p, _i, C.POINTER(C.c_size_t)], _i),
    "vsz_dbatch_create": ([_p, _i, _p, _sz, _p, C.POINTER(C.c_void_p)], _i),
    "vsz_dbatch_decompress": ([_p, _p], _i),
    "vsz_dbatch_destroy": ([_p], None),
    "vsz_autotune_workspace_bytes": ([_p, _i, C.POINTER(C.c_size_t), _d, C.POINTER(C.c_size_t)], _i),
    "vsz_autotune_block_size": ([_p, _i, C.POINTER(C.c_size_t), _p, _d, _i, _p, _sz, C.POINTER(C.c_int),
                                 C.POINTER(C.c_double), _p], _i),
    "vsz_autotune_block_size_host": ([_p, _i, C.POINTER(C.c_size_t), _p, _d, _i, C.POINTER(C.c_int),
                                      C.POINTER(C.c_double)], _i),
    "vsz_server_create": ([_sz, _i, C.POINTER(C.c_void_p)], _i),
    "vsz_server_submit": ([_p, _p, C.POINTER(C.c_uint64)], _i),
    "vsz_server_wait": ([_p, C.c_uint64, _d, _p], _i),
    "vsz_server_release": ([_p, C.c_uint64], _i),
    "vsz_server_cancel": ([_p, C.c_uint64], _i),
    "vsz_server_stats": ([_p, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_size_t),
                          C.POINTER(C.c_int)], _i),
    "vsz_server_destroy": ([_p], None),
    "vsz_huffman_encode_tmp_bytes": ([_sz], _sz),
    "vsz_huffman_encode": ([_p, _sz, _p, _i, _p, _p, _p, _p, _sz, _p], _i),
    "vsz_huffman_decode_tmp_bytes": ([_sz, _sz, _i], _sz),
    "vsz_huffman_decode": ([_p, _sz, _sz, _i, _p, _p, _sz, _p], _i),
    "vsz_dualquant_decompress_tmp_bytes": ([_i, C.POINTER(C.c_size_t)], _sz),
    "vsz_dualquant_decompress": ([_i, C.POINTER(C.c_size_t), _i, _i, _p, _p, C.c_uint64, _p, _p, _p, _sz, _p], _i),
    "vsz_compress_bounds": ([C.POINTER(Params), _i, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t),
                             C.POINTER(C.c_size_t)], _i),
    "vsz_compress": ([C.POINTER(Params), _i, C.POINTER(C.c_size_t), _p, _p, _sz, _p, _sz, _p, _p], _i),
    "vsz_archive_parse": ([_p, _sz, C.POINTER(ArchiveDesc)], _i),
    "vsz_decompress_bounds": ([C.POINTER(ArchiveDesc), C.POINTER(DecompressOpts), C.POINTER(C.c_size_t)], _i),
    "vsz_decompress": ([C.POINTER(ArchiveDesc), C.POINTER(DecompressOpts), _p, _p, _sz, _p, _p, _p], _i),
    "vsz_compress_host": ([C.POINTER(Params), _i, C.POINTER(C.c_size_t), _p, C.POINTER(C.c_void_p),
                           C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), C.POINTER(C.c_size_t),
                           C.POINTER(C.c_size_t)], _i),
    "vsz_compress_host_into": ([C.POINTER(Params), _i, C.POINTER(C.c_size_t), _p, _p, _sz, C.POINTER(C.c_size_t),
                                C.POINTER(C.c_size_t), C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)], _i),
    "vsz_compress_host_bound": ([C.POINTER(Params), _i, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)], _i),
    "vsz_decompress_host": ([_p, _sz, _sz, _sz, C.POINTER(DecompressOpts), C.POINTER(C.c_void_p),
                             C.POINTER(C.c_size_t)], _i),
    "vsz_decompress_host_into": ([_p, _sz, _sz, _sz, C.POINTER(DecompressOpts), _p, _sz, C.POINTER(C.c_size_t)], _i),
    "vsz_free_host": ([_p], None),
    "vsz_host_op_create": ([C.POINTER(_p)], _i),
    "vsz_host_op_destroy": ([_p], None),
    "vsz_host_op_compress": ([_p, C.POINTER(Params), _i, C.POINTER(C.c_size_t), _p, _p, _sz, _p], _i),
    "vsz_host_op_decompress": ([_p, _p, _sz, _p, _p, _sz, _p], _i),
    "vsz_host_op_wait": ([_p], _i),
    "vsz_lossless_compress": ([_i, _p, _sz, C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)], _i),
    "vsz_lossless_decompress": ([_p, _sz, _sz, C.POINTER(C.c_void_p), C.POINTER(C.c_size_t)], _i),
    "vsz_lossless_detect": ([_p, _sz], _i),
    "vsz_deflate_bounds": ([_sz, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)], _i),
    "vsz_deflate": ([_p, _sz, _p, _sz, _p, _sz, _p, _p], _i),
    "vsz_deflate_chunk_sizes": ([_p, _sz, _p, _p], _i),
    "vsz_deflate_chunk_bytes": ([], _sz),
    "vsz_inflate_bounds": ([_sz, C.POINTER(C.c_size_t)], _i),
    "vsz_inflate": ([_p, _sz, _p, _p, _sz, C.c_uint32, _p, _sz, _p, _sz, _p, _p], _i),
    "vsz_archive_parse_split": ([_p, _sz, _p, _sz, C.POINTER(ArchiveDesc)], _i),
    "vsz_profile_enable": ([_i], None),
    "vsz_profile_reset": ([], None),
    "vsz_profile_read": ([_p, _p, _p, _i], _i),
}


def library_path() -> str:
    return _build.LIB


def lib(build_if_missing: bool = True) -> C.CDLL:
    """Load libvecsz_gb300.so (building it with nvcc first if it is missing or stale)."""
    global _LIB
    if _LIB is None:
        path = _build.LIB
        if build_if_missing and (not os.path.exists(path) or _build._stale()):
            _build.build()
        if not os.path.exists(path):
            raise ImportError(f"vecsz_gb300: native library {path} is missing; run vecsz_gb300._build.build()")
        L = C.CDLL(path, mode=C.RTLD_GLOBAL)
        for name, (args, res) in _PROTOS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = res
        _LIB = L
    return _LIB


def exported_symbols() -> list[str]:
    return list(_PROTOS)


def check(status: int, what: str = "") -> None:
    if status != VSZ_OK:
        raise VszError(status, what)


def dims_arg(dims) -> C.Array:
    d = list(int(v) for v in dims) + [1] * (3 - len(dims))
    return (C.c_size_t * 3)(*d)
