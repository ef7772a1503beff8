"""vecsz_gb300: GB300-native (sm_103a) dual-quantization lossy compressor, compatible with vecSZ.

The compute path is libvecsz_gb300.so (hand-written CUDA kernels behind a C ABI, see
include/vecsz_gb300.h); this package binds it with ctypes.  There is no CPU fallback.
"""
from ._lib import VszError, lib, library_path  # noqa: F401
from .api import (BatchCompressor, BatchDecompressor, Compressed, DeviceCodec, HostOp, Server, compress,  # noqa: F401
                  decompress, make_params, pad_count, parse_archive, read_sz_file)

__all__ = ["VszError", "lib", "library_path", "BatchCompressor", "BatchDecompressor", "Compressed", "DeviceCodec",
           "HostOp", "Server", "compress", "decompress", "make_params", "pad_count", "parse_archive", "read_sz_file"]
