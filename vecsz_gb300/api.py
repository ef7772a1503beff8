"""Python host API over the C ABI.

Mirrors the reference's workflow (src/vecsz_interface.hh): `compress` is Compress<float,int>,
`decompress` is Decompress<float,int>, both on host arrays.  `DeviceCodec` keeps a field's
workspace resident on the GPU for repeated device-to-device compress/decompress (torch tensors
provide the device memory and streams).  Stage functions expose each kernel stage for tests.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib as L
from ._lib import (ArchiveDesc, DecompressOpts, Params, Result, VszError, check, dims_arg, lib)

_MODES = {"abs": L.MODE_ABS, "r2r": L.MODE_R2R}
_LOSSLESS = {None: L.LOSSLESS_NONE, "none": L.LOSSLESS_NONE, "zstd": L.LOSSLESS_ZSTD, "gzip": L.LOSSLESS_GZIP,
             "gzip-device": L.LOSSLESS_GZIP_DEVICE}


_PAD_MODES = {"none": L.PAD_NONE, "global": L.PAD_GLOBAL, "block": L.PAD_BLOCK, "edge": L.PAD_EDGE}
_PAD_TYPES = {"max": L.PADV_MAX, "min": L.PADV_MIN, "avg": L.PADV_AVG, "constant": L.PADV_CONST}


def make_params(eb=1e-4, mode="abs", dict_size=4096, block_size=8, lossless=None, strict=False,
                padding=None) -> Params:
    """Settings of one compress.  padding: the reference's -p string ("block,max", "global,avg",
    "edge,constant,2.5", ...; src/argument_parser/argparse.cc:399-415, which reads no sign), or a
    (mode, type, constant) tuple ("block", "avg", 0.0) that also takes negative constants; None
    for the zero halo."""
    m = _MODES[mode] if isinstance(mode, str) else int(mode)
    ll = _LOSSLESS[lossless] if (lossless is None or isinstance(lossless, str)) else int(lossless)
    p = Params(float(eb), m, int(dict_size), int(block_size), ll, 1 if strict else 0, L.PAD_NONE, L.PADV_CONST, 0.0)
    if isinstance(padding, str):
        check(lib().vsz_parse_padding(padding.encode(), C.byref(p)), "parse_padding")
    elif padding is not None:
        pm, pt, pc = padding
        p.pad_mode = _PAD_MODES[pm] if isinstance(pm, str) else int(pm)
        p.pad_type = _PAD_TYPES[pt] if isinstance(pt, str) else int(pt)
        p.pad_constant = float(pc)
    return p


def pad_count(dims, block_size: int, padding) -> int:
    """Pad values a packed block of this geometry holds with this padding (see make_params)."""
    p = make_params(block_size=block_size, padding=padding)
    return int(lib().vsz_pad_count(len(dims), dims_arg(dims), int(block_size), p.pad_mode))


@dataclass
class Compressed:
    """What Compress returns: the bytes main() writes after its 16-byte header, and the sizes."""
    data: bytes           # packed block (or lossless frame) followed by this library's trailer
    data_size: int        # packed block bytes (the reference's data_size)
    lossless_size: int    # lossless frame bytes, 0 without -L
    n_outlier: int

    def file_bytes(self) -> bytes:
        """The .sz file: u64 lossless_size, u64 data_size, payload (src/vecsz.cc:103-105)."""
        return (np.array([self.lossless_size, self.data_size], np.uint64).tobytes() + self.data)


def compress(data: np.ndarray, dims=None, eb: float = 1e-4, mode="abs", dict_size: int = 4096, block_size: int = 8,
             lossless=None, strict: bool = False, padding=None, dtype: str = "f32") -> Compressed:
    """Compress a field held in host memory (vecsz::interface::Compress).  padding: the
    reference's -p string, see make_params.  dtype "f64": the data are float64 and go through the
    f64 path (vsz_compress_host_f64: error bound guaranteed, 8-byte outliers)."""
    if dtype == "f64":
        x = np.ascontiguousarray(data, dtype=np.float64)
        if dims is None:
            dims = tuple(reversed(x.shape))
        p = make_params(eb, mode, dict_size, block_size, lossless, strict, padding)
        out = C.c_void_p(0)
        ob, ds, ls, no = C.c_size_t(0), C.c_size_t(0), C.c_size_t(0), C.c_size_t(0)
        check(lib().vsz_compress_host_f64(C.byref(p), len(dims), dims_arg(dims), x.ctypes.data_as(C.c_void_p),
                                          C.byref(out), C.byref(ob), C.byref(ds), C.byref(ls), C.byref(no)),
              "compress_f64")
        try:
            buf = C.string_at(out.value, ob.value)
        finally:
            lib().vsz_free_host(out)
        return Compressed(buf, ds.value, ls.value, no.value)
    if dtype != "f32":
        raise ValueError(f"dtype must be 'f32' or 'f64', not {dtype!r}")
    x = np.ascontiguousarray(data, dtype=np.float32)
    if dims is None:
        dims = tuple(reversed(x.shape))  # numpy (z, y, x) -> reference (x, y, z)
    p = make_params(eb, mode, dict_size, block_size, lossless, strict, padding)
    out = C.c_void_p(0)
    ob, ds, ls, no = C.c_size_t(0), C.c_size_t(0), C.c_size_t(0), C.c_size_t(0)
    check(lib().vsz_compress_host(C.byref(p), len(dims), dims_arg(dims), x.ctypes.data_as(C.c_void_p), C.byref(out),
                                  C.byref(ob), C.byref(ds), C.byref(ls), C.byref(no)), "compress")
    try:
        buf = C.string_at(out.value, ob.value)
    finally:
        lib().vsz_free_host(out)
    return Compressed(buf, ds.value, ls.value, no.value)


def decompress(archive, data_size: int = 0, lossless_size: int = 0, dict_size: int = 4096, block_size: int = 8,
               mode="abs", value_range: float = 0.0) -> np.ndarray:
    """Decompress (vecsz::interface::Decompress).  `archive` is a Compressed or raw bytes; the
    -d/-b/-m options matter only for archives without this library's trailer."""
    if isinstance(archive, Compressed):
        data_size, lossless_size, archive = archive.data_size, archive.lossless_size, archive.data
    a = np.frombuffer(archive, np.uint8)
    if _is_f64_archive(archive, data_size, lossless_size):
        out = C.c_void_p(0)
        n = C.c_size_t(0)
        check(lib().vsz_decompress_host_f64(a.ctypes.data_as(C.c_void_p), a.size, int(data_size), int(lossless_size),
                                            C.byref(out), C.byref(n)), "decompress_f64")
        try:
            res = np.frombuffer(C.string_at(out.value, n.value * 8), np.float64).copy()
        finally:
            lib().vsz_free_host(out)
        return res
    o = DecompressOpts(int(dict_size), int(block_size), _MODES[mode] if isinstance(mode, str) else int(mode),
                       float(value_range))
    out = C.c_void_p(0)
    n = C.c_size_t(0)
    check(lib().vsz_decompress_host(a.ctypes.data_as(C.c_void_p), a.size, int(data_size), int(lossless_size),
                                    C.byref(o), C.byref(out), C.byref(n)), "decompress")
    try:
        res = np.frombuffer(C.string_at(out.value, n.value * 4), np.float32).copy()
    finally:
        lib().vsz_free_host(out)
    return res


def _is_f64_archive(archive, data_size: int, lossless_size: int) -> bool:
    """Whether this library's trailer (after the packed block, or after the lossless frame) marks an
    f64 field: its mode word's bit 9."""
    t = int(lossless_size) if lossless_size else int(data_size)
    b = bytes(archive[t: t + 48]) if t else b""
    if len(b) < 48 or b[:4] != b"VSZT":
        return False
    return bool(int.from_bytes(b[32:36], "little") & 0x200)


def parse_archive(buf) -> ArchiveDesc:
    a = np.frombuffer(buf, np.uint8)
    d = ArchiveDesc()
    check(lib().vsz_archive_parse(a.ctypes.data_as(C.c_void_p), a.size, C.byref(d)), "archive_parse")
    return d


def read_sz_file(path: str):
    """(data, data_size, lossless_size) of a .sz file written by the reference or by this library."""
    raw = open(path, "rb").read()
    lossless_size, data_size = np.frombuffer(raw[:16], np.uint64)
    return raw[16:], int(data_size), int(lossless_size)


# ------------------------------------------------------------------------------------------------
# Device-resident codec (torch provides device memory and streams)
# ------------------------------------------------------------------------------------------------

def _torch():
    import torch
    return torch


def _ptr(t) -> C.c_void_p:
    return C.c_void_p(t.data_ptr())


def _stream_ptr(stream=None) -> C.c_void_p:
    torch = _torch()
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def deflate(data, stream=None):
    """The gzip pass on the device (vsz_deflate): bytes, a uint8 numpy array or a uint8 CUDA tensor
    -> (zlib stream bytes, stats {chunks, stored, fixed, dynamic})."""
    torch = _torch()
    if isinstance(data, torch.Tensor):
        d_in = data.contiguous().view(-1)
        n = int(d_in.numel())
    else:
        a = data.view(np.uint8).ravel() if isinstance(data, np.ndarray) else np.frombuffer(bytes(data), np.uint8)
        n = int(a.size)
        d_in = torch.from_numpy(a.copy()).cuda() if n else torch.zeros(1, dtype=torch.uint8, device="cuda")
    ws, cap = C.c_size_t(0), C.c_size_t(0)
    check(lib().vsz_deflate_bounds(n, C.byref(ws), C.byref(cap)), "deflate_bounds")
    d_ws = torch.empty(max(1, ws.value), dtype=torch.uint8, device=d_in.device)
    d_out = torch.empty(cap.value, dtype=torch.uint8, device=d_in.device)
    res = torch.zeros(8, dtype=torch.int64, device=d_in.device)
    check(lib().vsz_deflate(_ptr(d_in), n, _ptr(d_ws), ws.value, _ptr(d_out), cap.value, _ptr(res),
                            _stream_ptr(stream)), "deflate")
    r = res.cpu().numpy()
    if int(r[1]) != 0:
        raise VszError(int(r[1]), "deflate (device)")
    out = d_out[: int(r[0])].cpu().numpy().tobytes()
    sizes = np.zeros(int(r[2]), np.uint32)
    if sizes.size:
        check(lib().vsz_deflate_chunk_sizes(_ptr(d_ws), n, sizes.ctypes.data_as(C.c_void_p), _stream_ptr(stream)),
              "deflate_chunk_sizes")
        _torch().cuda.synchronize()
    return out, {"chunks": int(r[2]), "stored": int(r[3]), "fixed": int(r[4]), "dynamic": int(r[5]),
                 "chunk_bytes": sizes}


def inflate(stream_bytes: bytes, chunk_bytes, out_len: int) -> tuple[bytes, int]:
    """Inflate on the device (vsz_inflate) a stream vsz_deflate wrote, from its chunk sizes:
    (bytes, status); status VSZ_ERR_CORRUPT for streams it does not take."""
    torch = _torch()
    sizes = np.ascontiguousarray(chunk_bytes, np.uint32)
    offs = (2 + np.concatenate([[0], np.cumsum(sizes.astype(np.uint64))[:-1]])).astype(np.uint64) if sizes.size \
        else np.zeros(0, np.uint64)
    a = np.frombuffer(stream_bytes, np.uint8)
    d_s = torch.from_numpy(np.concatenate([a, np.zeros(16, np.uint8)])).cuda()
    d_off = torch.from_numpy(offs.view(np.int64).copy() if offs.size else np.zeros(1, np.int64)).cuda()
    d_sz = torch.from_numpy(sizes.view(np.int32).copy() if sizes.size else np.zeros(1, np.int32)).cuda()
    ws = C.c_size_t(0)
    check(lib().vsz_inflate_bounds(sizes.size, C.byref(ws)), "inflate_bounds")
    d_ws = torch.empty(ws.value, dtype=torch.uint8, device="cuda")
    d_out = torch.zeros(max(1, out_len), dtype=torch.uint8, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    adler = int.from_bytes(stream_bytes[-4:], "big") if len(stream_bytes) >= 4 else 0
    check(lib().vsz_inflate(_ptr(d_s), a.size, _ptr(d_off), _ptr(d_sz), sizes.size, adler, _ptr(d_out), out_len,
                            _ptr(d_ws), ws.value, _ptr(st), _stream_ptr()), "inflate")
    return d_out[:out_len].cpu().numpy().tobytes(), int(st.item())


class DeviceCodec:
    """Compress / decompress one field shape repeatedly with resident buffers.

    compress(d_in) writes the archive into self.archive (a uint8 CUDA tensor) and the vsz_result
    record into self.result (8 uint64); nothing is copied to the host unless you ask."""

    def __init__(self, dims, eb=1e-4, mode="abs", dict_size=1024, block_size=8, device="cuda", strict=False,
                 padding=None):
        torch = _torch()
        self.dims = tuple(int(v) for v in dims)
        self.n = int(np.prod(self.dims))
        self.params = make_params(eb, mode, dict_size, block_size, strict=strict, padding=padding)
        ws, cap = C.c_size_t(0), C.c_size_t(0)
        check(lib().vsz_compress_bounds(C.byref(self.params), len(self.dims), dims_arg(self.dims), C.byref(ws),
                                        C.byref(cap)), "compress_bounds")
        self.ws = torch.empty(ws.value, dtype=torch.uint8, device=device)
        self.archive = torch.zeros(cap.value + 64, dtype=torch.uint8, device=device)
        self.archive_cap = cap.value
        self.result = torch.zeros(8, dtype=torch.int64, device=device)
        self._dws = None
        self._desc = None

    def compress(self, d_in, stream=None) -> None:
        check(lib().vsz_compress(C.byref(self.params), len(self.dims), dims_arg(self.dims), _ptr(d_in), _ptr(self.ws),
                                 self.ws.numel(), _ptr(self.archive), self.archive_cap, _ptr(self.result),
                                 _stream_ptr(stream)), "compress")

    def result_host(self) -> Result:
        r = self.result.cpu().numpy().view(np.uint64)
        res = Result(*[int(v) for v in r])
        if res.status != 0:
            raise VszError(int(res.status), "compress (device)")
        return res

    def archive_bytes(self) -> bytes:
        r = self.result_host()
        return self.archive[: r.data_size + r.trailer_size].cpu().numpy().tobytes()

    def prepare_decompress(self, archive_host: bytes, opts: DecompressOpts | None = None) -> None:
        """Parse the archive's header on the host once and size the decompress workspace."""
        torch = _torch()
        self._desc = parse_archive(archive_host)
        self._opts = opts or DecompressOpts(self.params.dict_size, self.params.block_size, self.params.mode, 0.0)
        ws = C.c_size_t(0)
        check(lib().vsz_decompress_bounds(C.byref(self._desc), C.byref(self._opts), C.byref(ws)), "decompress_bounds")
        if self._dws is None or self._dws.numel() < ws.value:
            self._dws = torch.empty(ws.value, dtype=torch.uint8, device=self.archive.device)
        self._dstatus = torch.zeros(1, dtype=torch.int32, device=self.archive.device)

    def decompress(self, d_archive, d_out, stream=None) -> None:
        check(lib().vsz_decompress(C.byref(self._desc), C.byref(self._opts), _ptr(d_archive), _ptr(self._dws),
                                   self._dws.numel(), _ptr(d_out), _ptr(self._dstatus), _stream_ptr(stream)),
              "decompress")

    def decompress_status(self) -> int:
        return int(self._dstatus.item())


class HostOp:
    """One stream-ordered compress or decompress on pinned host buffers (vsz_host_op_*): calls
    enqueue the copies and kernels and return at once; wait() blocks until they are done.  Several
    ops overlap their host-to-device and device-to-host copies."""

    def __init__(self):
        h = C.c_void_p(0)
        check(lib().vsz_host_op_create(C.byref(h)), "host_op_create")
        self._h = h

    def compress(self, p: Params, dims, h_in_ptr: int, h_out_ptr: int, out_capacity: int, h_result_ptr: int):
        check(lib().vsz_host_op_compress(self._h, C.byref(p), len(dims), dims_arg(dims), C.c_void_p(h_in_ptr),
                                         C.c_void_p(h_out_ptr), int(out_capacity), C.c_void_p(h_result_ptr)),
              "host_op_compress")

    def decompress(self, h_archive_ptr: int, length: int, opts: DecompressOpts, h_out_ptr: int, out_capacity: int,
                   h_status_ptr: int):
        check(lib().vsz_host_op_decompress(self._h, C.c_void_p(h_archive_ptr), int(length), C.byref(opts),
                                           C.c_void_p(h_out_ptr), int(out_capacity), C.c_void_p(h_status_ptr)),
              "host_op_decompress")

    def wait(self):
        check(lib().vsz_host_op_wait(self._h), "host_op_wait")

    def close(self):
        if self._h:
            lib().vsz_host_op_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchCompressor:
    """Many device fields compressed in one launch sequence (vsz_batch_*).

    fields: list of dicts {"x": CUDA float32 tensor, "dims": dims, "eb", "mode", "dict_size",
    "block_size"}.  The archives land in per-field uint8 tensors (self.archives[i]); compress()
    may be called repeatedly (or captured in a CUDA graph) and recompresses the current inputs."""

    def __init__(self, fields, device="cuda"):
        torch = _torch()
        from ._lib import BatchField
        self.n = len(fields)
        self.fields = fields
        arr = (BatchField * self.n)()
        self.archives = []
        for i, f in enumerate(fields):
            dims = tuple(int(v) for v in f["dims"])
            p = make_params(f.get("eb", 1e-4), f.get("mode", "abs"), f.get("dict_size", 1024), f.get("block_size", 8),
                            strict=f.get("strict", False))
            ws, cap = C.c_size_t(0), C.c_size_t(0)
            check(lib().vsz_compress_bounds(C.byref(p), len(dims), dims_arg(dims), C.byref(ws), C.byref(cap)),
                  "compress_bounds")
            a = torch.zeros(cap.value + 64, dtype=torch.uint8, device=device)
            self.archives.append(a)
            arr[i].d_in = _ptr(f["x"]).value
            arr[i].ndim = len(dims)
            arr[i].dims = dims_arg(dims)
            arr[i].params = p
            arr[i].d_archive = _ptr(a).value
            arr[i].archive_capacity = cap.value
        self._arr = arr
        ws = C.c_size_t(0)
        check(lib().vsz_batch_workspace_bytes(arr, self.n, C.byref(ws)), "batch_workspace_bytes")
        self.ws = torch.empty(ws.value, dtype=torch.uint8, device=device)
        self.results = torch.zeros(8 * self.n, dtype=torch.int64, device=device)
        h = C.c_void_p(0)
        check(lib().vsz_batch_create(arr, self.n, _ptr(self.ws), self.ws.numel(), _ptr(self.results), C.byref(h)),
              "batch_create")
        self._h = h

    def compress(self, stream=None) -> None:
        check(lib().vsz_batch_compress(self._h, _stream_ptr(stream)), "batch_compress")

    def set_task_sizes(self, dq_units: int, enc_chunks: int) -> None:
        check(lib().vsz_batch_set_task_sizes(self._h, int(dq_units), int(enc_chunks)), "batch_set_task_sizes")

    def autotune(self, iterations: int = 2, stream=None):
        """Search the task sizes (vsz_batch_autotune); returns (dq_units, enc_chunks)."""
        a, b = C.c_int(0), C.c_int(0)
        check(lib().vsz_batch_autotune(self._h, int(iterations), C.byref(a), C.byref(b), _stream_ptr(stream)),
              "batch_autotune")
        return a.value, b.value

    def result(self, i) -> Result:
        r = self.results[8 * i: 8 * i + 8].cpu().numpy().view(np.uint64)
        return Result(*[int(v) for v in r])

    def archive_bytes(self, i) -> bytes:
        r = self.result(i)
        if r.status != 0:
            raise VszError(int(r.status), f"batch field {i}")
        return self.archives[i][: r.data_size + r.trailer_size].cpu().numpy().tobytes()

    def close(self) -> None:
        if self._h:
            lib().vsz_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class BatchDecompressor:
    """Many archives decompressed in one launch sequence (vsz_dbatch_*).

    archives: list of archives written by this library (bytes, or CUDA uint8 tensors with 16 readable
    bytes past the archive); block size 8, no padding, not strict.  The outputs land in per-field
    float32 tensors (self.outputs[i]); decompress() may be called repeatedly (or captured in a CUDA
    graph) and decodes the current contents of the archive buffers."""

    def __init__(self, archives, descs=None, device="cuda"):
        """descs (optional): vsz_archive_parse of each archive, for device archives whose bytes
        should not be copied back to parse them."""
        torch = _torch()
        from ._lib import DBatchField
        self.n = len(archives)
        arr = (DBatchField * self.n)()
        self.d_archives, self.outputs, self.descs = [], [], []
        for i, a in enumerate(archives):
            if isinstance(a, (bytes, bytearray)):
                desc = parse_archive(a) if descs is None else descs[i]
                d = torch.from_numpy(np.frombuffer(bytes(a) + bytes(64), np.uint8).copy()).to(device)
            else:
                desc = parse_archive(a.cpu().numpy().tobytes()) if descs is None else descs[i]
                d = a
            n = int(desc.dims[0]) * int(desc.dims[1]) * int(desc.dims[2])
            out = torch.empty(n, dtype=torch.float32, device=device)
            self.d_archives.append(d)
            self.outputs.append(out)
            self.descs.append(desc)
            arr[i].d_archive = _ptr(d).value
            arr[i].desc = desc
            arr[i].d_out = _ptr(out).value
        self._arr = arr
        ws = C.c_size_t(0)
        check(lib().vsz_dbatch_workspace_bytes(arr, self.n, C.byref(ws)), "dbatch_workspace_bytes")
        self.ws = torch.empty(ws.value, dtype=torch.uint8, device=device)
        self.status = torch.zeros(max(self.n, 1), dtype=torch.int32, device=device)
        h = C.c_void_p(0)
        check(lib().vsz_dbatch_create(arr, self.n, _ptr(self.ws), self.ws.numel(), _ptr(self.status), C.byref(h)),
              "dbatch_create")
        self._h = h

    def decompress(self, stream=None) -> None:
        check(lib().vsz_dbatch_decompress(self._h, _stream_ptr(stream)), "dbatch_decompress")

    def statuses(self):
        return [int(v) for v in self.status[: self.n].cpu().tolist()]

    def close(self) -> None:
        if self._h:
            lib().vsz_dbatch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(d_in, dims, eb=1e-4, mode="abs", dict_size=1024, sample_percent=10.0, iterations=2, link_gbs=0.0,
             stream=None) -> dict:
    """Field autotuner (vsz_autotune): each block size timed through compress + decompress on a
    leading slab and scored with the archive's transfer time over a link of link_gbs GB/s; cached
    per field class.  Returns the vsz_tune_result as a dict."""
    torch = _torch()
    from ._lib import TuneResult
    dims = tuple(int(v) for v in dims)
    p = make_params(eb, mode, dict_size, 8)
    ws = C.c_size_t(0)
    check(lib().vsz_autotune_bounds(C.byref(p), len(dims), dims_arg(dims), float(sample_percent), C.byref(ws)),
          "autotune_bounds")
    d_ws = torch.empty(ws.value, dtype=torch.uint8, device=d_in.device)
    r = TuneResult()
    check(lib().vsz_autotune(C.byref(p), len(dims), dims_arg(dims), _ptr(d_in), float(sample_percent), int(iterations),
                             float(link_gbs), _ptr(d_ws), ws.value, C.byref(r), _stream_ptr(stream)), "autotune")
    return {"block_size": r.block_size, "cached": bool(r.cached), "sample_elements": int(r.sample_elements),
            "candidates": [8, 16, 32, 64], "compress_ms": list(r.compress_ms), "decompress_ms": list(r.decompress_ms),
            "archive_bytes": [int(v) for v in r.archive_bytes], "score_ms": list(r.score_ms)}


def autotune_cache_clear() -> None:
    lib().vsz_autotune_cache_clear()


def autotune_block_size(d_in, dims, eb=1e-4, mode="abs", dict_size=1024, sample_percent=10.0, iterations=3):
    """GPU block-size autotuner (vsz_autotune_block_size, the CLI's -a): (best block size,
    {8: ms, 16: ms, 32: ms, 64: ms})."""
    torch = _torch()
    dims = tuple(int(v) for v in dims)
    p = make_params(eb, mode, dict_size, 8)
    ws = C.c_size_t(0)
    check(lib().vsz_autotune_workspace_bytes(C.byref(p), len(dims), dims_arg(dims), float(sample_percent),
                                             C.byref(ws)), "autotune_workspace_bytes")
    tmp = torch.empty(ws.value, dtype=torch.uint8, device=d_in.device)
    best = C.c_int(0)
    t = (C.c_double * 4)()
    check(lib().vsz_autotune_block_size(C.byref(p), len(dims), dims_arg(dims), _ptr(d_in), float(sample_percent),
                                        int(iterations), _ptr(tmp), ws.value, C.byref(best), t, _stream_ptr()),
          "autotune_block_size")
    return best.value, dict(zip((8, 16, 32, 64), list(t)))


class _CudaArray:
    def __init__(self, ptr, n, typestr):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": typestr, "data": (int(ptr), False),
                                         "version": 3, "strides": None}


def _device_view(ptr, nbytes, dtype="uint8"):
    """A torch tensor over raw device memory owned by the library (no copy)."""
    torch = _torch()
    if dtype == "float32":
        return torch.as_tensor(_CudaArray(ptr, nbytes // 4, "<f4"), device="cuda")
    return torch.as_tensor(_CudaArray(ptr, nbytes, "|u1"), device="cuda")


class Server:
    """Request server (vsz_server_*): compress / decompress requests admitted under a device-memory
    budget as stream slots and memory free up, their work overlapping on the device.

    submit_compress / submit_decompress return a ticket; wait(ticket) returns the Completion (its
    d_out points into the server's arena); output_tensor copies the output out; release frees it."""

    def __init__(self, budget_bytes, slots=8):
        h = C.c_void_p(0)
        check(lib().vsz_server_create(int(budget_bytes), int(slots), C.byref(h)), "server_create")
        self._h = h
        self._keep = {}

    def submit_compress(self, d_in, dims, eb=1e-4, mode="abs", dict_size=1024, block_size=8) -> int:
        from ._lib import REQ_COMPRESS, Request
        dims = tuple(int(v) for v in dims)
        r = Request()
        r.kind = REQ_COMPRESS
        r.d_in = _ptr(d_in).value
        r.ndim = len(dims)
        r.dims = dims_arg(dims)
        r.params = make_params(eb, mode, dict_size, block_size)
        t = C.c_uint64(0)
        check(lib().vsz_server_submit(self._h, C.byref(r), C.byref(t)), "server_submit")
        self._keep[t.value] = d_in
        return t.value

    def submit_decompress(self, d_archive, desc, opts) -> int:
        from ._lib import REQ_DECOMPRESS, Request
        r = Request()
        r.kind = REQ_DECOMPRESS
        r.d_in = _ptr(d_archive).value
        r.desc = desc
        r.opts = opts
        t = C.c_uint64(0)
        check(lib().vsz_server_submit(self._h, C.byref(r), C.byref(t)), "server_submit")
        self._keep[t.value] = d_archive
        return t.value

    def wait(self, ticket, timeout_s=60.0):
        from ._lib import Completion
        c = Completion()
        check(lib().vsz_server_wait(self._h, C.c_uint64(ticket), float(timeout_s), C.byref(c)), "server_wait")
        return c

    def output_view(self, c, dtype="uint8"):
        """Zero-copy torch view of a completion's device output (valid until release)."""
        return _device_view(c.d_out, c.out_bytes, dtype)

    def output_bytes(self, c) -> bytes:
        return self.output_view(c).cpu().numpy().tobytes() if c.out_bytes else b""

    def release(self, ticket) -> None:
        check(lib().vsz_server_release(self._h, C.c_uint64(ticket)), "server_release")
        self._keep.pop(ticket, None)

    def cancel(self, ticket) -> int:
        """Withdraw a queued request (vsz_server_cancel): 0, or the status why it could not be."""
        return int(lib().vsz_server_cancel(self._h, C.c_uint64(ticket)))

    def stats(self):
        d, b, u, q = C.c_uint64(0), C.c_uint64(0), C.c_size_t(0), C.c_int(0)
        check(lib().vsz_server_stats(self._h, C.byref(d), C.byref(b), C.byref(u), C.byref(q)), "server_stats")
        return {"completed": d.value, "input_bytes_completed": b.value, "arena_bytes_in_use": u.value,
                "queued": q.value}

    def close(self) -> None:
        if self._h:
            lib().vsz_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------------------------------------------------
# Stage-level calls on torch CUDA tensors (one per reference routine)
# ------------------------------------------------------------------------------------------------

def eb_setup(d_in, eb, mode="abs"):
    """Device constants for eb; returns (consts tensor, {eb_final, c, r, range}, status)."""
    torch = _torch()
    p = make_params(eb, mode, 2, 8)
    consts = torch.zeros(L.CONSTS_BYTES, dtype=torch.uint8, device=d_in.device)
    tmp = torch.zeros(16, dtype=torch.uint8, device=d_in.device)
    check(lib().vsz_eb_setup(C.byref(p), _ptr(d_in), d_in.numel(), _ptr(consts), _ptr(tmp), _stream_ptr()), "eb_setup")
    out = (C.c_double * 4)()
    st = C.c_int(0)
    check(lib().vsz_consts_read(_ptr(consts), out, C.byref(st), _stream_ptr()), "consts_read")
    return consts, {"eb_final": out[0], "c": out[1], "r": out[2], "range": out[3]}, st.value


def dualquant(d_in, dims, block_size, dict_size, consts):
    """Codes (u16 as int32 tensor), histogram (int64), scratch, segment counts."""
    torch = _torch()
    dev = d_in.device
    n = int(np.prod(dims))
    nseg = lib().vsz_outlier_segments(len(dims), dims_arg(dims))
    code = torch.zeros(n + 8, dtype=torch.int16, device=dev)
    scratch = torch.zeros(nseg * 128 + 4, dtype=torch.float32, device=dev)
    segc = torch.zeros(nseg + 16, dtype=torch.uint8, device=dev)
    hist = torch.zeros(dict_size, dtype=torch.int64, device=dev)
    check(lib().vsz_dualquant(len(dims), dims_arg(dims), block_size, dict_size, _ptr(d_in), _ptr(consts), _ptr(code),
                              _ptr(scratch), _ptr(segc), _ptr(hist), _stream_ptr()), "dualquant")
    return code[:n], hist, scratch, segc


def outlier_gather(dims, segc, scratch):
    torch = _torch()
    dev = segc.device
    nseg = lib().vsz_outlier_segments(len(dims), dims_arg(dims))
    tb = lib().vsz_outlier_gather_tmp_bytes(len(dims), dims_arg(dims))
    tmp = torch.zeros(tb, dtype=torch.uint8, device=dev)
    out = torch.zeros(nseg * 128 + 4, dtype=torch.float32, device=dev)
    cnt = torch.zeros(1, dtype=torch.int64, device=dev)
    check(lib().vsz_outlier_gather(len(dims), dims_arg(dims), _ptr(segc), _ptr(scratch), _ptr(out), _ptr(cnt),
                                   _ptr(tmp), tb, _stream_ptr()), "outlier_gather")
    k = int(cnt.item())
    return out[:k]


def huffman_build(hist, dict_size):
    """(codebook tensor, huffman head bytes tensor, info [node_count, tree_bytes, max_len, nodes])."""
    torch = _torch()
    dev = hist.device
    cb = torch.zeros(lib().vsz_codebook_bytes(dict_size), dtype=torch.uint8, device=dev)
    head = torch.zeros(lib().vsz_huff_head_max(dict_size) + 16, dtype=torch.uint8, device=dev)
    info = torch.zeros(4, dtype=torch.int32, device=dev)
    tb = lib().vsz_huffman_build_tmp_bytes(dict_size)
    tmp = torch.zeros(tb, dtype=torch.uint8, device=dev)
    check(lib().vsz_huffman_build(_ptr(hist), dict_size, _ptr(cb), _ptr(head), _ptr(info), _ptr(tmp), tb,
                                  _stream_ptr()), "huffman_build")
    torch.cuda.synchronize()
    st = int(tmp[:4].view(torch.int32).item())
    if st:
        raise VszError(st, "huffman_build")
    return cb, head, info.cpu().numpy()


def huffman_encode(code, cb, dict_size, max_bits_per_code=64, offset=0):
    """Payload bytes (host), total bits, per-512 chunk bits.  `offset` places the payload at that
    byte offset of the output buffer (to exercise unaligned starts)."""
    torch = _torch()
    dev = code.device
    n = code.numel()
    cap = offset + (n * max_bits_per_code + 7) // 8 + 64
    out = torch.zeros(cap, dtype=torch.uint8, device=dev)
    bits = torch.zeros(1, dtype=torch.int64, device=dev)
    chunks = torch.zeros((n + 511) // 512 + 8, dtype=torch.int16, device=dev)
    tb = lib().vsz_huffman_encode_tmp_bytes(n)
    tmp = torch.zeros(tb, dtype=torch.uint8, device=dev)
    check(lib().vsz_huffman_encode(_ptr(code), n, _ptr(cb), dict_size, C.c_void_p(out.data_ptr() + offset),
                                   _ptr(bits), _ptr(chunks), _ptr(tmp), tb, _stream_ptr()), "huffman_encode")
    torch.cuda.synchronize()
    st = int(tmp[:4].view(torch.int32).item())
    if st:
        raise VszError(st, "huffman_encode")
    b = int(bits.item())
    return out, b, chunks[: (n + 511) // 512]


def huffman_decode(d_huff, huff_bytes, n, dict_size):
    torch = _torch()
    dev = d_huff.device
    out = torch.zeros(n + 8, dtype=torch.int16, device=dev)
    tb = lib().vsz_huffman_decode_tmp_bytes(huff_bytes, n, dict_size)
    tmp = torch.zeros(tb, dtype=torch.uint8, device=dev)
    check(lib().vsz_huffman_decode(_ptr(d_huff), huff_bytes, n, dict_size, _ptr(out), _ptr(tmp), tb, _stream_ptr()),
          "huffman_decode")
    return out[:n]


def dualquant_decompress(dims, block_size, dict_size, code, outliers, consts):
    torch = _torch()
    dev = code.device
    n = int(np.prod(dims))
    out = torch.zeros(n + 8, dtype=torch.float32, device=dev)
    tb = lib().vsz_dualquant_decompress_tmp_bytes(len(dims), dims_arg(dims))
    tmp = torch.zeros(tb, dtype=torch.uint8, device=dev)
    check(lib().vsz_dualquant_decompress(len(dims), dims_arg(dims), block_size, dict_size, _ptr(code),
                                         _ptr(outliers) if outliers.numel() else C.c_void_p(tmp.data_ptr()),
                                         int(outliers.numel()), _ptr(consts), _ptr(out), _ptr(tmp), tb,
                                         _stream_ptr()), "dualquant_decompress")
    return out[:n]
