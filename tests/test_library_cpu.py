"""The C-ABI library without a GPU: it builds, loads, exports every entry point that
include/vecsz_gb300.h declares, and its host-only entry points (argument checks, archive parsing,
the lossless pass) behave.  No device compute is called here."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import oracle as O
import vecsz_gb300 as V
from vecsz_gb300 import _lib as L
from conftest import ROOT, golden_cases, load_golden

HEADER = os.path.join(ROOT, "include", "vecsz_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(vsz_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "vsz_compress" in names and "vsz_decompress" in names and "vsz_dualquant" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol():
    lib = V.lib()
    for name in declared_functions():
        assert hasattr(lib, name), f"{name} declared in include/vecsz_gb300.h but not exported"
    assert set(declared_functions()) <= set(L.exported_symbols())


def test_status_strings():
    lib = V.lib()
    for s in range(10):
        assert lib.vsz_status_string(s)
    assert b"sm_103a" in lib.vsz_version()


def _bounds(eb=1e-4, mode=0, dict_size=1024, bs=8, dims=(64, 64, 64)):
    p = L.Params(eb, mode, dict_size, bs, 0)
    ws, cap = C.c_size_t(0), C.c_size_t(0)
    rc = V.lib().vsz_compress_bounds(C.byref(p), len(dims), L.dims_arg(dims), C.byref(ws), C.byref(cap))
    return rc, ws.value, cap.value


def test_argument_checks():
    assert _bounds()[0] == L.VSZ_OK
    assert _bounds(eb=0.0)[0] == L.VSZ_ERR_INVALID
    assert _bounds(eb=-1.0)[0] == L.VSZ_ERR_INVALID
    assert _bounds(eb=float("nan"))[0] == L.VSZ_ERR_INVALID
    assert _bounds(mode=3)[0] == L.VSZ_ERR_INVALID
    assert _bounds(dict_size=1023)[0] == L.VSZ_ERR_INVALID
    assert _bounds(dict_size=131072)[0] == L.VSZ_ERR_INVALID
    assert _bounds(bs=12)[0] == L.VSZ_ERR_UNSUPPORTED
    assert _bounds(bs=0)[0] == L.VSZ_ERR_INVALID
    assert _bounds(dims=(0, 4))[0] == L.VSZ_ERR_INVALID
    rc, ws, cap = _bounds(dims=(512, 512, 512))
    assert rc == 0 and ws > 512 ** 3 * 2 and cap > 512 ** 3 * 4


@pytest.mark.parametrize("name", golden_cases())
def test_archive_parse_matches_oracle(name):
    g = load_golden(name)
    d = V.parse_archive(g["archive"].tobytes())
    h = O.parse_header(g["archive"].tobytes())
    assert d.ndim == h["ndim"] and tuple(d.dims[: d.ndim]) == h["dims"] and d.eb == h["eb"]
    assert (d.n_pad, d.huff_bytes, d.n_outlier) == h["lens"]
    assert d.data_size == g["data_size"] and not d.has_trailer
    nc = int.from_bytes(g["huff"][:4].tobytes(), "big")
    assert d.node_count == nc
    assert d.payload_offset + d.payload_bytes == d.outlier_offset


def test_archive_parse_rejects_garbage():
    lib = V.lib()
    d = L.ArchiveDesc()
    for buf in (b"", b"\x07\x00\x00\x00" + b"\x00" * 60, b"\x02\x00\x00\x00" + b"\xff" * 60):
        a = np.frombuffer(buf + b"\x00" * 8, np.uint8)
        rc = lib.vsz_archive_parse(a.ctypes.data_as(C.c_void_p), len(buf), C.byref(d))
        assert rc == L.VSZ_ERR_CORRUPT
    g = load_golden("d2_bump_64x45")
    a = g["archive"]
    rc = lib.vsz_archive_parse(a.ctypes.data_as(C.c_void_p), a.size - 1, C.byref(d))  # truncated
    assert rc == L.VSZ_ERR_CORRUPT


def test_lossless_reads_reference_zstd_frame():
    g = load_golden("d2_bump_64x45")
    frame = g["zstd_frame"]
    lib = V.lib()
    assert lib.vsz_lossless_detect(frame.ctypes.data_as(C.c_void_p), frame.size) == 1
    out, ol = C.c_void_p(0), C.c_size_t(0)
    rc = lib.vsz_lossless_decompress(frame.ctypes.data_as(C.c_void_p), frame.size, g["data_size"], C.byref(out),
                                     C.byref(ol))
    if rc == L.VSZ_ERR_UNSUPPORTED:
        pytest.skip("libzstd not present on this machine")
    assert rc == 0 and ol.value == g["data_size"]
    assert C.string_at(out.value, ol.value) == g["archive"].tobytes()
    lib.vsz_free_host(out)


@pytest.mark.parametrize("which", [L.LOSSLESS_ZSTD, L.LOSSLESS_GZIP])
def test_lossless_roundtrip(which):
    g = load_golden("d3_tail_19x23x29")
    a = g["archive"]
    lib = V.lib()
    out, ol = C.c_void_p(0), C.c_size_t(0)
    rc = lib.vsz_lossless_compress(which, a.ctypes.data_as(C.c_void_p), a.size, C.byref(out), C.byref(ol))
    if rc == L.VSZ_ERR_UNSUPPORTED:
        pytest.skip("lossless library not present")
    assert rc == 0
    frame = np.frombuffer(C.string_at(out.value, ol.value), np.uint8).copy()
    lib.vsz_free_host(out)
    assert lib.vsz_lossless_detect(frame.ctypes.data_as(C.c_void_p), frame.size) == (1 if which == 1 else 2)
    back, bl = C.c_void_p(0), C.c_size_t(0)
    assert lib.vsz_lossless_decompress(frame.ctypes.data_as(C.c_void_p), frame.size, a.size, C.byref(back),
                                       C.byref(bl)) == 0
    assert C.string_at(back.value, bl.value) == a.tobytes()
    lib.vsz_free_host(back)
