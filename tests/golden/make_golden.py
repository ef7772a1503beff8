"""Generates tests/golden/*.npz from the reference itself (szcompressor/vecSZ compiled from its
sources by oracle/ref/Makefile into oracle/_ref/libvszref.so; x86-64 only).

Each fixture holds a small seeded input field, its settings, and what the reference produced:
quant codes (c_lorenzo_*d1l), the gathered outlier list, the Huffman section (encode_withTree),
the packed block (Compress without -L), the zstd frame of Compress with -L zstd for one case, and
the reconstruction (Decompress; for 1D the per-block x_lorenzo_1d1l with a zero pad, because the
reference's 1D Decompress reads an uninitialised pad value).  The p*_ fixtures hold padded (-p)
cases: the input, the settings, the reference's packed block and its Decompress output, both run
on one OpenMP thread (the reference's pad index is shared between threads).

Run:  python tests/golden/make_golden.py      (needs the reference sources; rewrites the .npz)
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle as O  # noqa: E402
from vecsz_gb300 import fields  # noqa: E402


def walk(n, seed, scale=1.0):
    rng = np.random.default_rng(seed)
    return (np.cumsum(rng.standard_normal(n)) * scale).astype(np.float32)


def spiky(shape, seed):
    rng = np.random.default_rng(seed)
    x = rng.standard_normal(shape).astype(np.float32)
    idx = rng.choice(x.size, x.size // 10, replace=False)
    x.reshape(-1)[idx] = (rng.standard_cauchy(len(idx)) * 1e4).astype(np.float32)
    return x


# name, dims (x, y, z), block size, dict size, eb, r2r, field
CASES = [
    ("d1_walk_1003", (1003,), 8, 1024, 1e-3, False, lambda: walk(1003, 1)),
    ("d1_bs64_5000", (5000,), 64, 65536, 1e-5, False, lambda: walk(5000, 2, 0.1)),
    ("d2_bump_64x45", (64, 45), 8, 1024, 1e-4, False, lambda: fields.bump_field_2d(45, 64, seed=3)),
    ("d2_tailcols_77x41", (77, 41), 8, 1024, 1e-4, False, lambda: fields.bump_field_2d(41, 77, seed=4)),
    ("d2_bs32_100x90", (100, 90), 32, 256, 1e-2, False, lambda: fields.bump_field_2d(90, 100, seed=5)),
    ("d2_const_40x24", (40, 24), 8, 1024, 1e-3, False, lambda: np.full((24, 40), 0.37, np.float32)),
    ("d3_tail_19x23x29", (19, 23, 29), 8, 1024, 1e-3, False, lambda: fields.grf_3d(29, 23, 19, seed=6)),
    ("d3_bs16_r2r_33x17x9", (33, 17, 9), 16, 4096, 1e-3, True, lambda: fields.grf_3d(9, 17, 33, seed=7)),
    ("d3_large_16x16x16", (16, 16, 16), 8, 1024, 1e-6, False, lambda: spiky((16, 16, 16), 8)),
    ("d3_adv_24x20x18", (24, 20, 18), 8, 1024, 1e-6, False, lambda: fields.adversarial_3d(18, 20, 24, seed=9)),
]
ZSTD_CASE = "d2_bump_64x45"


def corner_1d():
    """1D block padding with raw (not prequantized) pad values, eb 0.5 (r = 1), radius 512: the
    first block's residual 511.7 gives code 1024 (= 2R, one past the dictionary), the second's
    -511.7 gives code 0 although quantizable (its outlier value is 0), the last block is partial."""
    hi = [513.0, 1.3, 2, 3, 4, 5, 6, 7]
    lo = [-510.0, 1.7, 1.0, 0.5, 0, 0, 0, 0]
    return np.array(hi + lo + [3.0] * 8 + hi[:5], np.float32)


# Padding (-p) cases: name, dims, bs, dict, eb, r2r, pad mode, pad type, constant, field.
# 2D/3D block/edge with max/min/avg use whole-block fields: the reference reads an uninitialised
# buffer for cells outside the field, so only whole blocks are deterministic there; the pad values
# of phantom blocks (get_nblk counts one past the field) stay unpinned ("pad_pinned" mask).
PAD_CASES = [
    ("p1_block_max_1003", (1003,), 8, 1024, 1e-3, False, 2, 0, 0.0, lambda: walk(1003, 21, 0.05)),
    ("p1_block_min_corner", (29,), 8, 1024, 0.5, False, 2, 1, 0.0, corner_1d),
    ("p1_edge_avg_4096", (4096,), 16, 1024, 1e-4, False, 3, 2, 0.0, lambda: walk(4096, 22, 0.05)),
    ("p1_global_min_777", (777,), 64, 4096, 1e-3, False, 1, 1, 0.0, lambda: walk(777, 23, 0.05)),
    ("p2_block_max_64x48", (64, 48), 8, 1024, 1e-3, False, 2, 0, 0.0, lambda: fields.bump_field_2d(48, 64, seed=24)),
    ("p2_edge_avg_96x64", (96, 64), 16, 1024, 1e-4, False, 3, 2, 0.0, lambda: fields.bump_field_2d(64, 96, seed=25)),
    ("p2_global_avg_77x41", (77, 41), 8, 1024, 1e-4, False, 1, 2, 0.0, lambda: fields.bump_field_2d(41, 77, seed=26)),
    ("p2_block_const_77x41", (77, 41), 8, 1024, 1e-3, False, 2, 3, 12.5,
     lambda: fields.bump_field_2d(41, 77, seed=27)),
    ("p3_block_avg_24x16x32", (24, 16, 32), 8, 1024, 1e-3, False, 2, 2, 0.0,
     lambda: fields.grf_3d(32, 16, 24, seed=28)),
    ("p3_edge_max_24x16x16", (24, 16, 16), 8, 1024, 1e-4, False, 3, 0, 0.0,
     lambda: fields.grf_3d(16, 16, 24, seed=29)),
    ("p3_global_max_19x23x29", (19, 23, 29), 8, 1024, 1e-3, False, 1, 0, 0.0,
     lambda: fields.grf_3d(29, 23, 19, seed=30)),
    ("p3_edge_const_19x23x29", (19, 23, 29), 8, 1024, 1e-3, False, 3, 3, -3.25,
     lambda: fields.grf_3d(29, 23, 19, seed=31)),
    ("p3_edge_min_r2r_16x16x16", (16, 16, 16), 16, 4096, 1e-3, True, 3, 1, 0.0,
     lambda: fields.grf_3d(16, 16, 16, seed=32)),
]


def main():
    if not O.ref_available():
        O.build_ref()
    if not O.ref_available():
        raise SystemExit("the reference library could not be built here")
    tmp = tempfile.mkdtemp()
    for name, dims, bs, dct, eb, r2r, gen in CASES:
        x = np.ascontiguousarray(gen(), np.float32).ravel()
        n = x.size
        f = os.path.join(tmp, name + ".f32")
        archive, dsz, _, nout = O.ref_compress(x, dims, bs, dct, eb, r2r, 0, f)
        hdr = O.parse_header(archive)
        ebf = eb * (O.value_range(x) if r2r else 1.0)
        code, outl_dense = O.ref_dualquant(x, dims, bs, dct, ebf)
        outliers = O.gather_outliers(code, outl_dense)
        huff = O.ref_huffman_encode(code, dct)
        if len(dims) == 1:
            xhat = O.ref_xlorenzo(code, outl_dense, dims, bs, dct, ebf)
        else:
            xhat = O.ref_decompress(archive, dsz, 0, n, bs, dct, r2r, f)
        extra = {}
        if name == ZSTD_CASE:
            frame, dsz2, lsz, _ = O.ref_compress(x, dims, bs, dct, eb, r2r, 1, f)
            assert dsz2 == dsz
            extra["zstd_frame"] = np.frombuffer(frame, np.uint8)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"), x=x, dims=np.array(dims, np.int64), bs=bs, dict_size=dct, eb=eb,
            r2r=int(r2r), eb_final=ebf, code=code.astype(np.uint16), outliers=outliers,
            huff=np.frombuffer(huff, np.uint8), archive=np.frombuffer(archive, np.uint8), data_size=dsz,
            n_outlier=nout, xhat=xhat, **extra)
        print(f"{name}: n={n} outliers={nout} huff={len(huff)} archive={len(archive)} "
              f"lens={hdr['lens']}")
    for name, dims, bs, dct, eb, r2r, mode, ptype, cst, gen in PAD_CASES:
        x = np.ascontiguousarray(gen(), np.float32).ravel()
        n = x.size
        f = os.path.join(tmp, name + ".f32")
        archive, nout = O.ref_compress_pad(x, dims, bs, dct, eb, r2r, mode, ptype, cst, f)
        xhat = O.ref_decompress(archive, len(archive), 0, n, bs, dct, r2r, f)
        hdr = O.parse_header(archive)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"), x=x, dims=np.array(dims, np.int64), bs=bs, dict_size=dct, eb=eb,
            r2r=int(r2r), pad_mode=mode, pad_type=ptype, pad_const=np.float32(cst),
            pad_pinned=O.ref_pinned_pads(dims, bs, mode, ptype), archive=np.frombuffer(archive, np.uint8),
            n_outlier=nout, xhat=xhat)
        print(f"{name}: n={n} outliers={nout} archive={len(archive)} lens={hdr['lens']}")


if __name__ == "__main__":
    main()
