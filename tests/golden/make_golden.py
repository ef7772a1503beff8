"""Generates tests/golden/*.npz from the reference itself (szcompressor/vecSZ compiled from its
sources by oracle/ref/Makefile into oracle/_ref/libvszref.so; x86-64 only).

Each fixture holds a small seeded input field, its settings, and what the reference produced:
quant codes (c_lorenzo_*d1l), the gathered outlier list, the Huffman section (encode_withTree),
the packed block (Compress without -L), the zstd frame of Compress with -L zstd for one case, and
the reconstruction (Decompress; for 1D the per-block x_lorenzo_1d1l with a zero pad, because the
reference's 1D Decompress reads an uninitialised pad value).

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


if __name__ == "__main__":
    main()
