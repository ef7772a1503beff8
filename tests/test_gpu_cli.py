"""The `vecsz` command line on the GPU: compress, decompress and dry-run give the oracle's archive
bytes and reconstruction (the reference's), and the same as the library's host entry points; the
.sz file is [u64 lossless_size][u64 data_size][payload] (src/vecsz.cc:40-45)."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
import vecsz_gb300 as V
from vecsz_gb300 import _build, fields

pytestmark = pytest.mark.gpu


def run(*args):
    r = subprocess.run([_build.CLI, *args], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr + r.stdout
    return r


@pytest.fixture
def field(tmp_path):
    x = fields.grf_3d(32, 40, 48, seed=21).ravel()
    p = tmp_path / "field.f32"
    x.tofile(p)
    return x, str(p)


def read_sz(path):
    b = open(path, "rb").read()
    ls, ds = np.frombuffer(b[:16], np.uint64)
    return int(ls), int(ds), b[16:]


@pytest.mark.parametrize("mode,eb", [("r2r", 1e-4), ("abs", 1e-3)])
def test_cli_compress_decompress(cuda, field, mode, eb):
    x, path = field
    run("-z", "-t", "f32", "-m", mode, "-e", str(eb), "-d", "1024", "-l", "48,40,32", "-i", path)
    ls, ds, payload = read_sz(path + ".sz")
    ref = V.compress(x, (48, 40, 32), eb=eb, mode=mode, dict_size=1024, block_size=8)
    assert ls == 0 and ds == ref.data_size and payload == ref.data
    oa, _ = O.compress(x, (48, 40, 32), 8, 1024, eb, mode == "r2r")
    assert payload[:ds] == oa  # the packed block the reference writes
    run("-x", "-i", path + ".sz", "-o", path + ".x")
    y = np.fromfile(path + ".x", np.float32)
    np.testing.assert_array_equal(y.view(np.uint32), V.decompress(ref).view(np.uint32))
    vr = O.value_range(x) if mode == "r2r" else 0.0
    np.testing.assert_array_equal(y.view(np.uint32), O.decompress(oa, 8, 1024, vr).view(np.uint32))


def test_cli_dry_run_metrics(cuda, field):
    x, path = field
    r = run("-r", "-t", "f32", "-m", "abs", "-e", "1e-3", "-l", "48,40,32", "-i", path, "--show-histo", "-V")
    assert "PSNR" in r.stdout and "max.err.abs.val" in r.stdout and "histogram of original datum" in r.stdout
    line = next(s for s in r.stdout.splitlines() if "max.err.abs.val" in s)
    # the reference's rounding overshoot: at most eb plus two ulps of the value
    assert float(line.split()[-1]) <= 1e-3 + 2 * float(np.spacing(np.abs(x).max()))
    y = np.fromfile(path + ".sz.out", np.float32)
    ref = V.compress(x, (48, 40, 32), eb=1e-3, mode="abs", dict_size=4096, block_size=8)
    np.testing.assert_array_equal(y.view(np.uint32), V.decompress(ref).view(np.uint32))
    oa, _ = O.compress(x, (48, 40, 32), 8, 4096, 1e-3, False)
    np.testing.assert_array_equal(y.view(np.uint32), O.decompress(oa, 8, 4096).view(np.uint32))


@pytest.mark.parametrize("extra", [["-L", "gzip-gpu"], ["-L", "gzip"], ["-p", "block,avg"], ["-a", "--num-iter", "2"],
                                   ["-b", "16", "-s", "AVX512"]])
def test_cli_options(cuda, field, extra):
    x, path = field
    run("-z", "-t", "f32", "-m", "r2r", "-e", "1e-4", "-l", "48,40,32", "-i", path, "-o", path + ".sz", *extra)
    ls, ds, payload = read_sz(path + ".sz")
    if extra[0] == "-L":
        assert ls > 0 and payload[:2] in (b"\x78\x01", b"\x78\x5e")
    run("-x", "-i", path + ".sz")
    y = np.fromfile(path + ".sz.out", np.float32)
    assert y.size == x.size
    if extra[0] in ("-L", "-b"):
        bs = 16 if extra[0] == "-b" else 8
        ref = V.compress(x, (48, 40, 32), eb=1e-4, mode="r2r", dict_size=4096, block_size=bs)
        np.testing.assert_array_equal(y.view(np.uint32), V.decompress(ref).view(np.uint32))
        oa, _ = O.compress(x, (48, 40, 32), bs, 4096, 1e-4, True)
        if extra[0] == "-b":
            assert payload[:ds] == oa
        np.testing.assert_array_equal(y.view(np.uint32), O.decompress(oa, bs, 4096, O.value_range(x)).view(np.uint32))
    if extra[0] == "-p":
        ref = V.compress(x, (48, 40, 32), eb=1e-4, mode="r2r", dict_size=4096, block_size=8, padding="block,avg")
        assert payload == ref.data
        np.testing.assert_array_equal(y.view(np.uint32), V.decompress(ref).view(np.uint32))
        oa, _ = O.compress(x, (48, 40, 32), 8, 4096, 1e-4, True, pad_mode=O.PAD_BLOCK, pad_type=O.PADV_AVG)
        assert payload[:ds] == oa
    if extra[0] == "-a":
        rng = float(x.max()) - float(x.min())
        assert np.max(np.abs(y.astype(np.float64) - x)) <= 1e-4 * rng * (1 + 1e-5) + 2 * np.spacing(np.abs(x)).max()
