"""The named single-field configurations at their full sizes, through the C ABI:
  * 512^3 NYX-like field, r2r 1e-4 and 1e-3 -- the benchmark's own field (seed 1000): packed block
    byte-identical to the oracle's and reconstruction bit-identical; and on another seed the
    size-independent properties (deterministic archive, error bound within the reference's two-ulp
    overshoot, indexed and self-synchronising decoders agree, the trailer-free packed block decodes
    to the same field);
  * 1800x3600 CESM-like field (abs 1e-4) and 256x384x384 adversarial field (abs 1e-6: many
    outliers, a flat histogram, long codewords) -- packed blocks byte-identical to the oracle's and
    reconstructions bit-identical."""
import numpy as np
import pytest

import oracle as O
import vecsz_gb300 as V
from vecsz_gb300 import _lib as L
from vecsz_gb300 import fields

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("eb", [1e-4, 1e-3])
def test_nyx512_roundtrip_properties(cuda, eb):
    torch = cuda
    xt = fields.grf_3d_torch(512, 512, 512, seed=11).reshape(-1)
    codec = V.DeviceCodec((512, 512, 512), eb=eb, mode="r2r", dict_size=1024, block_size=8)
    codec.compress(xt)
    a1 = codec.archive_bytes()
    codec.compress(xt)
    assert codec.archive_bytes() == a1
    r = codec.result_host()
    assert 2.0 < 4 * xt.numel() / r.data_size < 40.0
    codec.prepare_decompress(a1)
    out = torch.empty_like(xt)
    d_arch = torch.from_numpy(np.concatenate([np.frombuffer(a1, np.uint8), np.zeros(64, np.uint8)])).cuda()
    codec.decompress(d_arch, out)
    assert codec.decompress_status() == 0
    ebf = codec._desc.eb_final
    err = (out.double() - xt.double()).abs()
    bound = ebf + 2.0 * torch.abs(xt.double()) * 2.0 ** -23
    assert bool((err <= bound).all())
    # trailer-free bytes: self-synchronising decode, same field
    y = V.decompress(a1[: r.data_size], r.data_size, 0, 1024, 8, "r2r", codec._desc.value_range)
    assert torch.equal(torch.from_numpy(y).cuda().view(torch.int32), out.view(torch.int32))


@pytest.mark.parametrize("eb", [1e-4, 1e-3])
def test_nyx512_bench_field_matches_oracle(cuda, eb):
    """The field bench.py times (512^3 NYX-like, seed 1000, r2r, dict 1024, block 8)."""
    torch = cuda
    xt = fields.grf_3d_torch(512, 512, 512, seed=1000).reshape(-1)
    x = xt.cpu().numpy()
    dims = (512, 512, 512)
    codec = V.DeviceCodec(dims, eb=eb, mode="r2r", dict_size=1024, block_size=8)
    codec.compress(xt)
    r = codec.result_host()
    a1 = codec.archive_bytes()
    oa, meta = O.compress(x, dims, 8, 1024, eb, True)
    assert r.n_outlier == meta["n_outlier"]
    assert a1[: r.data_size] == oa
    codec.prepare_decompress(a1)
    out = torch.empty_like(xt)
    d_arch = torch.from_numpy(np.concatenate([np.frombuffer(a1, np.uint8), np.zeros(64, np.uint8)])).cuda()
    codec.decompress(d_arch, out)
    assert codec.decompress_status() == 0
    want = O.decompress(oa, 8, 1024, O.value_range(x))
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32), want.view(np.uint32))


def test_cesm_fullsize_matches_oracle(cuda):
    x = fields.bump_field_2d(1800, 3600, seed=21).ravel()
    c = V.compress(x, (3600, 1800), eb=1e-4, mode="abs", dict_size=1024, block_size=8)
    oa, meta = O.compress(x, (3600, 1800), 8, 1024, 1e-4, False)
    assert c.data[: c.data_size] == oa
    np.testing.assert_array_equal(V.decompress(c).view(np.uint32), O.decompress(oa, 8, 1024).view(np.uint32))


def test_field_beyond_2_32_elements(cuda):
    """2048 x 2048 x 1032 (4.33e9 elements, 17.3 GB): element indices, byte offsets and payload bit
    offsets all pass 2^32.  Every plane from z = 1024 on starts at element index >= 2^32.  In abs
    mode a Lorenzo block's codes and reconstruction depend only on its own values, so block-aligned
    sub-boxes of the reconstruction must be bit-identical to the oracle's round trip of the same
    sub-box.  One of them straddles index 2^32 and one is at the field's end, both with outliers.
    The whole field is checked against the error bound."""
    torch = cuda
    nx, ny, nz = 2048, 2048, 1032
    n = nx * ny * nz
    assert n > 1 << 32
    if torch.cuda.mem_get_info()[0] < 160 * 2**30:
        pytest.skip("needs 160 GB of free device memory")
    eb = 1e-3
    z = torch.arange(nz, device="cuda", dtype=torch.float32).view(nz, 1, 1)
    y = torch.arange(ny, device="cuda", dtype=torch.float32).view(1, ny, 1)
    x = torch.arange(nx, device="cuda", dtype=torch.float32).view(1, 1, nx)
    xt = (torch.sin(x * 0.0123) + torch.cos(y * 0.0071)) * (1.0 + 0.5 * torch.sin(z * 0.0037))
    del x, y, z
    flat = xt.view(-1)
    flat[torch.arange(0, n, 999983, device="cuda")] += 1000.0  # outliers all over the field
    boxes = [(slice(1016, 1032), slice(1000, 1064), slice(512, 768)),  # planes both sides of 2^32
             (slice(1024, 1032), slice(1984, 2048), slice(1792, 2048))]  # the field's last block row
    for zz, yy, xx in boxes:
        xt[zz.start + 3, yy.start + 9, xx.start + 17] += 500.0
        xt[zz.stop - 2, yy.stop - 5, xx.stop - 30] -= 300.0

    codec = V.DeviceCodec((nx, ny, nz), eb=eb, mode="abs", dict_size=1024, block_size=8)
    codec.compress(flat)
    a1 = codec.archive_bytes()
    r = codec.result_host()
    assert r.n_outlier > n // 999983 and r.payload_bits > 1 << 32
    codec.prepare_decompress(a1)
    d_arch = torch.from_numpy(np.concatenate([np.frombuffer(a1, np.uint8), np.zeros(64, np.uint8)])).cuda()
    del a1
    out = torch.empty_like(flat)
    codec.decompress(d_arch, out)
    assert codec.decompress_status() == 0

    step = 1 << 28
    for s in range(0, n, step):
        xs = flat[s: s + step].double()
        err = (out[s: s + step].double() - xs).abs()
        assert bool((err <= eb + 2.0 * xs.abs() * 2.0 ** -23).all()), f"error bound broken in [{s}, {s + step})"
        del xs, err

    out3 = out.view(nz, ny, nx)
    for zz, yy, xx in boxes:
        sub = xt[zz, yy, xx].contiguous().cpu().numpy().ravel()
        dims = (xx.stop - xx.start, yy.stop - yy.start, zz.stop - zz.start)
        oa, meta = O.compress(sub, dims, 8, 1024, eb, False)
        assert meta["n_outlier"] > 0
        want = O.decompress(oa, 8, 1024)
        got = out3[zz, yy, xx].contiguous().cpu().numpy().ravel()
        np.testing.assert_array_equal(got.view(np.uint32), want.view(np.uint32))


def test_adversarial_fullsize_matches_oracle(cuda):
    x = fields.adversarial_3d(256, 384, 384, seed=22).ravel()
    dims = (384, 384, 256)
    c = V.compress(x, dims, eb=1e-6, mode="abs", dict_size=1024, block_size=8)
    oa, meta = O.compress(x, dims, 8, 1024, 1e-6, False)
    assert c.n_outlier == meta["n_outlier"] and c.n_outlier > 0
    assert c.data[: c.data_size] == oa
    np.testing.assert_array_equal(V.decompress(c).view(np.uint32), O.decompress(oa, 8, 1024).view(np.uint32))


def test_dequant_check_cached_per_workspace(cuda, monkeypatch):
    """Fields of 2^22 elements and more check the separable pass's two-operation dequantization
    once per error bound and keep the result in the decompress workspace: decompressing through one
    workspace fields with the same bound (a hit), another bound (a new check) and the first bound
    again gives the oracle's reconstruction each time; bytes planted where the result is kept, with
    a wrong check word, are not taken for a result."""
    torch = cuda
    monkeypatch.setenv("VSZ_DQ_NO_WAVEFRONT", "1")  # 2^24 elements: else the wavefront pass
    dims = (256, 256, 256)
    cases = [(fields.grf_3d(256, 256, 256, seed=s).ravel() * 0.01, eb) for s, eb in ((1, 1e-4), (2, 1e-4), (3, 1e-3))]
    cases.append(cases[0])
    codec = V.DeviceCodec(dims, eb=1e-4, mode="abs", dict_size=1024, block_size=8)
    for i, (x, eb) in enumerate(cases + [cases[1]]):
        oa, meta = O.compress(x, dims, 8, 1024, eb, False)
        want = O.decompress(oa, 8, 1024)
        c = V.compress(x, dims, eb=eb, mode="abs", dict_size=1024, block_size=8)
        assert c.data[: c.data_size] == oa
        codec.prepare_decompress(c.data, L.DecompressOpts(1024, 8, 0, 0.0))
        if i == len(cases):
            # the slot after the constants (workspace offset 256): c_d's bits, a mode, a bad check word
            key = np.array([2.0 * eb], np.float64).view(np.uint64)[0]
            junk = np.array([key, 1, 0, 12345], np.uint64).view(np.uint8)
            codec._dws[256:288].copy_(torch.from_numpy(junk.copy()))
        out = torch.empty(x.size, dtype=torch.float32, device="cuda")
        d_arch = torch.from_numpy(np.concatenate([np.frombuffer(c.data, np.uint8), np.zeros(64, np.uint8)])).cuda()
        codec.decompress(d_arch, out)
        assert codec.decompress_status() == 0
        np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32), want.view(np.uint32))
