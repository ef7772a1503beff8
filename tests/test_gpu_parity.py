"""Parity of the CUDA path (through the C ABI) with the reference: every stage bit-exact against
the golden fixtures the reference produced, whole archives byte-identical, reconstructions
bit-identical, and random settings checked against the pinned oracle."""
import numpy as np
import pytest

import oracle as O
import vecsz_gb300 as V
from vecsz_gb300 import api, fields
from conftest import golden_cases, load_golden

pytestmark = pytest.mark.gpu
CASES = golden_cases()


def dev(cuda, a):
    return cuda.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("name", CASES)
def test_stages_match_reference(cuda, name):
    g = load_golden(name)
    x = dev(cuda, g["x"])
    consts, info, st = api.eb_setup(x, g["eb"], "r2r" if g["r2r"] else "abs")
    assert st == 0
    assert info["eb_final"] == g["eb_final"]
    code, hist, scratch, segc = api.dualquant(x, g["dims"], g["bs"], g["dict_size"], consts)
    cuda.cuda.synchronize()
    code_h = code.cpu().numpy().view(np.uint16)
    np.testing.assert_array_equal(code_h, g["code"])
    np.testing.assert_array_equal(hist.cpu().numpy(), np.bincount(g["code"].astype(np.int64),
                                                                  minlength=g["dict_size"]))
    outl = api.outlier_gather(g["dims"], segc, scratch)
    np.testing.assert_array_equal(outl.cpu().numpy().view(np.uint32), g["outliers"].view(np.uint32))
    cb, head, binfo = api.huffman_build(hist, g["dict_size"])
    nc, tree_bytes = int(binfo[0]), int(binfo[1])
    head_len = 8 + tree_bytes
    assert head.cpu().numpy()[:head_len].tobytes() == g["huff"][:head_len].tobytes()
    for off in (0, 1, 3):
        pay, bits, chunks = api.huffman_encode(code, cb, g["dict_size"], offset=off)
        nbytes = (bits + 7) // 8
        assert pay.cpu().numpy()[off:off + nbytes].tobytes() == g["huff"][head_len:].tobytes()
    # reconstruction from the reference's own codes and outliers
    d_out = api.dualquant_decompress(g["dims"], g["bs"], g["dict_size"], code, outl, consts)
    np.testing.assert_array_equal(d_out.cpu().numpy().view(np.uint32), g["xhat"].view(np.uint32))


@pytest.mark.parametrize("name", CASES)
def test_huffman_decode_reference_section(cuda, name):
    g = load_golden(name)
    huff = np.concatenate([g["huff"], np.zeros(16, np.uint8)])
    d = dev(cuda, huff)
    out = api.huffman_decode(d, g["huff"].size, g["code"].size, g["dict_size"])
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint16), g["code"])


@pytest.mark.parametrize("name", CASES)
def test_archive_and_roundtrip_match_reference(cuda, name):
    g = load_golden(name)
    codec = V.DeviceCodec(g["dims"], eb=g["eb"], mode="r2r" if g["r2r"] else "abs", dict_size=g["dict_size"],
                          block_size=g["bs"])
    x = dev(cuda, g["x"])
    codec.compress(x)
    r = codec.result_host()
    assert r.data_size == g["data_size"] and r.n_outlier == g["n_outlier"]
    ab = codec.archive_bytes()
    assert ab[: r.data_size] == g["archive"].tobytes()
    # our archive (with trailer -> indexed decode)
    codec.prepare_decompress(ab)
    assert codec._desc.has_trailer
    out = cuda.empty(g["x"].size, dtype=cuda.float32, device="cuda")
    d_arch = dev(cuda, np.concatenate([np.frombuffer(ab, np.uint8), np.zeros(64, np.uint8)]))
    codec.decompress(d_arch, out)
    assert codec.decompress_status() == 0
    np.testing.assert_array_equal(out.cpu().numpy().view(np.uint32), g["xhat"].view(np.uint32))
    # the reference's archive (no trailer -> self-synchronising decode), -d/-b/-m as given
    vr = O.value_range(g["x"]) if g["r2r"] else 0.0
    y = V.decompress(g["archive"].tobytes(), g["data_size"], 0, g["dict_size"], g["bs"],
                     "r2r" if g["r2r"] else "abs", vr)
    np.testing.assert_array_equal(y.view(np.uint32), g["xhat"].view(np.uint32))


def test_reference_zstd_archive(cuda):
    g = load_golden("d2_bump_64x45")
    try:
        y = V.decompress(g["zstd_frame"].tobytes(), g["data_size"], g["zstd_frame"].size, g["dict_size"], g["bs"])
    except V.VszError as e:
        if e.status == 6:
            pytest.skip("libzstd not present")
        raise
    np.testing.assert_array_equal(y.view(np.uint32), g["xhat"].view(np.uint32))


def _random_case(seed):
    rng = np.random.default_rng(1000 + seed)
    ndim = 1 + seed % 3
    if ndim == 1:
        dims = (int(rng.integers(1, 300000)),)
    elif ndim == 2:
        dims = (int(rng.integers(1, 700)), int(rng.integers(1, 400)))
    else:
        dims = tuple(int(rng.integers(1, 70)) for _ in range(3))
    n = int(np.prod(dims))
    bs = int(rng.choice([8, 8, 16, 32, 64]))
    dct = int(rng.choice([256, 1024, 1024, 4096, 65536]))
    eb = float(10 ** rng.uniform(-6, -1))
    kind = seed % 4
    if kind == 0:
        x = (np.cumsum(rng.standard_normal(n)) * 10 ** rng.uniform(-2, 3)).astype(np.float32)
    elif kind == 1:
        x = rng.standard_normal(n).astype(np.float32)
    elif kind == 2:
        x = (rng.standard_normal(n) * 1e6).astype(np.float32)  # |s| well above 2^24
    else:
        x = np.sin(np.arange(n) * 0.01).astype(np.float32) + 2.0
    r2r = bool(rng.integers(0, 2))
    return dims, bs, dct, eb, r2r, x


@pytest.fixture(params=["wavefront", "block"])
def dq_kernel(request, monkeypatch):
    """Small 3D fields run the wavefront reverse Lorenzo, or (VSZ_DQ_NO_WAVEFRONT) the block-8
    kernels that larger fields take."""
    if request.param == "block":
        monkeypatch.setenv("VSZ_DQ_NO_WAVEFRONT", "1")
    return request.param


@pytest.mark.parametrize("seed", range(24))
def test_random_settings_match_oracle(cuda, seed, dq_kernel):
    dims, bs, dct, eb, r2r, x = _random_case(seed)
    if r2r and O.value_range(x) == 0:
        r2r = False
    a_or, meta = O.compress(x, dims, bs, dct, eb, r2r)
    c = V.compress(x, dims, eb, "r2r" if r2r else "abs", dct, bs)
    assert c.data_size == len(a_or)
    assert c.data[: c.data_size] == a_or
    assert c.n_outlier == meta["n_outlier"]
    y = V.decompress(c)
    y_or = O.decompress(a_or, bs, dct, O.value_range(x) if r2r else 0.0)
    np.testing.assert_array_equal(y.view(np.uint32), y_or.view(np.uint32))


@pytest.mark.parametrize("dims", [(1,), (7,), (128,), (129,), (1, 1), (3, 1), (1, 9), (130, 2), (8, 8), (9, 9),
                                  (1, 1, 1), (2, 3, 5), (1, 1, 9), (129, 1, 1), (8, 8, 8), (9, 9, 9)])
def test_edge_shapes_match_oracle(cuda, dims, dq_kernel):
    rng = np.random.default_rng(sum(dims))
    x = np.cumsum(rng.standard_normal(int(np.prod(dims)))).astype(np.float32)
    for bs in (8, 16):
        a_or, _ = O.compress(x, dims, bs, 1024, 1e-3, False)
        c = V.compress(x, dims, 1e-3, "abs", 1024, bs)
        assert c.data[: c.data_size] == a_or
        y = V.decompress(c)
        np.testing.assert_array_equal(y.view(np.uint32), O.decompress(a_or, bs, 1024).view(np.uint32))


@pytest.mark.parametrize("d0", [5, 8, 13, 40, 64, 100, 128, 136, 200, 256, 264])
def test_outlier_dense_rows_match_oracle(cuda, d0, dq_kernel):
    """At least a tenth of the codes are outliers, on rows that one warp covers whole (d0 <= 256:
    an outlier's rank is carried from row to row; d0 <= 128: several y-blocks per warp) and on
    wider rows, 16-byte aligned rows or not, in 2D and 3D."""
    rng = np.random.default_rng(d0)
    for dims, sigma in (((d0, 37, 19), 0.03), ((d0, 150), 0.04)):
        x = (rng.standard_normal(int(np.prod(dims))) * sigma).astype(np.float32)
        a_or, meta = O.compress(x, dims, 8, 1024, 1e-4, False)
        assert meta["n_outlier"] > 0.1 * x.size  # all of them for 2D rows of d0 < 8
        c = V.compress(x, dims, 1e-4, "abs", 1024, 8)
        assert c.data[: c.data_size] == a_or
        y = V.decompress(c)
        np.testing.assert_array_equal(y.view(np.uint32), O.decompress(a_or, 8, 1024).view(np.uint32))


def test_large_3d_roundtrip_properties(cuda):
    """256^3 r2r field: deterministic archive, error bound (reference overshoot <= 2 ulp),
    indexed and self-synchronising decoders agree."""
    torch = cuda
    xt = fields.grf_3d_torch(256, 256, 256, seed=5)
    codec = V.DeviceCodec((256, 256, 256), eb=1e-4, mode="r2r", dict_size=1024, block_size=8)
    codec.compress(xt)
    a1 = codec.archive_bytes()
    codec.compress(xt)
    assert codec.archive_bytes() == a1
    r = codec.result_host()
    codec.prepare_decompress(a1)
    out = torch.empty_like(xt)
    d_arch = torch.from_numpy(np.concatenate([np.frombuffer(a1, np.uint8), np.zeros(64, np.uint8)])).cuda()
    codec.decompress(d_arch, out)
    assert codec.decompress_status() == 0
    ebf = codec._desc.eb_final
    err = (out.double() - xt.double()).abs()
    ulp = torch.from_numpy(np.spacing(np.abs(xt.cpu().numpy())).astype(np.float64)).cuda()
    assert bool((err <= ebf + 2 * ulp).all())
    # the same bytes without the trailer go through self-synchronisation
    y = V.decompress(a1[: r.data_size], r.data_size, 0, 1024, 8, "r2r", codec._desc.value_range)
    np.testing.assert_array_equal(y, out.cpu().numpy().ravel())


def test_corrupt_archive_is_reported(cuda):
    g = load_golden("d3_tail_19x23x29")
    bad = bytearray(g["archive"].tobytes())
    hoff = 4 * 4 + 8 + 24
    bad[hoff:hoff + 4] = (10 ** 6).to_bytes(4, "big")  # node count larger than the tree
    with pytest.raises(V.VszError):
        V.decompress(bytes(bad), g["data_size"], 0, g["dict_size"], g["bs"])
    with pytest.raises(V.VszError):
        V.decompress(g["archive"].tobytes()[:100], g["data_size"], 0, g["dict_size"], g["bs"])


def test_zero_range_r2r_is_an_error(cuda):
    x = np.full(1000, 3.0, np.float32)
    with pytest.raises(V.VszError) as e:
        V.compress(x, (1000,), 1e-3, "r2r", 1024, 8)
    assert e.value.status == 7


@pytest.fixture
def device_tree_builder():
    from vecsz_gb300 import _lib as L
    prev = L.lib().vsz_set_tree_builder(L.TREE_DEVICE)
    yield
    L.lib().vsz_set_tree_builder(prev)


@pytest.mark.parametrize("seed", range(0, 24, 3))
def test_device_tree_builder_matches_oracle(cuda, device_tree_builder, seed):
    """vsz_compress with the one-CTA device tree builder (the host builder is the default)."""
    dims, bs, dct, eb, r2r, x = _random_case(seed)
    if r2r and O.value_range(x) == 0:
        r2r = False
    a_or, meta = O.compress(x, dims, bs, dct, eb, r2r)
    c = V.compress(x, dims, eb, "r2r" if r2r else "abs", dct, bs)
    assert c.data[: c.data_size] == a_or and c.n_outlier == meta["n_outlier"]


def test_compress_replayed_from_cuda_graph(cuda):
    """vsz_compress captured in a CUDA graph (the device tree builder is used under capture) and
    replayed on new input matches the oracle for that input."""
    torch = cuda
    dims = (64, 48, 40)
    xa = fields.grf_3d(40, 48, 64, seed=21).ravel()
    xb = (fields.grf_3d(40, 48, 64, seed=22).ravel() * 3.0).astype(np.float32)
    codec = V.DeviceCodec(dims, eb=1e-4, mode="r2r", dict_size=1024, block_size=8)
    xd = dev(cuda, xa)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        codec.compress(xd)  # eager first call: one-time kernel attributes are set outside capture
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        codec.compress(xd)
    for x in (xb, xa):
        xd.copy_(torch.from_numpy(x))
        g.replay()
        torch.cuda.synchronize()
        a_or, meta = O.compress(x, dims, 8, 1024, 1e-4, True)
        r = codec.result_host()
        assert r.data_size == len(a_or) and r.n_outlier == meta["n_outlier"]
        assert codec.archive_bytes()[: r.data_size] == a_or


def test_long_codewords_match_oracle(cuda):
    """Codewords past the 12-bit primary table: 13..20 bits resolve through the secondary
    table, longer ones walk the tree.  1D field with 2 eb = 1 whose Lorenzo differences d have
    P(|d| = k) ~ 2^-k, so code lengths reach the mid 20s; archive, indexed decode and
    self-synchronising decode all checked against the oracle."""
    rng = np.random.default_rng(77)
    n = 1 << 22
    k = np.minimum(rng.geometric(0.5, n) - 1, 40)
    d = k * rng.choice(np.array([-1, 1]), n)
    s = np.cumsum(d).astype(np.int64)
    s -= int(np.round(s.mean()))
    x = np.clip(s, -30000, 30000).astype(np.float32)
    a_or, meta = O.compress(x, (n,), 8, 65536, 0.5, False)
    lens, *_ = O.huffman_codebook(np.bincount(O.dualquant(x, (n,), 8, 65536, 0.5)[0], minlength=65536).astype(np.uint64),
                                  65536)
    assert lens.max() > 20  # both the secondary table and the walk are exercised
    c = V.compress(x, (n,), 0.5, "abs", 65536, 8)
    assert c.data[: c.data_size] == a_or
    y_or = O.decompress(a_or, 8, 65536)
    np.testing.assert_array_equal(V.decompress(c).view(np.uint32), y_or.view(np.uint32))  # indexed
    y = V.decompress(a_or, len(a_or), 0, 65536, 8)                                          # self-sync
    np.testing.assert_array_equal(y.view(np.uint32), y_or.view(np.uint32))


@pytest.mark.parametrize("seed", [0, 4, 9, 14, 19])
def test_general_kernels_match_oracle(cuda, monkeypatch, seed):
    """The general indexed Huffman decoder (taken by trees with codewords over 32 bits) and the
    general reverse-Lorenzo kernel, forced on fields the fast kernels would otherwise take."""
    monkeypatch.setenv("VSZ_DECODE_NO_WINDOW", "1")
    monkeypatch.setenv("VSZ_FORCE_GENERAL_DECOMPRESS", "1")
    dims, bs, dct, eb, r2r, x = _random_case(seed)
    if r2r and O.value_range(x) == 0:
        r2r = False
    a_or, _ = O.compress(x, dims, bs, dct, eb, r2r)
    c = V.compress(x, dims, eb, "r2r" if r2r else "abs", dct, bs)
    assert c.data[: c.data_size] == a_or
    y_or = O.decompress(a_or, bs, dct, O.value_range(x) if r2r else 0.0)
    np.testing.assert_array_equal(V.decompress(c).view(np.uint32), y_or.view(np.uint32))


def test_long_codewords_general_decoder(cuda, monkeypatch):
    monkeypatch.setenv("VSZ_DECODE_NO_WINDOW", "1")
    test_long_codewords_match_oracle(cuda)


def test_long_codewords_dict4096_match_oracle(cuda):
    """Dictionary 4096 and a last chunk of 265 codes: the window decoder's secondary table and its
    tree walk, for codewords over 12 and 20 bits."""
    rng = np.random.default_rng(78)
    n = (1 << 21) + 777
    k = np.minimum(rng.geometric(0.45, n) - 1, 30)
    d = k * rng.choice(np.array([-1, 1]), n)
    x = np.cumsum(d).astype(np.float64)
    x = np.clip(x - np.round(x.mean()), -1e6, 1e6).astype(np.float32)
    a_or, meta = O.compress(x, (n,), 8, 4096, 0.5, False)
    lens, *_ = O.huffman_codebook(np.bincount(O.dualquant(x, (n,), 8, 4096, 0.5)[0], minlength=4096).astype(np.uint64),
                                  4096)
    assert lens.max() > 20 and lens.max() <= 32
    c = V.compress(x, (n,), 0.5, "abs", 4096, 8)
    assert c.data[: c.data_size] == a_or
    y_or = O.decompress(a_or, 8, 4096)
    np.testing.assert_array_equal(V.decompress(c).view(np.uint32), y_or.view(np.uint32))


@pytest.mark.parametrize("dims,bs,mode", [((96, 40), 8, "abs"), ((37, 41, 43), 8, "abs"), ((5000,), 16, "abs"),
                                          ((64, 64, 16), 16, "abs"), ((37, 41, 43), 8, "r2r"), ((64, 64, 16), 16, "r2r")])
def test_nan_inputs_keep_reference_bits(cuda, dims, bs, mode):
    """NaN inputs (quiet with payloads, negative, signalling): the reference's arithmetic keeps a
    NaN operand's bits, quieted, where the GPU's would give its canonical NaN; outliers and
    reconstructions must carry the reference's bits, in abs and r2r mode (whose value range skips
    the NaNs)."""
    rng = np.random.default_rng(sum(dims) + bs)
    n = int(np.prod(dims))
    x = (np.cumsum(rng.standard_normal(n)) * 0.1).astype(np.float32)
    bits = x.view(np.uint32)
    idx = rng.choice(n, 12, replace=False)
    bits[idx[:4]] = 0x7fc01234
    bits[idx[4:8]] = 0xffc00001
    bits[idx[8:]] = 0x7f800005   # signalling
    bits[0] = 0x7fc0beef
    if mode == "r2r":
        bits[0] = x.view(np.uint32)[1]  # a finite first value: the range skips NaNs after it
    c = V.compress(x, dims, eb=1e-3, mode=mode, dict_size=1024, block_size=bs)
    oa, _ = O.compress(x, dims, bs, 1024, 1e-3, mode == "r2r")
    assert c.data[:c.data_size] == oa
    y = V.decompress(c)
    vr = O.value_range(x) if mode == "r2r" else 0.0
    np.testing.assert_array_equal(y.view(np.uint32), O.decompress(oa, bs, 1024, vr).view(np.uint32))


def test_host_ops_match_host_entry_points(cuda):
    """Stream-ordered host-buffer ops: the same archive bytes and reconstruction as the one-call
    host entry points, with two ops in flight on different fields."""
    import ctypes as C

    from vecsz_gb300 import _lib as L
    from vecsz_gb300.api import HostOp
    torch = cuda
    fields_ = [(fields.grf_3d(40, 48, 64, seed=31).ravel(), (64, 48, 40), "r2r", 1e-3),
               (fields.bump_field_2d(90, 200, seed=32).ravel(), (200, 90), "abs", 1e-4)]
    ops = [HostOp(), HostOp()]
    pinned = []
    for x, dims, mode, eb in fields_:
        p = V.make_params(eb, mode, 1024, 8)
        cap = C.c_size_t(0)
        L.check(L.lib().vsz_compress_host_bound(C.byref(p), len(dims), L.dims_arg(dims), C.byref(cap)))
        h_in = torch.from_numpy(x).pin_memory()
        h_arch = torch.zeros(cap.value, dtype=torch.uint8).pin_memory()
        h_res = torch.zeros(8, dtype=torch.int64).pin_memory()
        h_out = torch.zeros(x.size, dtype=torch.float32).pin_memory()
        h_st = torch.zeros(1, dtype=torch.int32).pin_memory()
        pinned.append((x, dims, mode, eb, p, cap.value, h_in, h_arch, h_res, h_out, h_st))
    for op, (x, dims, mode, eb, p, cap, h_in, h_arch, h_res, h_out, h_st) in zip(ops, pinned):
        op.compress(p, dims, h_in.data_ptr(), h_arch.data_ptr(), cap, h_res.data_ptr())
    for op, (x, dims, mode, eb, p, cap, h_in, h_arch, h_res, h_out, h_st) in zip(ops, pinned):
        op.wait()
        r = h_res.numpy()
        assert int(r[5]) == 0
        total = int(r[0] + r[1])
        ref = V.compress(x, dims, eb=eb, mode=mode, dict_size=1024, block_size=8)
        assert h_arch.numpy()[:total].tobytes() == ref.data
        opts = L.DecompressOpts(1024, 8, 1 if mode == "r2r" else 0, 0.0)
        op.decompress(h_arch.data_ptr(), total, opts, h_out.data_ptr(), x.size, h_st.data_ptr())
    for op, (x, dims, mode, eb, p, cap, h_in, h_arch, h_res, h_out, h_st) in zip(ops, pinned):
        op.wait()
        assert int(h_st.item()) == 0
        ref = V.compress(x, dims, eb=eb, mode=mode, dict_size=1024, block_size=8)
        np.testing.assert_array_equal(h_out.numpy().view(np.uint32), V.decompress(ref).view(np.uint32))
    # an archive that does not fit is reported, not written past the buffer
    x, dims, mode, eb, p, cap, h_in, h_arch, h_res, h_out, h_st = pinned[0]
    ops[0].compress(p, dims, h_in.data_ptr(), h_arch.data_ptr(), 16, h_res.data_ptr())
    ops[0].wait()
    assert int(h_res.numpy()[5]) == L.VSZ_ERR_CAPACITY
    for op in ops:
        op.close()


@pytest.mark.parametrize("offset", ["none", "all", "half", "nan"])
def test_separable_reverse_lorenzo_matches_oracle(cuda, offset, dq_kernel):
    """3D block-8 fields with few outliers take the separable reverse Lorenzo (block kernels; a
    field this small takes the wavefront pass unless VSZ_DQ_NO_WAVEFRONT is set); blocks whose
    values reach 2^21 (here: a large offset at abs 1e-3, all or half of the field) or hold a NaN
    are redone in the reference's order.  Every case must match the oracle bit for bit."""
    nz, ny, nx = 40, 48, 64
    z, y, xx = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    x = (np.sin(xx / 9.0) * np.cos(y / 7.0) + 0.3 * np.sin(z / 5.0 + xx / 13.0)).astype(np.float64)
    if offset == "all":
        x += 5000.0
    elif offset == "half":
        x[nz // 2:] += 5000.0
    x = x.astype(np.float32).ravel()
    if offset == "nan":
        x[12345] = np.nan
    dims = (nx, ny, nz)
    c = V.compress(x, dims, eb=1e-3, mode="abs", dict_size=1024, block_size=8)
    a_or, meta = O.compress(x, dims, 8, 1024, 1e-3, False)
    assert c.data[: c.data_size] == a_or
    assert meta["n_outlier"] * 64 < x.size  # the separable pass is taken
    y_or = O.decompress(a_or, 8, 1024)
    np.testing.assert_array_equal(V.decompress(c).view(np.uint32), y_or.view(np.uint32))


@pytest.mark.parametrize("case", ["small", "offset", "nan", "abs", "bs16", "bs32_tail"])
def test_3d_value_scales_match_oracle(cuda, case, dq_kernel):
    """3D fields over value scales (prequantized values far below and far above 2^21, a NaN, abs
    and r2r) and block sizes 8, 16 and 32 with tail columns: archives byte-identical to the
    oracle's, reconstructions bit-identical."""
    nz, ny, nx = 36, 40, 64 if case != "bs32_tail" else 61
    z, y, xx = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    x = (np.sin(xx / 9.0) * np.cos(y / 7.0) + 0.3 * np.sin(z / 5.0 + xx / 13.0)).astype(np.float64)
    if case == "offset":
        x = 1000.0 + 0.001 * x  # range 0.0026: |s| ~ 1000 / (2e-4 * 0.0026) >> 2^21
    x = x.astype(np.float32).ravel()
    if case == "nan":
        x[777] = np.nan
    bs = {"bs16": 16, "bs32_tail": 32}.get(case, 8)
    mode, eb = ("abs", 1e-3) if case == "abs" else ("r2r", 1e-4)
    dims = (nx, ny, nz)
    c = V.compress(x, dims, eb=eb, mode=mode, dict_size=1024, block_size=bs)
    a_or, meta = O.compress(x, dims, bs, 1024, eb, mode == "r2r")
    assert c.data[: c.data_size] == a_or
    vr = O.value_range(x) if mode == "r2r" else 0.0
    np.testing.assert_array_equal(V.decompress(c).view(np.uint32), O.decompress(a_or, bs, 1024, vr).view(np.uint32))


@pytest.mark.parametrize("dims,bs,mode", [((96, 40), 8, "abs"), ((37, 41, 43), 8, "abs"), ((64, 64, 16), 8, "abs"),
                                          ((5000,), 16, "abs"), ((64, 48, 16), 16, "abs")])
def test_infinite_and_huge_inputs_match_oracle(cuda, dims, bs, mode):
    """Infinities and values near the float limit: outliers, codes and reconstructions follow the
    reference's IEEE arithmetic (overflowing prequantization, infinite residuals)."""
    rng = np.random.default_rng(7 * sum(dims) + bs)
    n = int(np.prod(dims))
    x = (np.cumsum(rng.standard_normal(n)) * 0.1).astype(np.float32)
    idx = rng.choice(n, 12, replace=False)
    x[idx[:3]] = np.inf
    x[idx[3:6]] = -np.inf
    x[idx[6:9]] = np.float32(3.0e38)
    x[idx[9:]] = np.float32(-1.7e38)
    c = V.compress(x, dims, eb=1e-3, mode=mode, dict_size=1024, block_size=bs)
    oa, _ = O.compress(x, dims, bs, 1024, 1e-3, mode == "r2r")
    assert c.data[:c.data_size] == oa
    np.testing.assert_array_equal(V.decompress(c).view(np.uint32), O.decompress(oa, bs, 1024).view(np.uint32))


def test_growing_dictionaries_in_one_process(cuda):
    """Dictionaries that grow from call to call in one process (3D: shared histogram + previous
    planes up to 96 KB of shared memory; 1D: histogram up to 64 KB): every launch still fits its
    kernel's shared-memory opt-in, and archives and reconstructions match the oracle."""
    rng = np.random.default_rng(31)
    x3 = fields.grf_3d(24, 40, 64, seed=5).ravel()
    x1 = (np.cumsum(rng.standard_normal(70001)) * 0.05).astype(np.float32)
    for dct in (2048, 8192, 16384):
        for x, dims in ((x3, (64, 40, 24)), (x1, (70001,))):
            c = V.compress(x, dims, eb=1e-4, mode="r2r", dict_size=dct, block_size=8)
            oa, _ = O.compress(x, dims, 8, dct, 1e-4, True)
            assert c.data[: c.data_size] == oa
            y = O.decompress(oa, 8, dct, O.value_range(x))
            np.testing.assert_array_equal(V.decompress(c).view(np.uint32), y.view(np.uint32))
