"""The batched decompressor (vsz_dbatch_*): many archives of uneven shapes, dimensionalities, error
bounds and dictionaries in one launch sequence.  Every field's reconstruction must be bit-identical
to single-field vsz_decompress of the same archive (and to the oracle's on a few of them); a
damaged archive fails alone; the sequence replays from a CUDA graph; archives the batch does not
take (block sizes other than 8, padding, strict mode) are refused."""
import numpy as np
import pytest

import oracle as O
import vecsz_gb300 as V
from vecsz_gb300 import _lib as L
from vecsz_gb300 import fields

pytestmark = pytest.mark.gpu


def _mixed_archives(seed, n):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        nd = int(rng.choice([1, 2, 3], p=[0.2, 0.4, 0.4]))
        if nd == 1:
            dims = (int(rng.integers(1, 300000)),)
            x = (np.cumsum(rng.standard_normal(dims[0])) * 0.01).astype(np.float32)
        elif nd == 2:
            dims = (int(rng.integers(1, 900)), int(rng.integers(1, 600)))
            x = fields.bump_field_2d(dims[1], dims[0], seed=seed * 100 + i).ravel()
        else:
            dims = tuple(int(v) for v in rng.integers(1, 90, 3))
            x = fields.grf_3d(dims[2], dims[1], dims[0], seed=seed * 100 + i).ravel()
        mode = "r2r" if rng.random() < 0.7 else "abs"
        if mode == "r2r" and (x.size < 2 or float(x.max()) == float(x.min())):
            mode = "abs"
        eb = float(10 ** rng.uniform(-5, -2))
        dct = int(rng.choice([256, 1024, 1024, 4096, 65536]))
        c = V.compress(x, dims, eb=eb, mode=mode, dict_size=dct, block_size=8)
        out.append((x, dims, eb, mode, dct, c))
    return out


def test_dbatch_matches_single_field_decompress(cuda):
    items = _mixed_archives(5, 36)
    # a constant field (one-symbol tree), dense outliers (the adversarial field) and a 3D field
    # wide enough for the separable pass
    xc = np.full(70000, 3.25, np.float32)
    items.append((xc, (70000,), 1e-3, "abs", 1024, V.compress(xc, (70000,), 1e-3, "abs", 1024, 8)))
    xa = fields.adversarial_3d(24, 40, 64, seed=9).ravel()
    items.append((xa, (64, 40, 24), 1e-6, "abs", 1024, V.compress(xa, (64, 40, 24), 1e-6, "abs", 1024, 8)))
    xg = fields.grf_3d(40, 64, 256, seed=10).ravel()
    items.append((xg, (256, 64, 40), 1e-4, "r2r", 1024, V.compress(xg, (256, 64, 40), 1e-4, "r2r", 1024, 8)))
    b = V.BatchDecompressor([c.data for *_, c in items])
    b.decompress()
    cuda.cuda.synchronize()
    assert b.statuses() == [0] * len(items)
    for i, (x, dims, eb, mode, dct, c) in enumerate(items):
        want = V.decompress(c)
        got = b.outputs[i].cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), f"field {i} {dims} {mode} dict {dct}"
    # the oracle on three of them
    for i in (0, len(items) - 2, len(items) - 1):
        x, dims, eb, mode, dct, c = items[i]
        oa, _ = O.compress(x, dims, 8, dct, eb, mode == "r2r")
        assert c.data[: c.data_size] == oa
        y = O.decompress(oa, 8, dct, O.value_range(x) if mode == "r2r" else 0.0)
        np.testing.assert_array_equal(b.outputs[i].cpu().numpy().view(np.uint32), y.view(np.uint32))


def test_dbatch_graph_replay_and_damaged_field(cuda):
    torch = cuda
    items = _mixed_archives(6, 10)
    archives = [bytearray(c.data) for *_, c in items]
    # damage field 3's decode index (its first chunk's bit count, one more than the chunk holds):
    # its decode must fail alone
    d = V.parse_archive(bytes(archives[3]))
    assert d.has_trailer and d.n_chunks >= 1
    k = int(d.index_offset)
    v = int.from_bytes(archives[3][k: k + 2], "little") + 1
    archives[3][k: k + 2] = v.to_bytes(2, "little")
    b = V.BatchDecompressor([bytes(a) for a in archives])
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        b.decompress(s)
    s.synchronize()
    st = b.statuses()
    assert st[3] == L.VSZ_ERR_CORRUPT
    assert all(v == 0 for i, v in enumerate(st) if i != 3)
    first = [o.clone() for o in b.outputs]
    for o in b.outputs:
        o.fill_(float("nan"))
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        b.decompress(s)
    g.replay()
    torch.cuda.synchronize()
    for i, (x, dims, eb, mode, dct, c) in enumerate(items):
        if i == 3:
            continue
        assert torch.equal(b.outputs[i].view(torch.int32), first[i].view(torch.int32))
        assert np.array_equal(b.outputs[i].cpu().numpy().view(np.uint32), V.decompress(c).view(np.uint32))
    assert b.statuses()[3] == L.VSZ_ERR_CORRUPT


@pytest.mark.parametrize("kind", ["bs16", "pad", "strict"])
def test_dbatch_refuses_what_it_does_not_take(cuda, kind):
    x = fields.grf_3d(16, 16, 32, seed=3).ravel()
    if kind == "bs16":
        c = V.compress(x, (32, 16, 16), 1e-3, "abs", 1024, 16)
    elif kind == "pad":
        c = V.compress(x, (32, 16, 16), 1e-3, "abs", 1024, 8, padding="block,avg")
    else:
        c = V.compress(x, (32, 16, 16), 1e-3, "abs", 1024, 8, strict=True)
    with pytest.raises(L.VszError) as e:
        V.BatchDecompressor([c.data])
    assert e.value.status == L.VSZ_ERR_UNSUPPORTED
