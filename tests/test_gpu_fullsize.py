"""The named single-field configurations at their full sizes, through the C ABI:
  * 512^3 NYX-like field, r2r 1e-4 and 1e-3 -- size-independent properties (deterministic archive,
    error bound within the reference's two-ulp overshoot, indexed and self-synchronising decoders
    agree, the trailer-free packed block decodes to the same field);
  * 1800x3600 CESM-like field (abs 1e-4) and 256x384x384 adversarial field (abs 1e-6: many
    outliers, a flat histogram, long codewords) -- packed blocks byte-identical to the oracle's and
    reconstructions bit-identical."""
import numpy as np
import pytest

import oracle as O
import vecsz_gb300 as V
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


def test_cesm_fullsize_matches_oracle(cuda):
    x = fields.bump_field_2d(1800, 3600, seed=21).ravel()
    c = V.compress(x, (3600, 1800), eb=1e-4, mode="abs", dict_size=1024, block_size=8)
    oa, meta = O.compress(x, (3600, 1800), 8, 1024, 1e-4, False)
    assert c.data[: c.data_size] == oa
    np.testing.assert_array_equal(V.decompress(c).view(np.uint32), O.decompress(oa, 8, 1024).view(np.uint32))


def test_adversarial_fullsize_matches_oracle(cuda):
    x = fields.adversarial_3d(256, 384, 384, seed=22).ravel()
    dims = (384, 384, 256)
    c = V.compress(x, dims, eb=1e-6, mode="abs", dict_size=1024, block_size=8)
    oa, meta = O.compress(x, dims, 8, 1024, 1e-6, False)
    assert c.n_outlier == meta["n_outlier"] and c.n_outlier > 0
    assert c.data[: c.data_size] == oa
    np.testing.assert_array_equal(V.decompress(c).view(np.uint32), O.decompress(oa, 8, 1024).view(np.uint32))
