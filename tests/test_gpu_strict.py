"""Strict error-bound mode (VSZ_FLAG_STRICT_EB): every element of the reconstruction within eb of
the input, checked in double precision, on the inputs where the reference's own arithmetic misses
eb -- |x| / 2eb beyond float precision, rounding overshoot, and the reference's dropped 2D tail
columns -- and on ordinary smooth fields, where it costs little."""
import numpy as np
import pytest

import vecsz_gb300 as V
from vecsz_gb300 import fields

pytestmark = pytest.mark.gpu


def _max_err(x, y):
    return float(np.max(np.abs(x.astype(np.float64) - y.astype(np.float64))))


def _ebf(x, eb, mode):
    return eb * (float(x.max()) - float(x.min())) if mode == "r2r" else eb


def test_strict_fixes_what_the_reference_misses(cuda):
    cases = [
        (fields.adversarial_3d(24, 40, 64, seed=2).ravel(), (64, 40, 24), 1e-6, "abs", 8),   # huge |x| / 2eb
        (fields.bump_field_2d(60, 203, seed=3).ravel(), (203, 60), 1e-4, "abs", 8),          # 2D tail columns
    ]
    for x, dims, eb, mode, bs in cases:
        compat = V.compress(x, dims, eb, mode, 1024, bs)
        y0 = V.decompress(compat)
        assert _max_err(x, y0) > eb  # the reference's arithmetic misses eb here
        c = V.compress(x, dims, eb, mode, 1024, bs, strict=True)
        assert V.parse_archive(c.data).strict == 1
        y = V.decompress(c)
        assert _max_err(x, y) <= eb


@pytest.mark.parametrize("nd,bs", [(1, 8), (2, 8), (2, 16), (3, 8), (3, 16), (3, 64)])
def test_strict_smooth_fields(cuda, nd, bs):
    rng = np.random.default_rng(nd * 100 + bs)
    if nd == 1:
        x = (np.cumsum(rng.standard_normal(200003)) * 0.01).astype(np.float32)
        dims = (x.size,)
    elif nd == 2:
        x = fields.bump_field_2d(300, 517, seed=bs).ravel()
        dims = (517, 300)
    else:
        x = fields.grf_3d(40, 50, 93, seed=bs).ravel()
        dims = (93, 50, 40)
    for mode, eb in (("r2r", 1e-4), ("abs", 1e-3)):
        c = V.compress(x, dims, eb, mode, 1024, bs, strict=True)
        y = V.decompress(c)
        assert _max_err(x, y) <= _ebf(x, eb, mode)
        base = V.compress(x, dims, eb, mode, 1024, bs)
        assert c.data_size <= 1.25 * base.data_size + 4096


def test_batch_refuses_strict(cuda):
    x = cuda.zeros(4096, dtype=cuda.float32, device="cuda") + 1.0
    with pytest.raises(V.VszError) as e:
        V.BatchCompressor([{"x": x, "dims": (4096,), "eb": 1e-3, "mode": "abs", "dict_size": 1024,
                            "block_size": 8, "strict": True}])
    assert e.value.status == 6
