"""The oracle's own scene generator and view builder (oracle/oracle_scene.c)
give the product's tgx_generate_scene / tgx_make_view results byte for byte.

The CPU reference arm of bench.py builds its inputs with the oracle's copy so
that it never loads the product library; these tests make sure both arms
still see the same scene and camera."""
from __future__ import annotations

import numpy as np
import pytest

import tg_gb300 as tg
from oracle_lib import VIEW_DTYPE, OBJECT_DTYPE


def _same_scene(a, b):
    assert a.objects.tobytes() == b.objects.tobytes()
    assert np.array_equal(a.cluster_pointers, b.cluster_pointers)
    assert np.array_equal(a.cluster_idx_to_object_idx, b.cluster_idx_to_object_idx)
    assert np.array_equal(a.voxel_bits.reshape(-1), b.voxel_bits.reshape(-1))
    assert np.array_equal(a.material_idx.reshape(-1), b.material_idx.reshape(-1))
    assert a.luts.tobytes() == b.luts.tobytes()


def test_dtypes_match_the_product_binding():
    assert VIEW_DTYPE == tg.VIEW_DTYPE
    assert OBJECT_DTYPE == tg.OBJECT_DTYPE


@pytest.mark.parametrize("kw", [
    dict(kind=0, n_objects=1, min_cpa=4, max_cpa=4, seed=0, bernoulli_p=0.3, translation=(0.0, 0.0, 64.0),
         n_luts=32),
    dict(kind=1, n_objects=24, min_cpa=2, max_cpa=6, seed=1, noise_period=64.0, noise_threshold=0.5,
         box_min=(-300.0,) * 3, box_max=(300.0,) * 3, n_luts=32),
    dict(kind=1, n_objects=7, min_cpa=1, max_cpa=3, seed=9, noise_period=17.0, noise_threshold=0.4,
         box_min=(-50.0, 0.0, 10.0), box_max=(50.0, 20.0, 90.0), n_luts=3),
])
def test_generator_equals_product(oracle, kw):
    kw = dict(kw)
    kind, n, lo, hi, seed = (kw.pop(k) for k in ("kind", "n_objects", "min_cpa", "max_cpa", "seed"))
    _same_scene(oracle.generate_scene(kind, n, lo, hi, seed, **kw), tg.generate_scene(kind, n, lo, hi, seed, **kw))


def test_benchmark_scene_objects_equal_product(oracle):
    """The whole 512-object benchmark scene (about 3.7e5 clusters, 213 MB)."""
    kw = dict(noise_period=64.0, noise_threshold=0.5, box_min=(-1024.0,) * 3, box_max=(1024.0,) * 3, n_luts=32)
    a = oracle.generate_scene(1, 512, 2, 16, 1, **kw)
    b = tg.generate_scene(1, 512, 2, 16, 1, **kw)
    _same_scene(a, b)


@pytest.mark.parametrize("args", [
    ((0.0, 0.0, 0.0), 0.0, float(np.pi), float(np.pi / 3), 1920, 1080, 0.1, 4096.0),
    ((3.0, -2.0, 7.5), 0.31, -1.2, 1.1, 97, 53, 0.1, 200.0),
    ((-60.0, 0.0, 0.0), 0.0, float(np.pi / 2), 1.3, 128, 16, 0.5, 300.0),
])
def test_view_equals_product(oracle, args):
    assert oracle.make_view(*args).tobytes() == tg.make_view(*args).tobytes()
