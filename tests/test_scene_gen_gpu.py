"""The device scene generator equals the host generator byte for byte."""
from __future__ import annotations

import numpy as np
import pytest

import tg_gb300 as tg

pytestmark = pytest.mark.gpu

CASES = [
    dict(kind=0, n_objects=1, min_cpa=4, max_cpa=4, seed=0, bernoulli_p=0.3, translation=(0.0, 0.0, 64.0)),
    dict(kind=0, n_objects=37, min_cpa=1, max_cpa=6, seed=9, bernoulli_p=0.45, box_min=(-200.0,) * 3,
         box_max=(200.0,) * 3, n_luts=3),
    dict(kind=1, n_objects=23, min_cpa=2, max_cpa=9, seed=1, noise_period=64.0, noise_threshold=0.5,
         box_min=(-300.0,) * 3, box_max=(300.0,) * 3, n_luts=4),
    dict(kind=1, n_objects=5, min_cpa=3, max_cpa=5, seed=77, noise_period=13.0, noise_threshold=0.35,
         box_min=(-50.0,) * 3, box_max=(50.0,) * 3),
]


@pytest.mark.parametrize("case", range(len(CASES)))
def test_device_generator_equals_host(ctx, case):
    kw = dict(CASES[case])
    host = tg.generate_scene(kw.pop("kind"), kw.pop("n_objects"), kw.pop("min_cpa"), kw.pop("max_cpa"),
                             kw.pop("seed"), **kw)
    kw = dict(CASES[case])
    sc = ctx.generate_scene(kw.pop("kind"), kw.pop("n_objects"), kw.pop("min_cpa"), kw.pop("max_cpa"),
                            kw.pop("seed"), **kw)
    dev = sc.download()
    assert np.array_equal(host.objects.view(np.uint8), dev.objects.view(np.uint8))
    assert np.array_equal(host.cluster_pointers, dev.cluster_pointers)
    assert np.array_equal(host.cluster_idx_to_object_idx, dev.cluster_idx_to_object_idx)
    assert np.array_equal(host.voxel_bits, dev.voxel_bits)
    assert np.array_equal(host.material_idx, dev.material_idx)
    assert np.array_equal(host.luts.view(np.uint8), dev.luts.view(np.uint8))
    assert 0 < np.unpackbits(dev.voxel_bits.view(np.uint8)).mean() < 1
    sc.close()
