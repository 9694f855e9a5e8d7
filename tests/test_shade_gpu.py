"""The shading pass (shading.frag:116-316) on the GPU equals the CPU oracle bit
for bit, in every mode (direct GGX shading and the debug views)."""
from __future__ import annotations

import numpy as np
import pytest

import tg_gb300 as tg
from oracle_lib import shade_render
from scenes import cfg1_scene, cfg1_view, fuzz_scene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", ["cfg1", "fuzz"])
def test_shade_bit_exact_vs_oracle(ctx, oracle, which):
    import torch
    if which == "cfg1":
        s, view = cfg1_scene(), cfg1_view(128, 96)
    else:
        s = fuzz_scene(19, n_objects=7, box=30.0, max_cpa=4)
        s.objects["lut_idx"] = 0
        view = tg.make_view((0.0, 5.0, -70.0), 0.1, float(np.pi), 1.1, 96, 64, 0.1, 300.0)
    w, h = int(view["width"][0]), int(view["height"][0])
    sc = ctx.upload(s)
    vis = torch.empty(w * h, dtype=torch.int64, device="cuda")
    ctx.vis_render(sc, view, [vis])
    rgba = torch.empty(w * h * 4, dtype=torch.float32, device="cuda")
    visb = None
    for mode in range(10):
        ctx.shade(sc, view, vis, mode, rgba)
        ctx.sync()
        if visb is None:
            visb = vis.cpu().numpy().view(np.uint64)
            assert 50 < (visb != np.uint64(tg.VIS_EMPTY)).sum() < w * h
        g = rgba.cpu().numpy().reshape(-1, 4)
        ref = shade_render(oracle, s, view, visb, mode)
        assert np.array_equal(g.view(np.uint32), ref.view(np.uint32)), (mode, np.abs(g - ref).max())
    sky = visb == np.uint64(tg.VIS_EMPTY)
    assert np.all(g[sky] == [1.0, 0.0, 1.0, 1.0])
    with pytest.raises(tg.TgxError):
        ctx.shade(sc, view, vis, 10, rgba)
    sc.close()
