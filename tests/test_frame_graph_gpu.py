"""Batched frames as a CUDA graph (each job's sorting passes on its own
branch, one persistent tile launch over all jobs through a work queue):
replays equal individual tgx_vis_render calls bit for bit, across scenes,
uneven resolutions, repeated launches and new cameras."""
from __future__ import annotations

import numpy as np
import pytest

import tg_gb300 as tg
from scenes import cfg1_scene, fuzz_scene

pytestmark = pytest.mark.gpu


def _views(rng, sizes, far=300.0):
    out = []
    for w, h in sizes:
        pos = rng.uniform(-60.0, 60.0, 3)
        out.append(tg.make_view(tuple(pos), float(rng.uniform(-0.4, 0.4)), float(rng.uniform(0, 2 * np.pi)),
                                float(np.pi / 3), w, h, 0.1, far))
    return np.concatenate(out)


def test_frame_graph_equals_individual_calls(ctx):
    import torch
    rng = np.random.default_rng(3)
    scenes = [ctx.upload(fuzz_scene(31, n_objects=8, box=40.0, max_cpa=5)), ctx.upload(cfg1_scene())]
    sizes = [[(320, 240), (97, 61), (640, 480)], [(256, 256), (130, 70)]]
    views = [_views(rng, s) for s in sizes]
    ref = [[torch.empty(w * h, dtype=torch.int64, device="cuda") for w, h in s] for s in sizes]
    for sc, v, o in zip(scenes, views, ref):
        ctx.vis_render(sc, v, o)
    outs = [[torch.full((w * h,), 7, dtype=torch.int64, device="cuda") for w, h in s] for s in sizes]
    g = ctx.frame_graph([(sc, v, o) for sc, v, o in zip(scenes, views, outs)])
    # per job: cull, record origins with counts, prefix, finalize with the
    # group scan (small frames), bin fill; then one persistent tile launch
    # over both jobs' tiles
    assert g.kernels == 2 * 5 + 1
    for o in outs:
        for t in o:
            t.fill_(7)
    launches0 = ctx.launches()
    for _ in range(2):
        g.launch()
    ctx.sync()
    assert ctx.launches() - launches0 == 2 * g.kernels
    assert ctx.device_error().code == 0
    for a, b in zip(ref, outs):
        for x, y in zip(a, b):
            assert torch.equal(x, y)
    # new cameras, same resolutions
    views2 = [_views(rng, s) for s in sizes]
    for j, v in enumerate(views2):
        g.set_views(j, v)
    g.launch()
    for sc, v, o in zip(scenes, views2, ref):
        ctx.vis_render(sc, v, o)
    ctx.sync()
    for a, b in zip(ref, outs):
        for x, y in zip(a, b):
            assert torch.equal(x, y)
    with pytest.raises(tg.TgxError):
        g.set_views(0, _views(rng, [(320, 240), (97, 61), (640, 482)]))
    g.close()
    for sc in scenes:
        sc.close()
