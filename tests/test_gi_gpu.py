"""GPU parity of SVO traversal (tgx_svo_trace) and plain GI (tgx_gi_render)
against the CPU oracle, bit for bit, and of the traversal against the
reference's own tg_svo_traverse results (fixtures)."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import tg_gb300 as tg
from oracle_lib import OracleSvo, gi_render, svo_build_with_materials
from scenes import fuzz_scene, permute_clusters

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def gpu_trace(ctx, svo, o, d, max_steps=1 << 20):
    import torch
    to = torch.from_numpy(np.ascontiguousarray(o, np.float32)).cuda()
    td = torch.from_numpy(np.ascontiguousarray(d, np.float32)).cuda()
    t = torch.empty(len(o), dtype=torch.float32, device="cuda")
    v = torch.empty((len(o), 3), dtype=torch.int32, device="cuda")
    svo.trace(to, td, t, v, max_steps)
    ctx.sync()
    return t.cpu().numpy(), v.cpu().numpy()


@pytest.mark.parametrize("name", sorted(p.stem.replace("ref_trace_", "") for p in GOLD.glob("ref_trace_*.npz")))
def test_trace_matches_reference_hits(ctx, name):
    f = np.load(GOLD / f"ref_svo_{name}.npz")
    tr = np.load(GOLD / f"ref_trace_{name}.npz")
    s = tg.HostScene(f["objects"].view(tg.OBJECT_DTYPE), f["cluster_pointers"], f["c2o"], f["voxel_bits"])
    sc = ctx.upload(s)
    svo = ctx.svo_build(sc, f["mn"], 10)
    t, v = gpu_trace(ctx, svo, tr["origin"], tr["dir"])
    hit = t < 3e38
    assert np.array_equal(hit, tr["hit"] == 1)
    assert np.array_equal(v[hit], tr["voxel"][hit])
    svo.close()
    sc.close()


@pytest.mark.parametrize("seed,L", [(1, 8), (2, 9), (3, 10), (4, 11)])
def test_trace_bit_exact_vs_oracle(ctx, oracle, seed, L):
    s = permute_clusters(fuzz_scene(seed, n_objects=6, box=float(min(2 ** (L - 1) - 40, 150)), max_cpa=4), seed)
    mn = [-(2.0 ** (L - 1))] * 3
    blocks, words, _ = oracle.svo_build(s, mn, L)
    osvo = OracleSvo(oracle, blocks, words, None, mn, L)
    rng = np.random.default_rng(seed)
    n = 20000
    o = rng.uniform(-(2 ** (L - 1)) * 0.9, (2 ** (L - 1)) * 0.9, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d[::5, 0] = 0.0
    d[::7, 1] = 0.0
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    sc = ctx.upload(s)
    svo = ctx.svo_build(sc, mn, L)
    for steps in (1 << 20, 40):
        t, v = gpu_trace(ctx, svo, o, d, steps)
        ot, ov, oax, ost = osvo.trace(o, d, steps)
        assert np.array_equal(t.view(np.uint32), ot.view(np.uint32))
        hit = ot < 3e38
        assert np.array_equal(v[hit], ov[hit])
        if steps > 40:
            assert hit.sum() > 100
        else:
            assert ((ot >= 3e38) & (ost == 40)).sum() > 0   # some rays ran out of steps
    svo.close()
    sc.close()


@pytest.mark.parametrize("bounces,spp", [(1, 4), (2, 2)])
def test_gi_bit_exact_vs_oracle(ctx, oracle, bounces, spp):
    import torch
    s = fuzz_scene(17, n_objects=6, box=30.0, max_cpa=4)
    s.luts = np.ascontiguousarray(s.luts[:256])
    s.objects["lut_idx"] = 0
    mn = [-128.0, -128.0, -128.0]
    L = 8
    blocks, words, mats = svo_build_with_materials(oracle, s, mn, L)
    osvo = OracleSvo(oracle, blocks, words, mats, mn, L)
    view = tg.make_view((0.0, 5.0, -70.0), 0.1, float(np.pi), 1.1, 64, 48, 0.1, 300.0)
    params = tg.gi_params(spp=spp, bounces=bounces, seed=2, max_steps=256)
    sc = ctx.upload(s)
    svo = ctx.svo_build(sc, mn, L)
    vis = torch.empty(64 * 48, dtype=torch.int64, device="cuda")
    ctx.vis_render(sc, view, [vis])
    rgb = torch.empty(64 * 48 * 3, dtype=torch.float32, device="cuda")
    ctx.gi_render(sc, svo, view, vis, params, rgb)
    ctx.sync()
    assert ctx.device_error().code == 0
    g = rgb.cpu().numpy().reshape(-1, 3)
    visb = vis.cpu().numpy().view(np.uint64)
    ref = gi_render(oracle, osvo, s, view, params, visb)
    assert np.array_equal(g.view(np.uint32), ref.view(np.uint32)), np.abs(g - ref).max()
    assert (visb != np.uint64(tg.VIS_EMPTY)).sum() > 200
    svo.close()
    sc.close()
