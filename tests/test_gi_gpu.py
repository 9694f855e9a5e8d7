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
    # aim most rays at the region that holds the objects
    aim = rng.uniform(-120.0, 120.0, (n, 3))
    d = aim - o
    d[::3] = rng.normal(size=(len(d[::3]), 3))
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
    work = ctx.gi_work()   # the traversal's own counts of this frame
    assert 0 < work.rays and work.rays <= work.dda_steps <= 256 * work.rays
    assert (visb != np.uint64(tg.VIS_EMPTY)).sum() > 200
    svo.close()
    sc.close()


def _scene_setup(ctx, seed=17):
    import torch
    s = fuzz_scene(seed, n_objects=6, box=30.0, max_cpa=4)
    s.objects["lut_idx"] = 0
    mn = [-128.0, -128.0, -128.0]
    sc = ctx.upload(s)
    svo = ctx.svo_build(sc, mn, 8)
    view = tg.make_view((0.0, 5.0, -70.0), 0.1, float(np.pi), 1.1, 96, 64, 0.1, 300.0)
    vis = torch.empty(96 * 64, dtype=torch.int64, device="cuda")
    ctx.vis_render(sc, view, [vis])
    return s, sc, svo, view, vis


def test_cached_gi_with_zero_cache_equals_plain_sky_only(ctx):
    """No sun and an all-zero cache: a bounce that hits contributes 0 in both
    paths, one that misses sees the sky, so cached GI equals plain 1-bounce GI
    bit for bit."""
    import torch
    s, sc, svo, view, vis = _scene_setup(ctx)
    cache = tg.Cache(ctx, seed=1)
    cache.set_weights(np.zeros(cache.n_params, np.float32))
    params = tg.gi_params(spp=4, bounces=1, seed=2, sun_radiance=(0.0, 0.0, 0.0), sky_radiance=(0.4, 0.5, 0.6))
    cp = tg.cache_gi_params((-40.0,) * 3, (40.0,) * 3, n_train=0, train_steps=0)
    a = torch.empty(96 * 64 * 3, dtype=torch.float32, device="cuda")
    b = torch.empty_like(a)
    ctx.gi_render(sc, svo, view, vis, params, a)
    ctx.gi_render_cached(sc, svo, cache, view, vis, params, cp, b)
    ctx.sync()
    assert ctx.device_error().code == 0
    assert torch.equal(a, b)
    cache.close(); svo.close(); sc.close()


def test_cached_gi_learns_toward_the_plain_estimate(ctx):
    """Online training over frames brings the cached 2-bounce GI toward a
    high-spp plain 2-bounce render of the same frame."""
    import torch
    s, sc, svo, view, vis = _scene_setup(ctx, seed=23)
    ref = torch.empty(96 * 64 * 3, dtype=torch.float32, device="cuda")
    ctx.gi_render(sc, svo, view, vis, tg.gi_params(spp=256, bounces=2, seed=9), ref)
    cache = tg.Cache(ctx, seed=2)
    cp = tg.cache_gi_params((-40.0,) * 3, (40.0,) * 3, n_train=8192, train_spp=16, train_steps=4, lr=1e-2)
    out = torch.empty_like(ref)
    hit = (vis.cpu().numpy().view(np.uint64) != np.uint64(tg.VIS_EMPTY))
    r = ref.cpu().numpy().reshape(-1, 3)[hit]

    def relmse():
        x = out.cpu().numpy().reshape(-1, 3)[hit]
        return float(np.mean((x - r) ** 2 / (r ** 2 + 1e-2)))

    errs = []
    for f in range(40):
        ctx.gi_render_cached(sc, svo, cache, view, vis, tg.gi_params(spp=4, bounces=2, seed=2, frame=f), cp, out)
        if f in (0, 39):
            ctx.sync()
            errs.append(relmse())
    assert ctx.device_error().code == 0
    assert errs[1] < 0.5 * errs[0], errs
    cache.close(); svo.close(); sc.close()


def _cached_relmse_after(ctx, sc, svo, view, vis, ref, hit, cp, frames=40, spp=4):
    import torch
    cache = tg.Cache(ctx, seed=2)
    out = torch.empty_like(ref)
    for f in range(frames):
        ctx.gi_render_cached(sc, svo, cache, view, vis, tg.gi_params(spp=spp, bounces=2, seed=2, frame=f), cp, out)
    ctx.sync()
    assert ctx.device_error().code == 0
    cache.close()
    r = ref.cpu().numpy().reshape(-1, 3)[hit]
    x = out.cpu().numpy().reshape(-1, 3)[hit]
    return float(np.mean((x - r) ** 2 / (r ** 2 + 1e-2))), out


def test_pixel_point_network_lowers_the_error(ctx):
    """The cache's second network, trained on the pixels' own sample means,
    lowers the error of 4-spp cached GI against a 256-spp plain render.  With
    weight 0 it trains but leaves every pixel bit-equal to cached GI without
    it (bounce network frozen: its training batch comes from hits appended in
    arbitrary order, so two trained runs differ in the last bits)."""
    import torch
    s, sc, svo, view, vis = _scene_setup(ctx, seed=23)
    ref = torch.empty(96 * 64 * 3, dtype=torch.float32, device="cuda")
    ctx.gi_render(sc, svo, view, vis, tg.gi_params(spp=256, bounces=2, seed=9), ref)
    hit = (vis.cpu().numpy().view(np.uint64) != np.uint64(tg.VIS_EMPTY))
    box = ((-40.0,) * 3, (40.0,) * 3)
    frozen = dict(n_train=0, train_spp=8, train_steps=4, lr=1e-2)
    _, out0 = _cached_relmse_after(ctx, sc, svo, view, vis, ref, hit, tg.cache_gi_params(*box, **frozen), frames=8)
    _, out_off = _cached_relmse_after(ctx, sc, svo, view, vis, ref, hit,
                                      tg.cache_gi_params(*box, **frozen, primary_weight=0.0, n_train_primary=4096),
                                      frames=8)
    assert torch.equal(out0, out_off)
    base = dict(n_train=8192, train_spp=8, train_steps=4, lr=1e-2)
    e0, _ = _cached_relmse_after(ctx, sc, svo, view, vis, ref, hit, tg.cache_gi_params(*box, **base))
    e1, _ = _cached_relmse_after(ctx, sc, svo, view, vis, ref, hit,
                                 tg.cache_gi_params(*box, **base, primary_weight=1.0, n_train_primary=4096))
    assert e1 < 0.9 * e0, (e0, e1)   # 0.70-0.81 over runs: the training batches vary run to run
    with pytest.raises(tg.TgxError):
        cache = tg.Cache(ctx, seed=2)
        try:
            ctx.gi_render_cached(sc, svo, cache, view, vis, tg.gi_params(spp=4, bounces=2),
                                 tg.cache_gi_params(*box, **base, primary_weight=1.5), torch.empty_like(ref))
        finally:
            cache.close()
    svo.close(); sc.close()


def test_shrinkage_is_one_weight_per_pixel_between_samples_and_network(ctx):
    """With both networks frozen, a 3-spp cached pixel is its samples' mean m
    moved toward the pixel-point network's prediction P by one weight k in
    [0, w] for all three channels: out - out(w=0) = k (out(P) - out(w=0)),
    where out(P) is the 1-spp render with w = 1 (P alone).  Direct light and
    albedo are the same in all three renders."""
    import torch
    s, sc, svo, view, vis = _scene_setup(ctx, seed=31)
    box = ((-40.0,) * 3, (40.0,) * 3)
    cache = tg.Cache(ctx, seed=3)
    out = torch.empty(96 * 64 * 3, dtype=torch.float32, device="cuda")
    train = tg.cache_gi_params(*box, n_train=8192, train_spp=8, train_steps=4, primary_weight=1.0,
                               n_train_primary=4096)
    for f in range(40):
        ctx.gi_render_cached(sc, svo, cache, view, vis, tg.gi_params(spp=4, bounces=2, seed=2, frame=f), train, out)
    w = 0.8
    renders = {}
    for name, spp, weight in (("m", 3, 0.0), ("P", 1, 1.0), ("blend", 3, w)):
        cp = tg.cache_gi_params(*box, n_train=0, train_steps=0, primary_weight=weight)
        o = torch.empty_like(out)
        ctx.gi_render_cached(sc, svo, cache, view, vis, tg.gi_params(spp=spp, bounces=2, seed=2, frame=9), cp, o)
        renders[name] = o
    ctx.sync()
    assert ctx.device_error().code == 0
    cache.close()
    hit = vis.cpu().numpy().view(np.uint64) != np.uint64(tg.VIS_EMPTY)
    m, p_, b = (renders[k].cpu().numpy().reshape(-1, 3)[hit].astype(np.float64) for k in ("m", "P", "blend"))
    d, e = p_ - m, b - m
    big = np.abs(d).max(axis=1) > 1e-2
    assert big.sum() > 200
    k = (e[big] * d[big]).sum(1) / (d[big] * d[big]).sum(1)
    assert np.abs(e[big] - k[:, None] * d[big]).max() < 1e-5
    assert k.min() > -1e-5 and k.max() < w + 1e-5
    assert np.ptp(k) > 0.05   # the weight varies over the pixels


def test_trace_steps_per_round_changes_no_result(ctx):
    """tgx_set_trace_steps only reschedules the persistent traversal: GI is bit-equal for every setting."""
    import torch
    s, sc, svo, view, vis = _scene_setup(ctx, seed=29)
    params = tg.gi_params(spp=2, bounces=2, seed=4)
    outs = []
    for k in (1, 3, 8, 64):
        ctx.set_trace_steps(k)
        rgb = torch.empty(96 * 64 * 3, dtype=torch.float32, device="cuda")
        ctx.gi_render(sc, svo, view, vis, params, rgb)
        outs.append(rgb)
    ctx.set_trace_steps(8)
    ctx.sync()
    assert ctx.device_error().code == 0
    for o in outs[1:]:
        assert torch.equal(outs[0], o)
    for bad in (0, 257):
        with pytest.raises(tg.TgxError):
            ctx.set_trace_steps(bad)
    svo.close(); sc.close()


@pytest.fixture(scope="module")
def bench_scene(oracle):
    """The benchmarked GI frame's inputs: the 512-object scene, its 4096^3 SVO
    around the camera as the oracle builds it (with materials), the 1080p view."""
    s = tg.generate_scene(1, 512, 2, 16, seed=1, noise_period=64.0, noise_threshold=0.5,
                          box_min=(-1024, -1024, -1024), box_max=(1024, 1024, 1024), n_luts=32)
    mn, L = [-2048.0] * 3, 12
    blocks, words, mats = svo_build_with_materials(oracle, s, mn, L, capacity=1 << 15)
    osvo = OracleSvo(oracle, blocks, words, mats, mn, L)
    view = tg.make_view((0.0, 0.0, 0.0), 0.0, float(np.pi), float(np.pi / 3), 1920, 1080, 0.1, 4096.0)
    yield s, mn, L, osvo, view, len(blocks)
    osvo.close()


@pytest.mark.parametrize("bounces,spp", [(1, 4), (2, 2)])
def test_gi_benchmark_frame_bands_bit_exact(ctx, oracle, bench_scene, bounces, spp):
    """Plain GI of the benchmarked frame (512 objects, 4096^3 SVO, 1920x1080,
    Philox seed 2, <= 256 SVO steps) against the oracle bit for bit on three
    bands of 16 rows spread over the frame (92,160 pixels); the SVO itself
    equals the oracle's block for block."""
    import torch
    s, mn, L, osvo, view, n_oracle_blocks = bench_scene
    sc = ctx.upload(s)
    svo = ctx.svo_build(sc, mn, L)
    assert svo.info().n_nonempty_blocks == n_oracle_blocks
    vis = torch.empty(1920 * 1080, dtype=torch.int64, device="cuda")
    ctx.vis_render(sc, view, [vis])
    params = tg.gi_params(spp=spp, bounces=bounces, seed=2, max_steps=256)
    rgb = torch.empty(1920 * 1080 * 3, dtype=torch.float32, device="cuda")
    ctx.gi_render(sc, svo, view, vis, params, rgb)
    ctx.sync()
    assert ctx.device_error().code == 0
    g = rgb.cpu().numpy().reshape(-1, 3)
    visb = vis.cpu().numpy().view(np.uint64)
    n_geo = 0
    for r0 in (200, 532, 900):
        rows = (r0, r0 + 16)
        ref = gi_render(oracle, osvo, s, view, params, visb, rows=rows)
        sl = slice(rows[0] * 1920, rows[1] * 1920)
        bad = np.nonzero((g[sl].view(np.uint32) != ref[sl].view(np.uint32)).any(axis=1))[0]
        assert len(bad) == 0, (rows, len(bad), bad[:5], g[sl][bad[:3]], ref[sl][bad[:3]])
        n_geo += int((visb[sl] != np.uint64(tg.VIS_EMPTY)).sum())
    assert n_geo > 5000
    svo.close()
    sc.close()


def test_cached_gi_keeps_its_gain_under_camera_and_object_motion(ctx):
    """The camera moves every frame, and so do two objects (tgx_svo_update):
    cached GI, trained online along the path, still has a lower error than
    plain GI of the same spp on the last frames, each scored against its own
    256-spp plain render.  A value-noise scene like the benchmark's, smaller."""
    import torch
    s = tg.generate_scene(1, 48, 2, 8, seed=3, noise_period=32.0, noise_threshold=0.5,
                          box_min=(-160.0,) * 3, box_max=(160.0,) * 3, n_luts=8)
    mn = [-256.0] * 3
    sc = ctx.upload(s)
    svo = ctx.svo_build(sc, mn, 9)
    base = s.objects.copy()
    vel = np.zeros((len(base), 3), np.float32)
    vel[:2] = (0.6, -0.3, 0.45)
    box = ((-220.0,) * 3, (220.0,) * 3)
    cp = tg.cache_gi_params(*box, n_train=16384, train_spp=16, train_steps=16, lr=1e-2, primary_weight=1.0,
                            n_train_primary=32768)
    cache = tg.Cache(ctx, seed=2)
    w, h = 256, 144
    vis = torch.empty(w * h, dtype=torch.int64, device="cuda")
    out = torch.empty(w * h * 3, dtype=torch.float32, device="cuda")
    ref = torch.empty_like(out)
    errs_cached, errs_plain = [], []
    for f in range(64):
        objs = base.copy()
        objs["translation"] += f * vel
        sc.set_objects(0, objs)
        svo.update(sc)
        view = tg.make_view((0.8 * f - 25.0, 3.0, -10.0 + 0.5 * f), 0.05, float(np.pi) + 0.004 * f, 1.0, w, h,
                            0.1, 600.0)
        ctx.vis_render(sc, view, [vis])
        ctx.gi_render_cached(sc, svo, cache, view, vis, tg.gi_params(spp=4, bounces=2, seed=2, frame=f), cp, out)
        if f >= 60:
            ctx.gi_render(sc, svo, view, vis, tg.gi_params(spp=256, bounces=2, seed=9, frame=f), ref)
            ctx.sync()
            hit = vis.cpu().numpy().view(np.uint64) != np.uint64(tg.VIS_EMPTY)
            r = ref.cpu().numpy().reshape(-1, 3)[hit]
            x = out.cpu().numpy().reshape(-1, 3)[hit]
            errs_cached.append(float(np.mean((x - r) ** 2 / (r ** 2 + 1e-2))))
            ctx.gi_render(sc, svo, view, vis, tg.gi_params(spp=4, bounces=2, seed=2, frame=f), out)
            ctx.sync()
            x = out.cpu().numpy().reshape(-1, 3)[hit]
            errs_plain.append(float(np.mean((x - r) ** 2 / (r ** 2 + 1e-2))))
            assert hit.sum() > 5000
    assert ctx.device_error().code == 0
    cache.close(); svo.close(); sc.close()
    print("relMSE cached", errs_cached, "plain", errs_plain)
    assert np.mean(errs_cached) < 0.7 * np.mean(errs_plain), (errs_cached, errs_plain)


def test_cached_gi_reaches_the_target_error_on_a_held_out_scene(ctx):
    """The shrinkage weight was tuned on the benchmark's 512-object scene
    (seed 1).  On the same generator with seed 2 (other sizes, poses, noise
    and LUTs), at 1920x1080 with the configured training budget, 4-spp cached
    2-bounce GI, scored as the benchmark scores it (60 online frames at 1 spp,
    then four at 4 spp), is within relMSE 0.01 of a 256-spp plain render
    (measured 0.0084; plain GI needs 14 spp for it)."""
    import torch
    s = tg.generate_scene(1, 512, 2, 16, seed=2, noise_period=64.0, noise_threshold=0.5,
                          box_min=(-1024.0,) * 3, box_max=(1024.0,) * 3, n_luts=32)
    view = tg.make_view((0.0, 0.0, 0.0), 0.0, float(np.pi), float(np.pi / 3), 1920, 1080, 0.1, 4096.0)
    sc = ctx.upload(s)
    svo = ctx.svo_build(sc, (-2048.0,) * 3, 12)
    vis = torch.empty(1920 * 1080, dtype=torch.int64, device="cuda")
    ctx.vis_render(sc, view, [vis])
    ref = torch.empty(1920 * 1080 * 3, dtype=torch.float32, device="cuda")
    out = torch.empty_like(ref)
    ctx.gi_render(sc, svo, view, vis, tg.gi_params(spp=256, bounces=2, seed=1234), ref)
    cp = tg.cache_gi_params((-1100.0,) * 3, (1100.0,) * 3, n_train=65536, train_spp=16, train_steps=16, lr=1e-2,
                            primary_weight=1.0, n_train_primary=131072)
    cache = tg.Cache(ctx, seed=7)
    # as the benchmark scores it: 60 online frames at 1 spp, then 4 frames at 4 spp, the last one scored
    for f in range(60):
        ctx.gi_render_cached(sc, svo, cache, view, vis, tg.gi_params(spp=1, bounces=2, seed=2, frame=f), cp, out)
    for f in range(4):
        ctx.gi_render_cached(sc, svo, cache, view, vis, tg.gi_params(spp=4, bounces=2, seed=2, frame=100 + f), cp,
                             out)
    ctx.sync()
    assert ctx.device_error().code == 0
    hit = vis.cpu().numpy().view(np.uint64) != np.uint64(tg.VIS_EMPTY)
    r = ref.cpu().numpy().reshape(-1, 3)[hit]
    x = out.cpu().numpy().reshape(-1, 3)[hit]
    err = float(np.mean((x - r) ** 2 / (r ** 2 + 1e-2)))
    cache.close(); svo.close(); sc.close()
    print("held-out scene, cached 4 spp relMSE", err)
    assert err <= 0.01, err
