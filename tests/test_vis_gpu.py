"""GPU parity of the visibility pass: the CUDA kernels through the C ABI
against the CPU oracle's transcription of visibility.frag, bit-exact."""
from __future__ import annotations

import numpy as np
import pytest

import tg_gb300 as tg
from scenes import cfg1_scene, cfg1_view, fuzz_scene, permute_clusters, single_cluster_scene

pytestmark = pytest.mark.gpu
EMPTY = np.uint64(0xFFFFFFFFFFFFFFFF)


def render(ctx, scene, views):
    import torch
    sc = ctx.upload(scene)
    outs = [torch.empty(int(v["width"]) * int(v["height"]), dtype=torch.int64, device="cuda") for v in views]
    ctx.vis_render(sc, views, outs)
    ctx.sync()
    err = ctx.device_error()
    assert err.code == 0, (err.code, err.where, err.detail)
    res = [o.cpu().numpy().view(np.uint64) for o in outs]
    sc.close()
    return res


def assert_same(gpu, ref):
    bad = np.nonzero(gpu != ref)[0]
    assert len(bad) == 0, f"{len(bad)} pixels differ, first {bad[:5]}: gpu {gpu[bad[:5]]} oracle {ref[bad[:5]]}"


def test_cfg1_bit_exact(ctx, oracle):
    s, v = cfg1_scene(), cfg1_view()
    (g,) = render(ctx, s, v)
    assert_same(g, oracle.vis_render(s, v, mode=1))
    assert (g != EMPTY).sum() > 10000


@pytest.mark.parametrize("seed", range(16))
def test_fuzz_scenes_bit_exact(ctx, oracle, seed):
    s = permute_clusters(fuzz_scene(seed, n_objects=6, box=40.0, max_cpa=4), seed)
    rng = np.random.default_rng(100 + seed)
    pos = rng.uniform(-10, 10, 3)
    v = tg.make_view(pos, rng.uniform(-0.5, 0.5), rng.uniform(-3, 3), rng.uniform(0.6, 1.6),
                     int(rng.integers(40, 200)), int(rng.integers(30, 150)), 0.1, float(rng.uniform(40, 200)))
    (g,) = render(ctx, s, v)
    assert_same(g, oracle.vis_render(s, v, mode=0))


def test_camera_inside_and_near_clusters(ctx, oracle):
    # camera inside an object: clusters straddle the camera plane (full-screen bins)
    s = fuzz_scene(11, n_objects=3, box=3.0, max_cpa=3, density=0.05)
    v = tg.make_view((0.5, 0.25, -0.75), 0.3, 1.0, 1.2, 96, 64, 0.1, 64.0)
    (g,) = render(ctx, s, v)
    assert_same(g, oracle.vis_render(s, v, mode=0))


def test_axis_aligned_rays_and_zero_direction_components(ctx, oracle):
    # identity rotation, camera on the axis: many ray components are exactly 0
    s = single_cluster_scene(range(0, 512, 3), translation=(0.0, 0.0, 12.0))
    v = cfg1_view(33, 33)
    (g,) = render(ctx, s, v)
    assert_same(g, oracle.vis_render(s, v, mode=0))


@pytest.mark.parametrize("view_i", range(3))
def test_diagonal_rays_from_lattice_points(ctx, oracle, view_i):
    # an axis-aligned 4x4x4-cluster object on the integer lattice, seen from
    # lattice points along diagonals: rays cross voxel edges at (nearly) equal
    # distances, so the hit voxel's entry axis is a near tie and the exact
    # three-axis maximum decides; power-of-two and other far planes
    rng = np.random.default_rng(7)
    objs = np.zeros(1, tg.OBJECT_DTYPE)
    objs["n_cluster_pointers_per_dim"] = (4, 4, 4)
    objs["translation"] = (0.0, 0.0, 0.0)
    objs["rotation"] = np.eye(4, dtype=np.float32).T.reshape(-1)
    words = (rng.random((64, 16, 32)) < 0.06).astype(np.uint64)
    words = (words << np.arange(32, dtype=np.uint64)).sum(axis=2).astype(np.uint32)
    s = tg.HostScene(objs, np.arange(64, dtype=np.uint32), np.zeros(64, np.uint32), words)
    pos, pitch, yaw, far = [((-24.0, 0.0, -24.0), 0.0, float(-3 * np.pi / 4), 128.0),
                            ((-24.0, -24.0, -24.0), 0.6154797, float(-3 * np.pi / 4), 100.0),
                            ((20.0, 8.0, -20.0), 0.0, float(3 * np.pi / 4), 4096.0)][view_i]
    v = tg.make_view(pos, pitch, yaw, 1.0, 160, 120, 0.1, far)
    (g,) = render(ctx, s, v)
    assert_same(g, oracle.vis_render(s, v, mode=0))
    assert (g != EMPTY).sum() > 100


def test_multi_view_batch_equals_single_views(ctx, oracle):
    s = fuzz_scene(21, n_objects=5, box=40.0)
    views = np.concatenate([
        tg.make_view((0, 0, -60), 0.0, float(np.pi), 1.0, 64, 48, 0.1, 200.0),
        tg.make_view((5, 3, 70), 0.2, 0.1, 0.9, 37, 53, 0.1, 200.0),
        tg.make_view((-60, 0, 0), 0.0, float(np.pi / 2), 1.3, 128, 16, 0.1, 200.0),
    ])
    outs = render(ctx, s, views)
    for i in range(len(views)):
        assert_same(outs[i], oracle.vis_render(s, views[i:i + 1], mode=1))


@pytest.mark.parametrize("tile", [(8, 4), (8, 8), (32, 8), (32, 16)])
def test_tile_shapes_agree(oracle, tile):
    s, v = cfg1_scene(), cfg1_view(100, 70)
    with tg.Context(0, tile=tile) as c:
        (g,) = render(c, s, v)
    assert_same(g, oracle.vis_render(s, v, mode=1))


def test_pipelined_host_buffers_equal_the_oracle(ctx, oracle):
    """tgx_vis_render_host_async: five frames of different cameras issued back
    to back into pinned and pageable host buffers, waited for with at most
    one frame in flight and then all; every buffer equals the oracle's render
    of its own camera.  The blocking call into a pinned buffer, too."""
    import torch
    s = cfg1_scene()
    sc = ctx.upload(s)
    views = [cfg1_view(72, 40 + 8 * k) for k in range(5)]
    # pinned buffers (written by the render) and pageable ones (device copy, then a copy out)
    outs = [torch.zeros(72 * (40 + 8 * k), dtype=torch.int64, pin_memory=k % 2 == 0).numpy().view(np.uint64)
            for k in range(5)]
    for k, (v, o) in enumerate(zip(views, outs)):
        ctx.vis_render_host_async(sc, v, [o])
        if k == 2:
            ctx.vis_host_wait(1)
    ctx.vis_host_wait(0)
    assert ctx.device_error().code == 0
    for v, o in zip(views, outs):
        assert_same(o, oracle.vis_render(s, v, mode=1))
    pinned = torch.zeros(72 * 40, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
    ctx.vis_render_host(sc, views[0], [pinned])
    assert_same(pinned, oracle.vis_render(s, views[0], mode=1))
    sc.close()


def test_large_frame_scan_path_equals_small_frames():
    """More than 512 groups of 256 tiles (here two 2048x1088 views in 8x4 tiles,
    139,264 tiles) take the one-CTA scan + finalize; each view alone (272
    groups) takes the direct finalize.  Both give the same buffers, and so
    does the render into pinned host buffers (written by the tile kernel
    directly), through either scan."""
    import torch
    s = fuzz_scene(41, n_objects=12, box=50.0, max_cpa=5)
    views = [tg.make_view((0.0, 5.0, -90.0), 0.05, float(np.pi), 1.1, 2048, 1088, 0.1, 300.0),
             tg.make_view((20.0, -5.0, 80.0), -0.1, 0.2, 0.9, 2048, 1088, 0.1, 300.0)]
    with tg.Context(0, tile=(8, 4)) as c:
        together = render(c, s, np.concatenate(views))
        alone = [render(c, s, v)[0] for v in views]
        sc = c.upload(s)
        pinned = [torch.zeros(2048 * 1088, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
                  for _ in views]
        c.vis_render_host(sc, np.concatenate(views), pinned)
        one = torch.zeros(2048 * 1088, dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
        c.vis_render_host(sc, views[1], [one])
        assert c.device_error().code == 0
        sc.close()
    for a, b, h in zip(together, alone, pinned):
        assert_same(a, b)
        assert_same(h, b)
        assert (a != EMPTY).sum() > 10000
    assert_same(one, alone[1])


def test_host_buffers_and_pick(ctx, oracle):
    s, v = cfg1_scene(), cfg1_view(64, 64)
    sc = ctx.upload(s)
    out = np.zeros(64 * 64, np.uint64)
    ctx.vis_render_host(sc, v, [out])
    ref = oracle.vis_render(s, v, mode=1)
    assert_same(out, ref)
    import torch
    d = torch.from_numpy(out.view(np.int64)).cuda()
    for (x, y) in [(32, 32), (0, 0), (40, 20)]:
        hit, depth, ptr, vox = ctx.pick(d, 64, 64, x, y)
        assert (hit, ptr if hit else None, vox if hit else None) == (
            tg.decode(int(ref[y * 64 + x]))[0],
            tg.decode(int(ref[y * 64 + x]))[2] if hit else None,
            tg.decode(int(ref[y * 64 + x]))[3] if hit else None)
    sc.close()


def test_empty_clusters_give_empty_buffer(ctx):
    s = single_cluster_scene([], translation=(0.0, 0.0, 10.0))
    (g,) = render(ctx, s, cfg1_view(40, 30))
    assert (g == EMPTY).all()


def test_rejects_bad_arguments(ctx):
    s = cfg1_scene()
    bad = tg.HostScene(s.objects, s.cluster_pointers + np.uint32(1000), s.cluster_idx_to_object_idx, s.voxel_bits)
    with pytest.raises(tg.TgxError) as e:
        ctx.upload(bad)
    assert e.value.status == 1
    sc = ctx.upload(s)
    v = cfg1_view(16, 16)
    v["width"] = 0
    import torch
    with pytest.raises(tg.TgxError):
        ctx.vis_render(sc, v, [torch.empty(1, dtype=torch.int64, device="cuda")])
    sc.close()


def test_cfg2_full_frame_bit_exact(ctx, oracle):
    """The benchmarked frame: 512 noise objects at 1920x1080, every pixel
    against the oracle (about 0.2 s on 16 host cores)."""
    s = tg.generate_scene(1, 512, 2, 16, seed=1, noise_period=64.0, noise_threshold=0.5,
                          box_min=(-1024, -1024, -1024), box_max=(1024, 1024, 1024), n_luts=32)
    v = tg.make_view((0.0, 0.0, 0.0), 0.0, float(np.pi), float(np.pi / 3), 1920, 1080, 0.1, 4096.0)
    ref = oracle.vis_render(s, v, mode=1)
    for tile in ((8, 8), (8, 16), (16, 16)):
        with tg.Context(0, tile=tile) as c:
            (g,) = render(c, s, v)
        assert_same(g, ref)
    assert (g != EMPTY).mean() > 0.05


def test_bin_overflow_takes_exact_record_scan(oracle):
    """With the bin storage pinned at its minimum the frame overflows it; the
    tile kernel then walks every record and must give the same buffer."""
    s = fuzz_scene(31, n_objects=8, box=30.0, max_cpa=4)
    v = tg.make_view((0.0, 0.0, -70.0), 0.0, float(np.pi), 1.2, 160, 120, 0.1, 256.0)
    with tg.Context(0, flags=tg.FLAG_MIN_BIN_CAPACITY) as c:
        (g,) = render(c, s, v)
        st = c.vis_stats()
    assert st.bin_entries > 64
    assert_same(g, oracle.vis_render(s, v, mode=1))


def test_repeated_frames_reuse_scratch(ctx, oracle):
    """Many frames in a row on one context (capacity grown from earlier frames)."""
    import torch
    s = fuzz_scene(41, n_objects=6, box=40.0)
    sc = ctx.upload(s)
    views = [tg.make_view((0.0, 0.0, -80.0 + 10 * i), 0.05 * i, float(np.pi) + 0.1 * i, 1.0, 96, 72, 0.1, 256.0)
             for i in range(6)]
    outs = [torch.empty(96 * 72, dtype=torch.int64, device="cuda") for _ in views]
    for v, o in zip(views, outs):
        ctx.vis_render(sc, v, [o])
    ctx.sync()
    assert ctx.device_error().code == 0
    for v, o in zip(views, outs):
        assert_same(o.cpu().numpy().view(np.uint64), oracle.vis_render(s, v, mode=1))
    sc.close()


def test_lost_bitmask_copy_times_out_and_the_context_stays_usable(oracle):
    """The device-side timeout path, with nothing faulting: under
    TGX_FLAG_TEST_LOST_COPY the tile's first batch waits for 64 bytes that no
    copy delivers, its bounded wait (about a second) runs out, the tile stops
    staging and the status word reports TGX_ERR_TIMEOUT at the tile kernel
    (where 5, detail = the tile).  A frame on a fresh context afterwards is
    bit-exact, so the GPU context stayed healthy."""
    import time
    import torch
    s, v = cfg1_scene(), cfg1_view(16, 16)   # one 16x16 tile that sees the object
    with tg.Context(0, tile=(16, 16), flags=tg.FLAG_TEST_LOST_COPY) as c:
        sc = c.upload(s)
        out = torch.empty(16 * 16, dtype=torch.int64, device="cuda")
        t0 = time.perf_counter()
        c.vis_render(sc, v, [out])
        c.sync()
        dt = time.perf_counter() - t0
        err = c.device_error()
        sc.close()
    assert (err.code, err.where, err.detail) == (5, 5, 0), (err.code, err.where, err.detail)
    assert 0.9 < dt < 30.0, dt   # the wait and the drain each run out after about a second
    with tg.Context(0, tile=(16, 16)) as c:
        (g,) = render(c, s, v)
    ref = oracle.vis_render(s, v, mode=1)
    assert_same(g, ref)
    assert (ref != EMPTY).sum() > 20


def test_work_counting_variant_gives_the_same_buffer_and_consistent_counts(oracle):
    """tgx_vis_count_work: the tile kernel's counting variant renders the same
    buffer, and its counters add up (every evaluated pair is a slab miss, a
    sure hit or an exact test; DDAs and hits only come from those)."""
    s = fuzz_scene(61, n_objects=8, box=40.0, max_cpa=4)
    v = tg.make_view((0.0, 0.0, -70.0), 0.05, float(np.pi), 1.1, 200, 120, 0.1, 256.0)
    ref = oracle.vis_render(s, v, mode=1)
    with tg.Context(0, tile=(8, 8)) as c:
        c.vis_count_work(True)
        (g,) = render(c, s, v)
        w = c.vis_work().as_dict()
        c.vis_count_work(False)
        (g2,) = render(c, s, v)
    assert_same(g, ref)
    assert_same(g2, ref)
    n_hit = int((ref != EMPTY).sum())
    assert w["pairs"] == w["slab_misses"] + w["sure_hits"] + w["exact_tests"], w
    assert w["ddas"] <= w["sure_hits"] + w["exact_tests"]
    assert w["ddas"] >= w["sure_hits"]
    assert n_hit <= w["hits"] <= w["ddas"] <= w["dda_steps"] <= 22 * w["ddas"]
    assert 0 < w["dir_setups"] <= w["pairs"] + w["depth_skips"]
    assert w["batches"] > 0


@pytest.mark.parametrize("buckets,batch,drain", [(8, 16, 16), (32, 48, 24), (16, 1, 1), (8, 7, 32), (32, 32, 8)])
def test_tuning_settings_change_no_result(oracle, buckets, batch, drain):
    """tgx_set_vis_tuning: depth buckets, staged batch size and pairs per DDA
    round only reschedule the pass; every setting gives the oracle's buffer.
    The scene puts many clusters on each tile (several batches per tile)."""
    s = fuzz_scene(71, n_objects=10, box=25.0, max_cpa=5)
    v = tg.make_view((0.0, 2.0, -60.0), 0.05, float(np.pi), 1.0, 150, 110, 0.1, 256.0)
    ref = oracle.vis_render(s, v, mode=1)
    for tile in ((8, 8), (16, 16)):
        with tg.Context(0, tile=tile) as c:
            c.set_vis_tuning(buckets, batch, drain)
            (g,) = render(c, s, v)
            st = c.vis_stats()
        assert_same(g, ref)
    assert st.bin_entries > 4 * st.tiles
    with tg.Context(0) as c:
        for bad in ((12, 0, 0), (0, 49, 0), (0, 0, 33)):
            with pytest.raises(tg.TgxError):
                c.set_vis_tuning(*bad)


def test_scene_upload_fails_cleanly_past_the_memory_budget(oracle):
    """Allocation failure made on the host: with a budget too small for the
    scene store the upload fails with TGX_ERR_OUT_OF_MEMORY partway through
    its allocations, frees what it took, and the context stays usable: the
    same upload under a larger budget renders the oracle's buffer, and the
    budget accounting returns to zero when the scene is destroyed."""
    s, v = cfg1_scene(), cfg1_view(64, 48)
    need = 96 + 64 * 4 * 2 + 64 * 64 + 9 * 4   # object, pointers, map, bits, rotation
    with tg.Context(0) as c:
        c.set_memory_budget(64 * 8 + 96)    # room for the objects and the pointers, not the bits
        with pytest.raises(tg.TgxError) as e:
            c.upload(s)
        assert e.value.status == 2
        assert c.memory() == (64 * 8 + 96, 0)
        c.set_memory_budget(1 << 20)
        (g,) = render(c, s, v)
        assert c.memory() == (1 << 20, 0)
        sc = c.upload(s)
        held = c.memory()[1]
        assert held >= need
        c.set_memory_budget(held + 100)
        with pytest.raises(tg.TgxError):
            c.upload(s)                    # a second copy does not fit
        assert c.memory()[1] == held
        sc.close()
        assert c.memory()[1] == 0
        c.set_memory_budget(0)
    assert_same(g, oracle.vis_render(s, v, mode=1))
