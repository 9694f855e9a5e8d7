"""GPU tests of the incremental SVO update (tgx_scene_set_objects +
tgx_svo_update), the insert-on-move the reference leaves commented out
(tg_svo_insert_object, tgvk_raytracer.c:982-989): after objects move, the
updated SVO must equal a fresh tgx_svo_build of the moved scene -- voxel
words, block counts, traversal hits and material-dependent GI, bit for bit --
and the CPU oracle's voxel set."""
from __future__ import annotations

import numpy as np
import pytest

import tg_gb300 as tg
from scenes import fuzz_scene

pytestmark = pytest.mark.gpu

MN = [-256.0, -256.0, -256.0]
L = 9


def rotation_cm(rng) -> np.ndarray:
    """A random rotation as tg's column-major 4x4 (float32[16])."""
    axis = rng.normal(size=3)
    axis /= np.linalg.norm(axis)
    a = rng.uniform(0, 2 * np.pi)
    k = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]], [-axis[1], axis[0], 0]])
    r = np.eye(3) + np.sin(a) * k + (1 - np.cos(a)) * (k @ k)
    m = np.eye(4, dtype=np.float32)
    m[:3, :3] = r
    return m.T.reshape(-1).astype(np.float32)


def moved(objects, idx, rng, box=60.0):
    out = objects.copy()
    for i in idx:
        out["translation"][i] = rng.uniform(-box, box, 3).astype(np.float32)
        out["rotation"][i] = rotation_cm(rng)
    return out


def with_objects(s: tg.HostScene, objects) -> tg.HostScene:
    return tg.HostScene(objects, s.cluster_pointers, s.cluster_idx_to_object_idx, s.voxel_bits, s.material_idx, s.luts)


def snapshot(ctx, sc, svo):
    """Everything observable about an SVO: voxel blocks, counts, trace hits and GI."""
    import torch
    ctx.sync()
    err = ctx.device_error()
    assert err.code == 0, (err.code, err.where, err.detail)
    xyz, words = svo.download()
    info = svo.info()
    rng = np.random.default_rng(5)
    n = 4096
    o = torch.tensor(rng.uniform(-150, 150, (n, 3)).astype(np.float32), device="cuda")
    d = rng.normal(size=(n, 3))
    d = torch.tensor((d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32), device="cuda")
    t = torch.empty(n, dtype=torch.float32, device="cuda")
    v = torch.empty((n, 3), dtype=torch.int32, device="cuda")
    svo.trace(o, d, t, v, max_steps=512)
    view = tg.make_view((0.0, 5.0, -140.0), 0.1, float(np.pi), 1.1, 64, 48, 0.1, 600.0)
    vis = torch.empty(64 * 48, dtype=torch.int64, device="cuda")
    ctx.vis_render(sc, view, [vis])
    rgb = torch.empty(64 * 48 * 3, dtype=torch.float32, device="cuda")
    ctx.gi_render(sc, svo, view, vis, tg.gi_params(spp=2, bounces=2, seed=3, max_steps=256), rgb)
    ctx.sync()
    return dict(xyz=xyz, words=words, n_blocks=info.n_blocks, nonempty=info.n_nonempty_blocks,
                t=t.cpu().numpy(), voxel=v.cpu().numpy(), vis=vis.cpu().numpy(), rgb=rgb.cpu().numpy())


def assert_same(a, b):
    sa = {tuple(x) for x in a["xyz"]}
    sb = {tuple(x) for x in b["xyz"]}
    assert sa == sb, (len(sa), len(sb), sorted(sa - sb)[:5], sorted(sb - sa)[:5])
    for k in a:
        assert np.array_equal(np.asarray(a[k]), np.asarray(b[k])), k


def fresh(ctx, s, objects, materials=True):
    sc = ctx.upload(with_objects(s, objects))
    svo = ctx.svo_build(sc, MN, L, materials=materials)
    snap = snapshot(ctx, sc, svo)
    svo.close()
    sc.close()
    return snap


def scene(seed=21, n=8, n_luts=3):
    """A fuzz scene with `n_luts` LUTs of different albedo, spread over the objects."""
    s = fuzz_scene(seed, n_objects=n, box=60.0, max_cpa=4)
    base = s.luts[:256]
    luts = np.concatenate([base] * n_luts)
    for k in range(1, n_luts):
        luts["albedo"][256 * k:256 * (k + 1)] = np.roll(base["albedo"], k, axis=1) * np.float32(0.5 + 0.2 * k)
    s.luts = np.ascontiguousarray(luts)
    s.objects["lut_idx"] = np.arange(n) % n_luts
    return s


def test_update_equals_full_rebuild_over_a_sequence_of_moves(ctx):
    s = scene()
    rng = np.random.default_rng(1)
    sc = ctx.upload(s)
    svo = ctx.svo_build(sc, MN, L)
    objs = s.objects.copy()
    # one object, several, all, then far away (pool growth) and back (slot reuse)
    for step, idx in enumerate([[3], [0, 5, 6], list(range(len(objs))), [2], [2]]):
        objs = moved(objs, idx, rng, box=180.0 if step == 3 else 60.0)
        sc.set_objects(0, objs)
        assert svo.update(sc) == len(idx)
        assert_same(snapshot(ctx, sc, svo), fresh(ctx, s, objs))
    assert svo.update(sc) == 0
    svo.close()
    sc.close()


def test_update_matches_oracle_voxels(ctx, oracle):
    s = scene(seed=4, n=5)
    rng = np.random.default_rng(2)
    sc = ctx.upload(s)
    svo = ctx.svo_build(sc, MN, L)
    objs = moved(s.objects, [1, 4], rng)
    sc.set_objects(1, objs[1:5])
    assert svo.update(sc) == 2
    xyz, words = svo.download()
    oxyz, owords, _ = oracle.svo_build(with_objects(s, objs), MN, L)
    assert len(oxyz) > 0
    assert np.array_equal(xyz, oxyz) and np.array_equal(words, owords)
    svo.close()
    sc.close()


@pytest.mark.parametrize("materials", [True, False])
def test_update_after_a_lut_change(ctx, materials):
    s = scene(seed=9, n=6)
    sc = ctx.upload(s)
    svo = ctx.svo_build(sc, MN, L, materials=materials)
    objs = s.objects.copy()
    objs["lut_idx"][2] = (int(objs["lut_idx"][2]) + 1) % (len(s.luts) // 256)   # a LUT change counts as a move
    sc.set_objects(0, objs)
    assert svo.update(sc) == 1
    assert_same(snapshot(ctx, sc, svo), fresh(ctx, s, objs, materials=materials))
    svo.close()
    sc.close()


def test_set_objects_moves_visibility(ctx):
    import torch
    s = scene(seed=12, n=4)
    objs = moved(s.objects, [0, 3], np.random.default_rng(3))
    view = tg.make_view((0.0, 5.0, -140.0), 0.1, float(np.pi), 1.1, 128, 96, 0.1, 600.0)
    a = torch.empty(128 * 96, dtype=torch.int64, device="cuda")
    b = torch.empty_like(a)
    sc = ctx.upload(s)
    sc.set_objects(0, objs)
    ctx.vis_render(sc, view, [a])
    sc2 = ctx.upload(with_objects(s, objs))
    ctx.vis_render(sc2, view, [b])
    ctx.sync()
    assert torch.equal(a, b)
    sc.close()
    sc2.close()


def test_set_objects_rejects_layout_changes(ctx):
    s = scene(seed=13, n=3)
    sc = ctx.upload(s)
    objs = s.objects.copy()
    objs["first_cluster_pointer"][1] += 1
    with pytest.raises(tg.TgxError):
        sc.set_objects(0, objs)
    with pytest.raises(tg.TgxError):
        sc.set_objects(2, s.objects[:2])
    objs = s.objects.copy()
    objs["lut_idx"][0] = 10 ** 6
    with pytest.raises(tg.TgxError):
        sc.set_objects(0, objs[:1])
    sc.close()


def test_update_rejects_another_scene(ctx):
    a = ctx.upload(scene(seed=14, n=3))
    b = ctx.upload(scene(seed=14, n=4))
    svo = ctx.svo_build(a, MN, L)
    with pytest.raises(tg.TgxError):
        svo.update(b)
    svo.close()
    a.close()
    b.close()
