"""GPU parity of the one-bit SVO build: the voxel set tg_svo_create builds,
bit-exact, against the reference's own output (golden fixtures made from the
reference's C code) and against the CPU oracle at other side lengths."""
from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest

import tg_gb300 as tg
from scenes import fuzz_scene, permute_clusters

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"


def fixture_scene(f) -> tg.HostScene:
    return tg.HostScene(f["objects"].view(tg.OBJECT_DTYPE), f["cluster_pointers"], f["c2o"], f["voxel_bits"])


def build(ctx, scene, mn, L):
    sc = ctx.upload(scene)
    svo = ctx.svo_build(sc, mn, L)
    ctx.sync()
    err = ctx.device_error()
    assert err.code == 0, (err.code, err.where, err.detail)
    xyz, words = svo.download()
    info = svo.info()
    svo.close()
    sc.close()
    return xyz, words, info


@pytest.mark.parametrize("name", sorted(p.stem for p in GOLD.glob("ref_svo_*.npz")))
def test_matches_reference_tg_svo_create(ctx, name):
    f = np.load(GOLD / f"{name}.npz")
    xyz, words, info = build(ctx, fixture_scene(f), f["mn"], 10)
    assert np.array_equal(xyz, f["block_xyz"])
    assert np.array_equal(words, f["block_words"])
    assert info.n_nonempty_blocks == len(xyz)


@pytest.mark.parametrize("seed,L", [(0, 10), (1, 11), (2, 12), (3, 9), (4, 7)])
def test_matches_oracle_other_extents(ctx, oracle, seed, L):
    s = permute_clusters(fuzz_scene(seed, n_objects=5, box=float(min(2 ** (L - 1) - 40, 200)), max_cpa=4), seed)
    mn = [-(2 ** (L - 1))] * 3
    xyz, words, info = build(ctx, s, mn, L)
    oxyz, owords, samples = oracle.svo_build(s, mn, L)
    assert len(oxyz) > 0
    assert np.array_equal(xyz, oxyz)
    assert np.array_equal(words, owords)


def test_benchmark_scene_4096_matches_oracle(ctx, oracle):
    """The benchmarked SVO: the 512-object scene in the 4096^3 cube around the
    camera (15,856 non-empty blocks), block for block against the oracle."""
    s = tg.generate_scene(1, 512, 2, 16, seed=1, noise_period=64.0, noise_threshold=0.5,
                          box_min=(-1024, -1024, -1024), box_max=(1024, 1024, 1024), n_luts=32)
    mn = [-2048.0] * 3
    xyz, words, info = build(ctx, s, mn, 12)
    oxyz, owords, _ = oracle.svo_build(s, mn, 12, capacity=1 << 15)
    assert len(oxyz) > 10000
    assert np.array_equal(xyz, oxyz)
    assert np.array_equal(words, owords)


@pytest.mark.parametrize("L", [13, 14])
def test_largest_extents_match_oracle(ctx, oracle, L):
    """Side lengths 8192 and 16384 (the large configuration's SVO): a small
    scene placed near the cube's far corner, at the origin and near its near
    corner, so block coordinates reach the top of the block table."""
    half = 2.0 ** (L - 1)
    s = permute_clusters(fuzz_scene(40 + L, n_objects=9, box=60.0, max_cpa=4), L)
    objs = s.objects.copy()
    for i, c in enumerate((half - 90.0, 0.0, -half + 90.0)):
        objs["translation"][3 * i:3 * i + 3] += np.float32(c)
    s = tg.HostScene(objs, s.cluster_pointers, s.cluster_idx_to_object_idx, s.voxel_bits, s.material_idx, s.luts)
    mn = [-half] * 3
    xyz, words, info = build(ctx, s, mn, L)
    oxyz, owords, _ = oracle.svo_build(s, mn, L)
    assert len(oxyz) > 0 and xyz.max() > half - 200 and xyz.min() < -half + 200
    assert np.array_equal(xyz, oxyz)
    assert np.array_equal(words, owords)


def test_offset_extent_and_clusters_outside(ctx, oracle):
    # objects partly outside the cube: only the inside voxels are built
    s = fuzz_scene(7, n_objects=6, box=120.0, max_cpa=5)
    mn = [-64, -100, 0]
    xyz, words, _ = build(ctx, s, mn, 7)
    oxyz, owords, _ = oracle.svo_build(s, mn, 7)
    assert np.array_equal(xyz, oxyz) and np.array_equal(words, owords)


def test_rejects_bad_extent(ctx):
    s = fuzz_scene(1, n_objects=1)
    sc = ctx.upload(s)
    with pytest.raises(tg.TgxError):
        ctx.svo_build(sc, [0, 0, 0], 5)
    with pytest.raises(tg.TgxError):
        ctx.svo_build(sc, [0.5, 0, 0], 10)
    sc.close()
