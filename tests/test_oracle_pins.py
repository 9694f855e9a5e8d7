"""Pins the CPU oracle against the reference's own CPU code.

Fixtures in tests/golden/ were produced by tests/golden/make_golden.py from
oracle/_ref/libtgref.so, i.e. the reference's tg_math.c, tg_physics.c,
tg_amanatides_woo.c and tg_sparse_voxel_octree.c compiled from its sources.
Every comparison is bit-exact.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from oracle_lib import Oracle, load_ref

GOLD = Path(__file__).resolve().parent / "golden"
OBJECT_DTYPE = np.dtype([("n_cluster_pointers_per_dim", np.uint32, 3), ("first_cluster_pointer", np.uint32),
                         ("translation", np.float32, 3), ("lut_idx", np.uint32), ("rotation", np.float32, 16)])


def P(a):
    return a.ctypes.data


@pytest.fixture(scope="module")
def prim():
    return np.load(GOLD / "ref_primitives.npz")


@pytest.fixture(scope="module")
def olib():
    lib = Oracle().lib
    vp = C.c_void_p
    lib.oracle_m4_inverse.argtypes = [vp, vp]
    lib.oracle_m4_mul.argtypes = [vp, vp, vp]
    lib.oracle_ray_aabb.argtypes = [vp, vp, vp, vp, vp, vp]
    lib.oracle_aabb_obb_flat.argtypes = [vp, vp, vp]
    lib.oracle_cluster_dda.argtypes = [vp, vp, vp, vp]
    return lib


def test_m4_inverse_matches_tgm_m4_inverse(prim, olib):
    src, want = prim["inv_in"], prim["inv_out"]
    got = np.zeros_like(want)
    for i in range(len(src)):
        olib.oracle_m4_inverse(P(src[i]), P(got[i]))
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_m4_mul_matches_tgm_m4_mul(prim, olib):
    a, b, want = prim["mul_a"], prim["mul_b"], prim["mul_ab"]
    got = np.zeros_like(want)
    for i in range(len(a)):
        olib.oracle_m4_mul(P(a[i]), P(b[i]), P(got[i]))
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_ray_aabb_matches_tg_intersect_ray_aabb(prim, olib):
    o, d, mn, mx = prim["ray_o"], prim["ray_d"], prim["ray_mn"], prim["ray_mx"]
    for i in range(len(o)):
        e, x = np.zeros(1, np.float32), np.zeros(1, np.float32)
        h = olib.oracle_ray_aabb(P(o[i]), P(d[i]), P(mn[i]), P(mx[i]), P(e), P(x))
        assert h == prim["ray_hit"][i]
        # enter/exit agree up to the sign of zero (GLSL vs C min/max tie rule)
        assert e[0] == prim["ray_enter"][i] and x[0] == prim["ray_exit"][i]


def test_obb_test_matches_tg_intersect_aabb_obb(prim, olib):
    mn, mx = np.zeros(3, np.float32), np.full(3, 8.0, np.float32)
    c = prim["sat_corners"]
    got = np.array([olib.oracle_aabb_obb_flat(P(mn), P(mx), P(c[i])) for i in range(len(c))])
    assert np.array_equal(got, prim["sat_result"])
    assert 0 < got.sum() < len(got)


def test_cluster_dda_matches_tg_amanatides_woo(prim, olib):
    s, d, g = prim["aw_start"], prim["aw_dir"], prim["aw_grid"]
    hits = 0
    for i in range(len(s)):
        v = np.zeros(3, np.int32)
        h = olib.oracle_cluster_dda(P(s[i]), P(d[i]), P(g[i]), P(v))
        assert h == prim["aw_hit"][i], i
        if h:
            hits += 1
            assert np.array_equal(v, prim["aw_voxel"][i]), i
    assert hits > len(s) // 4


@pytest.mark.parametrize("name", sorted(p.stem for p in GOLD.glob("ref_svo_*.npz")))
def test_svo_oracle_matches_tg_svo_create(name):
    f = np.load(GOLD / f"{name}.npz")
    objs = f["objects"].view(OBJECT_DTYPE)

    class S:
        pass

    sc = S()
    sc.objects, sc.cluster_pointers, sc.cluster_idx_to_object_idx, sc.voxel_bits = (
        objs, f["cluster_pointers"], f["c2o"], f["voxel_bits"])
    blocks, words, _ = Oracle().svo_build(sc, f["mn"], 10)
    assert np.array_equal(blocks, f["block_xyz"])
    assert np.array_equal(words, f["block_words"])
    assert len(blocks) > 0


def test_reference_library_reproduces_fixtures():
    """Where the reference could be built here, it still produces the fixtures."""
    ref = load_ref()
    if ref is None:
        pytest.skip("reference sources not available on this machine")
    f = np.load(GOLD / "ref_primitives.npz")
    out = np.zeros(16, np.float32)
    vp = C.c_void_p
    for i in range(8):
        axis = np.ascontiguousarray(f["aa_axis"][i])
        ref.tgref_angle_axis(C.c_float(f["aa_angle"][i]), vp(P(axis)), vp(P(out)))
        assert np.array_equal(out.view(np.uint32), f["aa_m4"][i].view(np.uint32))
