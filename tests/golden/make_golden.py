"""Generates the golden fixtures in tests/golden/ by running the reference's
own CPU code (oracle/_ref/libtgref.so, built by oracle/build_ref.sh from the
reference sources).  Run from the repository root:

    oracle/build_ref.sh <reference checkout root> && python tests/golden/make_golden.py

Fixtures:
  ref_primitives.npz   tgm_m4_angle_axis, tgm_m4_inverse, tgm_m4_mul,
                       tg_intersect_ray_aabb, tg_intersect_aabb_obb_ignore_contact
                       and tg_amanatides_woo on seeded inputs
  ref_svo_<name>.npz   tg_svo_create over [-512, 512)^3 on seeded scenes:
                       the scene arrays and the non-empty 32^3 blocks
                       (world min corner + 1024 bit words), sorted by index
  ref_trace_<name>.npz tg_svo_traverse on that SVO for seeded rays: hit flag,
                       distance and the world voxel of the hit
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))
from oracle_lib import load_ref  # noqa: E402

OBJECT_DTYPE = np.dtype([("n_cluster_pointers_per_dim", np.uint32, 3), ("first_cluster_pointer", np.uint32),
                         ("translation", np.float32, 3), ("lut_idx", np.uint32), ("rotation", np.float32, 16)])


def P(a):
    return a.ctypes.data_as(C.c_void_p)


def unit_axis(rng):
    """Random unit axis whose float magnitude is exactly 1 (tgm_m4_angle_axis asserts it, tg_math.c:1876)."""
    while True:
        a = rng.normal(size=3).astype(np.float32)
        a = (a / np.float32(np.sqrt(np.float32((a * a).sum())))).astype(np.float32)
        mag = np.float32(np.sqrt(np.float32(a[0] * a[0] + a[1] * a[1] + a[2] * a[2])))
        if mag == np.float32(1.0):
            return a


def pack_bits(bits):
    n = bits.shape[0]
    w = np.packbits(bits.reshape(n, 16, 32)[:, :, ::-1], axis=2).reshape(n, 16, 4)
    return np.ascontiguousarray(w).view(">u4").astype(np.uint32).reshape(n, 16)


def primitives(ref, rng):
    out = {}
    n = 256
    angles = rng.uniform(-7, 7, n).astype(np.float32)
    axes = np.stack([unit_axis(rng) for _ in range(n)])
    rots = np.zeros((n, 16), np.float32)
    for i in range(n):
        ref.tgref_angle_axis(C.c_float(angles[i]), P(axes[i]), P(rots[i]))
    out["aa_angle"], out["aa_axis"], out["aa_m4"] = angles, axes, rots
    mats = rng.uniform(-3, 3, (n, 16)).astype(np.float32)
    mats[: n // 2] = rots[: n // 2]
    mats[: n // 2, 12:15] = rng.uniform(-100, 100, (n // 2, 3)).astype(np.float32)
    inv = np.zeros_like(mats)
    for i in range(n):
        ref.tgref_m4_inverse(P(mats[i]), P(inv[i]))
    out["inv_in"], out["inv_out"] = mats, inv
    a = rng.uniform(-5, 5, (n, 16)).astype(np.float32)
    b = rng.uniform(-5, 5, (n, 16)).astype(np.float32)
    ab = np.zeros_like(a)
    for i in range(n):
        ref.tgref_m4_mul(P(a[i]), P(b[i]), P(ab[i]))
    out["mul_a"], out["mul_b"], out["mul_ab"] = a, b, ab
    m = 4096
    o = rng.uniform(-12, 20, (m, 3)).astype(np.float32)
    d = rng.normal(size=(m, 3)).astype(np.float32)
    d[::7, 0] = 0.0
    d[::11, 1] = 0.0
    d[::13, 2] = 0.0
    mn = np.zeros((m, 3), np.float32)
    mx = np.full((m, 3), 8.0, np.float32)
    mn[m // 2:] = rng.integers(-4, 4, (m - m // 2, 3)).astype(np.float32)
    mx[m // 2:] = mn[m // 2:] + 1.0
    ent = np.zeros(m, np.float32)
    ext = np.zeros(m, np.float32)
    hit = np.zeros(m, np.int32)
    for i in range(m):
        e, x = C.c_float(), C.c_float()
        hit[i] = ref.tgref_ray_aabb(P(o[i]), P(d[i]), P(mn[i]), P(mx[i]), C.byref(e), C.byref(x))
        ent[i], ext[i] = e.value, x.value
    out.update(ray_o=o, ray_d=d, ray_mn=mn, ray_mx=mx, ray_enter=ent, ray_exit=ext, ray_hit=hit)
    # box-vs-OBB test on transformed unit cubes
    k = 2048
    corners = np.zeros((k, 24), np.float32)
    sat = np.zeros(k, np.int32)
    unit = np.array([[x, y, z] for z in (0, 1) for y in (0, 1) for x in (0, 1)], np.float32)
    for i in range(k):
        r = rots[i % n].reshape(4, 4).T[:3, :3]
        s = np.float32(rng.uniform(2, 20))
        t = rng.uniform(-16, 24, 3).astype(np.float32)
        cs = (unit * s) @ r.T + t
        corners[i] = cs.astype(np.float32).reshape(-1)
        sat[i] = ref.tgref_aabb_obb(P(np.zeros(3, np.float32)), P(np.full(3, 8.0, np.float32)), P(corners[i]))
    out["sat_corners"], out["sat_result"] = corners, sat
    # 8^3 DDA from points on the grid's faces
    q = 1024
    grids = (rng.random((q, 512)) < 0.15)
    gw = pack_bits(grids)
    starts = rng.uniform(0, 8, (q, 3)).astype(np.float32)
    face = rng.integers(0, 3, q)
    starts[np.arange(q), face] = np.where(rng.random(q) < 0.5, 0.0, 8.0).astype(np.float32)
    dirs = rng.normal(size=(q, 3)).astype(np.float32)
    dirs[np.arange(q), face] = np.abs(dirs[np.arange(q), face]) * np.where(starts[np.arange(q), face] == 0, 1, -1)
    dirs = (dirs / np.sqrt((dirs.astype(np.float64) ** 2).sum(1, keepdims=True))).astype(np.float32)
    vox = np.zeros((q, 3), np.int32)
    aw_hit = np.zeros(q, np.int32)
    ext8 = np.full(3, 8.0, np.float32)
    for i in range(q):
        aw_hit[i] = ref.tgref_amanatides_woo(P(starts[i]), P(dirs[i]), P(ext8), P(gw[i]), P(vox[i]))
    out.update(aw_start=starts, aw_dir=dirs, aw_grid=gw, aw_hit=aw_hit, aw_voxel=vox)
    return out


def svo_scene(ref, rng, yonly: bool):
    n_obj = int(rng.integers(1, 5))
    dims = rng.integers(1, 5, size=(n_obj, 3)).astype(np.uint32)
    firsts = np.zeros(n_obj, np.uint32)
    tot = 0
    for i in range(n_obj):
        firsts[i] = tot
        tot += int(np.prod(dims[i]))
    trans = rng.uniform(-100, 100, size=(n_obj, 3)).astype(np.float32)
    angles = rng.uniform(0, 6.28, n_obj).astype(np.float32)
    axes = np.stack([np.array([0, 1, 0], np.float32) if yonly else unit_axis(rng) for _ in range(n_obj)])
    cp = np.arange(tot, dtype=np.uint32)
    perm = rng.permutation(tot).astype(np.uint32)   # cluster pointer -> cluster index indirection
    cp = perm
    c2o = np.zeros(tot, np.uint32)
    for i in range(n_obj):
        c2o[perm[firsts[i]:firsts[i] + np.prod(dims[i])]] = i
    bits = rng.random((tot, 512)) < rng.uniform(0.1, 0.5)
    bits[rng.random(tot) < 0.15] = False   # some empty clusters
    words = pack_bits(bits)
    mn = np.array([-512, -512, -512], np.float32)
    nb = ref.tgref_svo_build(C.c_uint32(n_obj), P(dims), P(firsts), P(trans), P(angles), P(axes), C.c_uint32(tot),
                             P(cp), P(c2o), C.c_uint32(tot), P(words), P(mn))
    if nb < 0:
        return None
    cap = 8192
    rb = np.zeros((cap, 3), np.int32)
    rw = np.zeros((cap, 1024), np.uint32)
    n = ref.tgref_svo_blocks(P(rb), P(rw), C.c_int(cap))
    key = ((rb[:n, 2] + 512) // 32 * 32 + (rb[:n, 1] + 512) // 32) * 32 + (rb[:n, 0] + 512) // 32
    o = np.argsort(key)
    rot = np.zeros((n_obj, 16), np.float32)
    for i in range(n_obj):
        ref.tgref_angle_axis(C.c_float(angles[i]), P(axes[i]), P(rot[i]))
    objs = np.zeros(n_obj, OBJECT_DTYPE)
    objs["n_cluster_pointers_per_dim"] = dims
    objs["first_cluster_pointer"] = firsts
    objs["translation"] = trans
    objs["rotation"] = rot
    sc = dict(objects=objs.view(np.uint8), cluster_pointers=cp, c2o=c2o, voxel_bits=words, mn=mn,
              angles=angles, axes=axes, block_xyz=rb[:n][o], block_words=rw[:n][o])
    # rays through the region of the scene, traversed by the reference's own tg_svo_traverse
    m = 4000
    lo = sc["block_xyz"].min(0) - 40
    hi = sc["block_xyz"].max(0) + 72
    orig = rng.uniform(lo, hi, (m, 3)).astype(np.float32)
    d = rng.normal(size=(m, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    hit = np.zeros(m, np.int32)
    dist = np.zeros(m, np.float32)
    vox = np.zeros((m, 3), np.int32)
    ref.tgref_svo_traverse(C.c_uint32(m), P(orig), P(d), P(hit), P(dist), P(vox))
    trace = dict(origin=orig, dir=d, hit=hit, distance=dist, voxel=vox)
    return sc, trace


def main():
    ref = load_ref()
    if ref is None:
        sys.exit("oracle/_ref/libtgref.so missing: run oracle/build_ref.sh first")
    rng = np.random.default_rng(20261203)
    np.savez_compressed(HERE / "ref_primitives.npz", **primitives(ref, rng))
    made = 0
    for name, yonly in (("yaxis", True), ("general", False)):
        k = 0
        seed = 0
        while k < 3:
            res = svo_scene(ref, np.random.default_rng(1000 * (1 + yonly) + seed), yonly)
            seed += 1
            if res is None:
                continue
            sc, trace = res
            np.savez_compressed(HERE / f"ref_svo_{name}_{k}.npz", **sc)
            np.savez_compressed(HERE / f"ref_trace_{name}_{k}.npz", **trace)
            k += 1
            made += 1
    print(f"wrote ref_primitives.npz and {made} SVO fixtures")


if __name__ == "__main__":
    main()
