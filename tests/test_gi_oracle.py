"""CPU checks of the traversal and GI oracle (the semantics the CUDA path must
reproduce), pinned where the reference has code:

- traversal: every hit voxel equals the reference's tg_svo_traverse
  (tg_sparse_voxel_octree.c:558-740) on its own SVO, for 24k fixture rays;
- Philox4x32-10: the published known-answer vectors (Salmon et al. 2011,
  Random123 kat_vectors);
- GI: energy and sampling sanity on a closed form (a plane under a sun).
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np
import pytest

import tg_gb300 as tg
from oracle_lib import OracleSvo, gi_render, svo_build_with_materials
from scenes import fuzz_scene

GOLD = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("name", sorted(p.stem.replace("ref_trace_", "") for p in GOLD.glob("ref_trace_*.npz")))
def test_traversal_matches_tg_svo_traverse(oracle, name):
    svo = np.load(GOLD / f"ref_svo_{name}.npz")
    tr = np.load(GOLD / f"ref_trace_{name}.npz")
    o = OracleSvo(oracle, svo["block_xyz"], svo["block_words"], None, svo["mn"], 10)
    t, vox, ax, steps = o.trace(tr["origin"], tr["dir"])
    ok = tr["hit"] >= 0
    assert ok.all()
    hit = t < 3e38
    assert np.array_equal(hit, tr["hit"] == 1)
    assert hit.sum() > 10
    assert np.array_equal(vox[hit], tr["voxel"][hit])
    # distances: the reference reports the (negative) entry distance behind the
    # origin when the ray starts inside the hit voxel; this traversal reports 0
    inside = ((tr["origin"] >= tr["voxel"]) & (tr["origin"] < tr["voxel"] + 1)).all(axis=1) & hit
    assert (t[inside] == 0).all() and (tr["distance"][inside] <= 0).all()
    rest = hit & ~inside
    assert (np.abs(t[rest] - tr["distance"][rest]) <= 2e-4 + 2e-6 * t[rest]).all()


def test_philox_known_answers(oracle):
    lib = oracle.lib
    lib.oracle_philox.argtypes = [C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p]
    cases = [
        ((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
        ((0xffffffff,) * 4, (0xffffffff, 0xffffffff), (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
        ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
         (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
    ]
    for ctr, key, want in cases:
        c = np.array(ctr, np.uint32)
        out = np.zeros(4, np.uint32)
        lib.oracle_philox(c.ctypes.data, key[0], key[1], out.ctypes.data)
        assert tuple(int(x) for x in out) == want


def test_gi_plane_under_sun_matches_closed_form(oracle):
    """A flat slab of voxels, normal +y, sun straight above, black sky, one
    bounce that can only escape: radiance = albedo/pi * E_sun exactly."""
    objs = np.zeros(1, tg.OBJECT_DTYPE)
    objs["n_cluster_pointers_per_dim"] = (4, 1, 4)
    objs["translation"] = (0.0, -4.0, 0.0)
    objs["rotation"] = np.eye(4, dtype=np.float32).T.reshape(-1)
    bits = np.zeros((16, 16), np.uint32)
    for c in range(16):
        for v in range(512):
            if (v >> 3) & 7 == 7:          # top layer of every cluster only
                bits[c, v >> 5] |= np.uint32(1 << (v & 31))
    mat = np.full((16, 512), 3, np.uint8)
    luts = np.zeros(256, tg.MATERIAL_DTYPE)
    luts["albedo"] = (0.6, 0.4, 0.2)
    s = tg.HostScene(objs, np.arange(16, dtype=np.uint32), np.zeros(16, np.uint32), bits, mat, luts)
    mn = [-64.0, -64.0, -64.0]
    blocks, words, mats = svo_build_with_materials(oracle, s, mn, 7)
    osvo = OracleSvo(oracle, blocks, words, mats, mn, 7)
    view = tg.make_view((0.0, 20.0, 0.0), -float(np.pi / 2), 0.0, 0.6, 16, 16, 0.1, 100.0)
    vis = oracle.vis_render(s, view, mode=0)
    assert (vis != np.uint64(tg.VIS_EMPTY)).all()
    p = tg.gi_params(spp=4, bounces=1, sun_dir=(0.0, 1.0, 0.0), sun_radiance=(1.0, 1.0, 1.0),
                     sky_radiance=(0.0, 0.0, 0.0))
    rgb = gi_render(oracle, osvo, s, view, p, vis)
    want = np.array([0.6, 0.4, 0.2], np.float32) * np.float32(0.318309886)
    assert np.allclose(rgb, want[None, :], rtol=1e-6)


def test_gi_sky_and_determinism(oracle):
    s = fuzz_scene(3, n_objects=3, box=20.0, max_cpa=3)
    mn = [-64.0, -64.0, -64.0]
    blocks, words, mats = svo_build_with_materials(oracle, s, mn, 7)
    osvo = OracleSvo(oracle, blocks, words, mats, mn, 7)
    view = tg.make_view((0.0, 0.0, -50.0), 0.0, float(np.pi), 1.0, 40, 30, 0.1, 200.0)
    vis = oracle.vis_render(s, view, mode=0)
    p = tg.gi_params(spp=4, bounces=2, seed=7)
    a = gi_render(oracle, osvo, s, view, p, vis)
    b = gi_render(oracle, osvo, s, view, p, vis)
    assert np.array_equal(a, b)
    sky = vis == np.uint64(tg.VIS_EMPTY)
    assert sky.any() and (~sky).any()
    assert np.allclose(a[sky], p["sky_radiance"][0])
    assert (a[~sky] >= 0).all() and np.isfinite(a).all()
    p2 = tg.gi_params(spp=4, bounces=2, seed=8)
    c = gi_render(oracle, osvo, s, view, p2, vis)
    assert not np.array_equal(a[~sky], c[~sky])


def test_traversal_levels(oracle):
    """Levels of the traversal: 1, 4, 8, 32, then every other block-pyramid level up to 2^(L-1)."""
    lib = oracle.lib
    for L in range(6, 15):
        lg = np.zeros(16, np.uint32)
        n = lib.oracle_svo_levels(C.c_uint32(L), C.c_void_p(lg.ctypes.data))
        want = [0, 2, 3, 5] + list(range(7, L - 1, 2))
        if want[-1] != L - 1:
            want.append(L - 1)
        assert list(lg[:n]) == want
        # the closed form the CUDA traversal evaluates per level
        closed = [0 if li == 0 else li + 1 if li <= 2 else min(2 * li - 1, L - 1) for li in range(n)]
        assert closed == want


def test_sub_block_masks(oracle):
    rng = np.random.default_rng(5)
    for p in (0.0, 0.001, 0.01, 0.2):
        bits = (rng.random((32, 32, 32)) < p)           # z, y, x
        words = np.packbits(bits.reshape(-1).astype(np.uint8), bitorder="little").view(np.uint32).copy()
        out = np.zeros(32, np.uint32)
        oracle.lib.oracle_svo_sub_masks(C.c_void_p(words.ctypes.data), C.c_void_p(out.ctypes.data))
        c4 = bits.reshape(8, 4, 8, 4, 8, 4).any(axis=(1, 3, 5)).reshape(-1)
        c8 = bits.reshape(4, 8, 4, 8, 4, 8).any(axis=(1, 3, 5)).reshape(-1)
        want = np.zeros(32, np.uint32)
        want[:16] = np.packbits(c4.astype(np.uint8), bitorder="little").view(np.uint32)
        want[16:18] = np.packbits(c8.astype(np.uint8), bitorder="little").view(np.uint32)
        assert np.array_equal(out, want)


def _sample(oracle, n, key, first, count, bounce=0, frame=0, seed=2):
    p = tg.gi_params(spp=count, bounces=1, seed=seed, frame=frame)
    nn = np.asarray(n, np.float32)
    out = np.zeros((count, 3), np.float32)
    oracle.lib.oracle_sample_cosine(C.c_void_p(nn.ctypes.data), C.c_uint32(key), C.c_uint32(first),
                                    C.c_uint32(count), C.c_uint32(bounce), C.c_void_p(p.ctypes.data),
                                    C.c_void_p(out.ctypes.data))
    return out


def test_sampler_is_cosine_weighted_and_stratified(oracle):
    """The randomised R2 + concentric-map sampler gives unit directions in the
    hemisphere with the cosine density (E[cos] = 2/3, E[cos^2] = 1/2), and
    the mean over the samples of one key varies far less across keys than
    independent samples would (stratification)."""
    n = np.array([0.36, -0.48, 0.8], np.float32)
    d = np.concatenate([_sample(oracle, n, key, 0, 64) for key in range(256)])
    assert np.allclose(np.linalg.norm(d, axis=1), 1.0, atol=2e-6)
    c = d @ n.astype(np.float64)
    assert (c >= -1e-6).all()
    assert abs(c.mean() - 2.0 / 3.0) < 0.005
    assert abs((c ** 2).mean() - 0.5) < 0.005
    means = c.reshape(256, 64).mean(axis=1)
    iid_var = c.var() / 64
    assert means.var() < 0.1 * iid_var
    # other keys, bounces and frames rotate the point set differently
    a = _sample(oracle, n, 5, 0, 8)
    assert not np.array_equal(a, _sample(oracle, n, 6, 0, 8))
    assert not np.array_equal(a, _sample(oracle, n, 5, 0, 8, bounce=1))
    assert not np.array_equal(a, _sample(oracle, n, 5, 0, 8, frame=1))
    assert np.array_equal(a[3:], _sample(oracle, n, 5, 3, 5))
