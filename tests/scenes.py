"""Scene helpers shared by the tests (seeded, small enough for the oracle)."""
from __future__ import annotations

import numpy as np

import tg_gb300 as tg


def permute_clusters(scene: tg.HostScene, seed: int) -> tg.HostScene:
    """Same geometry, but cluster pointer p -> cluster index perm[p] (exercises the indirection)."""
    n = scene.n_clusters
    perm = np.random.default_rng(seed).permutation(n).astype(np.uint32)
    bits = np.zeros_like(scene.voxel_bits)
    bits[perm] = scene.voxel_bits[scene.cluster_pointers]
    c2o = np.zeros(n, np.uint32)
    c2o[perm] = scene.cluster_idx_to_object_idx[scene.cluster_pointers]
    mat = None
    if scene.material_idx is not None:
        mat = np.zeros_like(scene.material_idx)
        mat[perm] = scene.material_idx[scene.cluster_pointers]
    return tg.HostScene(scene.objects, perm, c2o, bits, mat, scene.luts)


def cfg1_scene() -> tg.HostScene:
    """1 object of 4x4x4 clusters, Bernoulli(0.3) bits from seed 0, random rotation, translation (0,0,64)."""
    return tg.generate_scene(0, 1, 4, 4, seed=0, bernoulli_p=0.3, translation=(0.0, 0.0, 64.0))


def cfg1_view(w: int = 256, h: int = 256):
    """Pinhole at the origin looking +z (tg looks down -z at yaw 0), 60 degree vFOV, near 0.1, far 256."""
    return tg.make_view((0.0, 0.0, 0.0), 0.0, float(np.pi), float(np.pi / 3), w, h, 0.1, 256.0)


def fuzz_scene(seed: int, n_objects: int = 5, box: float = 60.0, max_cpa: int = 4, density: float = 0.25):
    s = tg.generate_scene(0 if density else 1, n_objects, 1, max_cpa, seed=seed, bernoulli_p=density,
                          translation=(0.0, 0.0, 0.0))
    rng = np.random.default_rng(seed)
    objs = s.objects.copy()
    objs["translation"] = rng.uniform(-box, box, size=(n_objects, 3)).astype(np.float32)
    return tg.HostScene(objs, s.cluster_pointers, s.cluster_idx_to_object_idx, s.voxel_bits, s.material_idx, s.luts)


def single_cluster_scene(bits_set, translation=(0.0, 0.0, 20.0), rotation=None):
    objs = np.zeros(1, tg.OBJECT_DTYPE)
    objs["n_cluster_pointers_per_dim"] = (1, 1, 1)
    objs["translation"] = translation
    objs["rotation"] = (np.eye(4, dtype=np.float32) if rotation is None else rotation).T.reshape(-1)
    words = np.zeros((1, 16), np.uint32)
    for v in bits_set:
        words[0, v // 32] |= np.uint32(1 << (v % 32))
    return tg.HostScene(objs, np.zeros(1, np.uint32), np.zeros(1, np.uint32), words)
