"""Known-answer tests of the visibility oracle (hand-derived expectations),
pinning the semantics of visibility.frag: image orientation, packing,
camera inside a cluster, far-plane cut, and that the oracle's conservative
rectangles never drop a fragment the brute-force pass would write."""
from __future__ import annotations

import numpy as np
import pytest

import tg_gb300 as tg
from scenes import cfg1_scene, cfg1_view, fuzz_scene, permute_clusters, single_cluster_scene

EMPTY = np.uint64(0xFFFFFFFFFFFFFFFF)


def pixel_dir(v, px, py):
    v = v[0]
    fx = (px + 0.5) / v["width"]
    fy = 1.0 - (py + 0.5) / v["height"]
    a = v["ray_bl"][:3] * (1 - fy) + v["ray_tl"][:3] * fy
    b = v["ray_br"][:3] * (1 - fy) + v["ray_tr"][:3] * fy
    d = (a * (1 - fx) + b * fx).astype(np.float64)
    return d / np.linalg.norm(d)


def test_full_cluster_front_face(oracle):
    s = single_cluster_scene(range(512), translation=(0.0, 0.0, 20.0))
    v = cfg1_view(64, 64)
    img = oracle.vis_render(s, v, mode=0).reshape(64, 64)
    for (px, py) in [(32, 32), (31, 31), (30, 34)]:
        d = pixel_dir(v, px, py)
        t = 16.0 / d[2]
        hitp = d * t
        x = int(np.floor(4 + hitp[0]))
        y = int(np.floor(4 + hitp[1]))
        hit, depth, ptr, vox = tg.decode(int(img[py, px]))
        assert hit and ptr == 0
        assert vox == 0 * 64 + y * 8 + x
        assert abs(depth * 256.0 - t) < 2e-4
    # pixels whose ray misses the box stay empty
    assert img[0, 0] == EMPTY


def test_image_orientation_top_row_is_up(oracle):
    # a cluster above the view axis shows up in the top half of the image
    s = single_cluster_scene(range(512), translation=(0.0, 10.0, 40.0))
    img = oracle.vis_render(s, cfg1_view(64, 64), mode=0).reshape(64, 64)
    rows = np.nonzero((img != EMPTY).any(axis=1))[0]
    assert len(rows) and rows.max() < 32


def test_camera_inside_voxel_gives_depth_zero(oracle):
    # camera at the object centre = cluster-space (4,4,4), voxel 4*64+4*8+4
    s = single_cluster_scene([292], translation=(0.0, 0.0, 0.0))
    img = oracle.vis_render(s, cfg1_view(16, 16), mode=0)
    assert (img == np.uint64((0 << 40) | (0 << 9) | 292)).all()


def test_far_plane_cut(oracle):
    s = single_cluster_scene(range(512), translation=(0.0, 0.0, 300.0))
    img = oracle.vis_render(s, cfg1_view(32, 32), mode=0)
    assert (img == EMPTY).all()


def test_single_voxel_only_where_rays_cross_it(oracle):
    s = single_cluster_scene([7 * 64 + 7 * 8 + 7], translation=(0.0, 0.0, 20.0))
    img = oracle.vis_render(s, cfg1_view(64, 64), mode=0)
    hits = img[img != EMPTY]
    assert len(hits) > 0
    assert ((hits & np.uint64(511)) == 511).all()


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_rect_culling_equals_brute_force(oracle, seed):
    s = permute_clusters(fuzz_scene(seed, n_objects=4, box=30.0), seed)
    v = tg.make_view((0.0, 0.0, 0.0), 0.1 * seed, 0.7 * seed, 1.0, 48, 40, 0.1, 128.0)
    a = oracle.vis_render(s, v, mode=0)
    b = oracle.vis_render(s, v, mode=1)
    assert np.array_equal(a, b)


def test_cfg1_has_hits(oracle):
    img = oracle.vis_render(cfg1_scene(), cfg1_view(), mode=1)
    n = int((img != EMPTY).sum())
    assert 10000 < n < 40000


def test_ray_parallel_to_a_slab_it_misses_is_no_fragment(oracle):
    """Identity rotation and a yaw-0 view of odd width give the centre column
    rays an exactly-zero x component.  A cluster displaced in x is crossed by
    no such ray, so the rasterised reference never shades it there; the
    shader's slab test alone (collide.inc:5-10) would accept it."""
    s = single_cluster_scene(range(512), translation=(20.0, 0.0, -40.0))
    v = tg.make_view((0.0, 0.0, 0.0), 0.0, 0.0, 1.0, 33, 17, 0.1, 256.0)
    assert v["ray_bl"][0][0] == -v["ray_br"][0][0]
    a = oracle.vis_render(s, v, mode=0).reshape(17, 33)
    assert (a[:, 16] == EMPTY).all()
    assert np.array_equal(a.reshape(-1), oracle.vis_render(s, v, mode=1))
