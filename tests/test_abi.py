"""CPU checks of the C-ABI library: it loads, exports every entry point
include/tgx.h declares, and its host-only functions behave."""
from __future__ import annotations

import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import tg_gb300 as tg
from conftest import has_gpu

ROOT = Path(__file__).resolve().parents[1]


def declared_functions() -> set[str]:
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names |= set(re.findall(r"\b(tgx_[a-z0-9_]+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(str(tg.LIB_PATH))
    names = declared_functions()
    assert "tgx_vis_render" in names and "tgx_svo_build" in names
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    assert set(tg.EXPORTS) <= names


def test_abi_version_and_status_strings():
    assert tg.lib.tgx_abi_version() == 1
    assert tg.lib.tgx_status_string(0) == b"ok"
    assert b"capacity" in tg.lib.tgx_status_string(4)


@pytest.mark.skipif(has_gpu(), reason="checks the no-device error path")
def test_create_without_device_fails_cleanly():
    with pytest.raises(tg.TgxError) as e:
        tg.Context(0)
    assert e.value.status == 7


def test_struct_sizes_match_reference_layout():
    # tg_object_data_ssbo is 96 bytes (tgvk_raytracer.c:35-42); the camera UBO
    # plus the size header are 96 bytes too.
    assert tg.OBJECT_DTYPE.itemsize == 96
    assert tg.VIEW_DTYPE.itemsize == 96
    assert tg.MATERIAL_DTYPE.itemsize == 16


def test_generator_is_deterministic_and_shaped():
    a = tg.generate_scene(0, 1, 4, 4, seed=0, bernoulli_p=0.3, translation=(0, 0, 64))
    b = tg.generate_scene(0, 1, 4, 4, seed=0, bernoulli_p=0.3, translation=(0, 0, 64))
    assert a.voxel_bits.shape == (64, 16)
    assert np.array_equal(a.voxel_bits, b.voxel_bits)
    assert np.array_equal(a.objects.view(np.uint8), b.objects.view(np.uint8))
    density = np.unpackbits(a.voxel_bits.view(np.uint8)).mean()
    assert 0.27 < density < 0.33
    r = a.objects["rotation"][0].reshape(4, 4).T[:3, :3].astype(np.float64)
    assert np.allclose(r @ r.T, np.eye(3), atol=1e-5) and abs(np.linalg.det(r) - 1) < 1e-5
    assert np.array_equal(a.objects["translation"][0], [0, 0, 64])


def test_generator_noise_scene():
    s = tg.generate_scene(1, 6, 2, 5, seed=1, noise_period=64.0, noise_threshold=0.5,
                          box_min=(-100, -100, -100), box_max=(100, 100, 100), n_luts=4)
    dims = s.objects["n_cluster_pointers_per_dim"]
    assert dims.min() >= 2 and dims.max() <= 5
    assert s.n_clusters == int(np.prod(dims, axis=1).sum())
    assert np.array_equal(s.cluster_pointers, np.arange(s.n_clusters))
    assert s.luts.shape == (4 * 256,)
    assert (s.luts["albedo"] >= 0.05).all() and (s.luts["albedo"] <= 0.95).all()
    d = np.unpackbits(s.voxel_bits.view(np.uint8)).mean()
    assert 0.2 < d < 0.8


def test_make_view_corner_rays_match_tg_camera():
    v = tg.make_view((0, 0, 0), 0.0, float(np.pi), float(np.pi / 3), 256, 256, 0.1, 256.0)[0]
    for k in ("ray_bl", "ray_br", "ray_tr", "ray_tl"):
        assert abs(np.linalg.norm(v[k][:3]) - 1) < 1e-6
    # looking along +z with a 60 degree vertical field of view: half angle 30 degrees
    c = (v["ray_bl"] + v["ray_br"] + v["ray_tr"] + v["ray_tl"])[:3]
    c /= np.linalg.norm(c)
    assert np.allclose(c, [0, 0, 1], atol=1e-6)
    up = (v["ray_tl"] + v["ray_tr"])[:3]
    up /= np.linalg.norm(up)
    assert abs(np.degrees(np.arccos(np.dot(up, c))) - 30.0) < 1e-3


def test_decode_matches_get_hovered_voxel_layout():
    packed = (123456 << 40) | (7777 << 9) | 300
    hit, depth, ptr, vox = tg.decode(packed)
    assert hit and ptr == 7777 and vox == 300 and abs(depth - 123456 / 16777215) < 1e-7
    hit, depth, ptr, vox = tg.decode(tg.VIS_EMPTY)
    assert not hit and depth == 1.0 and ptr == 0xFFFFFFFF


C_PROGRAM = r"""
#include <stdio.h>
#include <stddef.h>
#include "tgx.h"
int main(void)
{
    tgx_view v;
    const float pos[3] = {0.0f, 0.0f, 0.0f};
    if (tgx_abi_version() != TGX_ABI_VERSION) return 2;
    if (tgx_make_view(pos, 0.0f, 3.14159265f, 1.0471976f, 64, 48, 0.1f, 256.0f, &v) != TGX_OK) return 3;
    printf("tgx_object %zu\n", sizeof(tgx_object));
    printf("tgx_view %zu\n", sizeof(tgx_view));
    printf("tgx_material %zu\n", sizeof(tgx_material));
    printf("tgx_scene_desc %zu\n", sizeof(tgx_scene_desc));
    printf("tgx_config %zu\n", sizeof(tgx_config));
    printf("tgx_device_error %zu\n", sizeof(tgx_device_error));
    printf("tgx_vis_stats %zu\n", sizeof(tgx_vis_stats));
    printf("tgx_vis_work %zu\n", sizeof(tgx_vis_work));
    printf("tgx_gi_work %zu\n", sizeof(tgx_gi_work));
    printf("tgx_svo_info %zu\n", sizeof(tgx_svo_info));
    printf("tgx_gi_params %zu\n", sizeof(tgx_gi_params));
    printf("tgx_cache_gi_params %zu\n", sizeof(tgx_cache_gi_params));
    printf("tgx_gen_params %zu\n", sizeof(tgx_gen_params));
    printf("view_width %u\n", v.width);
    return 0;
}
"""


def test_header_compiles_as_c99_and_layouts_match_the_binding(tmp_path):
    """An engine's C translation unit: the header compiles as strict C99,
    links against the library, and every struct has the size the Python
    binding assumes."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("no C compiler")
    src = tmp_path / "engine.c"
    src.write_text(C_PROGRAM)
    exe = tmp_path / "engine"
    lib_dir = tg.LIB_PATH.parent
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-pedantic", "-I", str(ROOT / "include"), str(src),
                    "-L", str(lib_dir), "-ltgx", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    sizes = {k: int(v) for k, v in (line.split() for line in out.strip().splitlines())}
    assert sizes["view_width"] == 64
    assert sizes["tgx_object"] == tg.OBJECT_DTYPE.itemsize
    assert sizes["tgx_view"] == tg.VIEW_DTYPE.itemsize
    assert sizes["tgx_material"] == tg.MATERIAL_DTYPE.itemsize
    assert sizes["tgx_scene_desc"] == C.sizeof(tg.SceneDesc)
    assert sizes["tgx_config"] == C.sizeof(tg.Config)
    assert sizes["tgx_device_error"] == C.sizeof(tg.DeviceError)
    assert sizes["tgx_vis_stats"] == C.sizeof(tg.VisStats)
    assert sizes["tgx_vis_work"] == C.sizeof(tg.VisWork)
    assert sizes["tgx_gi_work"] == C.sizeof(tg.GiWork)
    assert sizes["tgx_svo_info"] == C.sizeof(tg.SvoInfo)
    assert sizes["tgx_gi_params"] == tg.GI_PARAMS_DTYPE.itemsize
    assert sizes["tgx_cache_gi_params"] == tg.CACHE_GI_DTYPE.itemsize
    assert sizes["tgx_gen_params"] == C.sizeof(tg.GenParams)
