"""tg_gb300 -- Python mirror of the tgx C ABI (include/tgx.h).

The compute path is libtgx.so (CUDA for sm_103a behind an ``extern "C"``
boundary).  This module only binds it with ctypes and converts numpy / torch
buffers to plain pointers, the way tg's C host code would call it:

    tg_raytracer_create / create_object / render / clear / get_hovered_voxel
        -> Context, Scene (tgx_scene_upload), Context.vis_render, Context.pick

There is no fallback: if the library is missing, importing raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "libtgx.so"

TGX_OK = 0
STATUS_NAMES = {
    0: "TGX_OK", 1: "TGX_ERR_INVALID_ARGUMENT", 2: "TGX_ERR_OUT_OF_MEMORY", 3: "TGX_ERR_CUDA",
    4: "TGX_ERR_CAPACITY", 5: "TGX_ERR_TIMEOUT", 6: "TGX_ERR_NOT_SUPPORTED", 7: "TGX_ERR_NO_DEVICE",
    8: "TGX_ERR_DEVICE_FAULT",
}
VIS_EMPTY = 0xFFFFFFFFFFFFFFFF
FLAG_MIN_BIN_CAPACITY = 1
FLAG_TEST_LOST_COPY = 2

# numpy views of the C structs -------------------------------------------------

OBJECT_DTYPE = np.dtype([
    ("n_cluster_pointers_per_dim", np.uint32, 3),
    ("first_cluster_pointer", np.uint32),
    ("translation", np.float32, 3),
    ("lut_idx", np.uint32),
    ("rotation", np.float32, 16),
])
assert OBJECT_DTYPE.itemsize == 96

VIEW_DTYPE = np.dtype([
    ("camera", np.float32, 4), ("ray_bl", np.float32, 4), ("ray_br", np.float32, 4),
    ("ray_tr", np.float32, 4), ("ray_tl", np.float32, 4), ("near_plane", np.float32),
    ("far_plane", np.float32), ("width", np.uint32), ("height", np.uint32),
])
assert VIEW_DTYPE.itemsize == 96

MATERIAL_DTYPE = np.dtype([("albedo", np.float32, 3), ("roughness", np.float32)])

GI_PARAMS_DTYPE = np.dtype([
    ("spp", np.uint32), ("bounces", np.uint32), ("max_steps", np.uint32), ("frame", np.uint32),
    ("seed", np.uint64), ("sun_dir", np.float32, 3), ("sun_radiance", np.float32, 3),
    ("sky_radiance", np.float32, 3), ("offset", np.float32),
])
assert GI_PARAMS_DTYPE.itemsize == 64


CACHE_GI_DTYPE = np.dtype([("n_train", np.uint32), ("train_spp", np.uint32), ("train_steps", np.uint32),
                           ("lr", np.float32), ("box_min", np.float32, 3), ("box_max", np.float32, 3),
                           ("primary_weight", np.float32), ("n_train_primary", np.uint32),
                           ("primary_variance_scale", np.float32)])


def cache_gi_params(box_min, box_max, n_train: int = 65536, train_spp: int = 16, train_steps: int = 4,
                    lr: float = 1e-2, primary_weight: float = 0.0, n_train_primary: int = 0,
                    primary_variance_scale: float = 0.0) -> np.ndarray:
    p = np.zeros(1, CACHE_GI_DTYPE)
    p["n_train"], p["train_spp"], p["train_steps"], p["lr"] = n_train, train_spp, train_steps, lr
    p["box_min"], p["box_max"] = box_min, box_max
    p["primary_weight"], p["n_train_primary"] = primary_weight, n_train_primary
    p["primary_variance_scale"] = primary_variance_scale
    return p


def gi_params(spp: int = 4, bounces: int = 1, seed: int = 2, max_steps: int = 256, frame: int = 0,
              sun_dir=(0.3, 0.8, 0.5), sun_radiance=(3.0, 2.9, 2.7), sky_radiance=(0.25, 0.3, 0.4),
              offset: float = 1.0) -> np.ndarray:
    """A tgx_gi_params record; sun_dir is normalised here."""
    p = np.zeros(1, GI_PARAMS_DTYPE)
    d = np.asarray(sun_dir, np.float64)
    p["spp"], p["bounces"], p["max_steps"], p["frame"], p["seed"] = spp, bounces, max_steps, frame, seed
    p["sun_dir"] = (d / np.linalg.norm(d)).astype(np.float32)
    p["sun_radiance"], p["sky_radiance"], p["offset"] = sun_radiance, sky_radiance, offset
    return p


class VisJob(C.Structure):
    _fields_ = [("scene", C.c_void_p), ("views", C.c_void_p), ("n_views", C.c_uint32),
                ("d_visbuf", C.POINTER(C.c_void_p))]


class SceneDesc(C.Structure):
    _fields_ = [
        ("n_objects", C.c_uint32), ("objects", C.c_void_p),
        ("n_cluster_pointers", C.c_uint32), ("cluster_pointers", C.c_void_p),
        ("n_clusters", C.c_uint32), ("cluster_idx_to_object_idx", C.c_void_p),
        ("voxel_bits", C.c_void_p), ("material_idx", C.c_void_p),
        ("n_luts", C.c_uint32), ("luts", C.c_void_p),
    ]


class Config(C.Structure):
    _fields_ = [("device", C.c_int), ("stream", C.c_void_p), ("tile_w", C.c_uint32),
                ("tile_h", C.c_uint32), ("flags", C.c_uint32), ("trace_steps", C.c_uint32)]


class DeviceError(C.Structure):
    _fields_ = [("code", C.c_uint32), ("where", C.c_uint32), ("detail", C.c_uint64)]


class GenParams(C.Structure):
    _fields_ = [
        ("kind", C.c_uint32), ("n_objects", C.c_uint32), ("min_clusters_per_axis", C.c_uint32),
        ("max_clusters_per_axis", C.c_uint32), ("bernoulli_p", C.c_float), ("noise_period", C.c_float),
        ("noise_threshold", C.c_float), ("seed", C.c_uint64), ("box_min", C.c_float * 3),
        ("box_max", C.c_float * 3), ("fixed_translation", C.c_float * 3), ("n_luts", C.c_uint32),
        ("threads", C.c_uint32),
    ]


class GenScene(C.Structure):
    _fields_ = [
        ("desc", SceneDesc), ("objects", C.c_void_p), ("cluster_pointers", C.c_void_p),
        ("cluster_idx_to_object_idx", C.c_void_p), ("voxel_bits", C.c_void_p),
        ("material_idx", C.c_void_p), ("luts", C.c_void_p),
    ]


class VisStats(C.Structure):
    _fields_ = [("visible_clusters", C.c_uint32), ("bin_entries", C.c_uint32), ("tiles", C.c_uint32),
                ("dda_overruns", C.c_uint32)]


class GiWork(C.Structure):
    """tgx_gi_work: the last GI call's SVO traversal work."""
    _fields_ = [("dda_steps", C.c_uint64), ("rays", C.c_uint64)]


class VisWork(C.Structure):
    """tgx_vis_work: the visibility tile kernel's own work counts."""
    _fields_ = [(n, C.c_uint64) for n in ("pairs", "depth_skips", "dir_setups", "slab_misses", "sure_hits",
                                          "exact_tests", "ddas", "dda_steps", "hits", "batches")]

    def as_dict(self) -> dict:
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class SvoInfo(C.Structure):
    _fields_ = [("min", C.c_float * 3), ("extent_log2", C.c_uint32), ("blocks_per_axis", C.c_uint32),
                ("n_blocks", C.c_uint32), ("n_nonempty_blocks", C.c_uint32), ("n_pairs", C.c_uint32),
                ("device_bytes", C.c_uint64)]


# library --------------------------------------------------------------------

EXPORTS = [
    "tgx_abi_version", "tgx_status_string", "tgx_last_error_string", "tgx_create", "tgx_destroy",
    "tgx_stream", "tgx_sync", "tgx_last_device_error", "tgx_launch_count", "tgx_scene_upload",
    "tgx_scene_destroy", "tgx_vis_render", "tgx_vis_render_host", "tgx_vis_decode", "tgx_pick",
    "tgx_svo_build", "tgx_svo_destroy", "tgx_svo_get_info", "tgx_svo_download", "tgx_svo_trace",
    "tgx_generate_scene", "tgx_free_generated_scene", "tgx_make_view", "tgx_trace_enable", "tgx_trace_reset",
    "tgx_trace_slots", "tgx_trace_get", "tgx_vis_get_stats", "tgx_gi_render", "tgx_cache_n_params",
    "tgx_cache_create", "tgx_cache_destroy", "tgx_cache_infer", "tgx_cache_train_step", "tgx_cache_last_loss",
    "tgx_cache_gradient", "tgx_cache_get_weights", "tgx_cache_set_weights", "tgx_cache_save", "tgx_cache_load",
    "tgx_gi_render_cached", "tgx_frame_graph_create", "tgx_frame_graph_launch", "tgx_frame_graph_set_views",
    "tgx_frame_graph_kernels", "tgx_frame_graph_destroy", "tgx_svo_build_flags", "tgx_generate_scene_device",
    "tgx_scene_counts", "tgx_scene_download", "tgx_shade", "tgx_svo_update", "tgx_scene_set_objects",
    "tgx_set_trace_steps", "tgx_vis_render_host_async", "tgx_vis_host_wait", "tgx_vis_count_work",
    "tgx_vis_get_work", "tgx_gi_get_work", "tgx_set_vis_tuning", "tgx_set_memory_budget", "tgx_get_memory",
]


def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(LIB_PATH))
    vp, u32, u64, i32 = C.c_void_p, C.c_uint32, C.c_uint64, C.c_int
    sig = {
        "tgx_abi_version": (u32, []),
        "tgx_status_string": (C.c_char_p, [i32]),
        "tgx_last_error_string": (C.c_char_p, []),
        "tgx_create": (i32, [C.POINTER(Config), C.POINTER(vp)]),
        "tgx_destroy": (None, [vp]),
        "tgx_stream": (vp, [vp]),
        "tgx_sync": (i32, [vp]),
        "tgx_last_device_error": (i32, [vp, C.POINTER(DeviceError)]),
        "tgx_launch_count": (u64, [vp]),
        "tgx_scene_upload": (i32, [vp, C.POINTER(SceneDesc), C.POINTER(vp)]),
        "tgx_scene_destroy": (None, [vp, vp]),
        "tgx_vis_render": (i32, [vp, vp, vp, u32, C.POINTER(vp)]),
        "tgx_vis_render_host": (i32, [vp, vp, vp, u32, C.POINTER(vp)]),
        "tgx_vis_render_host_async": (i32, [vp, vp, vp, u32, C.POINTER(vp)]),
        "tgx_vis_host_wait": (i32, [vp, u32]),
        "tgx_vis_decode": (i32, [u64, C.POINTER(C.c_float), C.POINTER(u32), C.POINTER(u32)]),
        "tgx_pick": (i32, [vp, vp, u32, u32, u32, u32, C.POINTER(C.c_float), C.POINTER(u32), C.POINTER(u32), C.POINTER(i32)]),
        "tgx_svo_build": (i32, [vp, vp, vp, u32, C.POINTER(vp)]),
        "tgx_svo_build_flags": (i32, [vp, vp, vp, u32, u32, C.POINTER(vp)]),
        "tgx_generate_scene_device": (i32, [vp, C.POINTER(GenParams), C.POINTER(vp)]),
        "tgx_scene_counts": (i32, [vp, C.POINTER(u32), C.POINTER(u32), C.POINTER(u32), C.POINTER(u32)]),
        "tgx_scene_download": (i32, [vp, vp, vp, vp, vp, vp, vp, vp]),
        "tgx_shade": (i32, [vp, vp, vp, vp, u32, vp]),
        "tgx_svo_update": (i32, [vp, vp, vp, C.POINTER(u32)]),
        "tgx_set_trace_steps": (i32, [vp, u32]),
        "tgx_scene_set_objects": (i32, [vp, vp, u32, u32, vp]),
        "tgx_svo_destroy": (None, [vp, vp]),
        "tgx_svo_get_info": (i32, [vp, vp, C.POINTER(SvoInfo)]),
        "tgx_svo_download": (i32, [vp, vp, vp, vp, u32, C.POINTER(u32)]),
        "tgx_svo_trace": (i32, [vp, vp, u32, vp, vp, u32, vp, vp]),
        "tgx_generate_scene": (i32, [C.POINTER(GenParams), C.POINTER(GenScene)]),
        "tgx_free_generated_scene": (None, [C.POINTER(GenScene)]),
        "tgx_make_view": (i32, [vp, C.c_float, C.c_float, C.c_float, u32, u32, C.c_float, C.c_float, vp]),
        "tgx_trace_enable": (i32, [vp, i32]),
        "tgx_vis_get_stats": (i32, [vp, C.POINTER(VisStats)]),
        "tgx_vis_count_work": (i32, [vp, i32]),
        "tgx_vis_get_work": (i32, [vp, C.POINTER(VisWork)]),
        "tgx_gi_get_work": (i32, [vp, C.POINTER(GiWork)]),
        "tgx_set_vis_tuning": (i32, [vp, u32, u32, u32]),
        "tgx_set_memory_budget": (i32, [vp, u64]),
        "tgx_get_memory": (i32, [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]),
        "tgx_gi_render": (i32, [vp, vp, vp, vp, vp, vp, vp]),
        "tgx_cache_n_params": (u32, []),
        "tgx_gi_render_cached": (i32, [vp, vp, vp, vp, vp, vp, vp, vp, vp]),
        "tgx_cache_create": (i32, [vp, u64, C.POINTER(vp)]),
        "tgx_cache_destroy": (None, [vp, vp]),
        "tgx_cache_infer": (i32, [vp, vp, u32, vp, vp]),
        "tgx_cache_train_step": (i32, [vp, vp, u32, vp, vp, C.c_float]),
        "tgx_cache_last_loss": (i32, [vp, vp, C.POINTER(C.c_float)]),
        "tgx_cache_gradient": (i32, [vp, vp, u32, vp, vp, vp, C.POINTER(C.c_float)]),
        "tgx_cache_get_weights": (i32, [vp, vp, vp]),
        "tgx_cache_set_weights": (i32, [vp, vp, vp]),
        "tgx_cache_save": (i32, [vp, vp, C.c_char_p]),
        "tgx_cache_load": (i32, [vp, vp, C.c_char_p]),
        "tgx_frame_graph_create": (i32, [vp, C.POINTER(VisJob), u32, C.POINTER(vp)]),
        "tgx_frame_graph_launch": (i32, [vp, vp]),
        "tgx_frame_graph_set_views": (i32, [vp, vp, u32, vp]),
        "tgx_frame_graph_kernels": (u32, [vp]),
        "tgx_frame_graph_destroy": (None, [vp, vp]),
        "tgx_trace_reset": (i32, [vp]),
        "tgx_trace_slots": (u32, []),
        "tgx_trace_get": (i32, [vp, u32, C.POINTER(C.c_char_p), C.POINTER(C.c_double), C.POINTER(u64)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


lib = _load()


class TgxError(RuntimeError):
    def __init__(self, status: int, where: str):
        msg = lib.tgx_last_error_string().decode(errors="replace")
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


def check(status: int, where: str) -> None:
    if status != TGX_OK:
        raise TgxError(status, where)


def _ptr(a) -> int:
    """Address of a numpy array or torch tensor (host or device)."""
    if a is None:
        return 0
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data


# scenes -----------------------------------------------------------------------

class HostScene:
    """A tg scene store held in numpy arrays (tg_scene, tgvk_raytracer.h:90-108)."""

    def __init__(self, objects, cluster_pointers, cluster_idx_to_object_idx, voxel_bits,
                 material_idx=None, luts=None):
        self.objects = np.ascontiguousarray(objects, dtype=OBJECT_DTYPE)
        self.cluster_pointers = np.ascontiguousarray(cluster_pointers, dtype=np.uint32)
        self.cluster_idx_to_object_idx = np.ascontiguousarray(cluster_idx_to_object_idx, dtype=np.uint32)
        self.voxel_bits = np.ascontiguousarray(voxel_bits, dtype=np.uint32).reshape(-1, 16)
        self.material_idx = None if material_idx is None else np.ascontiguousarray(material_idx, dtype=np.uint8).reshape(-1, 512)
        self.luts = None if luts is None else np.ascontiguousarray(luts, dtype=MATERIAL_DTYPE)

    @property
    def n_clusters(self) -> int:
        return self.voxel_bits.shape[0]

    def desc(self) -> SceneDesc:
        d = SceneDesc()
        d.n_objects = len(self.objects)
        d.objects = _ptr(self.objects)
        d.n_cluster_pointers = len(self.cluster_pointers)
        d.cluster_pointers = _ptr(self.cluster_pointers)
        d.n_clusters = self.n_clusters
        d.cluster_idx_to_object_idx = _ptr(self.cluster_idx_to_object_idx)
        d.voxel_bits = _ptr(self.voxel_bits)
        d.material_idx = _ptr(self.material_idx)
        d.n_luts = 0 if self.luts is None else len(self.luts) // 256
        d.luts = _ptr(self.luts)
        return d


def gen_params(kind: int, n_objects: int, min_cpa: int, max_cpa: int, seed: int, *,
               bernoulli_p: float = 0.3, noise_period: float = 64.0, noise_threshold: float = 0.5,
               box_min=(0.0, 0.0, 0.0), box_max=(0.0, 0.0, 0.0), translation=(0.0, 0.0, 0.0),
               n_luts: int = 1, threads: int = 0) -> GenParams:
    p = GenParams(kind=kind, n_objects=n_objects, min_clusters_per_axis=min_cpa, max_clusters_per_axis=max_cpa,
                  bernoulli_p=bernoulli_p, noise_period=noise_period, noise_threshold=noise_threshold, seed=seed,
                  n_luts=n_luts, threads=threads)
    p.box_min[:] = box_min
    p.box_max[:] = box_max
    p.fixed_translation[:] = translation
    return p


def generate_scene(kind: int, n_objects: int, min_cpa: int, max_cpa: int, seed: int, **kw) -> HostScene:
    """Seeded synthetic scene (tgx_generate_scene); arrays are copied into numpy."""
    p = gen_params(kind, n_objects, min_cpa, max_cpa, seed, **kw)
    g = GenScene()
    check(lib.tgx_generate_scene(C.byref(p), C.byref(g)), "tgx_generate_scene")
    try:
        d = g.desc
        n_cl = d.n_clusters

        def arr(ptr, dtype, count):
            buf = (C.c_char * (count * np.dtype(dtype).itemsize)).from_address(ptr)
            return np.frombuffer(buf, dtype=dtype, count=count).copy()

        scene = HostScene(
            arr(g.objects, OBJECT_DTYPE, d.n_objects),
            arr(g.cluster_pointers, np.uint32, d.n_cluster_pointers),
            arr(g.cluster_idx_to_object_idx, np.uint32, n_cl),
            arr(g.voxel_bits, np.uint32, n_cl * 16),
            arr(g.material_idx, np.uint8, n_cl * 512),
            arr(g.luts, MATERIAL_DTYPE, d.n_luts * 256),
        )
    finally:
        lib.tgx_free_generated_scene(C.byref(g))
    return scene


def make_view(position, pitch: float, yaw: float, fov_y: float, width: int, height: int,
              near: float = 0.1, far: float = 256.0) -> np.ndarray:
    """One tgx_view (tg camera corner rays, tgvk_core.c:382-444) as a numpy record."""
    v = np.zeros(1, dtype=VIEW_DTYPE)
    pos = np.asarray(position, dtype=np.float32)
    check(lib.tgx_make_view(_ptr(pos), pitch, yaw, fov_y, width, height, near, far, _ptr(v)), "tgx_make_view")
    return v


def decode(packed: int):
    """tgx_vis_decode: (hit, depth, cluster_pointer, voxel_idx)."""
    d, cp, vx = C.c_float(), C.c_uint32(), C.c_uint32()
    hit = lib.tgx_vis_decode(C.c_uint64(packed), C.byref(d), C.byref(cp), C.byref(vx))
    return bool(hit), d.value, cp.value, vx.value


# context ----------------------------------------------------------------------

class Context:
    """tgx_ctx: one device, one stream."""

    def __init__(self, device: int = 0, stream: int | None = None, tile: tuple[int, int] = (16, 16), flags: int = 0,
                 trace_steps: int = 0):
        cfg = Config(device=device, stream=stream or 0, tile_w=tile[0], tile_h=tile[1], flags=flags,
                     trace_steps=trace_steps)
        h = C.c_void_p()
        check(lib.tgx_create(C.byref(cfg), C.byref(h)), "tgx_create")
        self.handle = h

    def close(self) -> None:
        if self.handle:
            lib.tgx_destroy(self.handle)
            self.handle = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self) -> int:
        return lib.tgx_stream(self.handle) or 0

    def sync(self) -> None:
        check(lib.tgx_sync(self.handle), "tgx_sync")

    def set_trace_steps(self, steps: int) -> None:
        """tgx_set_trace_steps: DDA steps per lane between ray-queue refills."""
        check(lib.tgx_set_trace_steps(self.handle, steps), "tgx_set_trace_steps")

    def launches(self) -> int:
        return int(lib.tgx_launch_count(self.handle))

    def device_error(self) -> DeviceError:
        e = DeviceError()
        lib.tgx_last_device_error(self.handle, C.byref(e))
        return e

    def trace(self, enable: bool) -> None:
        check(lib.tgx_trace_enable(self.handle, int(enable)), "tgx_trace_enable")

    def trace_reset(self) -> None:
        check(lib.tgx_trace_reset(self.handle), "tgx_trace_reset")

    def trace_read(self) -> dict[str, tuple[float, int]]:
        """{kernel name: (summed device ms, launches)} for kernels launched since the last reset."""
        out = {}
        for i in range(lib.tgx_trace_slots()):
            name, ms, n = C.c_char_p(), C.c_double(), C.c_uint64()
            check(lib.tgx_trace_get(self.handle, i, C.byref(name), C.byref(ms), C.byref(n)), "tgx_trace_get")
            if n.value:
                out[name.value.decode()] = (ms.value, int(n.value))
        return out

    def upload(self, scene: HostScene) -> "Scene":
        d = scene.desc()
        h = C.c_void_p()
        check(lib.tgx_scene_upload(self.handle, C.byref(d), C.byref(h)), "tgx_scene_upload")
        return Scene(self, h)

    def vis_render(self, scene: "Scene", views: np.ndarray, outs) -> None:
        """Device outputs: `outs` is a list of device tensors (int64/uint64, W*H each)."""
        views = np.ascontiguousarray(views, dtype=VIEW_DTYPE)
        ptrs = (C.c_void_p * len(views))(*[_ptr(o) for o in outs])
        check(lib.tgx_vis_render(self.handle, scene.handle, _ptr(views), len(views), ptrs), "tgx_vis_render")

    def vis_render_host(self, scene: "Scene", views: np.ndarray, outs) -> None:
        """Host outputs: `outs` is a list of uint64 numpy arrays (W*H each); blocking."""
        views = np.ascontiguousarray(views, dtype=VIEW_DTYPE)
        ptrs = (C.c_void_p * len(views))(*[_ptr(o) for o in outs])
        check(lib.tgx_vis_render_host(self.handle, scene.handle, _ptr(views), len(views), ptrs),
              "tgx_vis_render_host")

    def vis_render_host_async(self, scene: "Scene", views: np.ndarray, outs) -> None:
        """Pipelined host outputs (tgx_vis_render_host_async): returns before
        the buffers are filled; `outs` (uint64 arrays, pinned for overlap) are
        ready after vis_host_wait."""
        views = np.ascontiguousarray(views, dtype=VIEW_DTYPE)
        ptrs = (C.c_void_p * len(views))(*[_ptr(o) for o in outs])
        check(lib.tgx_vis_render_host_async(self.handle, scene.handle, _ptr(views), len(views), ptrs),
              "tgx_vis_render_host_async")

    def vis_host_wait(self, max_in_flight: int = 0) -> None:
        """Waits until at most `max_in_flight` pipelined host renders are pending."""
        check(lib.tgx_vis_host_wait(self.handle, max_in_flight), "tgx_vis_host_wait")

    def generate_scene(self, kind: int, n_objects: int, min_cpa: int, max_cpa: int, seed: int, **kw) -> "Scene":
        """The generate_scene scene built in device memory (tgx_generate_scene_device)."""
        p = gen_params(kind, n_objects, min_cpa, max_cpa, seed, **kw)
        h = C.c_void_p()
        check(lib.tgx_generate_scene_device(self.handle, C.byref(p), C.byref(h)), "tgx_generate_scene_device")
        return Scene(self, h)

    def shade(self, scene: "Scene", view: np.ndarray, visbuf, mode: int, rgba) -> None:
        """tgx_shade: device visbuf (W*H u64) -> device rgba (W*H*4 float32)."""
        view = np.ascontiguousarray(view, dtype=VIEW_DTYPE).reshape(1)
        check(lib.tgx_shade(self.handle, scene.handle, _ptr(view), _ptr(visbuf), mode, _ptr(rgba)), "tgx_shade")

    def frame_graph(self, jobs) -> "FrameGraph":
        """Captures a batched frame: `jobs` is a list of (scene, views, outs) with device
        outputs; returns a FrameGraph whose launch() replays all of it with one graph launch."""
        return FrameGraph(self, jobs)

    def svo_build(self, scene: "Scene", mn, extent_log2: int, materials: bool = True) -> Svo:
        """materials=False leaves out the per-voxel material grid (TGX_SVO_NO_MATERIALS)."""
        m = np.asarray(mn, dtype=np.float32)
        h = C.c_void_p()
        check(lib.tgx_svo_build_flags(self.handle, scene.handle, _ptr(m), extent_log2, 0 if materials else 1,
                                      C.byref(h)), "tgx_svo_build")
        return Svo(self, h)

    def gi_render(self, scene: "Scene", svo: "Svo", view: np.ndarray, visbuf, params: np.ndarray, rgb) -> None:
        """Device buffers: visbuf (W*H u64 as int64), rgb (W*H*3 float32)."""
        view = np.ascontiguousarray(view, dtype=VIEW_DTYPE).reshape(1)
        params = np.ascontiguousarray(params, dtype=GI_PARAMS_DTYPE).reshape(1)
        check(lib.tgx_gi_render(self.handle, scene.handle, svo.handle, _ptr(view), _ptr(visbuf), _ptr(params),
                                _ptr(rgb)), "tgx_gi_render")

    def gi_render_cached(self, scene: "Scene", svo: "Svo", cache: "Cache", view: np.ndarray, visbuf,
                         params: np.ndarray, cache_params: np.ndarray, rgb) -> None:
        view = np.ascontiguousarray(view, dtype=VIEW_DTYPE).reshape(1)
        params = np.ascontiguousarray(params, dtype=GI_PARAMS_DTYPE).reshape(1)
        cp = np.ascontiguousarray(cache_params, dtype=CACHE_GI_DTYPE).reshape(1)
        check(lib.tgx_gi_render_cached(self.handle, scene.handle, svo.handle, cache.handle, _ptr(view), _ptr(visbuf),
                                       _ptr(params), _ptr(cp), _ptr(rgb)), "tgx_gi_render_cached")

    def vis_stats(self) -> VisStats:
        st = VisStats()
        check(lib.tgx_vis_get_stats(self.handle, C.byref(st)), "tgx_vis_get_stats")
        return st

    def set_memory_budget(self, nbytes: int) -> None:
        """tgx_set_memory_budget: cap on the bytes of this context's scene stores (0: none)."""
        check(lib.tgx_set_memory_budget(self.handle, nbytes), "tgx_set_memory_budget")

    def memory(self) -> tuple[int, int]:
        """tgx_get_memory: (budget, bytes held by live scene stores)."""
        b, u = C.c_uint64(), C.c_uint64()
        check(lib.tgx_get_memory(self.handle, C.byref(b), C.byref(u)), "tgx_get_memory")
        return b.value, u.value

    def set_vis_tuning(self, depth_buckets: int = 0, batch: int = 0, drain: int = 0) -> None:
        """tgx_set_vis_tuning: depth buckets per tile (8/16/32), clusters per staged batch (1..48) and pairs per
        DDA round (1..32); 0 keeps the default.  Results do not depend on them."""
        check(lib.tgx_set_vis_tuning(self.handle, depth_buckets, batch, drain), "tgx_set_vis_tuning")

    def vis_count_work(self, enable: bool) -> None:
        """tgx_vis_count_work: later renders run the tile kernel's counting variant."""
        check(lib.tgx_vis_count_work(self.handle, int(enable)), "tgx_vis_count_work")

    def gi_work(self) -> GiWork:
        """tgx_gi_get_work: the last GI call's traversal steps and rays (blocking)."""
        w = GiWork()
        check(lib.tgx_gi_get_work(self.handle, C.byref(w)), "tgx_gi_get_work")
        return w

    def vis_work(self) -> VisWork:
        """tgx_vis_get_work: the last counted render's work totals (blocking)."""
        w = VisWork()
        check(lib.tgx_vis_get_work(self.handle, C.byref(w)), "tgx_vis_get_work")
        return w

    def pick(self, d_visbuf, w: int, h: int, x: int, y: int):
        d, cp, vx, hit = C.c_float(), C.c_uint32(), C.c_uint32(), C.c_int()
        check(lib.tgx_pick(self.handle, _ptr(d_visbuf), w, h, x, y, C.byref(d), C.byref(cp), C.byref(vx),
                           C.byref(hit)), "tgx_pick")
        return bool(hit.value), d.value, cp.value, vx.value


class FrameGraph:
    """tgx_frame_graph: the visibility passes of many (scene, views) jobs as one CUDA graph."""

    def __init__(self, ctx: "Context", jobs):
        self.ctx = ctx
        self._keep = []
        arr = (VisJob * len(jobs))()
        for i, (scene, views, outs) in enumerate(jobs):
            v = np.ascontiguousarray(views, dtype=VIEW_DTYPE).reshape(-1)
            ptrs = (C.c_void_p * len(v))(*[_ptr(o) for o in outs])
            self._keep += [v, ptrs, outs]
            arr[i].scene = scene.handle
            arr[i].views = v.ctypes.data
            arr[i].n_views = len(v)
            arr[i].d_visbuf = ptrs
        h = C.c_void_p()
        check(lib.tgx_frame_graph_create(ctx.handle, arr, len(jobs), C.byref(h)), "tgx_frame_graph_create")
        self.handle = h

    @property
    def kernels(self) -> int:
        return int(lib.tgx_frame_graph_kernels(self.handle))

    def launch(self) -> None:
        check(lib.tgx_frame_graph_launch(self.ctx.handle, self.handle), "tgx_frame_graph_launch")

    def set_views(self, job: int, views) -> None:
        v = np.ascontiguousarray(views, dtype=VIEW_DTYPE).reshape(-1)
        check(lib.tgx_frame_graph_set_views(self.ctx.handle, self.handle, job, _ptr(v)), "tgx_frame_graph_set_views")

    def close(self) -> None:
        if self.handle and self.ctx.handle:
            lib.tgx_frame_graph_destroy(self.ctx.handle, self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Svo:
    """tgx_svo: the one-bit voxel set of tg_svo_create on the device."""

    def __init__(self, ctx: "Context", handle):
        self.ctx = ctx
        self.handle = handle

    def info(self) -> SvoInfo:
        i = SvoInfo()
        check(lib.tgx_svo_get_info(self.ctx.handle, self.handle, C.byref(i)), "tgx_svo_get_info")
        return i

    def download(self):
        """(block_xyz int32[n,3], words uint32[n,1024]) of the non-empty blocks, sorted by block index."""
        n = C.c_uint32()
        check(lib.tgx_svo_download(self.ctx.handle, self.handle, None, None, 0, C.byref(n)), "tgx_svo_download")
        xyz = np.zeros((n.value, 3), np.int32)
        words = np.zeros((n.value, 1024), np.uint32)
        check(lib.tgx_svo_download(self.ctx.handle, self.handle, _ptr(xyz), _ptr(words), n.value, C.byref(n)),
              "tgx_svo_download")
        return xyz, words

    def update(self, scene: "Scene") -> int:
        """tgx_svo_update: follow the scene's moved objects; returns how many moved."""
        n = C.c_uint32()
        check(lib.tgx_svo_update(self.ctx.handle, self.handle, scene.handle, C.byref(n)), "tgx_svo_update")
        return n.value

    def trace(self, origins, dirs, t_out, voxel_out, max_steps: int = 4096) -> None:
        """Device arrays: origins/dirs float32[n,3], t_out float32[n], voxel_out int32[n,3]."""
        n = origins.shape[0]
        check(lib.tgx_svo_trace(self.ctx.handle, self.handle, n, _ptr(origins), _ptr(dirs), max_steps, _ptr(t_out),
                                _ptr(voxel_out)), "tgx_svo_trace")

    def close(self) -> None:
        if self.handle and self.ctx.handle:
            lib.tgx_svo_destroy(self.ctx.handle, self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Cache:
    """tgx_cache: the learned radiance cache MLP (inputs n x 9, outputs n x 3, device memory)."""

    def __init__(self, ctx: "Context", seed: int = 0):
        self.ctx = ctx
        h = C.c_void_p()
        check(lib.tgx_cache_create(ctx.handle, seed, C.byref(h)), "tgx_cache_create")
        self.handle = h
        self.n_params = int(lib.tgx_cache_n_params())

    def infer(self, x, out) -> None:
        check(lib.tgx_cache_infer(self.ctx.handle, self.handle, x.shape[0], _ptr(x), _ptr(out)), "tgx_cache_infer")

    def train_step(self, x, target, lr: float = 1e-2) -> None:
        check(lib.tgx_cache_train_step(self.ctx.handle, self.handle, x.shape[0], _ptr(x), _ptr(target), lr),
              "tgx_cache_train_step")

    def last_loss(self) -> float:
        v = C.c_float()
        check(lib.tgx_cache_last_loss(self.ctx.handle, self.handle, C.byref(v)), "tgx_cache_last_loss")
        return v.value

    def gradient(self, x, target):
        g = np.zeros(self.n_params, np.float32)
        loss = C.c_float()
        check(lib.tgx_cache_gradient(self.ctx.handle, self.handle, x.shape[0], _ptr(x), _ptr(target), _ptr(g),
                                     C.byref(loss)), "tgx_cache_gradient")
        return loss.value, g

    def get_weights(self) -> np.ndarray:
        w = np.zeros(self.n_params, np.float32)
        check(lib.tgx_cache_get_weights(self.ctx.handle, self.handle, _ptr(w)), "tgx_cache_get_weights")
        return w

    def set_weights(self, w) -> None:
        w = np.ascontiguousarray(w, np.float32)
        check(lib.tgx_cache_set_weights(self.ctx.handle, self.handle, _ptr(w)), "tgx_cache_set_weights")

    def save(self, path) -> None:
        check(lib.tgx_cache_save(self.ctx.handle, self.handle, str(path).encode()), "tgx_cache_save")

    def load(self, path) -> None:
        check(lib.tgx_cache_load(self.ctx.handle, self.handle, str(path).encode()), "tgx_cache_load")

    def close(self) -> None:
        if self.handle and self.ctx.handle:
            lib.tgx_cache_destroy(self.ctx.handle, self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Scene:
    def __init__(self, ctx: Context, handle):
        self.ctx = ctx
        self.handle = handle

    def download(self) -> HostScene:
        """The scene's arrays back in host memory (tgx_scene_download)."""
        n = [C.c_uint32() for _ in range(4)]
        check(lib.tgx_scene_counts(self.handle, *[C.byref(x) for x in n]), "tgx_scene_counts")
        n_obj, n_cp, n_cl, n_lut = (x.value for x in n)
        objs = np.zeros(n_obj, OBJECT_DTYPE)
        cp = np.zeros(n_cp, np.uint32)
        c2o = np.zeros(n_cl, np.uint32)
        bits = np.zeros((n_cl, 16), np.uint32)
        mat = np.zeros(n_cl * 512, np.uint8)
        luts = np.zeros(n_lut * 256, MATERIAL_DTYPE)
        check(lib.tgx_scene_download(self.ctx.handle, self.handle, _ptr(objs), _ptr(cp), _ptr(c2o), _ptr(bits),
                                     _ptr(mat), _ptr(luts) if n_lut else None), "tgx_scene_download")
        return HostScene(objs, cp, c2o, bits, mat, luts if n_lut else None)

    def set_objects(self, first: int, objects) -> None:
        """tgx_scene_set_objects: new poses (or LUTs) for objects first .. first+len-1 (OBJECT_DTYPE records)."""
        objs = np.ascontiguousarray(objects, OBJECT_DTYPE)
        check(lib.tgx_scene_set_objects(self.ctx.handle, self.handle, first, objs.shape[0], _ptr(objs)),
              "tgx_scene_set_objects")

    def close(self) -> None:
        if self.handle and self.ctx.handle:
            lib.tgx_scene_destroy(self.ctx.handle, self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
