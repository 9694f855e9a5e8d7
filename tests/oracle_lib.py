"""ctypes bindings of the CPU oracle (oracle/_build/liboracle.so) and of the
reference's own CPU code (oracle/_ref/libtgref.so, present only where the
reference sources were available at build time).  Test infrastructure."""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
ORACLE_SO = ROOT / "oracle" / "_build" / "liboracle.so"
REF_SO = ROOT / "oracle" / "_ref" / "libtgref.so"


def _p(a) -> int:
    return 0 if a is None else a.ctypes.data


def load_oracle() -> C.CDLL:
    lib = C.CDLL(str(ORACLE_SO))
    vp, u32, u64 = C.c_void_p, C.c_uint32, C.c_uint64
    lib.oracle_vis_pair.restype = C.c_int
    lib.oracle_vis_pair.argtypes = [vp, vp, vp, vp, vp, u32, u32, u32, vp]
    lib.oracle_vis_render.restype = u64
    lib.oracle_vis_render.argtypes = [vp, u32, vp, vp, vp, vp, vp, C.c_int, u32, u32, C.c_int]
    lib.oracle_svo_build.restype = C.c_int64
    lib.oracle_svo_build.argtypes = [vp, u32, u32, vp, vp, vp, vp, u32, vp, vp, u32, vp]
    return lib


def load_ref() -> C.CDLL | None:
    if not REF_SO.exists():
        return None
    try:
        lib = C.CDLL(str(REF_SO))
    except OSError:   # built for another machine (the library ships with the tree)
        return None
    lib.tgref_last_assert.restype = C.c_char_p
    return lib


# numpy layouts of include/tgx.h's records, kept here so that this module
# never loads the product library (bench.py's CPU reference arm uses it alone)
OBJECT_DTYPE = np.dtype([
    ("n_cluster_pointers_per_dim", np.uint32, 3), ("first_cluster_pointer", np.uint32),
    ("translation", np.float32, 3), ("lut_idx", np.uint32), ("rotation", np.float32, 16),
])
VIEW_DTYPE = np.dtype([
    ("camera", np.float32, 4), ("ray_bl", np.float32, 4), ("ray_br", np.float32, 4),
    ("ray_tr", np.float32, 4), ("ray_tl", np.float32, 4), ("near_plane", np.float32),
    ("far_plane", np.float32), ("width", np.uint32), ("height", np.uint32),
])
MATERIAL_DTYPE = np.dtype([("albedo", np.float32, 3), ("roughness", np.float32)])
assert OBJECT_DTYPE.itemsize == 96 and VIEW_DTYPE.itemsize == 96


class _GenParams(C.Structure):
    """tgx_gen_params (include/tgx.h)."""
    _fields_ = [
        ("kind", C.c_uint32), ("n_objects", C.c_uint32), ("min_clusters_per_axis", C.c_uint32),
        ("max_clusters_per_axis", C.c_uint32), ("bernoulli_p", C.c_float), ("noise_period", C.c_float),
        ("noise_threshold", C.c_float), ("seed", C.c_uint64), ("box_min", C.c_float * 3),
        ("box_max", C.c_float * 3), ("fixed_translation", C.c_float * 3), ("n_luts", C.c_uint32),
        ("threads", C.c_uint32),
    ]


class OracleScene:
    """A scene store in numpy arrays with the fields the oracle reads."""

    def __init__(self, objects, cluster_pointers, cluster_idx_to_object_idx, voxel_bits, material_idx, luts):
        self.objects = objects
        self.cluster_pointers = cluster_pointers
        self.cluster_idx_to_object_idx = cluster_idx_to_object_idx
        self.voxel_bits = voxel_bits
        self.material_idx = material_idx
        self.luts = luts


class Oracle:
    def __init__(self):
        self.lib = load_oracle()
        lib = self.lib
        vp = C.c_void_p
        lib.oracle_gen_objects.restype = C.c_uint64
        lib.oracle_gen_objects.argtypes = [vp, vp]
        lib.oracle_gen_fill.argtypes = [vp, vp, C.c_uint32, vp, vp, vp, vp, vp]
        lib.oracle_make_view.restype = C.c_int
        lib.oracle_make_view.argtypes = [vp, C.c_float, C.c_float, C.c_float, C.c_uint32, C.c_uint32, C.c_float,
                                         C.c_float, vp]

    def generate_scene(self, kind: int, n_objects: int, min_cpa: int, max_cpa: int, seed: int, *,
                       bernoulli_p: float = 0.3, noise_period: float = 64.0, noise_threshold: float = 0.5,
                       box_min=(0.0, 0.0, 0.0), box_max=(0.0, 0.0, 0.0), translation=(0.0, 0.0, 0.0),
                       n_luts: int = 1, threads: int = 0) -> OracleScene:
        """The seeded synthetic scene, from the oracle's own generator (oracle_scene.c);
        the arguments mean what they mean for the product's tgx_generate_scene."""
        p = _GenParams(kind=kind, n_objects=n_objects, min_clusters_per_axis=min_cpa,
                       max_clusters_per_axis=max_cpa, bernoulli_p=bernoulli_p, noise_period=noise_period,
                       noise_threshold=noise_threshold, seed=seed, n_luts=n_luts, threads=threads)
        p.box_min[:] = box_min
        p.box_max[:] = box_max
        p.fixed_translation[:] = translation
        objects = np.zeros(n_objects, OBJECT_DTYPE)
        n = int(self.lib.oracle_gen_objects(C.byref(p), _p(objects)))
        assert n > 0, "scene too large"
        cp = np.zeros(n, np.uint32)
        c2o = np.zeros(n, np.uint32)
        bits = np.zeros((n, 16), np.uint32)
        mats = np.zeros((n, 512), np.uint8)
        luts = np.zeros(max(1, n_luts) * 256, MATERIAL_DTYPE)
        self.lib.oracle_gen_fill(C.byref(p), _p(objects), n, _p(cp), _p(c2o), _p(bits), _p(mats), _p(luts))
        return OracleScene(objects, cp, c2o, bits, mats, luts)

    def make_view(self, position, pitch: float, yaw: float, fov_y: float, width: int, height: int,
                  near: float = 0.1, far: float = 256.0) -> np.ndarray:
        """tg's pinhole view (oracle_make_view) as a one-record array."""
        v = np.zeros(1, VIEW_DTYPE)
        pos = np.asarray(position, np.float32)
        assert self.lib.oracle_make_view(_p(pos), pitch, yaw, fov_y, width, height, near, far, _p(v)) == 0
        return v

    def vis_render(self, scene, view, mode: int = 1, rows=None, threads: int = 0) -> np.ndarray:
        v = np.ascontiguousarray(view).reshape(1)
        W, H = int(v["width"][0]), int(v["height"][0])
        out = np.full(W * H, np.uint64(0xFFFFFFFFFFFFFFFF), dtype=np.uint64)
        r0, r1 = (0, H) if rows is None else rows
        self.pairs = self.lib.oracle_vis_render(
            _p(scene.objects), len(scene.cluster_pointers), _p(scene.cluster_pointers),
            _p(scene.cluster_idx_to_object_idx), _p(scene.voxel_bits), _p(v), _p(out), mode, r0, r1, threads)
        return out

    def vis_pair(self, scene, view, cluster_pointer: int, px: int, py: int):
        v = np.ascontiguousarray(view).reshape(1)
        out = np.zeros(1, np.uint64)
        hit = self.lib.oracle_vis_pair(_p(scene.objects), _p(scene.cluster_pointers),
                                       _p(scene.cluster_idx_to_object_idx), _p(scene.voxel_bits), _p(v),
                                       cluster_pointer, px, py, _p(out))
        return int(out[0]) if hit else None

    def svo_build(self, scene, mn, extent_log2: int, capacity: int = 1 << 16):
        mn = np.asarray(mn, np.float32)
        blocks = np.zeros((capacity, 3), np.int32)
        words = np.zeros((capacity, 1024), np.uint32)
        samples = np.zeros(1, np.uint64)
        n = self.lib.oracle_svo_build(_p(scene.objects), len(scene.objects), len(scene.cluster_pointers),
                                      _p(scene.cluster_pointers), _p(scene.cluster_idx_to_object_idx),
                                      _p(scene.voxel_bits), _p(mn), extent_log2, _p(blocks), _p(words),
                                      capacity, _p(samples))
        assert n <= capacity, "capacity too small"
        return blocks[:n].copy(), words[:n].copy(), int(samples[0])


GI_PARAMS_DTYPE = np.dtype([
    ("spp", np.uint32), ("bounces", np.uint32), ("max_steps", np.uint32), ("frame", np.uint32),
    ("seed", np.uint64), ("sun_dir", np.float32, 3), ("sun_radiance", np.float32, 3),
    ("sky_radiance", np.float32, 3), ("offset", np.float32),
])
assert GI_PARAMS_DTYPE.itemsize == 64


class OracleSvo:
    """The oracle's view of an SVO (non-empty blocks + optional materials)."""

    def __init__(self, oracle: "Oracle", block_xyz, words, mats, mn, L):
        lib = oracle.lib
        vp, u32 = C.c_void_p, C.c_uint32
        lib.oracle_svo_open.restype = vp
        lib.oracle_svo_open.argtypes = [vp, vp, vp, u32, vp, u32]
        lib.oracle_svo_close.argtypes = [vp]
        lib.oracle_trace_batch.argtypes = [vp, u32, vp, vp, u32, vp, vp, vp, vp]
        self.lib = lib
        self._keep = (np.ascontiguousarray(block_xyz, np.int32), np.ascontiguousarray(words, np.uint32),
                      None if mats is None else np.ascontiguousarray(mats, np.uint16), np.asarray(mn, np.float32))
        b, w, m, mnv = self._keep
        self.h = lib.oracle_svo_open(_p(b), _p(w), _p(m), len(b), _p(mnv), L)
        self.mn = mnv
        self.L = L

    def trace(self, o, d, max_steps: int = 1 << 20):
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        n = len(o)
        t = np.zeros(n, np.float32)
        vox = np.zeros((n, 3), np.int32)
        ax = np.zeros(n, np.int32)
        steps = np.zeros(n, np.uint32)
        self.lib.oracle_trace_batch(self.h, n, _p(o), _p(d), max_steps, _p(t), _p(vox), _p(ax), _p(steps))
        return t, vox, ax, steps

    def close(self):
        if self.h:
            self.lib.oracle_svo_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def svo_build_with_materials(oracle: "Oracle", scene, mn, L, capacity: int = 1 << 14):
    lib = oracle.lib
    vp, u32 = C.c_void_p, C.c_uint32
    lib.oracle_svo_build_mat.restype = C.c_int64
    lib.oracle_svo_build_mat.argtypes = [vp, u32, u32, vp, vp, vp, vp, vp, u32, vp, vp, vp, u32, vp]
    mnv = np.asarray(mn, np.float32)
    blocks = np.zeros((capacity, 3), np.int32)
    words = np.zeros((capacity, 1024), np.uint32)
    mats = np.zeros((capacity, 32768), np.uint16)
    samples = np.zeros(1, np.uint64)
    n = lib.oracle_svo_build_mat(_p(scene.objects), len(scene.objects), len(scene.cluster_pointers),
                                 _p(scene.cluster_pointers), _p(scene.cluster_idx_to_object_idx),
                                 _p(scene.voxel_bits), _p(scene.material_idx), _p(mnv), L, _p(blocks), _p(words),
                                 _p(mats), capacity, _p(samples))
    assert n <= capacity
    return blocks[:n].copy(), words[:n].copy(), mats[:n].copy()


def gi_render(oracle: "Oracle", osvo: OracleSvo, scene, view, params, visbuf, rows=None, threads: int = 0):
    lib = oracle.lib
    vp, u32 = C.c_void_p, C.c_uint32
    lib.oracle_gi_render.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, u32, u32, C.c_int]
    v = np.ascontiguousarray(view).reshape(1)
    W, H = int(v["width"][0]), int(v["height"][0])
    out = np.zeros((H * W, 3), np.float32)
    r0, r1 = (0, H) if rows is None else rows
    p = np.ascontiguousarray(params, GI_PARAMS_DTYPE).reshape(1)
    lib.oracle_gi_render(osvo.h, _p(scene.objects), _p(scene.cluster_pointers), _p(scene.cluster_idx_to_object_idx),
                         _p(scene.material_idx), _p(scene.luts), _p(v), _p(p),
                         _p(np.ascontiguousarray(visbuf, np.uint64)), _p(out), r0, r1, threads)
    return out


class OracleMlp:
    """FP64 oracle of the radiance-cache network (oracle/oracle_mlp.c)."""

    def __init__(self, oracle: "Oracle"):
        lib = oracle.lib
        vp, u32 = C.c_void_p, C.c_uint32
        lib.oracle_mlp_n_params.restype = C.c_int
        lib.oracle_mlp_encode.argtypes = [vp, u32, vp]
        lib.oracle_mlp_forward.argtypes = [vp, vp, u32, vp]
        lib.oracle_mlp_loss_grad.restype = C.c_double
        lib.oracle_mlp_loss_grad.argtypes = [vp, vp, vp, u32, vp]
        lib.oracle_mlp_adam.argtypes = [vp, vp, vp, vp, u32, u32, C.c_double, C.c_double, C.c_double, C.c_double]
        self.lib = lib
        self.n_params = lib.oracle_mlp_n_params()

    def encode(self, x):
        x = np.ascontiguousarray(x, np.float32)
        out = np.zeros((len(x), 216), np.float64)
        self.lib.oracle_mlp_encode(_p(x), len(x), _p(out))
        return out

    def forward(self, w, x):
        x = np.ascontiguousarray(x, np.float32)
        w = np.ascontiguousarray(w, np.float64)
        out = np.zeros((len(x), 3), np.float64)
        self.lib.oracle_mlp_forward(_p(w), _p(x), len(x), _p(out))
        return out

    def loss_grad(self, w, x, t):
        x = np.ascontiguousarray(x, np.float32)
        t = np.ascontiguousarray(t, np.float32)
        w = np.ascontiguousarray(w, np.float64)
        g = np.zeros(self.n_params, np.float64)
        loss = self.lib.oracle_mlp_loss_grad(_p(w), _p(x), _p(t), len(x), _p(g))
        return loss, g

    def adam(self, w, m, v, g, step, lr=1e-2, b1=0.9, b2=0.99, eps=1e-15):
        self.lib.oracle_mlp_adam(_p(w), _p(m), _p(v), _p(np.ascontiguousarray(g, np.float64)), self.n_params, step,
                                 lr, b1, b2, eps)


def shade_render(oracle: "Oracle", scene, view, visbuf, mode: int) -> np.ndarray:
    """oracle_shade_render: RGBA float32 [H*W, 4] of the shading pass."""
    v = np.ascontiguousarray(view).reshape(1)
    W, H = int(v["width"][0]), int(v["height"][0])
    out = np.zeros((W * H, 4), np.float32)
    vb = np.ascontiguousarray(visbuf, np.uint64)
    oracle.lib.oracle_shade_render(C.c_void_p(_p(scene.objects)), C.c_void_p(_p(scene.cluster_pointers)),
                                   C.c_void_p(_p(scene.cluster_idx_to_object_idx)), C.c_void_p(_p(scene.material_idx)),
                                   C.c_void_p(_p(scene.luts)), C.c_void_p(_p(v)), C.c_void_p(_p(vb)),
                                   C.c_uint32(mode), C.c_void_p(_p(out)))
    return out
