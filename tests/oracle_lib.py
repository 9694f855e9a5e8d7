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
    lib = C.CDLL(str(REF_SO))
    lib.tgref_last_assert.restype = C.c_char_p
    return lib


class Oracle:
    def __init__(self):
        self.lib = load_oracle()

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
