"""The no-allocation visibility entry point (tgx_vis_render_noalloc).

It serves callers that cannot call cudaMalloc themselves (an engine or plugin
host that owns every device allocation).  It keeps all its scratch in one
fixed device array inside the library instead.  This test calls it through
the C ABI with the scene in device memory the test owns, twice in a row with
different views. Each result must equal the regular tgx_vis_render output for
the same view, bit for bit (the tolerance of all visibility tests). That
shows the shared scratch is reset between calls. The file name sorts last,
so a run that stops at the first failure has run every other test first.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import tg_gb300 as tg

pytestmark = pytest.mark.gpu


def _bind():
    fn = tg.lib.tgx_vis_render_noalloc
    vp = C.c_void_p
    fn.restype = C.c_int
    fn.argtypes = [vp, vp, C.c_uint32, vp, C.c_uint32, vp, vp, vp, vp, C.POINTER(tg.DeviceError)]
    return fn


def test_no_alloc_entry_point_matches_vis_render():
    import torch

    noalloc = _bind()
    scene = tg.generate_scene(1, 24, 2, 6, seed=5, noise_period=16.0, noise_threshold=0.5,
                              box_min=(-120.0, -120.0, -120.0), box_max=(120.0, 120.0, 120.0), n_luts=2)
    views = [tg.make_view((0.0, 0.0, 0.0), 0.0, float(np.pi), float(np.pi / 3), 320, 200, 0.1, 512.0),
             tg.make_view((10.0, 5.0, -30.0), 0.2, 0.4, 1.1, 257, 131, 0.1, 512.0)]

    # the regular entry point (context-owned scratch) gives the expected buffers
    expected = []
    with tg.Context(0) as ctx:
        sc = ctx.upload(scene)
        for v in views:
            out = torch.empty(int(v["width"][0]) * int(v["height"][0]), dtype=torch.int64, device="cuda")
            ctx.vis_render(sc, v, [out])
            ctx.sync()
            assert ctx.device_error().code == 0
            expected.append(out.cpu().numpy().view(np.uint64).copy())
        sc.close()

    dev = torch.device("cuda", 0)
    d_objects = torch.from_numpy(scene.objects.view(np.uint8).copy()).to(dev)
    d_ptrs = torch.from_numpy(scene.cluster_pointers.view(np.int32).copy()).to(dev)
    d_c2o = torch.from_numpy(scene.cluster_idx_to_object_idx.view(np.int32).copy()).to(dev)
    d_bits = torch.from_numpy(scene.voxel_bits.reshape(-1).view(np.int32).copy()).to(dev)
    torch.cuda.synchronize()
    for v, want in zip(views, expected):
        out = torch.full((int(v["width"][0]) * int(v["height"][0]),), -7, dtype=torch.int64, device=dev)
        err = tg.DeviceError()
        st = noalloc(None, d_objects.data_ptr(), len(scene.objects), d_ptrs.data_ptr(), len(scene.cluster_pointers),
                     d_c2o.data_ptr(), d_bits.data_ptr(), v.ctypes.data, out.data_ptr(), C.byref(err))
        assert st == 0, tg.lib.tgx_last_error_string()
        assert err.code == 0
        got = out.cpu().numpy().view(np.uint64)
        assert np.array_equal(got, want), int((got != want).sum())
        assert (got != np.uint64(tg.VIS_EMPTY)).sum() > 100


def test_no_alloc_entry_point_rejects_oversized_inputs():
    noalloc = _bind()
    v = tg.make_view((0.0, 0.0, 0.0), 0.0, 0.0, 1.0, 8000, 8000, 0.1, 100.0)
    st = noalloc(None, 1, 1, 1, 1, 1, 1, v.ctypes.data, 1, None)
    assert st == 4 and b"tiles" in tg.lib.tgx_last_error_string()
    st = noalloc(None, 1, 70000, 1, 1, 1, 1, v.ctypes.data, 1, None)
    assert st == 4 and b"objects" in tg.lib.tgx_last_error_string()
