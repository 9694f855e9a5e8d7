"""The no-allocation visibility entry point (tgx_vis_render_noalloc).

It serves callers that cannot call cudaMalloc themselves (an engine or plugin
host that owns every device allocation).  It keeps all its scratch in one
fixed device array inside the library instead.  These tests call it through
the C ABI with the scene in device memory the test owns.  Every result must
equal the regular tgx_vis_render output for the same view, bit for bit (the
tolerance of all visibility tests).  Calls in a row go small -> large ->
small on a caller's stream, one of them without the status read-back, so
stale scratch from a larger frame would show.  A frame that needs more bin
entries than the fixed bins hold takes the exact record-scan path and still
matches.  The file name sorts last, so a run that stops at the first failure
has run every other test first.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import tg_gb300 as tg

pytestmark = pytest.mark.gpu

NA_BINS = 1 << 18   # the fixed bins of the entry point (include/tgx.h)


def _bind():
    fn = tg.lib.tgx_vis_render_noalloc
    vp = C.c_void_p
    fn.restype = C.c_int
    fn.argtypes = [vp, vp, C.c_uint32, vp, C.c_uint32, vp, vp, vp, vp, C.POINTER(tg.DeviceError)]
    return fn


def _expected(scene, views):
    """tgx_vis_render with 16x16 tiles (the entry point's tile): the buffers
    and each frame's bin-entry count."""
    import torch
    out_bufs, entries = [], []
    with tg.Context(0, tile=(16, 16)) as ctx:
        sc = ctx.upload(scene)
        for v in views:
            out = torch.empty(int(v["width"][0]) * int(v["height"][0]), dtype=torch.int64, device="cuda")
            ctx.vis_render(sc, v, [out])
            ctx.sync()
            assert ctx.device_error().code == 0
            out_bufs.append(out.cpu().numpy().view(np.uint64).copy())
            entries.append(int(ctx.vis_stats().bin_entries))
        sc.close()
    return out_bufs, entries


def _device_scene(scene):
    import torch
    dev = torch.device("cuda", 0)
    arrays = (torch.from_numpy(scene.objects.view(np.uint8).copy()).to(dev),
              torch.from_numpy(scene.cluster_pointers.view(np.int32).copy()).to(dev),
              torch.from_numpy(scene.cluster_idx_to_object_idx.view(np.int32).copy()).to(dev),
              torch.from_numpy(scene.voxel_bits.reshape(-1).view(np.int32).copy()).to(dev))
    torch.cuda.synchronize()
    return arrays


def _call(fn, stream, scene, dev_arrays, view, out, err):
    d_objects, d_ptrs, d_c2o, d_bits = dev_arrays
    return fn(stream, d_objects.data_ptr(), len(scene.objects), d_ptrs.data_ptr(), len(scene.cluster_pointers),
              d_c2o.data_ptr(), d_bits.data_ptr(), view.ctypes.data, out.data_ptr(),
              None if err is None else C.byref(err))


def test_no_alloc_entry_point_matches_vis_render():
    import torch

    noalloc = _bind()
    scene = tg.generate_scene(1, 24, 2, 6, seed=5, noise_period=16.0, noise_threshold=0.5,
                              box_min=(-120.0, -120.0, -120.0), box_max=(120.0, 120.0, 120.0), n_luts=2)
    views = [tg.make_view((10.0, 5.0, -30.0), 0.2, 0.4, 1.1, 160, 100, 0.1, 512.0),
             tg.make_view((0.0, 0.0, 0.0), 0.0, float(np.pi), float(np.pi / 3), 1280, 720, 0.1, 512.0),
             tg.make_view((-20.0, 8.0, 15.0), -0.1, 2.2, 0.9, 257, 131, 0.1, 512.0)]
    expected, _ = _expected(scene, views)
    arrays = _device_scene(scene)

    # twice in a row on the legacy default stream, with the status read-back
    for v, want in zip(views[:2], expected[:2]):
        out = torch.full((int(v["width"][0]) * int(v["height"][0]),), -7, dtype=torch.int64, device="cuda")
        err = tg.DeviceError()
        st = _call(noalloc, None, scene, arrays, v, out, err)
        assert st == 0, tg.lib.tgx_last_error_string()
        assert err.code == 0
        got = out.cpu().numpy().view(np.uint64)
        assert np.array_equal(got, want), int((got != want).sum())
        assert (got != np.uint64(tg.VIS_EMPTY)).sum() > 100

    # small -> large -> small on a caller's stream; the middle call does not wait
    stream = torch.cuda.Stream()
    outs = [torch.full((int(v["width"][0]) * int(v["height"][0]),), -7, dtype=torch.int64, device="cuda")
            for v in views]
    torch.cuda.synchronize()
    for k, (v, out) in enumerate(zip(views, outs)):
        err = None if k == 1 else tg.DeviceError()
        st = _call(noalloc, C.c_void_p(stream.cuda_stream), scene, arrays, v, out, err)
        assert st == 0, tg.lib.tgx_last_error_string()
        assert err is None or err.code == 0
    stream.synchronize()
    for out, want in zip(outs, expected):
        got = out.cpu().numpy().view(np.uint64)
        assert np.array_equal(got, want), int((got != want).sum())


def test_no_alloc_bin_overflow_takes_the_exact_record_scan():
    """128 noise objects close in front of the camera at 1920x1080: the frame
    needs more (cluster, tile) entries than the fixed bins hold, so every tile
    scans all visible clusters.  Still equal to tgx_vis_render, twice in a row."""
    import torch

    noalloc = _bind()
    scene = tg.generate_scene(1, 128, 6, 10, seed=12, noise_period=20.0, noise_threshold=0.58,
                              box_min=(-90.0, -50.0, 70.0), box_max=(90.0, 50.0, 170.0), n_luts=1)
    view = tg.make_view((0.0, 0.0, 0.0), 0.0, float(np.pi), float(np.pi / 3), 1920, 1080, 0.1, 1024.0)
    (want,), (entries,) = _expected(scene, [view])
    assert entries > NA_BINS, entries
    arrays = _device_scene(scene)
    for _ in range(2):
        out = torch.full((1920 * 1080,), -7, dtype=torch.int64, device="cuda")
        err = tg.DeviceError()
        st = _call(noalloc, None, scene, arrays, view, out, err)
        assert st == 0 and err.code == 0, (st, err.code, tg.lib.tgx_last_error_string())
        got = out.cpu().numpy().view(np.uint64)
        assert np.array_equal(got, want), int((got != want).sum())
    assert (want != np.uint64(tg.VIS_EMPTY)).mean() > 0.3


def test_no_alloc_entry_point_rejects_oversized_inputs():
    noalloc = _bind()
    v = tg.make_view((0.0, 0.0, 0.0), 0.0, 0.0, 1.0, 8000, 8000, 0.1, 100.0)
    st = noalloc(None, 1, 1, 1, 1, 1, 1, v.ctypes.data, 1, None)
    assert st == 4 and b"tiles" in tg.lib.tgx_last_error_string()
    st = noalloc(None, 1, 70000, 1, 1, 1, 1, v.ctypes.data, 1, None)
    assert st == 4 and b"objects" in tg.lib.tgx_last_error_string()
