"""Autotuners: the visibility pass's screen-tile shape, and the SVO
traversal's DDA steps per ray-queue round.

The tile shape sets the CTA size of k_vis_tiles (one thread per pixel) and
the binning granularity.  The tuner renders a few frames of the caller's own
scene and views with each candidate shape, times them with CUDA events on
the library stream (tgx_trace_*), and keeps the fastest.

The traversal's steps per round set how long a lane of the persistent
k_trace_queue runs its ray before the warp refills finished lanes from the
ray queue (fewer: lanes idle less; more: refills cost less).  The tuner times
a few GI frames of the caller's frame per candidate and keeps the fastest.

Results are cached per (GPU, workload) in a JSON file next to this module.
"""
from __future__ import annotations

import json
import os
from pathlib import Path

import numpy as np

CANDIDATES = ((8, 8), (16, 8), (8, 16), (16, 16), (32, 8))
CACHE = Path(__file__).resolve().parent / "_tuning.json"


def _key(gpu: str, views: np.ndarray, n_clusters: int) -> str:
    sizes = "+".join(f"{int(v['width'])}x{int(v['height'])}" for v in views)
    return f"{gpu}|{sizes}|{int(np.log2(max(n_clusters, 1)))}"


def tune_visibility(scene, views, candidates=CANDIDATES, frames: int = 5, device: int = 0, use_cache: bool = True):
    """Returns (best_tile, {tile: ms per frame})."""
    import torch
    import tg_gb300 as tg

    views = np.ascontiguousarray(views, dtype=tg.VIEW_DTYPE)
    gpu = torch.cuda.get_device_name(device)
    key = _key(gpu, views, scene.n_clusters)
    cache = {}
    if use_cache and CACHE.exists():
        try:
            cache = json.loads(CACHE.read_text())
        except ValueError:
            cache = {}
        if key in cache:
            e = cache[key]
            return tuple(e["best"]), {tuple(map(int, k.split("x"))): v for k, v in e["ms"].items()}
    outs = [torch.empty(int(v["width"]) * int(v["height"]), dtype=torch.int64, device=f"cuda:{device}") for v in views]
    results = {}
    for tile in candidates:
        with tg.Context(device, tile=tile) as ctx:
            sc = ctx.upload(scene)
            for _ in range(2):
                ctx.vis_render(sc, views, outs)
            ctx.sync()
            ctx.trace_reset()
            ctx.trace(True)
            for _ in range(frames):
                ctx.vis_render(sc, views, outs)
            tr = ctx.trace_read()
            ctx.trace(False)
            sc.close()
        results[tile] = sum(ms for ms, _ in tr.values()) / frames
    best = min(results, key=results.get)
    if use_cache:
        cache[key] = {"best": list(best), "ms": {f"{t[0]}x{t[1]}": v for t, v in results.items()}}
        tmp = CACHE.with_suffix(".tmp")
        tmp.write_text(json.dumps(cache, indent=1))
        os.replace(tmp, CACHE)
    return best, results


TRACE_CANDIDATES = (2, 4, 8, 16)


def tune_gi_traversal(ctx, scene, svo, view, visbuf, candidates=TRACE_CANDIDATES, frames: int = 3, device: int = 0,
                      use_cache: bool = True):
    """Picks tgx_set_trace_steps for plain 1-bounce 4-spp GI on the caller's frame
    (scene, SVO, view and its visibility buffer); leaves ctx set to the best.
    Returns (best_steps, {steps: ms per frame})."""
    import torch
    import tg_gb300 as tg

    view = np.ascontiguousarray(view, dtype=tg.VIEW_DTYPE).reshape(1)
    gpu = torch.cuda.get_device_name(device)
    info = svo.info()
    key = f"gi|{gpu}|{int(view[0]['width'])}x{int(view[0]['height'])}|{int(info.n_nonempty_blocks).bit_length()}"
    cache = {}
    if use_cache and CACHE.exists():
        try:
            cache = json.loads(CACHE.read_text())
        except ValueError:
            cache = {}
        if key in cache:
            best = int(cache[key]["best"])
            ctx.set_trace_steps(best)
            return best, {int(k): v for k, v in cache[key]["ms"].items()}
    n = int(view[0]["width"]) * int(view[0]["height"]) * 3
    rgb = torch.empty(n, dtype=torch.float32, device="cuda")
    params = tg.gi_params(spp=4, bounces=1, seed=2, max_steps=256)
    stream = torch.cuda.ExternalStream(ctx.stream)
    times = {}
    with torch.cuda.stream(stream):
        for k in candidates:
            ctx.set_trace_steps(k)
            ctx.gi_render(scene, svo, view, visbuf, params, rgb)   # warm-up
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(frames):
                ctx.gi_render(scene, svo, view, visbuf, params, rgb)
            e1.record(stream)
            ctx.sync()
            times[k] = round(e0.elapsed_time(e1) / frames, 4)
    best = min(times, key=times.get)
    ctx.set_trace_steps(best)
    if use_cache:
        cache[key] = {"best": best, "ms": {str(k): v for k, v in times.items()}}
        try:
            CACHE.write_text(json.dumps(cache, indent=1))
        except OSError:
            pass
    return best, times
