"""Autotuners: the visibility pass's tile shape and tuning, and the SVO
traversal's DDA steps per ray-queue round.

Visibility: four settings change the speed of a frame but never a result
(tested bit for bit):
  - the tile shape: the CTA size of k_vis_tiles (one thread per pixel) and
    the binning granularity;
  - the depth buckets per tile (8, 16, 32): how finely a tile's clusters are
    sorted near to far, so a tile stops once all its pixels are nearer;
  - the batch: clusters staged per shared-memory batch (16, 32, 48);
  - the drain: (pixel, cluster) pairs a warp gathers by ballot before its
    lanes run their DDAs (16, 24, 32), i.e. rays per warp round.
The tuner runs the caller's own frame (one scene and its views, or a whole
batched frame graph) with each candidate, times it with CUDA events on the
library stream (best of three runs) and keeps the fastest, moving away from
the current choice only for a gain above 1 %: first over the tile shapes
with the other settings at their defaults, then one setting at a time
(coordinate descent).

Traversal: how long a lane of the persistent k_trace_queue runs its ray
before the warp refills finished lanes from the ray queue.

Results are cached per (GPU, workload) in a JSON file next to this module.
"""
from __future__ import annotations

import json
import os
from pathlib import Path

import numpy as np

CANDIDATES = ((8, 8), (16, 8), (8, 16), (16, 16), (32, 8))
DEPTH_BUCKETS = (8, 16, 32)
BATCHES = (16, 32, 48)
DRAINS = (16, 24, 32)
DEFAULTS = {"depth_buckets": 16, "batch": 48, "drain": 32}
CACHE = Path(__file__).resolve().parent / "_tuning.json"


def _key(gpu: str, views: np.ndarray, n_clusters: int) -> str:
    sizes = "+".join(f"{int(v['width'])}x{int(v['height'])}" for v in views)
    return f"{gpu}|{sizes}|{int(np.log2(max(n_clusters, 1)))}"


def _read_cache() -> dict:
    if CACHE.exists():
        try:
            return json.loads(CACHE.read_text())
        except ValueError:
            return {}
    return {}


def _write_cache(cache: dict) -> None:
    try:
        tmp = CACHE.with_suffix(".tmp")
        tmp.write_text(json.dumps(cache, indent=1))
        os.replace(tmp, CACHE)
    except OSError:
        pass


def _label(cfg: dict) -> str:
    t = cfg["tile"]
    return f"{t[0]}x{t[1]}/b{cfg['depth_buckets']}/n{cfg['batch']}/d{cfg['drain']}"


def coordinate_search(measure, tiles=CANDIDATES, depth_buckets=DEPTH_BUCKETS, batches=BATCHES, drains=DRAINS,
                      margin: float = 0.01):
    """Coordinate search over the visibility settings: the tile shapes first
    (from the defaults), then the depth buckets, the batch and the drain, one
    at a time from the best so far.  measure(cfg) returns a frame time; each
    distinct setting is measured once.  A candidate replaces the current
    choice only when it is faster by more than `margin` (run-to-run noise
    would otherwise pick settings at random).  Returns (best config dict,
    {label: measured time})."""
    times = {}

    def run(cfg):
        lab = _label(cfg)
        if lab not in times:
            times[lab] = measure(cfg)
        return times[lab]

    def better(cand, cur):
        return run(cand) < run(cur) * (1.0 - margin)

    best = {"tile": tiles[0], **DEFAULTS}
    for t in tiles:
        cand = {**best, "tile": t}
        if better(cand, best):
            best = cand
    for name, values in (("depth_buckets", depth_buckets), ("batch", batches), ("drain", drains)):
        for v in values:
            cand = {**best, name: v}
            if better(cand, best):
                best = cand
    return best, times


def tune_workload(make_frame, device: int = 0, frames: int = 5, tiles=CANDIDATES, depth_buckets=DEPTH_BUCKETS,
                  batches=BATCHES, drains=DRAINS, reps: int = 3, margin: float = 0.01):
    """Coordinate search (coordinate_search) over the visibility settings for
    one workload, timed on the GPU.

    make_frame(ctx) sets up the workload on a fresh context and returns
    (render, close): render() issues one whole frame on the context's stream,
    close() frees what make_frame made.  Each candidate is timed `reps` times
    over `frames` frames and keeps its best time.  Returns (best config dict,
    {label: ms per frame})."""
    import torch
    import tg_gb300 as tg

    def measure(cfg):
        with tg.Context(device, tile=cfg["tile"]) as ctx:
            ctx.set_vis_tuning(cfg["depth_buckets"], cfg["batch"], cfg["drain"])
            render, close = make_frame(ctx)
            stream = torch.cuda.ExternalStream(ctx.stream)
            for _ in range(2):
                render()
            ctx.sync()
            best_ms = None
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                for _ in range(frames):
                    render()
                e1.record(stream)
                ctx.sync()
                ms = e0.elapsed_time(e1) / frames
                best_ms = ms if best_ms is None else min(best_ms, ms)
            err = ctx.device_error()
            if err.code:
                raise RuntimeError(f"tuning frame failed: device status {err.code} at {err.where}")
            close()
        return round(best_ms, 4)

    return coordinate_search(measure, tiles, depth_buckets, batches, drains, margin)


def tune_visibility(scene, views, frames: int = 5, device: int = 0, use_cache: bool = True, **space):
    """The visibility settings for rendering `views` of `scene` (a HostScene)
    with tgx_vis_render.  Returns (best config dict, {label: ms per frame})."""
    import torch
    import tg_gb300 as tg

    views = np.ascontiguousarray(views, dtype=tg.VIEW_DTYPE)
    gpu = torch.cuda.get_device_name(device)
    key = "vis2|" + _key(gpu, views, scene.n_clusters)
    cache = _read_cache() if use_cache else {}
    if key in cache:
        e = cache[key]
        return {**e["best"], "tile": tuple(e["best"]["tile"])}, e["ms"]
    outs = [torch.empty(int(v["width"]) * int(v["height"]), dtype=torch.int64, device=f"cuda:{device}") for v in views]

    def make_frame(ctx):
        sc = ctx.upload(scene)
        return (lambda: ctx.vis_render(sc, views, outs)), sc.close

    best, times = tune_workload(make_frame, device, frames, **space)
    if use_cache:
        cache[key] = {"best": {**best, "tile": list(best["tile"])}, "ms": times}
        _write_cache(cache)
    return best, times


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
