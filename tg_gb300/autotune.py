"""Autotuner for the visibility pass: picks the screen-tile shape.

The tile shape sets the CTA size of k_vis_tiles (one thread per pixel) and
the binning granularity.  The tuner renders a few frames of the caller's own
scene and views with each candidate shape, times them with CUDA events on
the library stream (tgx_trace_*), and keeps the fastest.  Results are cached
per (GPU, view sizes, scene size) in a JSON file next to this module.
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
