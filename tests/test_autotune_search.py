"""The autotuner's coordinate search over the visibility settings, on
synthetic frame times (no GPU): it walks the tile shapes, then the depth
buckets, the batch and the drain from the best so far; it measures each
setting once; it keeps the current choice unless a candidate is faster by
more than the margin."""
from __future__ import annotations

from tg_gb300.autotune import CANDIDATES, DEFAULTS, coordinate_search


def separable_cost(tile_ms, bucket_ms, batch_ms, drain_ms):
    def cost(cfg):
        return (tile_ms[cfg["tile"]] + bucket_ms[cfg["depth_buckets"]] + batch_ms[cfg["batch"]] +
                drain_ms[cfg["drain"]])
    return cost


def test_finds_the_coordinate_optimum_and_measures_each_setting_once():
    tile_ms = {(8, 8): 0.10, (16, 8): 0.09, (8, 16): 0.12, (16, 16): 0.08, (32, 8): 0.11}
    bucket_ms = {8: 0.010, 16: 0.020, 32: 0.030}
    batch_ms = {16: 0.005, 32: 0.001, 48: 0.009}
    drain_ms = {16: 0.004, 24: 0.002, 32: 0.006}
    calls = []
    cost = separable_cost(tile_ms, bucket_ms, batch_ms, drain_ms)

    def measure(cfg):
        calls.append(dict(cfg))
        return cost(cfg)

    best, times = coordinate_search(measure)
    assert best == {"tile": (16, 16), "depth_buckets": 8, "batch": 32, "drain": 24}
    labels = [f"{c['tile'][0]}x{c['tile'][1]}/b{c['depth_buckets']}/n{c['batch']}/d{c['drain']}" for c in calls]
    assert len(labels) == len(set(labels)) == len(times)
    # the tiles from the defaults, then one new setting per remaining value of each coordinate
    assert len(calls) == len(CANDIDATES) + 2 + 2 + 2
    assert calls[0] == {"tile": CANDIDATES[0], **DEFAULTS}


def test_margin_keeps_the_current_choice_against_noise():
    tile_ms = {t: 0.100 for t in CANDIDATES}
    tile_ms[(16, 8)] = 0.0995          # 0.5 % faster: inside a 1 % margin
    tile_ms[(32, 8)] = 0.0980          # 2 % faster: taken
    flat = {v: 0.0 for v in (8, 16, 24, 32, 48)}
    best, _ = coordinate_search(separable_cost(tile_ms, flat, flat, flat), margin=0.01)
    assert best["tile"] == (32, 8)
    tile_ms[(32, 8)] = 0.0995
    best, _ = coordinate_search(separable_cost(tile_ms, flat, flat, flat), margin=0.01)
    assert best["tile"] == CANDIDATES[0]
    best, _ = coordinate_search(separable_cost(tile_ms, flat, flat, flat), margin=0.0)
    assert best["tile"] == (16, 8)


def test_restricted_space():
    tile_ms = {(8, 8): 0.2, (8, 16): 0.1}
    flat = {v: 0.0 for v in (8, 16, 24, 32, 48)}
    best, times = coordinate_search(separable_cost(tile_ms, flat, flat, flat), tiles=((8, 8), (8, 16)),
                                    depth_buckets=(16,), batches=(48,), drains=(32,))
    assert best == {"tile": (8, 16), **DEFAULTS}
    assert len(times) == 2
