"""Host-side pieces of bench.py, on canned input (no GPU): the clock
sampler's reading of nvidia-smi's CSV lines (median SM clock under load, the
maximum clock, the throttle reasons seen), which decides whether a run is
valid; the relMSE that scores cached against plain GI; the seeded camera
path of the motion study."""
from __future__ import annotations

import sys
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
import bench  # noqa: E402

IDLE = "0, 2070, 2070, 812.40, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active"


def sampler(lines):
    s = bench.ClockSampler(0)
    s.lines = list(lines)
    return s.summary()


def test_clean_run_has_no_reasons():
    r = sampler([IDLE, IDLE.replace("2070, 2070", "2055, 2070")])
    assert r["reasons"] == [] and r["samples"] == 2
    assert r["sm_max_mhz"] == 2070.0 and r["sm_mhz"] == (2070.0 + 2055.0) / 2


def test_power_cap_and_thermal_reasons_are_reported():
    cap = "0, 1980, 2070, 1399.00, 0x0000000000000004, Not Active, Not Active, Not Active, Active"
    hot = "0, 1500, 2070, 900.00, 0x0000000000000040, Not Active, Active, Not Active, Not Active"
    r = sampler([IDLE, cap, hot])
    assert r["reasons"] == ["hw_thermal_slowdown", "sw_power_cap"]
    assert r["sm_mhz"] == 1980.0 and r["samples"] == 3


def test_malformed_and_unavailable_lines_are_skipped():
    r = sampler(["", "garbage", "0, [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A], [N/A]", IDLE])
    assert r["samples"] == 1 and r["sm_mhz"] == 2070.0


def test_no_samples():
    r = sampler([])
    assert r == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_rel_mse_matches_its_definition_over_masked_pixels():
    import numpy as np
    rng = np.random.default_rng(3)
    r = rng.uniform(0.0, 2.0, (40, 3)).astype(np.float32)
    x = r + rng.normal(0.0, 0.1, (40, 3)).astype(np.float32)
    mask = rng.random(40) < 0.6
    want = np.mean([((x[i, c] - r[i, c]) ** 2) / (r[i, c] ** 2 + 1e-2)
                    for i in range(40) if mask[i] for c in range(3)])
    got = bench.rel_mse(x.reshape(-1), r.reshape(-1), mask)
    assert abs(got - want) <= 1e-6 * want
    assert bench.rel_mse(r.reshape(-1), r.reshape(-1), mask) == 0.0


def test_camera_path_is_seeded_and_moves_two_voxels_per_frame():
    import numpy as np
    a = [bench.camera_path(f) for f in range(5)]
    b = [bench.camera_path(f) for f in range(5)]
    for (pa, ya, wa), (pb, yb, wb) in zip(a, b):
        assert np.array_equal(pa, pb) and ya == yb and wa == wb
    steps = [np.linalg.norm(a[f + 1][0] - a[f][0]) for f in range(4)]
    assert np.allclose(steps, 2.0)
