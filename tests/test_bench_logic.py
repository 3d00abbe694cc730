"""Host-side logic of bench.py (no GPU): the equal-RMSE interpolation of the
radiance-cache comparison and the reference row bands."""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402


def test_equal_rmse_interpolates_in_log_space():
    # rmse = 0.02 / sqrt(ds), time = 10 + ds ms
    ladder = [(ds, 10.0 + ds, 0.02 / ds ** 0.5) for ds in (1, 2, 4, 8, 16)]
    ms, ds, ok = bench.equal_rmse_time(ladder, 0.02 / 3.0)   # ds = 9 exactly
    assert ok
    assert abs(ds - 9.0) < 1e-9
    assert abs(ms - 19.0) < 1e-9


def test_equal_rmse_outside_the_ladder_is_a_bound():
    ladder = [(1, 11.0, 0.02), (4, 14.0, 0.01)]
    ms, ds, ok = bench.equal_rmse_time(ladder, 0.001)
    assert not ok and ds == 4 and ms == 14.0
    ms, ds, ok = bench.equal_rmse_time(ladder, 0.05)
    assert not ok and ds == 1 and ms == 11.0


def test_reference_bands_cover_the_image():
    bands = bench.reference_bands(1080)
    assert len(bands) == bench.REF_BANDS
    assert all(0 <= a < b <= 1080 and b - a == 8 for a, b in bands)
    assert bands[0][0] < 68 and bands[-1][1] > 1000
    assert all(b0[1] <= b1[0] for b0, b1 in zip(bands, bands[1:]))


def test_committed_profile_figures_are_read():
    # the machine-read lines of the committed ncu summary the roofline quotes
    for kind in ("trace", "shadow", "gather", "trace_packet"):
        prof = bench.committed_profile(kind)
        assert prof["source"] == os.path.join("profiles", "roofline_kernels_960x540.md")
        assert 1.0 <= prof["threads_per_instruction"] <= 32.0, kind
        assert 0.0 < prof["issue_active"] <= 100.0, kind
    assert bench.committed_profile("trace_packet")["dram_bytes_per_unit"] is None
    assert bench.committed_profile("trace")["dram_bytes_per_unit"] > 0.0
    # the camera rays' packets run at a higher SIMT efficiency than the thread-per-ray kernel
    assert bench.committed_profile("trace_packet")["threads_per_instruction"] > bench.committed_profile("trace")["threads_per_instruction"]
