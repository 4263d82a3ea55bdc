"""The fixed-timestep frame driver (fl_timestep_*) against the reference's own
tests of TimestepController (app/crates/fluid-lab/src/timestep.rs:251-420),
through the C ABI on the CPU host (no device needed)."""
import numpy as np
import pytest

from fluidgb import Timestep

F = np.float32
FIXED = float(F(1.0) / F(120.0))
MAX_RENDER_DT = float(F(1.0) / F(30.0))


def close(a, b):
    assert abs(a - b) < 1e-6, (a, b)


@pytest.fixture
def lib(fluidlib):
    return fluidlib


def test_one_hundred_twentieth_frame_with_cap_one_runs_realtime(lib):
    tc = Timestep(FIXED, 1, lib)
    assert tc.steps_for_frame(FIXED) == 1
    s = tc.last_stats()
    assert s["substeps"] == 1 and s["natural_substeps"] == 1 and s["max_substeps"] == 1
    assert not s["substep_cap_hit"]
    close(s["fixed_dt"], FIXED)
    close(s["wall_dt"], FIXED)
    close(s["sim_advanced"], FIXED)
    close(s["real_time_factor"], 1.0)
    assert s["policy_label"] == "fixed-drop-cap"
    assert tc.total_dropped() == 0.0


def test_sixty_hz_frame_with_cap_one_reports_half_realtime(lib):
    tc = Timestep(FIXED, 1, lib)
    assert tc.steps_for_frame(1.0 / 60.0) == 1
    s = tc.last_stats()
    assert s["natural_substeps"] == 2 and s["substep_cap_hit"]
    close(s["wall_dt"], 1.0 / 60.0)
    close(s["sim_advanced"], FIXED)
    close(s["real_time_factor"], 0.5)
    close(s["dropped_this_frame"], FIXED)
    close(tc.total_dropped(), FIXED)
    assert abs(s["accumulated_after"]) < 1e-6


def test_large_hitch_uses_raw_wall_time_for_realtime_factor(lib):
    tc = Timestep(FIXED, 1, lib)
    assert tc.steps_for_frame(1.0) == 1
    s = tc.last_stats()
    assert s["natural_substeps"] == 4 and s["substep_cap_hit"]
    close(s["accumulated_before"], MAX_RENDER_DT)
    close(s["wall_dt"], 1.0)
    close(s["sim_advanced"], FIXED)
    close(s["real_time_factor"], FIXED)
    close(s["dropped_this_frame"], 3.0 * FIXED)
    close(tc.total_dropped(), 3.0 * FIXED)
    assert abs(s["accumulated_after"]) < 1e-6


def test_scaled_time_advances_fractional_wall_time(lib):
    tc = Timestep(FIXED, 4, lib)
    assert tc.steps_for_frame(1.0 / 60.0, 0.25) == 0
    s = tc.last_stats()
    close(s["wall_dt"], 1.0 / 60.0)
    close(s["sim_time_scale"], 0.25)
    close(s["accumulated_before"], 1.0 / 240.0)
    close(s["sim_advanced"], 0.0)
    close(s["real_time_factor"], 0.0)
    assert tc.steps_for_frame(1.0 / 60.0, 0.25) == 1
    s = tc.last_stats()
    close(s["sim_advanced"], FIXED)
    close(s["real_time_factor"], 0.5)
    assert abs(s["accumulated_after"]) < 1e-6


def test_two_steps_per_half_period_frame(lib):
    tc = Timestep(FIXED, 4, lib)
    assert tc.steps_for_frame(1.0 / 60.0) == 2
    assert abs(tc.accumulator()) < 1e-6
    assert tc.total_dropped() == 0.0
    s = tc.last_stats()
    assert s["substeps"] == 2 and s["dropped_this_frame"] == 0.0 and s["natural_substeps"] == 2
    assert not s["substep_cap_hit"]


def test_large_frame_clamped_and_capped(lib):
    tc = Timestep(FIXED, 4, lib)
    assert tc.steps_for_frame(1.0) == 4
    assert tc.total_dropped() == 0.0 and tc.last_stats()["dropped_this_frame"] == 0.0
    tc2 = Timestep(FIXED, 2, lib)
    assert tc2.steps_for_frame(1.0) == 2
    assert tc2.total_dropped() > 0.0
    assert abs(tc2.accumulator()) < 1e-6
    assert tc2.last_stats()["dropped_this_frame"] > 0.0
    assert abs(tc2.last_stats()["accumulated_after"]) < 1e-6


def test_tiny_frames_accumulate(lib):
    tc = Timestep(FIXED, 4, lib)
    assert sum(tc.steps_for_frame(0.002) for _ in range(5)) == 1
    assert tc.total_dropped() == 0.0


def test_large_frame_drops_excess_and_records_stats(lib):
    tc = Timestep(FIXED, 1, lib)
    assert tc.steps_for_frame(1.0) == 1
    s = tc.last_stats()
    assert s["substeps"] == 1 and s["natural_substeps"] == 4 and s["substep_cap_hit"]
    close(s["dropped_this_frame"], 3.0 * FIXED)


def test_reset_zeroes_accumulator_and_frame_stats_but_keeps_dropped(lib):
    tc = Timestep(FIXED, 1, lib)
    tc.steps_for_frame(1.0)
    dropped = tc.total_dropped()
    tc.steps_for_frame(0.005)
    tc.reset()
    assert tc.accumulator() == 0.0 and tc.total_dropped() == dropped
    s = tc.last_stats()
    assert s["substeps"] == 0 and s["wall_dt"] == 0.0 and s["sim_time_scale"] == 1.0


def test_manual_export_and_idle_records(lib):
    tc = Timestep(FIXED, 4, lib)
    tc.record_manual_steps(1.0 / 60.0, 1, 1.0)
    s = tc.last_stats()
    assert s["substeps"] == 1 and s["natural_substeps"] == 0 and s["max_substeps"] == 4
    close(s["real_time_factor"], 0.5)
    tc.record_export_steps(0.05, 6)
    s = tc.last_stats()
    assert s["substeps"] == 6 and s["max_substeps"] == 6 and s["natural_substeps"] == 6
    assert s["policy_label"] == "fixed-explicit-export" and s["sim_time_scale"] == 1.0
    close(s["sim_advanced"], 6 * FIXED)
    tc.record_idle_frame(float("nan"), float("inf"))
    s = tc.last_stats()
    assert s["substeps"] == 0 and s["wall_dt"] == 0.0 and s["sim_time_scale"] == 0.0


def test_non_finite_and_negative_deltas_are_sanitised(lib):
    tc = Timestep(FIXED, 4, lib)
    for bad in (float("nan"), float("inf"), -1.0):
        assert tc.steps_for_frame(bad) == 0
    assert tc.accumulator() == 0.0
