"""fl_frame / fl_export_frame (FluidApp::frame and export_frame, lib.rs:352-394,
:570-590) drive the handle exactly like the equivalent fl_step calls."""
import numpy as np
import pytest

from fluidgb import Fluid, Timestep, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from fluidgb import _abi, build
    build.build()
    return _abi.load_library()


def test_frames_match_direct_steps(lib):
    p, parts, _ = scenes.workload("dam32")
    fixed = float(p.geom[2])
    a = Fluid(p, parts.shape[0])
    b = Fluid(p, parts.shape[0])
    a.set_particles(parts)
    b.set_particles(parts)
    ts = Timestep(fixed, 4, lib)
    ref = Timestep(fixed, 4, lib)
    total = 0
    # 60 Hz frames, a hitch, a slow-motion stretch, then paused with two manual steps
    frames = [(1000.0 / 60.0, 1.0)] * 5 + [(250.0, 1.0)] + [(1000.0 / 60.0, 0.3)] * 4
    for ms, speed in frames:
        n, _ = ts.frame(a, ms, speed)
        assert n == ref.steps_for_frame(np.float32(ms) / np.float32(1000.0), speed)
        b.step(n)
        total += n
    pending = 2
    for _ in range(3):
        n, pending = ts.frame(a, 1000.0 / 60.0, 1.0, paused=True, pending_steps=pending)
        b.step(n)
        total += n
    assert pending == 0 and ts.last_stats()["substeps"] == 0
    ts.export_frame(a, 3, 3 * fixed)
    b.step(3)
    total += 3
    assert ts.last_stats()["policy_label"] == "fixed-explicit-export"
    assert a.stats()["substeps"] == b.stats()["substeps"] == total
    xa, ia = a.get_particles()
    xb, ib = b.get_particles()
    assert np.array_equal(xa, xb) and np.array_equal(ia, ib)
    a.close()
    b.close()


@pytest.mark.parametrize("mode", [0, 1, 2])
def test_grid_slice_matches_oracle_restatement(lib, oracle, mode):
    """fl_grid_slice (slice.wgsl per-cell arithmetic) vs the oracle's C
    restatement on the same grid, value for value, at k = nz/2 and k = 5."""
    p, parts, _ = scenes.workload("dam32")
    g = Fluid(p, parts.shape[0])
    g.set_particles(parts)
    g.step(30)
    grid = g.get_grid()
    dims = p.grid
    for k in (None, 5):
        img = g.grid_slice(mode, k)
        ref = oracle.grid_slice(dims, grid["cell_type"], grid["pressure"], grid["u"], grid["v"], grid["w"], mode, k)
        assert np.array_equal(img, ref), (mode, k, np.argwhere(img != ref)[:3])
        assert img[..., 3].sum() > 0
    g.close()


@pytest.mark.parametrize("preset", [0, 1, 2])
def test_seeded_particles_match_the_reference_layout(lib, oracle, preset):
    """fl_seed_particles (one thread per particle, LCG jumped ahead) equals the
    reference's sequential generate_particles (the oracle's restatement) bit
    for bit, on the registry-default 80x40x80 tank; the handle then steps."""
    import ctypes
    from fluidgb import FlParams
    from fluidgb._abi import scene_blocks, scene_particle_count, seed_count
    p = FlParams()
    assert lib.fl_params_default(ctypes.byref(p), 80, 40, 80, 2.0 / 64.0, None) == 0
    blocks = scene_blocks(preset, 1.0, 0.2, lib)
    budget = scene_particle_count((80, 40, 80), blocks, 10.0, 0, lib)
    n = seed_count(p, blocks, budget, lib)
    g = Fluid(p, n)
    assert g.seed(blocks, budget) == n
    x, ids = g.get_particles()
    n_ref, x_ref = oracle.ref_generate_particles(p, blocks, budget, n)
    assert n_ref == n
    assert np.array_equal(x, x_ref) and np.array_equal(ids, np.arange(n, dtype=np.uint32))
    g.step(2)
    assert g.stats()["device_status"] == 0
    g.reset()
    assert np.array_equal(g.get_particles()[0], x_ref)
    g.close()


def test_stage_times_and_the_reference_rollup(lib):
    """Profiled substeps give every stage a positive time, and the coarse
    rollup {prep, pressure, finish} (timing.rs PREP_END / FINISH_START)
    partitions the stage totals; profiling leaves the results unchanged."""
    p, parts, _ = scenes.workload("dam32")
    a = Fluid(p, parts.shape[0])
    b = Fluid(p, parts.shape[0])
    a.set_particles(parts)
    b.set_particles(parts)
    a.set_profiling(True)
    a.step(3)
    b.step(3)
    stages, n = a.stage_times()
    coarse, n2 = a.coarse_times()
    assert n == n2 == 3
    assert all(v > 0.0 for v in stages.values()), stages
    assert abs(sum(coarse.values()) - sum(stages.values())) <= 1e-9 * sum(stages.values())
    assert coarse["pressure"] == stages["cg"]
    xa, ia = a.get_particles()
    xb, ib = b.get_particles()
    assert np.array_equal(xa, xb) and np.array_equal(ia, ib)
    a.reset_stage_times()
    assert a.coarse_times() == ({"prep": 0.0, "pressure": 0.0, "finish": 0.0}, 0)
    a.close()
    b.close()
