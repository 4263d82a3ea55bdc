"""CUDA path vs the CPU oracle, through the C ABI, on a GB300.

In the reference-arithmetic mode (FL_CG_F32) every stage of the step is an
exact restatement of the oracle's f32 arithmetic, so the comparison is exact
(value equality) for bins, cell types, P2G, the CG pressure, projection and the
advected particles — over many steps.  The FP64-reduction mode is compared with
a stated tolerance.
"""
import numpy as np
import pytest

from fluidgb import FL_CG_F64, FL_CG_F64_IEEE, Fluid, scenes
from fluidgb import _abi

pytestmark = pytest.mark.gpu

GRID_KEYS = ("u", "v", "w", "u_saved", "v_saved", "w_saved", "pressure", "cell_type", "counts", "offsets")


@pytest.fixture(scope="module")
def lib():
    from fluidgb import build
    build.build()
    return _abi.load_library()


def make_pair(oracle, params, parts, capacity=None):
    cap = capacity or max(parts.shape[0], 1)
    g = Fluid(params, cap)
    o = oracle.OracleFluid(params, cap)
    g.set_particles(parts)
    o.set_particles(parts)
    return g, o


def assert_same_state(g, o, where=""):
    xg, ig = g.get_particles()
    xo, io = o.get_particles()
    gg, go = g.get_grid(), o.get_grid()
    for k in GRID_KEYS:
        if not np.array_equal(gg[k], go[k]):
            bad = np.flatnonzero(gg[k] != go[k])
            raise AssertionError("%s %s differs at %d entries, first %d: gpu %r oracle %r" % (
                where, k, bad.size, bad[0], gg[k][bad[0]], go[k][bad[0]]))
    if not np.array_equal(g.get_divergence(), o.get_divergence()):
        raise AssertionError("%s divergence differs" % where)
    bg, bo = g.get_bins(), o.get_bins()
    for name, a, b in zip(("counts", "offsets", "perm"), bg, bo):
        assert np.array_equal(a, b), "%s bins.%s" % (where, name)
    assert np.array_equal(ig, io), where + " ids"
    if not np.array_equal(xg, xo):
        bad = np.flatnonzero(np.any(xg != xo, axis=1))
        raise AssertionError("%s particles differ in %d rows; first %d gpu %r oracle %r" % (
            where, bad.size, bad[0], xg[bad[0]], xo[bad[0]]))
    sg, so = g.stats(), o.stats()
    for k in ("liquid_cells", "cg_iterations", "stray_particles"):
        assert sg[k] == so[k], "%s stats.%s gpu %s oracle %s" % (where, k, sg[k], so[k])
    assert sg["device_status"] == 0


def test_bins_are_bit_exact_and_stable(lib, oracle):
    p, parts, _ = scenes.workload("dam32")
    g, o = make_pair(oracle, p, parts)
    # shuffle so that the stable order is not the identity
    rng = np.random.default_rng(1)
    sh = parts[rng.permutation(parts.shape[0])]
    g.set_particles(sh)
    o.set_particles(sh)
    g.step(1)
    o.step(1)
    counts, offsets, perm = g.get_bins()
    co, oo, po = o.get_bins()
    assert np.array_equal(counts, co) and np.array_equal(offsets, oo) and np.array_equal(perm, po)
    # stable: inside a bucket the pre-sort slots increase
    for c in np.flatnonzero(counts > 1)[:2000]:
        seg = perm[offsets[c]:offsets[c] + counts[c]].astype(np.int64)
        assert np.all(np.diff(seg) > 0)


@pytest.mark.parametrize("steps", [1, 5])
def test_step_is_bit_exact_dam32(lib, oracle, steps):
    p, parts, _ = scenes.workload("dam32")
    g, o = make_pair(oracle, p, parts)
    for s in range(steps):
        g.step(1)
        o.step(1)
        assert_same_state(g, o, "step %d" % s)


def test_full_dam32_rollout_is_bit_exact(lib, oracle):
    """The 32^3 dam break of the first benchmark configuration, all 120 steps."""
    p, parts, spec = scenes.workload("dam32")
    g, o = make_pair(oracle, p, parts)
    for chunk in range(4):
        g.step(30)
        o.step(30)
        assert_same_state(g, o, "after %d steps" % (30 * (chunk + 1)))


@pytest.mark.parametrize("opts", [
    dict(friction=0.35), dict(dilation=1), dict(stiffness=0.0), dict(advect_order=2), dict(warm=0),
    dict(threshold=2), dict(gravity=(1.5, -9.81, -2.0)),
], ids=lambda d: "-".join(d))
def test_step_options_are_bit_exact(lib, oracle, opts):
    p, parts, _ = scenes.workload("dam32")
    if "friction" in opts:
        p.phys[3] = opts["friction"]
    if "dilation" in opts:
        p.cls[1] = opts["dilation"]
    if "stiffness" in opts:
        p.spc[1] = opts["stiffness"]
    if "advect_order" in opts:
        p.advect_order = opts["advect_order"]
    if "warm" in opts:
        p.dims[3] = opts["warm"]
    if "threshold" in opts:
        p.cls[0] = opts["threshold"]
    if "gravity" in opts:
        p.grav[0], p.grav[1], p.grav[2] = opts["gravity"]
    g, o = make_pair(oracle, p, parts)
    for s in range(4):
        g.step(1)
        o.step(1)
        assert_same_state(g, o, "step %d" % s)


def test_non_power_of_two_cell_size_and_strays(lib, oracle):
    """h = 1/24 is inexact in f32: the division-form bin and the multiply-form
    P2G cell disagree for particles on cell faces; those go through the stray
    pass.  Particles placed exactly on faces force many such ties."""
    n = 24
    p = scenes.params_for(n, iters=60, tol=1e-4)
    parts = scenes.seed_particles(n, scenes.box(0.6, 0.5, 0.7), seed=7)
    h = np.float32(1.0) / np.float32(n)
    inv_h = np.float32(1.0) / h
    # coordinates one ulp below a cell face where x/h and x*inv_h floor differently
    ties = []
    for k in range(1, n - 1):
        x = np.nextafter(np.float32(k) * h, np.float32(-1.0))
        if np.floor(x / h) != np.floor(x * inv_h):
            ties.append(x)
    assert len(ties) >= 4
    ties = np.array(ties, np.float32)
    rng = np.random.default_rng(5)
    for axis in (0, 1, 2):
        sel = np.flatnonzero(rng.random(parts.shape[0]) < 0.1)
        near = np.abs(ties[None, :] - parts[sel, axis][:, None]).argmin(axis=1)
        parts[sel, axis] = ties[near]
    g, o = make_pair(oracle, p, parts)
    g.step(1)
    o.step(1)
    assert o.stats()["stray_particles"] > 0
    assert_same_state(g, o, "step 0")
    for s in range(3):
        g.step(1)
        o.step(1)
        assert_same_state(g, o, "step %d" % (s + 1))


def test_out_of_domain_particles_are_clamped_like_the_reference(lib, oracle):
    p = scenes.params_for(16, iters=30, tol=1e-4)
    parts = scenes.seed_particles(16, scenes.box(0.5, 0.5), seed=3)
    parts[0, :3] = [-5.0, -5.0, -5.0]
    parts[1, :3] = [9.0, 9.0, 9.0]
    parts[2, :3] = [0.5, 2.0, -1.0]
    g, o = make_pair(oracle, p, parts)
    g.step(1)
    o.step(1)
    assert_same_state(g, o, "step 0")


def test_empty_and_tiny_particle_sets(lib, oracle):
    p = scenes.params_for(16, iters=10, tol=0.0)
    for n in (0, 1, 3):
        parts = scenes.seed_particles(16, scenes.box(0.5, 0.5))[:n]
        g, o = make_pair(oracle, p, parts, capacity=8)
        g.step(2)
        o.step(2)
        assert_same_state(g, o, "n=%d" % n)


@pytest.mark.parametrize("form", [FL_CG_F64, FL_CG_F64_IEEE], ids=["float-float", "ieee-double"])
def test_fp64_reductions_match_oracle_to_tolerance(lib, oracle, form):
    """FL_CG_F64 (float-float) and FL_CG_F64_IEEE (double) inner products
    against the oracle's double dots.  Summation order differs from the
    oracle's (1e-16 relative), so alpha/beta may differ in the last f32 bit;
    state must agree to 1e-5 relative after 3 steps."""
    p, parts, _ = scenes.workload("dam32", precision=form)
    g, o = make_pair(oracle, p, parts)
    g.step(3)
    o.step(3)
    xg, ig = g.get_particles()
    xo, io = o.get_particles()
    assert np.array_equal(ig, io)
    assert np.allclose(xg, xo, rtol=1e-5, atol=1e-6)
    gg, go = g.get_grid(), o.get_grid()
    for k in ("u", "v", "w"):
        scale = max(np.abs(go[k]).max(), 1e-6)
        assert np.abs(gg[k] - go[k]).max() <= 1e-5 * scale + 1e-7, k
    sc = np.abs(go["pressure"]).max()
    assert np.abs(gg["pressure"] - go["pressure"]).max() <= 1e-5 * sc
    assert abs(g.stats()["cg_iterations"] - o.stats()["cg_iterations"]) <= 1


@pytest.mark.parametrize("precision", [0, FL_CG_F64, FL_CG_F64_IEEE])
def test_gpu_run_is_deterministic(lib, precision):
    p, parts, _ = scenes.workload("dam32", precision=precision)
    outs = []
    for _ in range(2):
        g = Fluid(p, parts.shape[0])
        g.set_particles(parts)
        g.step(10)
        outs.append(g.get_particles())
        g.close()
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])


def test_impulse_reset_and_checkpoint_resume(lib, oracle):
    p, parts, _ = scenes.workload("dam32")
    g, o = make_pair(oracle, p, parts)
    g.apply_impulse([0.3, 0.1, -0.2])
    o.apply_impulse([0.3, 0.1, -0.2])
    g.step(3)
    o.step(3)
    assert_same_state(g, o, "after impulse")
    blob = g.save_state()
    g.step(4)
    ref = g.get_particles()
    g.load_state(blob)
    g.step(4)
    again = g.get_particles()
    assert np.array_equal(ref[0], again[0]) and np.array_equal(ref[1], again[1])
    g.reset()
    x, ids = g.get_particles()
    assert np.array_equal(x, parts) and np.array_equal(ids, np.arange(parts.shape[0], dtype=np.uint32))


def test_live_params_update(lib, oracle):
    p, parts, _ = scenes.workload("dam32")
    g, o = make_pair(oracle, p, parts)
    g.step(2)
    o.step(2)
    q = p.copy()
    q.phys[2] = 0.5
    q.dims[2] = 12
    q.grav[0] = 2.0
    g.set_params(q)
    o.set_params(q)
    g.step(2)
    o.step(2)
    assert_same_state(g, o, "after live update")
    bad = p.copy()
    bad.gdim[0] = 33
    with pytest.raises(_abi.FluidError):
        g.set_params(bad)


def test_step_device_buffer_matches_handle_path(lib):
    torch = pytest.importorskip("torch")
    p, parts, _ = scenes.workload("dam32")
    g = Fluid(p, parts.shape[0])
    g.set_particles(parts)
    g.step(1)
    want = g.get_particles(with_ids=False)
    d = torch.from_numpy(parts.copy()).cuda().contiguous()
    h = Fluid(p, parts.shape[0])
    torch.cuda.synchronize()
    h.step_device(d.data_ptr(), parts.shape[0])
    h.sync()
    got = d.cpu().numpy()
    assert np.array_equal(got, want)


def test_solve_pressure_matches_oracle_and_reference_thresholds(lib, oracle):
    from test_oracle_kats import _l2_after, divergent_tank
    d, ct, u, v, w, div0 = divergent_tank(oracle)
    pg, sg = _abi.solve_pressure(ct, div0, d, 1.0, 1.0, 1.0, 40)
    po, so = oracle.solve_pressure(ct, div0, d, 1.0, 1.0, 1.0, 40)
    assert np.array_equal(pg, po)
    assert sg["cg_iterations"] == so["cg_iterations"] == 40
    l2_before = oracle.ref_l2_divergence(div0, ct)
    pj = oracle.ref_jacobi_solve(d, 1.0, 1.0, 1.0, ct, div0, 200)
    l2 = _l2_after(oracle, d, ct, u, v, w, pg)
    assert l2 < 0.01 * l2_before and l2 <= _l2_after(oracle, d, ct, u, v, w, pj)
    # warm start and tolerance exit
    pw, sw = _abi.solve_pressure(ct, div0, d, 1.0, 1.0, 1.0, 40, warm_start=True, pressure_in=pg, tolerance=0.1)
    pwo, swo = oracle.solve_pressure(ct, div0, d, 1.0, 1.0, 1.0, 40, warm_start=True, pressure_in=pg,
                                     tolerance=0.1)
    assert np.array_equal(pw, pwo) and sw["cg_iterations"] == swo["cg_iterations"] < 40
    # f64 inner products
    o64, _ = oracle.solve_pressure(ct, div0, d, 1.0, 1.0, 1.0, 40, precision=1)
    for form in (FL_CG_F64, FL_CG_F64_IEEE):
        p64, s64 = _abi.solve_pressure(ct, div0, d, 1.0, 1.0, 1.0, 40, precision=form)
        assert np.allclose(p64, o64, rtol=1e-5, atol=1e-5 * np.abs(o64).max()), form


def test_128_grid_one_step_bit_exact(lib, oracle):
    """The ~2M-particle 128^3 headline workload: one substep against the oracle."""
    p, parts, _ = scenes.workload("dam128_2m")
    g, o = make_pair(oracle, p, parts)
    g.step(1)
    o.step(1)
    assert_same_state(g, o, "128^3 step 0")


def test_256_grid_two_steps_bit_exact(lib, oracle):
    """The 256^3, 18.8M-particle block: its CG holds more active chunks than one
    staging window (plan-order exchange slots, windowed reduction) and more
    liquid cells per block than the shared-memory cell list (the unlisted-cell
    path) — both bit-exact against the oracle."""
    p, parts, _ = scenes.workload("block256")
    g, o = make_pair(oracle, p, parts)
    for s in range(2):
        g.step(1)
        o.step(1)
        assert_same_state(g, o, "256^3 step %d" % s)
    g.close()
    o.close()


@pytest.mark.parametrize("workload,steps", [("dam128", 1), ("sphere_pool128", 2), ("block64", 3)])
def test_configuration_scenes_bit_exact(lib, oracle, workload, steps):
    """The other configurations' scenes, from their seeded initial states:
    the full-depth 128^3 dam break (4.19M particles), the sphere falling into
    the pool, and the 64^3 block with N(0, 0.1^2) initial velocities."""
    p, parts, _ = scenes.workload(workload)
    g, o = make_pair(oracle, p, parts)
    for s in range(steps):
        g.step(1)
        o.step(1)
        assert_same_state(g, o, "%s step %d" % (workload, s))
    g.close()
    o.close()


def test_128_grid_thirty_steps_bit_exact(lib, oracle):
    """The benchmarked configuration (128^3, 2,000,376 particles, CG <= 200 at
    1e-5) over 30 substeps: every substep of the first five, then every fifth,
    compared with the oracle by value equality (fluid.rs:1436-1715 per substep)."""
    p, parts, _ = scenes.workload("dam128_2m")
    g, o = make_pair(oracle, p, parts)
    done = 0
    for k in (1, 2, 3, 4, 5, 10, 15, 20, 25, 30):
        g.step(k - done)
        o.step(k - done)
        done = k
        assert_same_state(g, o, "128^3 after %d steps" % k)
    g.close()
    o.close()


@pytest.mark.parametrize("form", [FL_CG_F64, FL_CG_F64_IEEE], ids=["float-float", "ieee-double"])
def test_128_grid_fp64_reductions_track_the_oracle(lib, oracle, form):
    """The extended-precision forms on the benchmarked configuration, 20
    substeps.  Before every substep the oracle (the reference step with double
    inner products) takes the GPU's particles and warm-start pressure, and
    both take the step; the float-float or IEEE-double reductions then agree
    with the oracle's to 1e-5 relative in face velocity and pressure, 1e-6 in
    position, and in the iteration count to within one."""
    p, parts, _ = scenes.workload("dam128_2m", precision=form)
    n = parts.shape[0]
    g = Fluid(p, n)
    g.set_particles(parts)
    o = oracle.OracleFluid(p, n)
    worst = {"velocity": 0.0, "pressure": 0.0, "position": 0.0}
    for s in range(20):
        x_in, id_in = g.get_particles()
        p_in = g.get_grid()["pressure"]
        g.step(1)
        o.set_particles(x_in)
        o.set_pressure(p_in)
        o.step(1)
        gg, og = g.get_grid(), o.get_grid()
        vscale = max(max(np.abs(og[k]).max() for k in ("u", "v", "w")), 1e-30)
        dv = max(np.abs(gg[k].astype(np.float64) - og[k]).max() for k in ("u", "v", "w")) / vscale
        pscale = max(np.abs(og["pressure"]).max(), 1e-30)
        dp = np.abs(gg["pressure"].astype(np.float64) - og["pressure"]).max() / pscale
        xg, ig = g.get_particles()
        xo, io = o.get_particles()
        assert np.array_equal(ig, id_in[io]), "step %d: bin order" % s
        dx = np.abs(xg[:, 0:3].astype(np.float64) - xo[:, 0:3]).max()
        worst["velocity"] = max(worst["velocity"], dv)
        worst["pressure"] = max(worst["pressure"], dp)
        worst["position"] = max(worst["position"], dx)
        assert dv <= 1e-5 and dp <= 1e-5 and dx <= 1e-6, (s, dv, dp, dx)
        assert abs(g.stats()["cg_iterations"] - o.stats()["cg_iterations"]) <= 1, s
        assert g.stats()["device_status"] == 0
    print("form %d vs oracle over 20 substeps of dam128_2m: max rel velocity %.2e, pressure %.2e, "
          "max abs position %.2e" % (form, worst["velocity"], worst["pressure"], worst["position"]))
    g.close()
    o.close()
