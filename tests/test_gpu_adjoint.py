"""Adjoint of the substep (fl_step_record / fl_step_adjoint) against central
finite differences of the FP64 oracle forward.

Loss: squared distance of the particle centre of mass to a target after a
short rollout; gradients w.r.t. the initial per-particle velocity and the
gravity vector, through the checkpointed rollout and torch.autograd.Function.
The finite-difference forward is the oracle's double-precision step with
unrounded P2G accumulation and a tight CG (a smooth function of its inputs);
the adjoint linearises the GPU forward (f32 state, FP64 CG reductions), with
the P2G normalisation taken at its unquantised sums.  Without that, the 2^16
fixed-point quantum at low-weight surface faces, amplified by 1/sum(w) in the
position derivative, put the 4-step gradient off by 66%.
"""
import numpy as np
import pytest

from fluidgb import FL_CG_F64, FL_CG_F64_IEEE, scenes

pytestmark = pytest.mark.gpu

TARGET = np.array([0.7, 0.2, 0.5])


def blob(x, y, z):
    return (x > 0.3) & (x < 0.7) & (y > 0.35) & (y < 0.65) & (z > 0.3) & (z < 0.7)


def floor_blob(x, y, z):
    """A blob on the floor: its lower cells lie inside the wall-friction band
    (2.5 h above the wall clamp, g2p.wgsl:173-184), clear of the clamp itself."""
    return (x > 0.3) & (x < 0.7) & (y > 0.1) & (y < 0.3) & (z > 0.3) & (z < 0.7)


def setup_case(n=20, steps=4, seed=11, region=blob, advect_order=1, friction=0.0):
    """A blob falling freely, away from the walls (no wall clamps in the run)."""
    p = scenes.params_for(n, iters=500, tol=1e-6, precision=FL_CG_F64, stiffness=0.0, advect_order=advect_order)
    p.phys[3] = friction
    parts = scenes.seed_particles(n, region, seed=seed, vel_sigma=0.1)
    return p, parts, steps


def fd_errors(oracle, p, parts, steps, gv, gg, want=3, seed=3):
    """Relative errors of the adjoint's directional derivatives against
    central differences of the FP64 oracle, on random directions whose +-eps
    runs keep every cell type of the unperturbed run."""
    n = parts.shape[0]
    oracle.set_exact_p2g(True)
    try:
        base_g = np.array([0.0, np.float32(-9.81), 0.0], np.float64)
        _, ct0 = oracle_run(oracle, p, parts, steps, None, 0.0, base_g)
        rng = np.random.default_rng(seed)
        eps = 1e-6  # converged: 1e-5 .. 1e-7 agree to ~1e-5 relative on this scene
        errs = []
        tries = 0
        while len(errs) < want and tries < 12:
            tries += 1
            dv = rng.standard_normal((n, 3))
            dg = rng.standard_normal(3)
            lp, ctp = oracle_run(oracle, p, parts, steps, dv, eps, base_g + eps * dg)
            lm, ctm = oracle_run(oracle, p, parts, steps, dv, -eps, base_g - eps * dg)
            if not (np.array_equal(ctp, ct0) and np.array_equal(ctm, ct0)):
                continue  # a cell changed type between the runs: redraw the direction
            fd = (lp - lm) / (2 * eps)
            ad = float((gv * dv).sum() + (gg * dg).sum())
            errs.append(abs(ad - fd) / max(abs(fd), 1e-12))
    finally:
        oracle.set_exact_p2g(False)
    return errs


def oracle_run(oracle, p, parts, steps, dv, eps, grav, dx=None):
    """FP64 oracle rollout from `parts` with velocity + eps*dv (and position
    + eps*dx) and gravity `grav` applied in double: (loss, cell types of every step)."""
    q = p.copy()
    q.dims[2] = 3000
    q.pressure_tolerance = 1e-9
    o = oracle.OracleFluid(q, parts.shape[0], "f64")
    o.set_particles(parts)
    o.set_gravity_d(grav)
    if dv is not None:
        o.add_velocity_d(dv, eps)
    if dx is not None:
        o.add_position_d(dx, eps)
    cts = []
    for _ in range(steps):
        o.step(1)
        cts.append(o.get_grid()["cell_type"].copy())
    c = o.mean_position_d()
    o.close()
    return float(((c - TARGET) ** 2).sum()), np.concatenate(cts)


def adjoint_grads(p, parts, steps, k):
    import torch
    from fluidgb.autograd import Rollout, RolloutFunction, com_loss
    roll = Rollout(p, parts.shape[0], steps, checkpoint_every=k, adj_cg_iters=3000, adj_cg_tol=1e-7)
    vel0 = torch.tensor(parts[:, 4:7], device="cuda", requires_grad=True)
    grav = torch.tensor([0.0, -9.81, 0.0], device="cuda", dtype=torch.float32, requires_grad=True)
    pos0 = torch.tensor(parts[:, 0:3], device="cuda")
    final = RolloutFunction.apply(vel0, grav, pos0, roll)
    loss = com_loss(final, torch.tensor(TARGET, dtype=torch.float32, device="cuda"))
    loss.backward()
    roll.close()
    return vel0.grad.detach().cpu().numpy().astype(np.float64), grav.grad.detach().cpu().numpy().astype(np.float64)


# 1e-3 relative at the horizons of a few substeps; over 12 substeps the f32
# forward's rounding, amplified along the horizon, is reported against a
# looser bound.
@pytest.mark.parametrize("steps,k,bound", [(1, 1, 1e-3), (4, 2, 1e-3), (12, 4, 1e-2)])
def test_adjoint_matches_finite_differences(oracle, steps, k, bound):
    pytest.importorskip("torch")
    from fluidgb import build
    build.build()
    p, parts, _ = setup_case(steps=steps)
    gv, gg = adjoint_grads(p, parts, steps, k)
    assert np.all(np.isfinite(gv)) and np.all(np.isfinite(gg))
    errs = fd_errors(oracle, p, parts, steps, gv, gg)
    print("forward Euler, %d steps: rel errors %s" % (steps, ["%.2e" % e for e in errs]))
    assert len(errs) >= 2
    assert max(errs) < bound, errs


@pytest.mark.parametrize("case", ["midpoint", "friction", "midpoint_friction"])
@pytest.mark.parametrize("steps", [1, 4])
def test_adjoint_of_midpoint_advection_and_wall_friction(oracle, case, steps):
    """The midpoint advection (advect_order 2: k1 = clamp(PIC(X)), midpoint
    gather of the final faces, k2 = clamp(fin(Xm))) and the wall-friction band
    (g2p.wgsl:173-184) differentiated by fl_step_adjoint, against central
    differences of the FP64 oracle running the same options."""
    pytest.importorskip("torch")
    from fluidgb import build
    build.build()
    opts = {"midpoint": dict(advect_order=2), "friction": dict(region=floor_blob, friction=0.35),
            "midpoint_friction": dict(region=floor_blob, friction=0.35, advect_order=2)}[case]
    p, parts, _ = setup_case(steps=steps, **opts)
    gv, gg = adjoint_grads(p, parts, steps, 2 if steps > 1 else 1)
    assert np.all(np.isfinite(gv)) and np.all(np.isfinite(gg))
    errs = fd_errors(oracle, p, parts, steps, gv, gg)
    print("%s, %d steps: rel errors %s" % (case, steps, ["%.2e" % e for e in errs]))
    assert len(errs) >= 2
    assert max(errs) < 1e-3, errs


def test_checkpointed_recompute_matches_forward():
    """The backward pass recomputes segments from checkpoints; the recomputed
    final state must equal the forward's bit for bit."""
    torch = pytest.importorskip("torch")
    from fluidgb.autograd import Rollout
    p, parts, steps = setup_case(steps=5)
    roll = Rollout(p, parts.shape[0], steps, checkpoint_every=2)
    final, ids = roll.forward(parts, (0.0, -9.81, 0.0))
    assert sorted(roll.checkpoints) == [0, 2, 4]
    buf = roll.checkpoints[4]
    roll.fluid.load_state_device(buf.data_ptr(), buf.numel())
    roll.fluid.step(1)
    again, ids2 = roll.fluid.get_particles()
    assert np.array_equal(final.cpu().numpy(), again) and np.array_equal(ids.cpu().numpy(), ids2)
    # the device checkpoint holds the same bytes as the host one
    roll.fluid.load_state_device(buf.data_ptr(), buf.numel())
    assert roll.fluid.save_state() == bytes(buf.cpu().numpy())
    # replaying every substep from the start with the logged pressure fields
    # (no CG) reproduces the forward bit for bit
    buf = roll.checkpoints[0]
    roll.fluid.load_state_device(buf.data_ptr(), buf.numel())
    for s in range(steps):
        roll.fluid.step_replay(roll.plog[s].data_ptr())
    again, ids2 = roll.fluid.get_particles()
    assert np.array_equal(final.cpu().numpy(), again) and np.array_equal(ids.cpu().numpy(), ids2)
    roll.close()


def test_pressure_log_recompute_gives_the_same_gradients():
    """Backward passes that recompute segments by replaying logged pressure
    fields and by re-solving record the same tapes, and the adjoint has no
    float atomics: the gradients agree bit for bit."""
    torch = pytest.importorskip("torch")
    from fluidgb.autograd import Rollout
    p, parts, steps = setup_case(steps=9)
    n = parts.shape[0]
    g = np.zeros((n, 8), np.float32)
    g[:, 0:3] = np.random.default_rng(6).standard_normal((n, 3)).astype(np.float32) / n
    out = []
    for plog in (False, True):
        roll = Rollout(p, n, steps, checkpoint_every=3, adj_cg_iters=500, adj_cg_tol=1e-6, pressure_log=plog)
        final, ids = roll.forward(parts, (0.0, -9.81, 0.0))
        g0, gg = roll.backward(torch.from_numpy(g).cuda()[ids])
        out.append((g0.cpu().numpy().copy(), np.asarray(gg).copy()))
        roll.close()
    rel = np.linalg.norm(out[1][0] - out[0][0]) / np.linalg.norm(out[0][0])
    relg = np.linalg.norm(out[1][1] - out[0][1]) / np.linalg.norm(out[0][1])
    print("pressure log vs re-solve: gradient rel. difference %.1e (particles), %.1e (gravity)" % (rel, relg))
    assert np.array_equal(out[1][0], out[0][0]) and np.array_equal(out[1][1], out[0][1])


@pytest.mark.parametrize("steps,k,what", [(1, 1, "pos"), (2, 1, "vel"), (4, 4, "vel"), (4, 2, "grav")])
def test_adjoint_position_and_chain_diagnostics(oracle, steps, k, what):
    """Directional derivatives w.r.t. initial positions (one step), initial
    velocities (2 and 4 steps, with and without checkpoints) and gravity, each
    alone: a failure here names the part of the chain that is off."""
    pytest.importorskip("torch")
    import torch
    from fluidgb.autograd import Rollout
    p, parts, _ = setup_case(steps=steps)
    n = parts.shape[0]
    roll = Rollout(p, n, steps, checkpoint_every=k, adj_cg_iters=3000, adj_cg_tol=1e-7)
    final, ids = roll.forward(parts, (0.0, np.float32(-9.81), 0.0))
    c = final[:, 0:3].cpu().numpy().astype(np.float64).mean(axis=0)
    g = np.zeros((n, 8), np.float32)
    g[:, 0:3] = (2.0 * (c - TARGET) / n).astype(np.float32)
    g0, g_grav = roll.backward(g)
    g0 = g0.cpu().numpy()
    roll.close()
    oracle.set_exact_p2g(True)
    try:
        base_g = np.array([0.0, np.float32(-9.81), 0.0], np.float64)
        rng = np.random.default_rng(5)
        d = rng.standard_normal((n, 3))
        eps = 1e-6
        if what == "pos":
            eps = 1e-7  # tent weights are piecewise linear: keep clear of the kinks
            lp, _ = oracle_run(oracle, p, parts, steps, None, eps, base_g, dx=d)
            lm, _ = oracle_run(oracle, p, parts, steps, None, -eps, base_g, dx=d)
            fd = (lp - lm) / (2 * eps)
            ad = float((g0[:, 0:3].astype(np.float64) * d).sum())
        elif what == "grav":
            dg = np.array([0.3, -1.0, 0.2])
            lp, _ = oracle_run(oracle, p, parts, steps, None, 0.0, base_g + eps * dg)
            lm, _ = oracle_run(oracle, p, parts, steps, None, 0.0, base_g - eps * dg)
            fd = (lp - lm) / (2 * eps)
            ad = float((np.asarray(g_grav) * dg).sum())
        else:
            lp, _ = oracle_run(oracle, p, parts, steps, d, eps, base_g)
            lm, _ = oracle_run(oracle, p, parts, steps, d, -eps, base_g)
            fd = (lp - lm) / (2 * eps)
            ad = float((g0[:, 4:7].astype(np.float64) * d).sum())
    finally:
        oracle.set_exact_p2g(False)
    print("%s steps %d k %d: adjoint %.6e fd %.6e rel %.2e" % (what, steps, k, ad, fd, abs(ad - fd) / abs(fd)))
    assert abs(ad - fd) <= 1e-2 * abs(fd)


def test_adjoint_warm_start_matches_cold_start():
    """The warm-started adjoint solve (each from the next step's lambda, same
    |r| <= tol |dL/dp| bound) gives the cold start's gradients to the solve's
    tolerance in fewer CG iterations, and a second backward pass repeats the
    first bit for bit (lambda is reset at its start; the face gradients are
    gathered per face in a fixed order, with no float atomics)."""
    torch = pytest.importorskip("torch")
    from fluidgb.autograd import Rollout
    p = scenes.params_for(32, iters=400, tol=1e-6, precision=FL_CG_F64, stiffness=0.0)
    parts = scenes.seed_particles(32, scenes.box(0.5, 0.4), vel_sigma=0.1)
    n, steps = parts.shape[0], 20
    g = np.zeros((n, 8), np.float32)
    g[:, 0:3] = np.random.default_rng(5).standard_normal((n, 3)).astype(np.float32) / n

    def grads(warm):
        roll = Rollout(p, n, steps, checkpoint_every=5, adj_cg_iters=400, adj_cg_tol=1e-6, adj_warm_start=warm)
        final, ids = roll.forward(parts, (0.0, -9.81, 0.0))
        gf = torch.from_numpy(g).cuda()[ids]
        g0, gg = roll.backward(gf)
        out = (g0.cpu().numpy().copy(), np.asarray(gg).copy(), list(roll.adj_cg_iterations))
        g1, gg1 = roll.backward(gf)
        rep = np.array_equal(g1.cpu().numpy(), out[0]) and np.array_equal(np.asarray(gg1), out[1])
        roll.close()
        return out + (rep,)

    gc, ggc, itc, repc = grads(False)
    gw, ggw, itw, repw = grads(True)
    rel = np.linalg.norm(gw - gc) / np.linalg.norm(gc)
    relg = np.linalg.norm(ggw - ggc) / np.linalg.norm(ggc)
    print("adjoint CG iterations: cold %d, warm %d; gradient rel. difference %.2e (particles), %.2e (gravity); "
          "repeats bit-identical: %s (cold) %s (warm)" % (sum(itc), sum(itw), rel, relg, repc, repw))
    assert repc and repw
    assert sum(itw) < sum(itc)
    assert rel < 1e-3 and relg < 1e-3


def test_adjoint_through_the_multigrid_solver():
    """A handle on FL_SOLVER_MGPCG solves its adjoint pressure systems with the
    multigrid preconditioner too: the gradients agree with the CG handle's to
    the solves' tolerance, in far fewer adjoint iterations."""
    torch = pytest.importorskip("torch")
    from fluidgb import FL_SOLVER_MGPCG
    from fluidgb.autograd import Rollout
    p = scenes.params_for(32, iters=400, tol=1e-6, precision=FL_CG_F64, stiffness=0.0)
    parts = scenes.seed_particles(32, scenes.box(0.5, 0.4), vel_sigma=0.1)
    n, steps = parts.shape[0], 12
    g = np.zeros((n, 8), np.float32)
    g[:, 0:3] = np.random.default_rng(7).standard_normal((n, 3)).astype(np.float32) / n
    out = []
    # (forward solver, adjoint solver): the CG handle, the MGPCG handle, and
    # the CG handle whose tape solves the adjoint through the preconditioner
    from fluidgb import FL_SOLVER_CG, FL_SOLVER_FOLLOW
    for solver, adj in ((0, FL_SOLVER_FOLLOW), (FL_SOLVER_MGPCG, FL_SOLVER_FOLLOW), (0, FL_SOLVER_MGPCG)):
        q = p.copy()
        q.pressure_solver = solver
        roll = Rollout(q, n, steps, checkpoint_every=4, adj_cg_iters=400, adj_cg_tol=1e-6, adj_solver=adj)
        final, ids = roll.forward(parts, (0.0, -9.81, 0.0))
        g0, gg = roll.backward(torch.from_numpy(g).cuda()[ids])
        out.append((g0.cpu().numpy().copy(), np.asarray(gg).copy(), sum(roll.adj_cg_iterations)))
        roll.close()
    for k, name in ((1, "MGPCG handle"), (2, "CG handle, MGPCG adjoint")):
        rel = np.linalg.norm(out[k][0] - out[0][0]) / np.linalg.norm(out[0][0])
        relg = np.linalg.norm(out[k][1] - out[0][1]) / np.linalg.norm(out[0][1])
        print("adjoint CG vs %s: iterations %d vs %d; gradient rel. difference %.2e (particles), %.2e (gravity)" % (
            name, out[0][2], out[k][2], rel, relg))
        assert out[k][2] * 2 < out[0][2]
        assert rel < 1e-3 and relg < 1e-3
    assert FL_SOLVER_CG == 0


@pytest.mark.parametrize("case", ["midpoint_friction", "strays"])
def test_backward_passes_repeat_bit_for_bit(case):
    """Two backward passes of the same rollout give identical gradients: the
    face gradients are gathered per face in a fixed order, the midpoint
    stencil's are summed as 64-bit integers, dL/dgravity from block partials
    in order.  Cases: the midpoint step with wall friction, and a step with
    stray particles (exact cell-face positions: the widened gather)."""
    torch = pytest.importorskip("torch")
    from fluidgb.autograd import Rollout
    if case == "strays":
        n = 24  # h = 1/24 is inexact in f32: particles on cell faces bin and scatter differently
        p = scenes.params_for(n, iters=300, tol=1e-6, precision=FL_CG_F64, stiffness=0.0)
        parts = scenes.seed_particles(n, blob, seed=7, vel_sigma=0.1)
        h = np.float32(1.0) / np.float32(n)
        sel = np.flatnonzero(np.random.default_rng(2).random(parts.shape[0]) < 0.2)
        for axis in (0, 1, 2):
            parts[sel, axis] = np.nextafter(np.round(parts[sel, axis] / h).astype(np.float32) * h, np.float32(-1.0))
    else:
        p, parts, _ = setup_case(steps=4, region=floor_blob, friction=0.35, advect_order=2)
    n, steps = parts.shape[0], 4
    g = np.zeros((n, 8), np.float32)
    g[:, 0:3] = np.random.default_rng(9).standard_normal((n, 3)).astype(np.float32) / n
    roll = Rollout(p, n, steps, checkpoint_every=2, adj_cg_iters=300, adj_cg_tol=1e-6)
    final, ids = roll.forward(parts, (0.0, -9.81, 0.0))
    gf = torch.from_numpy(g).cuda()[ids]
    g0, gg0 = roll.backward(gf)
    a = (g0.cpu().numpy().copy(), np.asarray(gg0).copy())
    g1, gg1 = roll.backward(gf)
    roll.close()
    assert np.all(np.isfinite(a[0])) and np.any(a[0] != 0)
    assert np.array_equal(g1.cpu().numpy(), a[0]) and np.array_equal(np.asarray(gg1), a[1])


def test_adjoint_with_ieee_double_reductions(oracle):
    """The adjoint pressure solve follows the handle's cg_precision: with
    IEEE-double inner products the 4-substep gradients meet the same 1e-3
    bound against the FP64 oracle's finite differences."""
    pytest.importorskip("torch")
    p, parts, steps = setup_case(steps=4)
    p.cg_precision = FL_CG_F64_IEEE
    gv, gg = adjoint_grads(p, parts, steps, 2)
    errs = fd_errors(oracle, p, parts, steps, gv, gg)
    print("IEEE-double CG, 4 steps: rel errors %s" % (["%.2e" % e for e in errs]))
    assert len(errs) >= 2
    assert max(errs) < 1e-3, errs
