"""Gradient check of the differentiable rollout at the 64^3 configuration.

Scene: 64^3 tank, fluid block x<0.5, y<0.4 at 8 particles per cell (384,400
particles), initial velocities N(0, 0.1^2) seeded, 60 substeps at dt 1/120,
checkpoints every 10.  Loss: |centre of mass - (0.7, 0.2, 0.5)|^2.  Gradients
w.r.t. the per-particle initial velocity and the gravity vector come from the
adjoint kernels through RolloutFunction (torch.autograd.Function); they are
compared with central finite differences, eps 1e-3, of the FP64 oracle forward
(unrounded P2G, CG to 1e-9) on 16 random directions.  Volume stiffness is 0:
its drift term is a function of integer particle counts, held fixed by the
adjoint.

Two horizons.  The default suite runs 3 substeps at eps 1e-6: there every
direction's +-eps runs keep the unperturbed run's cell types (at least 12 of
16 are required) and the median relative error over them must be at most
1e-3.  The configuration's own horizon and step (60 substeps, eps 1e-3) run
with FL_GRADCHECK64=1 (33 FP64 rollouts of 60 substeps take minutes on the
host cores) and are reported: at that horizon nearly every direction flips
cell types.  FL_GC_STEPS and FL_GC_EPS override the opt-in run's horizon and
step; every direction is printed, and with FL_GRADCHECK_OUT written as JSON.
The adjoint holds the discrete choices of the recorded forward fixed (bins,
cell types, clamps); a direction whose +-eps runs change cell types sees those
jumps in the finite difference, so each direction reports how many cell types
differ from the unperturbed run.
"""
import json
import os

import numpy as np
import pytest

from fluidgb import FL_CG_F64, scenes

pytestmark = pytest.mark.gpu

TARGET = np.array([0.7, 0.2, 0.5])
EVERY, DIRECTIONS = 10, 16
OPT_IN = os.environ.get("FL_GRADCHECK64") == "1"
# the configuration's horizon and step size; FL_GC_STEPS / FL_GC_EPS vary them
CONFIG_STEPS = int(os.environ.get("FL_GC_STEPS", "60"))
CONFIG_EPS = float(os.environ.get("FL_GC_EPS", "1e-3"))


def forward_fp64(oracle, p, parts, dv, eps, grav, steps):
    q = p.copy()
    q.dims[2] = 3000
    q.pressure_tolerance = 1e-9
    o = oracle.OracleFluid(q, parts.shape[0], "f64")
    o.set_particles(parts)
    o.set_gravity_d(grav)
    if dv is not None:
        o.add_velocity_d(dv, eps)
    cts = []
    for _ in range(steps):
        o.step(1)
        cts.append(o.get_grid()["cell_type"].copy())
    c = o.mean_position_d()
    o.close()
    return float(((c - TARGET) ** 2).sum()), np.stack(cts)


@pytest.mark.parametrize("horizon", [
    "short", pytest.param("configuration", marks=pytest.mark.skipif(
        not OPT_IN, reason="minutes of FP64 host rollouts: FL_GRADCHECK64=1"))])
def test_block64_rollout_gradients_against_fp64_finite_differences(oracle, horizon):
    STEPS, EPS = (3, 1e-6) if horizon == "short" else (CONFIG_STEPS, CONFIG_EPS)
    torch = pytest.importorskip("torch")
    from fluidgb import build
    from fluidgb.autograd import Rollout, RolloutFunction, com_loss
    build.build()
    spec = scenes.WORKLOADS["block64"]
    p = scenes.params_for(spec["n"], iters=500, tol=1e-6, precision=FL_CG_F64, stiffness=0.0)
    parts = scenes.seed_particles(spec["n"], spec["region"], vel_sigma=spec["vel_sigma"])
    n = parts.shape[0]
    roll = Rollout(p, n, STEPS, checkpoint_every=EVERY, adj_cg_iters=3000, adj_cg_tol=1e-7)
    vel0 = torch.tensor(parts[:, 4:7], device="cuda", requires_grad=True)
    grav = torch.tensor([0.0, -9.81, 0.0], device="cuda", dtype=torch.float32, requires_grad=True)
    pos0 = torch.tensor(parts[:, 0:3], device="cuda")
    final = RolloutFunction.apply(vel0, grav, pos0, roll)
    loss = com_loss(final, torch.tensor(TARGET, dtype=torch.float32, device="cuda"))
    loss.backward()
    gv = vel0.grad.detach().cpu().numpy().astype(np.float64)
    gg = grav.grad.detach().cpu().numpy().astype(np.float64)
    roll.close()
    assert np.all(np.isfinite(gv)) and np.all(np.isfinite(gg))

    oracle.set_threads(0)
    oracle.set_exact_p2g(True)
    rows = []
    try:
        base_g = np.array([0.0, np.float32(-9.81), 0.0], np.float64)
        _, ct0 = forward_fp64(oracle, p, parts, None, 0.0, base_g, STEPS)
        rng = np.random.default_rng(4)
        for k in range(DIRECTIONS):
            dv = rng.standard_normal((n, 3))
            dg = rng.standard_normal(3)
            lp, ctp = forward_fp64(oracle, p, parts, dv, EPS, base_g + EPS * dg, STEPS)
            lm, ctm = forward_fp64(oracle, p, parts, dv, -EPS, base_g - EPS * dg, STEPS)
            fd = (lp - lm) / (2 * EPS)
            ad = float((gv * dv).sum() + (gg * dg).sum())
            rel = abs(ad - fd) / max(abs(fd), 1e-12)
            changed = int(np.count_nonzero(ctp != ct0) + np.count_nonzero(ctm != ct0))
            rows.append({"direction": k, "adjoint": ad, "fd": fd, "rel_err": rel, "cell_type_changes": changed})
            print("direction %2d: adjoint %+.6e  fd %+.6e  rel err %.2e  cell-type changes %d" % (
                k, ad, fd, rel, changed))
    finally:
        oracle.set_exact_p2g(False)
    out = os.environ.get("FL_GRADCHECK_OUT")
    if out:
        with open(out, "w") as f:
            json.dump({"particles": n, "steps": STEPS, "checkpoint_every": EVERY, "eps": EPS, "rows": rows}, f,
                      indent=1)
    errs = np.array([r["rel_err"] for r in rows])
    smooth = [r["rel_err"] for r in rows if r["cell_type_changes"] == 0]
    print("steps %d eps %.0e: median rel err %.2e, max %.2e; %d of %d directions keep every cell type" % (
        STEPS, EPS, np.median(errs), errs.max(), len(smooth), len(rows)))
    # The finite difference measures the adjoint's derivative only where the
    # +-eps runs take the same discrete branch; on those directions the median
    # error is bounded (the f32 forward's rounding, amplified along the
    # horizon, sets the rest).
    if horizon == "short":
        assert len(smooth) >= 12, rows
        assert np.median(smooth) <= 1e-3, smooth
    elif smooth:
        assert np.median(smooth) < 1e-2, smooth
