"""The multigrid-preconditioned pressure solver (FL_SOLVER_MGPCG).

It solves the CG's system (same operator, right-hand side, warm start,
iteration cap and stopping test) with a multigrid V-cycle as preconditioner
(red-black Gauss-Seidel smoothing, the reference's pressure.wgsl sweep).  Its
pressure is checked against the system itself: the right-hand side comes from
the oracle's step on the same particles (its P2G, classification and
divergence are bit-exact with the GPU's), and the relative residual
|b - A p| / |b| is evaluated in float64.  The reference's CG on the same step
is measured beside it; both stop at the same tolerance.
"""
import numpy as np
import pytest

from fluidgb import FL_CG_F64, FL_SOLVER_MGPCG, Fluid, scenes

pytestmark = pytest.mark.gpu

SOLID, LIQ = 0, 1


def apply_A(ct, p):
    """(A p)_c = n_c p_c - sum of liquid neighbours (n_c: non-solid
    neighbours), on liquid cells; ct and p are (nz, ny, nx)."""
    liq = ct == LIQ
    ns = ct != SOLID
    q = np.zeros(ct.shape, np.float64)
    pp = np.where(liq, p, 0.0)
    for ax in range(3):
        for sh in (1, -1):
            q += np.roll(ns, sh, axis=ax) * pp - np.roll(pp, sh, axis=ax)
    return np.where(liq, q, 0.0)


def rel_residual(ct, div, p, scale):
    b = np.where(ct == LIQ, -scale * div.astype(np.float64), 0.0)
    r = b - apply_A(ct, p.astype(np.float64))
    return float(np.linalg.norm(r) / np.linalg.norm(b))


def run(p, parts, steps=1):
    g = Fluid(p, parts.shape[0])
    g.set_particles(parts)
    g.step(steps)
    grid = g.get_grid()
    st = g.stats()
    x, ids = g.get_particles()
    g.close()
    assert st["device_status"] == 0
    return grid, st, x, ids


# 10^3 runs on one block (it owns the level-0 cells and the coarse levels,
# stencils read from global memory); 12^3 on two (block 0 the coarse levels
# with its stencils in shared memory, block 1 every level-0 cell).
@pytest.mark.parametrize("dims", [(48, 48, 48), (37, 29, 33), (10, 10, 10), (12, 12, 12)])
def test_mgpcg_residual_against_the_system(oracle, dims):
    nx, ny, nz = dims
    p = scenes.params_for(nx, ny=ny, nz=nz, iters=1000, tol=1e-5, precision=FL_CG_F64, stiffness=0.0,
                          warm_start=False)
    parts = scenes.seed_particles(nx, scenes.box(0.5, 0.5), ny=ny, nz=nz)
    q = p.copy()
    q.pressure_solver = FL_SOLVER_MGPCG
    g_cg, s_cg, _, _ = run(p, parts)
    g_mg, s_mg, _, _ = run(q, parts)
    o = oracle.OracleFluid(p, parts.shape[0], "f32")
    o.set_particles(parts)
    o.step(1)
    div = o.get_divergence().reshape(nz, ny, nx)
    ct = o.get_grid()["cell_type"].reshape(nz, ny, nx)
    o.close()
    assert np.array_equal(ct, g_mg["cell_type"].reshape(nz, ny, nx))
    h = np.float32(1.0) / np.float32(nx)
    scale = float(np.float32(np.float32(np.float32(1000.0) * h) * h) / np.float32(p.geom[2]))
    res_cg = rel_residual(ct, div, g_cg["pressure"].reshape(nz, ny, nx), scale)
    res_mg = rel_residual(ct, div, g_mg["pressure"].reshape(nz, ny, nx), scale)
    print("%s: CG %d iterations, |b-Ap|/|b| %.2e; MGPCG %d iterations, %.2e" % (
        dims, s_cg["cg_iterations"], res_cg, s_mg["cg_iterations"], res_mg))
    if nx >= 32:
        assert s_mg["cg_iterations"] * 3 < s_cg["cg_iterations"]
    else:
        assert s_mg["cg_iterations"] < s_cg["cg_iterations"]
    # both stop on the recurrence residual at 1e-5; the f32 vectors leave the
    # true residual a few times above it
    assert res_cg < 1e-4 and res_mg < 1e-4
    assert res_mg <= 2.0 * max(res_cg, 1e-5)


def by_id(x, ids):
    out = np.empty_like(x)
    out[ids] = x
    return out[:, 0:3].astype(np.float64)


def test_mgpcg_steps_repeat_and_track_the_cg():
    """Ten warm-started substeps: two MGPCG handles agree bit for bit; the
    particles differ from the reference CG's (tolerance 1e-5) by no more than
    the CG's own result moves when its tolerance is tightened to 1e-6:
    differences at the tolerance, amplified alike by the flow."""
    n = 40
    p = scenes.params_for(n, iters=200, tol=1e-5)
    parts = scenes.seed_particles(n, scenes.box(0.4, 0.6))
    q = p.copy()
    q.pressure_solver = FL_SOLVER_MGPCG
    p6 = p.copy()
    p6.pressure_tolerance = 1e-6
    _, s1, x1, i1 = run(q, parts, 10)
    _, _, x2, i2 = run(q, parts, 10)
    _, s0, x0, i0 = run(p, parts, 10)
    _, _, x3, i3 = run(p6, parts, 10)
    assert np.array_equal(x1, x2) and np.array_equal(i1, i2)
    ref = by_id(x0, i0)
    d_mg = np.abs(by_id(x1, i1) - ref)
    d_t = np.abs(by_id(x3, i3) - ref)
    rms = lambda d: float(np.sqrt(np.mean(d * d)))
    print("10 substeps vs the CG at 1e-5: MGPCG max %.2e rms %.2e; CG at 1e-6 max %.2e rms %.2e; "
          "iterations of the last solve CG %d, MGPCG %d" % (
              d_mg.max(), rms(d_mg), d_t.max(), rms(d_t), s0["cg_iterations"], s1["cg_iterations"]))
    assert rms(d_mg) <= 3.0 * max(rms(d_t), 1e-7)
    assert s1["cg_iterations"] < s0["cg_iterations"]


def test_solver_switch_on_a_live_handle():
    n = 32
    p = scenes.params_for(n, iters=200, tol=1e-5)
    parts = scenes.seed_particles(n, scenes.box(0.4, 0.6))
    g = Fluid(p, parts.shape[0])
    g.set_particles(parts)
    g.step(2)
    it_cg = g.stats()["cg_iterations"]
    q = p.copy()
    q.pressure_solver = FL_SOLVER_MGPCG
    g.set_params(q)
    g.step(2)
    it_mg = g.stats()["cg_iterations"]
    g.set_params(p)
    g.step(1)
    st = g.stats()
    g.close()
    assert st["device_status"] == 0
    assert 0 < it_mg < it_cg
