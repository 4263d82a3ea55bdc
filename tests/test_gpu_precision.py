"""Precision study of the 128^3 sphere-into-pool scene against the FP64 oracle.

Scene: a sphere of radius 0.12 at (0.5, 0.75, 0.5) falling into a pool of
depth 0.3, 8 jittered particles per fluid cell, seed 0x5EED, 200 substeps.  For
each CG relative tolerance in {1e-3, 1e-4, 1e-5, 1e-6} and each form (the
reference's FP32 CG, FL_CG_F32, and the form with extended-precision
reductions in float-float, FL_CG_F64, and in IEEE double, FL_CG_F64_IEEE),
the GPU runs the scene; at substeps 1 and 200 the step
is repeated by the FP64 oracle from the GPU's state before it (particles and
the warm-start pressure), once at the same tolerance and iteration cap and once
converged (tolerance 1e-10).  Reported per step, max and RMS of
|gpu - oracle|: the final face velocities (u, v, w) and the normalised P2G
face velocities relative to the largest oracle face speed, the pressure
relative to the largest oracle pressure, and particle positions (absolute, in
units of the box).

The errors are printed; with FL_PRECISION_OUT set they are also written there
as JSON.  Bounds: the GPU's CG takes the oracle's iteration count within 3%;
at tolerance 1e-5 both forms agree with the FP64 oracle of the same step to
1e-5 RMS in face velocity, 1e-6 RMS in pressure and 1e-6 in every position.
The max-norm velocity error is reported, not bounded: the projection takes
differences of neighbouring pressures, which in the pool are ~40 times smaller
than the pressure itself, so the pressure's relative error (set by the CG
tolerance) is amplified on individual faces; once particles move, low-weight
free-surface faces add the f32-vs-f64 rounding of the fixed-point P2G terms
round(w v 2^16) (the p2g_velocity column, before the solve).
"""
import json
import os

import numpy as np
import pytest

from fluidgb import FL_CG_F32, FL_CG_F64, FL_CG_F64_IEEE, Fluid, scenes

pytestmark = pytest.mark.gpu

TOLS = (1e-3, 1e-4, 1e-5, 1e-6)
CHECK_STEPS = (1, 200)


def vel_err(g_grid, og, keys):
    """Max and RMS of |gpu - oracle| over all faces of the three components,
    relative to the largest oracle face speed of those components."""
    d = np.concatenate([np.abs(np.asarray(g_grid[k], np.float64) - np.asarray(og[k], np.float64)) for k in keys])
    scale = max(max(np.max(np.abs(np.asarray(og[k], np.float64))) for k in keys), 1e-30)
    return float(np.max(d) / scale), float(np.sqrt(np.mean(d * d)) / scale)


def compare(g_grid, g_parts_by_id, o, in_ids):
    og = o.get_grid()
    xo, io = o.get_particles()
    # oracle ids are rows of its input, which was the GPU's slot order
    pos_o = np.empty((xo.shape[0], 3), np.float64)
    pos_o[in_ids[io]] = xo[:, 0:3]
    pg, po = np.asarray(g_grid["pressure"], np.float64), np.asarray(og["pressure"], np.float64)
    ps = max(np.max(np.abs(po)), 1e-30)
    d = np.abs(g_parts_by_id[:, 0:3].astype(np.float64) - pos_o)
    return {
        "velocity": vel_err(g_grid, og, ("u", "v", "w")),           # final faces (after projection)
        "p2g_velocity": vel_err(g_grid, og, ("u_saved", "v_saved", "w_saved")),  # normalised P2G faces
        "pressure": (float(np.max(np.abs(pg - po)) / ps), float(np.sqrt(np.mean((pg - po) ** 2)) / ps)),
        "position_abs": (float(np.max(d)), float(np.sqrt(np.mean(d * d)))),
        "cg_iterations_oracle": o.stats()["cg_iterations"],
    }


def params(prec, tol, iters):
    spec = scenes.WORKLOADS["sphere_pool128"]
    return scenes.params_for(spec["n"], iters=iters, tol=tol, precision=prec)


def test_precision_study_sphere_pool128(lib_built, oracle):
    oracle.set_threads(0)
    p0, parts, spec = scenes.workload("sphere_pool128")
    n = parts.shape[0]
    o = oracle.OracleFluid(p0, n, "f64")
    results = []
    try:
        for tol in TOLS:
            for prec in (FL_CG_F32, FL_CG_F64, FL_CG_F64_IEEE):
                p = params(prec, tol, spec["iters"])
                g = Fluid(p, n)
                g.set_particles(parts)
                done = 0
                for k in CHECK_STEPS:
                    g.step(k - 1 - done)
                    done = k - 1
                    x_in, id_in = g.get_particles()
                    p_in = g.get_grid()["pressure"]
                    g.step(1)
                    done = k
                    grid = g.get_grid()
                    x1, id1 = g.get_particles()
                    st = g.stats()
                    assert st["device_status"] == 0
                    by_id = np.empty_like(x1)
                    by_id[id1] = x1
                    row = {"tol": tol, "form": {FL_CG_F32: "f32", FL_CG_F64: "f64-reductions",
                                                    FL_CG_F64_IEEE: "ieee-f64-reductions"}[prec], "step": k,
                           "cg_iterations": st["cg_iterations"], "particles": n}
                    for label, otol, oiters in (("same_tol", tol, spec["iters"]), ("converged", 1e-10, 5000)):
                        q = params(FL_CG_F32, otol, oiters)
                        o.set_params(q)
                        o.set_particles(x_in)
                        o.set_pressure(p_in)
                        o.step(1)
                        # oracle ids are rows of x_in; map them to the GPU's particle ids
                        row[label] = compare(grid, by_id, o, id_in)
                    results.append(row)
                    sm, cv = row["same_tol"], row["converged"]
                    print("tol %.0e %-15s step %3d iters %3d/%3d | same-tol vel max %.1e rms %.1e  p2g max %.1e  "
                          "p rms %.1e  x max %.1e | converged vel rms %.1e  p rms %.1e" % (
                              tol, row["form"], k, st["cg_iterations"], sm["cg_iterations_oracle"],
                              sm["velocity"][0], sm["velocity"][1], sm["p2g_velocity"][0], sm["pressure"][1],
                              sm["position_abs"][0], cv["velocity"][1], cv["pressure"][1]))
                g.close()
    finally:
        o.close()
        oracle.set_threads(0)
    out = os.environ.get("FL_PRECISION_OUT")
    if out:
        with open(out, "w") as f:
            json.dump(results, f, indent=1)
    for row in results:
        sm = row["same_tol"]
        it_o = sm["cg_iterations_oracle"]
        assert abs(row["cg_iterations"] - it_o) <= max(2, 0.03 * it_o), row
        if row["tol"] == 1e-5:
            assert sm["velocity"][1] <= 1e-5, (row["form"], row["step"], sm["velocity"])
            assert sm["pressure"][1] <= 1e-6, (row["form"], row["step"], sm["pressure"])
            assert sm["position_abs"][0] <= 1e-6, (row["form"], row["step"], sm["position_abs"])


@pytest.fixture(scope="module")
def lib_built():
    from fluidgb import _abi, build
    build.build()
    return _abi.load_library()
