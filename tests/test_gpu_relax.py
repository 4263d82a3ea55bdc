"""The reference's relaxation solvers on the GPU (fl_relax_pressure): Jacobi
(sim/pressure.rs:68-136) and red-black Gauss-Seidel (pressure.wgsl), bit for
bit against the oracle's restatements, on the reference's 16^3 divergent-tank
fixture and on the divergence of a 48^3 dam-break step."""
import numpy as np
import pytest

from fluidgb import FL_RELAX_JACOBI, FL_RELAX_RBGS, _abi, scenes

pytestmark = pytest.mark.gpu


def dam_field(oracle, n=48):
    p = scenes.params_for(n, stiffness=0.0)
    parts = scenes.seed_particles(n, scenes.box(0.5, 0.5))
    o = oracle.OracleFluid(p, parts.shape[0], "f32")
    o.set_particles(parts)
    o.step(1)
    div = o.get_divergence()
    ct = o.get_grid()["cell_type"]
    o.close()
    return (n, n, n), ct, div, float(np.float32(1.0) / np.float32(n)), float(np.float32(p.geom[2]))


@pytest.mark.parametrize("method", [FL_RELAX_JACOBI, FL_RELAX_RBGS])
def test_relax_matches_oracle(fluidlib, oracle, method):
    from test_oracle_kats import divergent_tank
    ref = oracle.ref_jacobi_solve if method == FL_RELAX_JACOBI else oracle.ref_rbgs_solve
    d, ct, _, _, _, div0 = divergent_tank(oracle)
    for iters in (1, 7, 200):
        g = _abi.relax_pressure(ct, div0, d, 1.0, 1.0, 1.0, method, iters)
        assert np.array_equal(g, ref(d, 1.0, 1.0, 1.0, ct, div0, iters)), iters
    d, ct, div, h, dt = dam_field(oracle)
    g = _abi.relax_pressure(ct, div, d, h, 1000.0, dt, method, 50)
    o = ref(d, h, 1000.0, dt, ct, div, 50)
    assert np.array_equal(g, o)
    assert np.any(g != 0.0)
