"""Failure detection without a GPU fault: a device-side wait that runs out.

Every wait in the solvers (the CG's exchange polls, the multigrid barrier) is
bounded by a limit on %globaltimer.  With the limit set below one poll's
latency, the first wait of the 128^3 solve that is not met at once expires:
the kernel records FL_TIMEOUT, every block returns, the substep finishes, and
the next fl_sync reports the status (the reference's device-lost status word,
gpu/mod.rs:245-250).  With the default limit restored, the handle keeps
working: the next substep, from a restored checkpoint, equals the oracle's bit
for bit (the CG) or a fresh handle's (the multigrid-preconditioned CG).
Nothing here traps, faults or hangs: the expiry is an ordinary return path.
"""
import numpy as np
import pytest

from fluidgb import FL_SOLVER_MGPCG, FL_TIMEOUT, Fluid, FluidError, scenes

from test_gpu_parity import assert_same_state, make_pair

pytestmark = pytest.mark.gpu

# Below the latency of one poll: any wait not met by its first poll expires
# (at 128^3 every solve has such waits: the blocks never all publish at once).
LIMIT_NS = 1


@pytest.fixture(scope="module")
def lib():
    from fluidgb import _abi, build
    build.build()
    return _abi.load_library()


def expire_once(g):
    """One substep with the short limit; the status comes back as FL_TIMEOUT."""
    g.set_wait_timeout(LIMIT_NS)
    g.step(1)
    with pytest.raises(FluidError) as e:
        g.sync()
    assert e.value.status == FL_TIMEOUT
    g.set_wait_timeout(0)
    g.sync()  # the status was cleared by the read that reported it
    assert g.stats()["device_status"] == 0


def test_cg_wait_expires_and_the_handle_recovers(lib, oracle):
    p, parts, _ = scenes.workload("dam128_2m")
    g, o = make_pair(oracle, p, parts)
    g.step(1)
    o.step(1)
    assert_same_state(g, o, "before")
    blob = g.save_state()
    expire_once(g)
    g.load_state(blob)
    g.step(1)
    o.step(1)
    assert_same_state(g, o, "after recovery")
    g.close()
    o.close()


def test_mgpcg_barrier_expires_and_the_handle_recovers(lib):
    p, parts, _ = scenes.workload("dam128_2m")
    p.pressure_solver = FL_SOLVER_MGPCG
    g = Fluid(p, parts.shape[0])
    g.set_particles(parts)
    g.step(1)
    blob = g.save_state()
    expire_once(g)
    g.load_state(blob)
    g.step(1)
    got = g.get_particles()
    ref = Fluid(p, parts.shape[0])
    ref.set_particles(parts)
    ref.step(2)
    want = ref.get_particles()
    assert np.array_equal(got[0], want[0]) and np.array_equal(got[1], want[1])
    g.close()
    ref.close()
