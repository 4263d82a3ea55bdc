"""fl_solve_pressure_noalloc: the pressure solve for callers that cannot call
cudaMalloc (no-allocation frame loops, plugins whose host owns all device
memory, processes that must not grow their footprint after start-up).

It runs the same CG as fl_solve_pressure with its scratch in one static device
array, on device buffers the caller owns.  This file is collected last so that
a failure here does not hide any other test; it must pass on its own in a
fresh process and after the rest of the suite.  The test allocates its own
buffers (with torch); the entry point under test allocates nothing.
"""
import ctypes

import numpy as np
import pytest

from fluidgb import FL_CG_F32, FL_CG_F64, FL_INVALID_ARG, FL_OK, FlStats
from fluidgb import _abi

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def lib():
    from fluidgb import build
    build.build()
    return _abi.load_library()


def tank(oracle):
    from test_oracle_kats import divergent_tank
    d, ct, u, v, w, div = divergent_tank(oracle)
    return d, ct, div


def random_case(n=48, seed=3):
    rng = np.random.default_rng(seed)
    d = (n, n, n)
    k, j, i = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij")
    ct = np.where((i == 0) | (j == 0) | (k == 0) | (i == n - 1) | (j == n - 1) | (k == n - 1), 0,
                  np.where((j < n // 2) | (rng.random((n, n, n)) < 0.3), 1, 2)).astype(np.uint8).ravel()
    div = (rng.standard_normal(n ** 3) * (ct == 1)).astype(np.float32)
    p0 = (rng.standard_normal(n ** 3) * (ct == 1)).astype(np.float32)
    return d, ct, div, p0


def noalloc(lib, torch, d, ct, div, p_init, iters, warm, tol, precision):
    ct_d = torch.from_numpy(ct).cuda()
    div_d = torch.from_numpy(div).cuda()
    p_d = torch.from_numpy(p_init.copy()).cuda()
    torch.cuda.synchronize()
    st = FlStats()
    r = lib.fl_solve_pressure_noalloc(d[0], d[1], d[2], ct_d.data_ptr(), div_d.data_ptr(), p_d.data_ptr(), 1.0,
                                      1.0, 1.0, iters, 1 if warm else 0, tol, precision, None, ctypes.byref(st))
    assert r == FL_OK, r
    return p_d.cpu().numpy(), st.as_dict()


@pytest.mark.parametrize("precision", [FL_CG_F32, FL_CG_F64])
@pytest.mark.parametrize("case", ["tank16", "random48_warm"])
def test_noalloc_matches_allocating_solve_twice_in_a_row(lib, oracle, precision, case):
    torch = pytest.importorskip("torch")
    if case == "tank16":
        d, ct, div = tank(oracle)
        p0, warm, tol, iters = np.zeros_like(div), False, 0.0, 40
    else:
        d, ct, div, p0 = random_case()
        warm, tol, iters = True, 1e-3, 120
    want, sw = _abi.solve_pressure(ct, div, d, 1.0, 1.0, 1.0, iters, warm_start=warm, pressure_in=p0,
                                   tolerance=tol, precision=precision)
    for call in range(2):  # the shared scratch keeps the previous call's contents
        got, sg = noalloc(lib, torch, d, ct, div, p0, iters, warm, tol, precision)
        # same kernels and launch shape as fl_solve_pressure: identical bits
        # (the tolerance the parity tests use for the f32 CG is exact)
        assert np.array_equal(got, want), "call %d" % call
        assert sg["cg_iterations"] == sw["cg_iterations"]
        assert sg["rs_final"] == sw["rs_final"]


@pytest.mark.parametrize("precision", [FL_CG_F32, FL_CG_F64])
def test_noalloc_grid_changes_between_calls(lib, oracle, precision):
    """The shared scratch keeps the last call's plan, chunk flags, exchange
    words and vector entries: a 48^3 solve, then the 16^3 tank, then 48^3
    again, each equal bit for bit to the allocating solve."""
    torch = pytest.importorskip("torch")
    d48, ct48, div48, p48 = random_case()
    d16, ct16, div16 = tank(oracle)
    cases = [(d48, ct48, div48, p48, True, 1e-3, 120), (d16, ct16, div16, np.zeros_like(div16), False, 0.0, 40),
             (d48, ct48, div48, p48, True, 1e-3, 120)]
    for i, (d, ct, div, p0, warm, tol, iters) in enumerate(cases):
        want, sw = _abi.solve_pressure(ct, div, d, 1.0, 1.0, 1.0, iters, warm_start=warm, pressure_in=p0,
                                       tolerance=tol, precision=precision)
        got, sg = noalloc(lib, torch, d, ct, div, p0, iters, warm, tol, precision)
        assert np.array_equal(got, want), "call %d (%s)" % (i, d)
        assert sg["cg_iterations"] == sw["cg_iterations"]


def test_noalloc_rejects_overlapping_buffers(lib):
    torch = pytest.importorskip("torch")
    n = 16
    buf = torch.zeros(n ** 3, dtype=torch.float32, device="cuda")
    ct = torch.zeros(n ** 3, dtype=torch.uint8, device="cuda")
    r = lib.fl_solve_pressure_noalloc(n, n, n, ct.data_ptr(), buf.data_ptr(), buf.data_ptr(), 1.0, 1.0, 1.0, 10, 0,
                                      0.0, FL_CG_F32, None, None)
    assert r == FL_INVALID_ARG
    assert b"overlap" in lib.fl_last_error(None)


def test_noalloc_rejects_grids_beyond_its_limit(lib):
    torch = pytest.importorskip("torch")
    n = 65  # 274,625 cells > FL_NOALLOC_MAX_CELLS = 262,144
    div = torch.zeros(n ** 3, dtype=torch.float32, device="cuda")
    pres = torch.zeros(n ** 3, dtype=torch.float32, device="cuda")
    ct = torch.zeros(n ** 3, dtype=torch.uint8, device="cuda")
    r = lib.fl_solve_pressure_noalloc(n, n, n, ct.data_ptr(), div.data_ptr(), pres.data_ptr(), 1.0, 1.0, 1.0, 10, 0,
                                      0.0, FL_CG_F32, None, None)
    assert r == FL_INVALID_ARG
    assert b"no-allocation limit" in lib.fl_last_error(None)
