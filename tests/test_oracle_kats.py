"""Pin the CPU oracle to the reference's own known-answer tests.

The reference (Rust) cannot be built here, so its test files are the golden
source: each test below restates one of them with the same inputs and the
same assertions, against the oracle's restatement of the function under test.
Paths are within the reference project (app/crates/fluid-lab/src/...).
"""
import numpy as np
import pytest

F = np.float32


def lcg_u32(state, count):
    """state = state*1664525 + 1013904223 (wrapping u32); yields the states."""
    out = np.empty(count, np.uint32)
    s = int(state)
    for i in range(count):
        s = (s * 1664525 + 1013904223) & 0xFFFFFFFF
        out[i] = s
    return out


def lcg01(state, count):
    """(st >> 8) as f32 / 2^24, lib.rs:1219-1222 and fluid.rs:1875-1878."""
    s = lcg_u32(state, count)
    return (s >> np.uint32(8)).astype(np.float32) / F(16777216.0)


def sample_positions(n, origin, h, dims):
    """lib.rs:1215-1231 sample_positions."""
    h = F(h)
    extent = [F(dims[a]) * h for a in range(3)]
    r = lcg01(0x9E3779B9, 3 * n).reshape(n, 3)
    o = [F(x) for x in origin]
    pos = np.empty((n, 3), np.float32)
    for a in range(3):
        pos[:, a] = o[a] + r[:, a] * extent[a]
    return pos


# ---------------------------------------------------------------- sort (lib.rs)

def test_exclusive_scan_matches_definition(oracle):  # lib.rs:1233-1239
    hist = np.array([3, 0, 5, 1, 0, 4], np.uint32)
    off = oracle.ref_exclusive_scan(hist)
    assert off.tolist() == [0, 3, 3, 8, 9, 9]
    assert off[5] + hist[5] == hist.sum()


def test_permutation_is_a_bijection(oracle):  # lib.rs:1241-1255
    dims, h, origin = (16, 8, 16), 0.1, (-0.8, -0.4, -0.8)
    pos = sample_positions(5000, origin, h, dims)
    perm, _ = oracle.ref_counting_sort(pos, origin, h, dims)
    assert perm.size == pos.shape[0]
    assert np.array_equal(np.sort(perm), np.arange(5000, dtype=np.uint32))


def test_each_bucket_shares_one_key_and_is_monotone(oracle):  # lib.rs:1257-1285
    dims, h, origin = (12, 6, 10), 0.1, (-0.6, -0.3, -0.5)
    pos = sample_positions(4000, origin, h, dims)
    perm, keys = oracle.ref_counting_sort(pos, origin, h, dims)
    sk = keys[perm]
    assert np.all(np.diff(sk.astype(np.int64)) >= 0)
    cells = dims[0] * dims[1] * dims[2]
    hist = np.bincount(keys, minlength=cells).astype(np.uint32)
    starts = oracle.ref_exclusive_scan(hist)
    for c in range(cells):
        s, e = int(starts[c]), int(starts[c] + hist[c])
        assert np.all(keys[perm[s:e]] == c)
    # stable: within a bucket, source indices increase
    for c in range(cells):
        s, e = int(starts[c]), int(starts[c] + hist[c])
        assert np.all(np.diff(perm[s:e].astype(np.int64)) > 0)


def test_clamps_out_of_bounds_positions_into_edge_cells(oracle):  # lib.rs:1287-1300
    dims, h, origin = (4, 4, 4), 1.0, (0.0, 0.0, 0.0)
    pos = np.array([[-100, -100, -100], [100, 100, 100]], np.float32)
    perm, keys = oracle.ref_counting_sort(pos, origin, h, dims)
    assert keys.max() < 64 and keys.min() == 0 and keys.max() == 63
    assert sorted(perm.tolist()) == [0, 1]


# ---------------------------------------------------------------- grid (sim/mod.rs)

def test_world_to_cell_roundtrips_centers_and_clamps_escapes(oracle):  # sim/mod.rs:246-260
    dims, h, origin = (8, 8, 8), 0.25, (-1.0, -1.0, -1.0)
    c = [origin[a] + (ijk + 0.5) * h for a, ijk in enumerate((3, 4, 5))]
    assert oracle.ref_world_to_cell(dims, h, origin, c) == (3, 4, 5)
    assert oracle.ref_world_to_cell(dims, h, origin, (-100, -100, -100)) == (0, 0, 0)
    assert oracle.ref_world_to_cell(dims, h, origin, (100, 100, 100)) == (7, 7, 7)


def test_world_to_cell_roundtrips_on_rectangular_tank(oracle):  # sim/mod.rs:305-330
    dims, h, origin = (5, 9, 7), F(0.3), (F(-0.75), F(1.35), F(-2.1))
    for k in range(dims[2]):
        for j in range(dims[1]):
            for i in range(dims[0]):
                c = [origin[a] + (F(ijk) + F(0.5)) * h for a, ijk in enumerate((i, j, k))]
                assert oracle.ref_world_to_cell(dims, h, origin, c) == (i, j, k)
    assert oracle.ref_world_to_cell(dims, h, origin, (-1e3, -1e3, -1e3)) == (0, 0, 0)
    assert oracle.ref_world_to_cell(dims, h, origin, (1e3, 1e3, 1e3)) == (4, 8, 6)


def test_boundary_cells_are_solid_interior_marked_by_occupancy(oracle):  # sim/mod.rs:263-276
    d = (6, 6, 6)
    idx = lambda i, j, k: i + 6 * (j + 6 * k)
    occ = np.zeros(216, np.uint8)
    occ[idx(2, 2, 2)] = 1
    ct = oracle.ref_classify(d, occ)
    assert ct[idx(0, 3, 3)] == 0 and ct[idx(5, 3, 3)] == 0 and ct[idx(3, 0, 3)] == 0
    assert ct[idx(2, 2, 2)] == 1
    assert ct[idx(3, 3, 3)] == 2


def test_particles_mark_their_containing_cells(oracle):  # sim/mod.rs:278-288
    d, h, o = (8, 8, 8), 1.0, (0.0, 0.0, 0.0)
    occ = np.zeros(512, np.uint8)
    for p in ([2.5, 3.5, 4.5], [5.5, 5.5, 5.5]):
        i, j, k = oracle.ref_world_to_cell(d, h, o, p)
        occ[i + 8 * (j + 8 * k)] = 1
    ct = oracle.ref_classify(d, occ)
    assert ct[2 + 8 * (3 + 8 * 4)] == 1 and ct[5 + 8 * (5 + 8 * 5)] == 1


def test_wall_aware_mac_gather_preserves_tangential_velocity_near_static_wall(oracle):  # sim/mod.rs:527-553
    d = (8, 8, 8)
    fin = oracle.ref_fill_wall_zeroed_faces(d, 1, 10.0)
    sav = oracle.ref_fill_wall_zeroed_faces(d, 1, 7.0)
    p = (1.05, 3.5, 3.5)
    old = oracle.ref_sample_mac_pair(d, 1.0, (0, 0, 0), 1, p, fin, sav, False)
    fixed = oracle.ref_sample_mac_pair(d, 1.0, (0, 0, 0), 1, p, fin, sav, True)
    assert abs(old[0] - 5.5) < 1e-6 and abs(old[1] - 3.85) < 1e-6
    assert abs(fixed[0] - 10.0) < 1e-6 and abs(fixed[1] - 7.0) < 1e-6


def test_wall_aware_mac_gather_preserves_away_from_ceiling_normal_velocity(oracle):  # sim/mod.rs:555-586
    d = (8, 8, 8)
    fin = oracle.ref_fill_wall_zeroed_faces(d, 1, -10.0)
    sav = oracle.ref_fill_wall_zeroed_faces(d, 1, -6.0)
    p = (3.5, 6.95, 3.5)
    old = oracle.ref_sample_mac_pair(d, 1.0, (0, 0, 0), 1, p, fin, sav, False)
    fixed = oracle.ref_sample_mac_pair(d, 1.0, (0, 0, 0), 1, p, fin, sav, True)
    assert abs(old[0] - -0.5) < 1e-5 and abs(old[1] - -0.3) < 1e-5
    assert abs(fixed[0] - -10.0) < 1e-6 and abs(fixed[1] - -6.0) < 1e-6


def test_all_64_tank_reproduces_the_original_unit_cube():  # sim/mod.rs:588-602
    n, H = 64, F(2.0) / F(64.0)
    assert abs(float(H * F(n)) - 2.0) < 1e-6
    assert abs(float(-F(n) * H / F(2.0)) - (-1.0)) < 1e-6


# ---------------------------------------------------------------- pressure (sim/pressure.rs)

def divergent_tank(oracle):
    """sim/pressure.rs:470-508: 16^3 tank, top interior layer air, LCG(12345) faces."""
    n = 16
    d = (n, n, n)
    idx = lambda i, j, k: i + n * (j + n * k)
    occ = np.zeros(n ** 3, np.uint8)
    for k in range(1, n - 1):
        for j in range(1, n - 1):
            for i in range(1, n - 1):
                if j != n - 2:
                    occ[idx(i, j, k)] = 1
    ct = oracle.ref_classify(d, occ)
    fu, fv, fw = (n + 1) * n * n, n * (n + 1) * n, n * n * (n + 1)
    r = lcg01(12345, fu + fv + fw) * F(2.0) - F(1.0)
    u, v, w = r[:fu].copy(), r[fu:fu + fv].copy(), r[fu + fv:].copy()
    zero_solid_faces(d, ct, u, v, w)
    div = oracle.ref_compute_divergence(d, 1.0, u, v, w, ct)
    return d, ct, u, v, w, div


def zero_solid_faces(d, ct, u, v, w):
    """sim/pressure.rs:570-609."""
    nx, ny, nz = d
    c3 = ct.reshape(nz, ny, nx)
    solid = c3 == 0
    U = u.reshape(nz, ny, nx + 1)
    lo = np.ones((nz, ny, nx + 1), bool)
    hi = np.ones((nz, ny, nx + 1), bool)
    lo[:, :, 1:] = solid
    hi[:, :, :nx] = solid
    U[lo | hi] = 0
    V = v.reshape(nz, ny + 1, nx)
    lo = np.ones((nz, ny + 1, nx), bool)
    hi = np.ones((nz, ny + 1, nx), bool)
    lo[:, 1:, :] = solid
    hi[:, :ny, :] = solid
    V[lo | hi] = 0
    W = w.reshape(nz + 1, ny, nx)
    lo = np.ones((nz + 1, ny, nx), bool)
    hi = np.ones((nz + 1, ny, nx), bool)
    lo[1:] = solid
    hi[:nz] = solid
    W[lo | hi] = 0


def test_jacobi_reduces_divergence_16cubed(oracle):  # sim/pressure.rs:513-567
    d, ct, u, v, w, div0 = divergent_tank(oracle)
    idx = lambda i, j, k: i + 16 * (j + 16 * k)
    assert ct[idx(8, 14, 8)] == 2 and ct[idx(8, 13, 8)] == 1
    l2_before = oracle.ref_l2_divergence(div0, ct)
    max_before = oracle.ref_max_abs_divergence(div0, ct)
    assert l2_before > 1.0
    p = oracle.ref_jacobi_solve(d, 1.0, 1.0, 1.0, ct, div0, 200)
    u1, v1, w1 = oracle.ref_subtract_gradient(d, 1.0, 1.0, 1.0, p, ct, u, v, w)
    div1 = oracle.ref_compute_divergence(d, 1.0, u1, v1, w1, ct)
    assert oracle.ref_l2_divergence(div1, ct) < 0.1 * l2_before
    assert oracle.ref_max_abs_divergence(div1, ct) < max_before


def _l2_after(oracle, d, ct, u, v, w, p):
    u1, v1, w1 = oracle.ref_subtract_gradient(d, 1.0, 1.0, 1.0, p, ct, u, v, w)
    return oracle.ref_l2_divergence(oracle.ref_compute_divergence(d, 1.0, u1, v1, w1, ct), ct)


def test_cg_beats_jacobi_16cubed(oracle):  # sim/pressure.rs:615-698
    d, ct, u, v, w, div0 = divergent_tank(oracle)
    l2_before = oracle.ref_l2_divergence(div0, ct)
    pj = oracle.ref_jacobi_solve(d, 1.0, 1.0, 1.0, ct, div0, 200)
    pc, k, _, _ = oracle.ref_cg_solve(d, 1.0, 1.0, 1.0, ct, div0, 40)
    l2_jac = _l2_after(oracle, d, ct, u, v, w, pj)
    l2_cg = _l2_after(oracle, d, ct, u, v, w, pc)
    assert l2_cg < 0.01 * l2_before
    assert l2_cg <= l2_jac


def test_rbgs_restatement_16cubed(oracle):
    """pressure.wgsl's red-black Gauss-Seidel (no reference test pins it):
    from zero, its first red phase is the first Jacobi sweep on the red cells
    (the same update, sim/pressure.rs:72-117, with every neighbour still 0);
    100 iterations remove more divergence than 200 Jacobi sweeps, as
    Gauss-Seidel should."""
    d, ct, u, v, w, div0 = divergent_tank(oracle)
    k, j, i = np.indices((16, 16, 16))
    red = (((i + j + k) & 1) == 0).ravel()
    g1 = oracle.ref_rbgs_solve(d, 1.0, 1.0, 1.0, ct, div0, 1)
    j1 = oracle.ref_jacobi_solve(d, 1.0, 1.0, 1.0, ct, div0, 1)
    assert np.array_equal(g1[red], j1[red])
    assert np.all(g1[ct != 1] == 0.0)
    l2_before = oracle.ref_l2_divergence(div0, ct)
    l2_gs = _l2_after(oracle, d, ct, u, v, w, oracle.ref_rbgs_solve(d, 1.0, 1.0, 1.0, ct, div0, 100))
    l2_jac = _l2_after(oracle, d, ct, u, v, w, oracle.ref_jacobi_solve(d, 1.0, 1.0, 1.0, ct, div0, 200))
    assert l2_gs < 0.1 * l2_before and l2_gs < l2_jac


def test_cg_zero_initial_guess_matches_fixed_iteration_output(oracle):  # sim/pressure.rs:700-721
    d, ct, u, v, w, div = divergent_tank(oracle)
    fixed, _, _, _ = oracle.ref_cg_solve(d, 1.0, 1.0, 1.0, ct, div, 40)
    zero = np.zeros(16 ** 3, np.float32)
    p0, k, rs0, rs1 = oracle.ref_cg_solve(d, 1.0, 1.0, 1.0, ct, div, 40, p_init=zero)
    assert k == 40
    assert np.array_equal(p0, fixed)
    assert rs0 > rs1


def test_cg_warm_initial_guess_reaches_lower_residual_with_fewer_iterations(oracle):  # sim/pressure.rs:723-763
    d, ct, u, v, w, div = divergent_tank(oracle)
    pz, kz, rz0, rz1 = oracle.ref_cg_solve(d, 1.0, 1.0, 1.0, ct, div, 12)
    pw, kw, rw0, rw1 = oracle.ref_cg_solve(d, 1.0, 1.0, 1.0, ct, div, 40, p_init=pz, tol=1.0)
    assert kw < kz
    assert rw1 <= rz1
    assert rw0 < rz0


def test_divergence_free_field_has_zero_divergence(oracle):  # sim/pressure.rs:765-783
    d = (8, 8, 8)
    occ = np.zeros(512, np.uint8)
    for k in range(1, 7):
        for j in range(1, 7):
            for i in range(1, 7):
                occ[i + 8 * (j + 8 * k)] = 1
    ct = oracle.ref_classify(d, occ)
    u = np.full(9 * 64, 3.0, np.float32)
    v = np.full(9 * 64, -2.0, np.float32)
    w = np.full(9 * 64, 1.5, np.float32)
    div = oracle.ref_compute_divergence(d, 0.5, u, v, w, ct)
    assert oracle.ref_max_abs_divergence(div, ct) < 1e-5


# ------------------------------------------- the step's (GPU-variant) CG against the same KATs

@pytest.mark.parametrize("precision", [0, 1])
def test_step_cg_meets_reference_cg_thresholds(oracle, precision):
    """The WGSL-variant CG the step runs (cg_*.wgsl; f32 tree dots or f64 dots)
    meets the reference CG's own acceptance bar on the 16^3 tank."""
    d, ct, u, v, w, div0 = divergent_tank(oracle)
    l2_before = oracle.ref_l2_divergence(div0, ct)
    pj = oracle.ref_jacobi_solve(d, 1.0, 1.0, 1.0, ct, div0, 200)
    p, st = oracle.solve_pressure(ct, div0, d, 1.0, 1.0, 1.0, 40, precision=precision)
    assert st["cg_iterations"] == 40
    l2 = _l2_after(oracle, d, ct, u, v, w, p)
    assert l2 < 0.01 * l2_before
    assert l2 <= _l2_after(oracle, d, ct, u, v, w, pj)


def test_step_cg_f64_dots_track_reference_cg(oracle):
    """With f64 inner products the step CG matches the reference CPU CG
    (f64 dots, f32 alpha/beta) to f32 rounding."""
    d, ct, u, v, w, div0 = divergent_tank(oracle)
    pr, _, _, _ = oracle.ref_cg_solve(d, 1.0, 1.0, 1.0, ct, div0, 40)
    p, _ = oracle.solve_pressure(ct, div0, d, 1.0, 1.0, 1.0, 40, precision=1)
    assert np.allclose(p, pr, rtol=1e-4, atol=1e-4 * np.abs(pr).max())
