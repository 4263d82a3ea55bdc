"""ctypes binding of the CPU oracle (oracle/fl_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, always as the checker of (or the baseline beside)
the CUDA path.  `OracleFluid` has the same methods as fluidgb.Fluid so parity
tests drive both identically.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import build_oracle  # noqa: E402

_fp = ctypes.POINTER(ctypes.c_float)
_u32 = ctypes.c_uint32
_u32p_t = ctypes.POINTER(ctypes.c_uint32)
_u8p_t = ctypes.POINTER(ctypes.c_uint8)
_lib = None


def _structs():
    # The parameter/stat/grid structs are the ABI's (include/fluidgb.h).
    pkg = os.path.join(os.path.dirname(HERE), "fluid-simulation_gb300")
    if pkg not in sys.path:
        sys.path.insert(0, pkg)
    from fluidgb._abi import FlGridView, FlParams, FlStats
    return FlParams, FlStats, FlGridView


FlParams, FlStats, FlGridView = _structs()


def load(build=True):
    global _lib
    if _lib is not None:
        return _lib
    path = build_oracle.build() if build else build_oracle.LIB
    lib = ctypes.CDLL(path)
    P = ctypes.POINTER(FlParams)
    for sfx in ("_f32", "_f64"):
        getattr(lib, "orc_create" + sfx).restype = ctypes.c_void_p
        getattr(lib, "orc_create" + sfx).argtypes = [P, _u32]
        getattr(lib, "orc_destroy" + sfx).argtypes = [ctypes.c_void_p]
        getattr(lib, "orc_destroy" + sfx).restype = None
        sigs = {
            "orc_set_params": [ctypes.c_void_p, P],
            "orc_set_particles": [ctypes.c_void_p, _fp, _u32],
            "orc_get_particles": [ctypes.c_void_p, _fp, _u32p_t],
            "orc_step": [ctypes.c_void_p, _u32],
            "orc_apply_impulse": [ctypes.c_void_p, _fp],
            "orc_reset": [ctypes.c_void_p],
            "orc_get_grid": [ctypes.c_void_p, ctypes.POINTER(FlGridView)],
            "orc_get_bins": [ctypes.c_void_p, _u32p_t, _u32p_t, _u32p_t],
            "orc_get_stats": [ctypes.c_void_p, ctypes.POINTER(FlStats)],
            "orc_get_divergence": [ctypes.c_void_p, _fp],
            "orc_set_gravity_d": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)],
            "orc_add_velocity_d": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_double],
            "orc_set_pressure": [ctypes.c_void_p, _fp],
            "orc_mean_position_d": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double)],
            "orc_add_position_d": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.c_double],
            "orc_solve_pressure": [_u32, _u32, _u32, _u8p_t, _fp, _fp, _fp, ctypes.c_float, ctypes.c_float,
                                   ctypes.c_float, _u32, _u32, ctypes.c_float, _u32, ctypes.POINTER(FlStats)],
        }
        for name, args in sigs.items():
            fn = getattr(lib, name + sfx)
            fn.argtypes = args
            fn.restype = ctypes.c_int
    lib.orc_set_exact_p2g.argtypes = [ctypes.c_int]
    lib.orc_set_threads.argtypes = [ctypes.c_int]
    lib.orc_get_threads.restype = ctypes.c_int
    lib.orc_ref_cell_key.restype = _u32
    lib.orc_ref_cell_key.argtypes = [_fp, _fp, ctypes.c_float, _u32p_t]
    lib.orc_ref_exclusive_scan.argtypes = [_u32p_t, _u32, _u32p_t]
    lib.orc_ref_counting_sort.argtypes = [_fp, _u32, _fp, ctypes.c_float, _u32p_t, _u32p_t, _u32p_t]
    lib.orc_ref_world_to_cell.restype = _u32
    lib.orc_ref_world_to_cell.argtypes = [_u32, _u32, _u32, ctypes.c_float, _fp, _fp, _u32p_t]
    lib.orc_ref_classify_cells.argtypes = [_u32, _u32, _u32, _u8p_t, _u8p_t]
    lib.orc_ref_sample_mac_pair.argtypes = [_u32, _u32, _u32, ctypes.c_float, _fp, ctypes.c_int, _fp, _fp, _fp,
                                            ctypes.c_int, _fp]
    lib.orc_ref_fill_wall_zeroed_faces.argtypes = [_u32, _u32, _u32, ctypes.c_int, ctypes.c_float, _fp]
    lib.orc_ref_compute_divergence.argtypes = [_u32, _u32, _u32, ctypes.c_float, _fp, _fp, _fp, _u8p_t, _fp]
    lib.orc_ref_jacobi_solve.argtypes = [_u32, _u32, _u32, ctypes.c_float, ctypes.c_float, ctypes.c_float, _u8p_t,
                                         _fp, _u32, _fp]
    lib.orc_ref_rbgs_solve.argtypes = [_u32, _u32, _u32, ctypes.c_float, ctypes.c_float, ctypes.c_float, _u8p_t,
                                       _fp, _u32, _fp]
    lib.orc_ref_apply_poisson.argtypes = [_u32, _u32, _u32, _u8p_t, _fp, _fp]
    lib.orc_ref_cg_solve.restype = _u32
    lib.orc_ref_cg_solve.argtypes = [_u32, _u32, _u32, ctypes.c_float, ctypes.c_float, ctypes.c_float, _u8p_t,
                                     _fp, _u32, _fp, ctypes.c_float, _fp, ctypes.POINTER(ctypes.c_double),
                                     ctypes.POINTER(ctypes.c_double)]
    lib.orc_ref_subtract_gradient.argtypes = [_u32, _u32, _u32, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                              _fp, _u8p_t, _fp, _fp, _fp]
    lib.orc_ref_l2_divergence.restype = ctypes.c_float
    lib.orc_ref_l2_divergence.argtypes = [_u32, _fp, _u8p_t]
    lib.orc_ref_max_abs_divergence.restype = ctypes.c_float
    lib.orc_ref_max_abs_divergence.argtypes = [_u32, _fp, _u8p_t]
    lib.orc_ref_generate_particles.restype = _u32
    lib.orc_ref_generate_particles.argtypes = [_fp, ctypes.c_float, _u32p_t, _fp, _u32, _u32, _fp, _u32]
    lib.orc_grid_slice.restype = None
    lib.orc_grid_slice.argtypes = [_u32, _u32, _u32, _u8p_t, _fp, _fp, _fp, _fp, _u32, _u32, _fp]
    _lib = lib
    return lib


def f32p(a):
    return a.ctypes.data_as(_fp)


def u32p(a):
    return a.ctypes.data_as(_u32p_t)


def u8p(a):
    return a.ctypes.data_as(_u8p_t)


def set_threads(n):
    load().orc_set_threads(int(n))


def set_exact_p2g(on):
    """_f64 oracle: unrounded P2G accumulation (smooth forward for finite differences)."""
    load().orc_set_exact_p2g(1 if on else 0)


class OracleFluid:
    """CPU oracle handle; precision 'f32' (reference arithmetic) or 'f64'."""

    def __init__(self, params, capacity, precision="f32"):
        self.lib = load()
        self.sfx = "_" + precision
        self.params = params.copy()
        self.h = getattr(self.lib, "orc_create" + self.sfx)(ctypes.byref(self.params), int(capacity))
        if not self.h:
            raise ValueError("oracle rejected the parameters")
        nx, ny, nz = params.grid
        self.dims = (nx, ny, nz)
        self.C = nx * ny * nz
        self.F = ((nx + 1) * ny * nz, nx * (ny + 1) * nz, nx * ny * (nz + 1))
        self.n = 0

    def _f(self, name):
        return getattr(self.lib, name + self.sfx)

    def close(self):
        if self.h:
            self._f("orc_destroy")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _c(self, st):
        if st != 0:
            raise RuntimeError("oracle call failed with status %d" % st)

    def set_params(self, params):
        self._c(self._f("orc_set_params")(self.h, ctypes.byref(params)))
        self.params = params.copy()

    def set_particles(self, parts):
        a = np.ascontiguousarray(parts, dtype=np.float32).reshape(-1, 8)
        self._c(self._f("orc_set_particles")(self.h, f32p(a), a.shape[0]))
        self.n = a.shape[0]

    def particle_count(self):
        return self.n

    def get_particles(self, with_ids=True):
        out = np.empty((self.n, 8), np.float32)
        ids = np.empty(self.n, np.uint32)
        self._c(self._f("orc_get_particles")(self.h, f32p(out), u32p(ids)))
        return (out, ids) if with_ids else out

    def step(self, substeps=1):
        self._c(self._f("orc_step")(self.h, substeps))

    def apply_impulse(self, dv):
        v = np.asarray(dv, np.float32)
        self._c(self._f("orc_apply_impulse")(self.h, f32p(v)))

    def reset(self):
        self._c(self._f("orc_reset")(self.h))

    def get_grid(self):
        fu, fv, fw = self.F
        g = {
            "u": np.empty(fu, np.float32), "v": np.empty(fv, np.float32), "w": np.empty(fw, np.float32),
            "u_saved": np.empty(fu, np.float32), "v_saved": np.empty(fv, np.float32),
            "w_saved": np.empty(fw, np.float32), "pressure": np.empty(self.C, np.float32),
            "cell_type": np.empty(self.C, np.uint8), "counts": np.empty(self.C, np.uint32),
            "offsets": np.empty(self.C, np.uint32),
        }
        v = FlGridView()
        for k in ("u", "v", "w", "u_saved", "v_saved", "w_saved", "pressure"):
            setattr(v, k, f32p(g[k]))
        v.cell_type = u8p(g["cell_type"])
        v.counts = u32p(g["counts"])
        v.offsets = u32p(g["offsets"])
        self._c(self._f("orc_get_grid")(self.h, ctypes.byref(v)))
        return g

    def set_gravity_d(self, g):
        a = np.ascontiguousarray(g, np.float64)
        self._c(self._f("orc_set_gravity_d")(self.h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))

    def add_velocity_d(self, dv, eps):
        a = np.ascontiguousarray(dv, np.float64).reshape(-1, 3)
        self._c(self._f("orc_add_velocity_d")(self.h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), eps))

    def add_position_d(self, dx, eps):
        a = np.ascontiguousarray(dx, np.float64).reshape(-1, 3)
        self._c(self._f("orc_add_position_d")(self.h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), eps))

    def set_pressure(self, p):
        """Warm-start pressure of the next step (precision-study hook)."""
        a = np.ascontiguousarray(p, np.float32)
        self._c(self._f("orc_set_pressure")(self.h, f32p(a)))

    def mean_position_d(self):
        out = np.zeros(3, np.float64)
        self._c(self._f("orc_mean_position_d")(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))))
        return out

    def get_divergence(self):
        out = np.empty(self.C, np.float32)
        self._c(self._f("orc_get_divergence")(self.h, f32p(out)))
        return out

    def get_bins(self):
        counts = np.empty(self.C, np.uint32)
        offsets = np.empty(self.C, np.uint32)
        perm = np.empty(self.n, np.uint32)
        self._c(self._f("orc_get_bins")(self.h, u32p(counts), u32p(offsets), u32p(perm)))
        return counts, offsets, perm

    def stats(self):
        s = FlStats()
        self._c(self._f("orc_get_stats")(self.h, ctypes.byref(s)))
        return s.as_dict()


def solve_pressure(cell_type, div, dims, h, rho, dt, max_iters, warm_start=False, pressure_in=None, tolerance=0.0,
                   precision=0, variant="f32"):
    lib = load()
    nx, ny, nz = dims
    ct = np.ascontiguousarray(cell_type, np.uint8)
    dv = np.ascontiguousarray(div, np.float32)
    pin = np.ascontiguousarray(pressure_in if pressure_in is not None else np.zeros_like(dv), np.float32)
    pout = np.empty_like(dv)
    st = FlStats()
    fn = getattr(lib, "orc_solve_pressure_" + variant)
    r = fn(nx, ny, nz, u8p(ct), f32p(dv), f32p(pin), f32p(pout), h, rho, dt, max_iters, 1 if warm_start else 0,
           tolerance, precision, ctypes.byref(st))
    if r != 0:
        raise RuntimeError("oracle solve failed %d" % r)
    return pout, st.as_dict()


# ---- restatements of the reference's Rust CPU functions ----

def ref_exclusive_scan(hist):
    lib = load()
    h = np.ascontiguousarray(hist, np.uint32)
    out = np.empty_like(h)
    lib.orc_ref_exclusive_scan(u32p(h), h.size, u32p(out))
    return out


def ref_counting_sort(pos3, origin, h, dims):
    lib = load()
    p = np.ascontiguousarray(pos3, np.float32).reshape(-1, 3)
    o = np.asarray(origin, np.float32)
    d = np.asarray(dims, np.uint32)
    perm = np.empty(p.shape[0], np.uint32)
    keys = np.empty(p.shape[0], np.uint32)
    lib.orc_ref_counting_sort(f32p(p), p.shape[0], f32p(o), h, u32p(d), u32p(perm), u32p(keys))
    return perm, keys


def ref_world_to_cell(dims, h, origin, p):
    lib = load()
    o = np.asarray(origin, np.float32)
    pp = np.asarray(p, np.float32)
    ijk = np.zeros(3, np.uint32)
    lib.orc_ref_world_to_cell(dims[0], dims[1], dims[2], h, f32p(o), f32p(pp), u32p(ijk))
    return tuple(int(x) for x in ijk)


def ref_classify(dims, occupied):
    lib = load()
    occ = np.ascontiguousarray(occupied, np.uint8)
    out = np.empty_like(occ)
    lib.orc_ref_classify_cells(dims[0], dims[1], dims[2], u8p(occ), u8p(out))
    return out


def ref_fill_wall_zeroed_faces(dims, axis, value):
    lib = load()
    nx, ny, nz = dims
    cnt = [(nx + 1) * ny * nz, nx * (ny + 1) * nz, nx * ny * (nz + 1)][axis]
    out = np.empty(cnt, np.float32)
    lib.orc_ref_fill_wall_zeroed_faces(nx, ny, nz, axis, value, f32p(out))
    return out


def ref_sample_mac_pair(dims, h, origin, axis, p, final_vel, saved_vel, wall_aware):
    lib = load()
    o = np.asarray(origin, np.float32)
    pp = np.asarray(p, np.float32)
    out = np.zeros(2, np.float32)
    fv = np.ascontiguousarray(final_vel, np.float32)
    sv = np.ascontiguousarray(saved_vel, np.float32)
    lib.orc_ref_sample_mac_pair(dims[0], dims[1], dims[2], h, f32p(o), axis, f32p(pp), f32p(fv), f32p(sv),
                                1 if wall_aware else 0, f32p(out))
    return float(out[0]), float(out[1])


def ref_compute_divergence(dims, h, u, v, w, ct):
    lib = load()
    out = np.empty(dims[0] * dims[1] * dims[2], np.float32)
    lib.orc_ref_compute_divergence(dims[0], dims[1], dims[2], h, f32p(np.ascontiguousarray(u, np.float32)),
                                   f32p(np.ascontiguousarray(v, np.float32)),
                                   f32p(np.ascontiguousarray(w, np.float32)), u8p(np.ascontiguousarray(ct, np.uint8)),
                                   f32p(out))
    return out


def ref_jacobi_solve(dims, h, rho, dt, ct, div, iters):
    lib = load()
    out = np.empty(dims[0] * dims[1] * dims[2], np.float32)
    lib.orc_ref_jacobi_solve(dims[0], dims[1], dims[2], h, rho, dt, u8p(np.ascontiguousarray(ct, np.uint8)),
                             f32p(np.ascontiguousarray(div, np.float32)), iters, f32p(out))
    return out


def ref_rbgs_solve(dims, h, rho, dt, ct, div, iters):
    lib = load()
    out = np.empty(dims[0] * dims[1] * dims[2], np.float32)
    lib.orc_ref_rbgs_solve(dims[0], dims[1], dims[2], h, rho, dt, u8p(np.ascontiguousarray(ct, np.uint8)),
                           f32p(np.ascontiguousarray(div, np.float32)), iters, f32p(out))
    return out


def ref_cg_solve(dims, h, rho, dt, ct, div, iters, p_init=None, tol=None):
    lib = load()
    out = np.empty(dims[0] * dims[1] * dims[2], np.float32)
    rs0 = ctypes.c_double()
    rs1 = ctypes.c_double()
    pi = None if p_init is None else np.ascontiguousarray(p_init, np.float32)
    k = lib.orc_ref_cg_solve(dims[0], dims[1], dims[2], h, rho, dt, u8p(np.ascontiguousarray(ct, np.uint8)),
                             f32p(np.ascontiguousarray(div, np.float32)), iters, None if pi is None else f32p(pi),
                             -1.0 if tol is None else tol, f32p(out), ctypes.byref(rs0), ctypes.byref(rs1))
    return out, int(k), rs0.value, rs1.value


def ref_subtract_gradient(dims, h, rho, dt, p, ct, u, v, w):
    lib = load()
    u = np.array(u, np.float32)
    v = np.array(v, np.float32)
    w = np.array(w, np.float32)
    lib.orc_ref_subtract_gradient(dims[0], dims[1], dims[2], h, rho, dt, f32p(np.ascontiguousarray(p, np.float32)),
                                  u8p(np.ascontiguousarray(ct, np.uint8)), f32p(u), f32p(v), f32p(w))
    return u, v, w


def ref_l2_divergence(div, ct):
    lib = load()
    return float(lib.orc_ref_l2_divergence(div.size, f32p(np.ascontiguousarray(div, np.float32)),
                                           u8p(np.ascontiguousarray(ct, np.uint8))))


def ref_max_abs_divergence(div, ct):
    lib = load()
    return float(lib.orc_ref_max_abs_divergence(div.size, f32p(np.ascontiguousarray(div, np.float32)),
                                                u8p(np.ascontiguousarray(ct, np.uint8))))


def grid_slice(dims, ct, p, u, v, w, mode, k=None):
    """The slice renderer's per-cell colours (orc_grid_slice): (ny, nx, 4) float32."""
    lib = load()
    nx, ny, nz = dims
    k = nz // 2 if k is None else k
    out = np.empty((ny, nx, 4), np.float32)
    arrs = [np.ascontiguousarray(a, np.float32) for a in (p, u, v, w)]
    ctc = np.ascontiguousarray(ct, np.uint8)
    lib.orc_grid_slice(nx, ny, nz, u8p(ctc), *[f32p(a) for a in arrs], mode, k, f32p(out))
    return out


def ref_generate_particles(params, blocks, particle_count, capacity):
    """generate_particles (fluid.rs:1838-1913), sequential: (n, particles[:n])."""
    lib = load()
    origin = np.array(params.origin[:3], np.float32)
    gdim = np.array(params.gdim[:3], np.uint32)
    b = np.array([[*blk.min, *blk.max] for blk in blocks], np.float32).reshape(-1)
    out = np.zeros((capacity, 8), np.float32)
    n = lib.orc_ref_generate_particles(f32p(origin), params.geom[0], u32p(gdim), f32p(b), len(blocks),
                                       particle_count, f32p(out), capacity)
    return n, out[:min(n, capacity)]

