"""ctypes binding of libfluidgb (include/fluidgb.h).

`Fluid` mirrors the reference's `GpuFluid` life cycle (gpu/fluid.rs): create
from a settings block, upload particles, step, live-update settings, impulse,
reset, and read back particles / grid / bins / stats.  Every call goes through
the C ABI; there is no Python or CPU fallback — if the shared library is
missing the import of the binding fails loudly.
"""
import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libfluidgb.so")

FL_OK, FL_INVALID_ARG, FL_OOM, FL_CUDA_ERROR, FL_NOT_CONVERGED, FL_TIMEOUT, FL_NO_DEVICE, FL_INTERNAL = range(8)
FL_CELL_SOLID, FL_CELL_LIQUID, FL_CELL_AIR = 0, 1, 2
FL_CG_F32, FL_CG_F64, FL_CG_F64_IEEE = 0, 1, 2
FL_SOLVER_CG, FL_SOLVER_MGPCG = 0, 1
FL_SOLVER_FOLLOW = 0xFFFFFFFF
FL_RELAX_JACOBI, FL_RELAX_RBGS = 0, 1

c_u32 = ctypes.c_uint32
c_f32 = ctypes.c_float


class FlParams(ctypes.Structure):
    """The reference's 128-byte Params (gpu/fluid.rs:25-39) + 32-byte extension."""
    _fields_ = [
        ("dims", c_u32 * 4), ("geom", c_f32 * 4), ("phys", c_f32 * 4), ("origin", c_f32 * 4),
        ("grav", c_f32 * 4), ("spc", c_f32 * 4), ("cls", c_f32 * 4), ("gdim", c_u32 * 4),
        ("pressure_tolerance", c_f32), ("cg_precision", c_u32), ("advect_order", c_u32),
        ("sort_period", c_u32), ("pressure_solver", c_u32), ("reserved", c_u32 * 3),
    ]

    def copy(self):
        p = FlParams()
        ctypes.memmove(ctypes.byref(p), ctypes.byref(self), ctypes.sizeof(FlParams))
        return p

    @property
    def grid(self):
        return tuple(int(x) for x in self.gdim[:3])


class FlStats(ctypes.Structure):
    _fields_ = [
        ("liquid_cells", c_u32), ("cg_iterations", c_u32), ("stray_particles", c_u32),
        ("device_status", c_u32), ("substeps", ctypes.c_uint64), ("rs_initial", ctypes.c_double),
        ("rs_final", ctypes.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_fp = ctypes.POINTER(ctypes.c_float)


class FlGridView(ctypes.Structure):
    _fields_ = [
        ("u", _fp), ("v", _fp), ("w", _fp), ("u_saved", _fp), ("v_saved", _fp), ("w_saved", _fp),
        ("pressure", _fp), ("cell_type", ctypes.POINTER(ctypes.c_uint8)),
        ("counts", ctypes.POINTER(c_u32)), ("offsets", ctypes.POINTER(c_u32)),
    ]


assert ctypes.sizeof(FlParams) == 160

FL_POLICY_FIXED_DROP_CAP, FL_POLICY_EXPLICIT_EXPORT = 0, 1
FL_PRESET_FALLING_BLOB, FL_PRESET_DAM_BREAK, FL_PRESET_DOUBLE_SPLASH = 0, 1, 2


class FlBlock(ctypes.Structure):
    """A liquid block in normalized tank space (scene/mod.rs LiquidBlock)."""
    _fields_ = [("min", c_f32 * 3), ("max", c_f32 * 3)]


class FlTimestepStats(ctypes.Structure):
    """TimestepFrameStats (timestep.rs:21-50)."""
    _fields_ = [
        ("substeps", c_u32), ("natural_substeps", c_u32), ("max_substeps", c_u32), ("substep_cap_hit", c_u32),
        ("fixed_dt", c_f32), ("accumulated_before", c_f32), ("accumulated_after", c_f32),
        ("dropped_this_frame", c_f32), ("sim_advanced", c_f32), ("wall_dt", c_f32), ("sim_time_scale", c_f32),
        ("real_time_factor", c_f32), ("policy", c_u32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}

# name -> (restype, argtypes)
SIGNATURES = {
    "fl_abi_version": (c_u32, []),
    "fl_status_string": (ctypes.c_char_p, [ctypes.c_int]),
    "fl_params_default": (ctypes.c_int, [ctypes.POINTER(FlParams), c_u32, c_u32, c_u32, c_f32, _fp]),
    "fl_create": (ctypes.c_int, [ctypes.POINTER(FlParams), c_u32, ctypes.POINTER(ctypes.c_void_p)]),
    "fl_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "fl_set_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(FlParams)]),
    "fl_get_params": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(FlParams)]),
    "fl_set_particles": (ctypes.c_int, [ctypes.c_void_p, _fp, c_u32]),
    "fl_get_particles": (ctypes.c_int, [ctypes.c_void_p, _fp, ctypes.POINTER(c_u32)]),
    "fl_particle_count": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(c_u32)]),
    "fl_step": (ctypes.c_int, [ctypes.c_void_p, c_u32]),
    "fl_step_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, c_u32]),
    "fl_step_host": (ctypes.c_int, [ctypes.c_void_p, _fp, _fp, c_u32, c_u32]),
    "fl_sync": (ctypes.c_int, [ctypes.c_void_p]),
    "fl_set_wait_timeout": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
    "fl_set_profiling": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "fl_get_stage_times": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_uint64)]),
    "fl_reset_stage_times": (ctypes.c_int, [ctypes.c_void_p]),
    "fl_section_name": (ctypes.c_char_p, [ctypes.c_uint32]),
    "fl_section_stage": (ctypes.c_int, [ctypes.c_uint32]),
    "fl_get_coarse_times": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_uint64)]),
    "fl_set_stream": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fl_apply_impulse": (ctypes.c_int, [ctypes.c_void_p, _fp]),
    "fl_reset": (ctypes.c_int, [ctypes.c_void_p]),
    "fl_get_grid": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(FlGridView)]),
    "fl_get_divergence": (ctypes.c_int, [ctypes.c_void_p, _fp]),
    "fl_get_bins": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(c_u32), ctypes.POINTER(c_u32),
                                   ctypes.POINTER(c_u32)]),
    "fl_get_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(FlStats)]),
    "fl_save_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)]),
    "fl_load_state": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "fl_solve_pressure": (ctypes.c_int, [c_u32, c_u32, c_u32, ctypes.POINTER(ctypes.c_uint8), _fp, _fp, _fp,
                                         c_f32, c_f32, c_f32, c_u32, c_u32, c_f32, c_u32,
                                         ctypes.POINTER(FlStats)]),
    "fl_relax_pressure": (ctypes.c_int, [c_u32, c_u32, c_u32, ctypes.POINTER(ctypes.c_uint8), _fp, c_f32, c_f32,
                                         c_f32, c_u32, c_u32, _fp]),
    "fl_solve_pressure_noalloc": (ctypes.c_int, [c_u32, c_u32, c_u32, ctypes.c_void_p, ctypes.c_void_p,
                                                 ctypes.c_void_p, c_f32, c_f32, c_f32, c_u32, c_u32, c_f32, c_u32,
                                                 ctypes.c_void_p, ctypes.POINTER(FlStats)]),
    "fl_get_particles_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fl_save_state_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)]),
    "fl_load_state_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]),
    "fl_set_particles_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, c_u32]),
    "fl_tape_create": (ctypes.c_int, [ctypes.c_void_p, c_u32, ctypes.POINTER(ctypes.c_void_p)]),
    "fl_tape_free": (ctypes.c_int, [ctypes.c_void_p]),
    "fl_tape_clear": (ctypes.c_int, [ctypes.c_void_p]),
    "fl_tape_set_adjoint_warm_start": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int]),
    "fl_tape_set_adjoint_solver": (ctypes.c_int, [ctypes.c_void_p, c_u32]),
    "fl_tape_count": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(c_u32)]),
    "fl_tape_last_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fl_step_record": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fl_copy_pressure_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fl_step_replay": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fl_step_adjoint": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, _fp, c_u32,
                                       c_f32]),
    "fl_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "fl_scene_blocks": (ctypes.c_int, [c_u32, c_f32, c_f32, ctypes.POINTER(FlBlock), ctypes.POINTER(c_u32)]),
    "fl_scene_seeded_fraction": (ctypes.c_int, [ctypes.POINTER(FlBlock), c_u32, ctypes.POINTER(c_f32)]),
    "fl_scene_particle_count": (ctypes.c_int, [c_u32, c_u32, c_u32, ctypes.POINTER(FlBlock), c_u32, c_f32, c_u32,
                                               ctypes.POINTER(c_u32)]),
    "fl_seed_count": (ctypes.c_int, [ctypes.POINTER(FlParams), ctypes.POINTER(FlBlock), c_u32, c_u32,
                                     ctypes.POINTER(c_u32)]),
    "fl_seed_particles": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(FlBlock), c_u32, c_u32,
                                         ctypes.POINTER(c_u32)]),
    "fl_grid_slice": (ctypes.c_int, [ctypes.c_void_p, c_u32, c_u32, _fp]),
    "fl_grid_slice_device": (ctypes.c_int, [ctypes.c_void_p, c_u32, c_u32, ctypes.c_void_p]),
    "fl_timestep_create": (ctypes.c_int, [c_f32, c_u32, ctypes.POINTER(ctypes.c_void_p)]),
    "fl_timestep_free": (ctypes.c_int, [ctypes.c_void_p]),
    "fl_timestep_steps_for_frame": (ctypes.c_int, [ctypes.c_void_p, c_f32, c_f32, ctypes.POINTER(c_u32)]),
    "fl_timestep_record_manual_steps": (ctypes.c_int, [ctypes.c_void_p, c_f32, c_u32, c_f32]),
    "fl_timestep_record_export_steps": (ctypes.c_int, [ctypes.c_void_p, c_f32, c_u32]),
    "fl_timestep_record_idle_frame": (ctypes.c_int, [ctypes.c_void_p, c_f32, c_f32]),
    "fl_timestep_reset": (ctypes.c_int, [ctypes.c_void_p]),
    "fl_timestep_last_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(FlTimestepStats)]),
    "fl_timestep_total_dropped": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(c_f32)]),
    "fl_timestep_accumulator": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(c_f32)]),
    "fl_timestep_policy_label": (ctypes.c_char_p, [c_u32]),
    "fl_frame": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, c_f32, ctypes.c_int,
                                ctypes.POINTER(c_u32), ctypes.POINTER(c_u32)]),
    "fl_export_frame": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, c_u32, ctypes.c_double]),
}

# FL_STAGE_* order (include/fluidgb.h)
STAGES = ("sort", "classify", "scatter", "prep", "cg", "gradient", "g2p")


def section_table(lib=None):
    """[(reference section name, stage that times it)] for the reference's
    detailed sections and CG categories (fl_section_name / fl_section_stage)."""
    lib = lib or load_library()
    out = []
    i = 0
    while True:
        name = lib.fl_section_name(i)
        if name is None:
            return out
        out.append((name.decode(), STAGES[lib.fl_section_stage(i)]))
        i += 1

_lib = None


def load_library(path=None):
    """Load libfluidgb.so (built by fluidgb.build).  Raises if it is missing."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError("libfluidgb.so not found at %s: run fluidgb.build.build() (needs nvcc)" % p)
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.fl_abi_version() != 1:
        raise RuntimeError("libfluidgb ABI version mismatch")
    if path is None:
        _lib = lib
    return lib


class FluidError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (_STATUS.get(status, status), msg))
        self.status = status


_STATUS = {0: "FL_OK", 1: "FL_INVALID_ARG", 2: "FL_OOM", 3: "FL_CUDA_ERROR", 4: "FL_NOT_CONVERGED",
           5: "FL_TIMEOUT", 6: "FL_NO_DEVICE", 7: "FL_INTERNAL"}


def _check(lib, status, handle=None):
    if status != FL_OK:
        msg = lib.fl_last_error(handle)
        raise FluidError(status, msg.decode() if msg else "")


def _f32p(a):
    return a.ctypes.data_as(_fp)


def _u32p(a):
    return a.ctypes.data_as(ctypes.POINTER(c_u32))


def default_params(nx, ny, nz, h, origin=None):
    """Registry defaults (settings/mod.rs) for an nx*ny*nz tank of cell size h."""
    lib = load_library()
    p = FlParams()
    o = None if origin is None else (ctypes.c_float * 3)(*origin)
    _check(lib, lib.fl_params_default(ctypes.byref(p), nx, ny, nz, h, o))
    return p


def face_counts(nx, ny, nz):
    return ((nx + 1) * ny * nz, nx * (ny + 1) * nz, nx * ny * (nz + 1))


class Fluid:
    """One simulation handle on the current CUDA device."""

    def __init__(self, params, capacity, lib=None):
        self.lib = lib or load_library()
        self.params = params.copy()
        self.capacity = int(capacity)
        h = ctypes.c_void_p()
        _check(self.lib, self.lib.fl_create(ctypes.byref(self.params), self.capacity, ctypes.byref(h)))
        self.h = h
        nx, ny, nz = params.grid
        self.dims = (nx, ny, nz)
        self.C = nx * ny * nz
        self.F = face_counts(nx, ny, nz)

    def close(self):
        if self.h:
            self.lib.fl_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _c(self, status):
        _check(self.lib, status, self.h)

    def set_params(self, params):
        self._c(self.lib.fl_set_params(self.h, ctypes.byref(params)))
        self.params = params.copy()

    def set_particles(self, parts):
        a = np.ascontiguousarray(parts, dtype=np.float32).reshape(-1, 8)
        self._c(self.lib.fl_set_particles(self.h, _f32p(a), a.shape[0]))

    def particle_count(self):
        n = c_u32()
        self._c(self.lib.fl_particle_count(self.h, ctypes.byref(n)))
        return n.value

    def get_particles(self, with_ids=True):
        n = self.particle_count()
        out = np.empty((n, 8), np.float32)
        ids = np.empty(n, np.uint32) if with_ids else None
        self._c(self.lib.fl_get_particles(self.h, _f32p(out), _u32p(ids) if with_ids else None))
        return (out, ids) if with_ids else out

    def step(self, substeps=1):
        self._c(self.lib.fl_step(self.h, substeps))

    def step_device(self, ptr, n):
        self._c(self.lib.fl_step_device(self.h, ctypes.c_void_p(ptr), n))

    def step_host(self, parts_in, parts_out, substeps=1):
        """Host buffers in/out (fl_step_host); arrays are (n, 8) float32."""
        n = parts_in.shape[0]
        self._c(self.lib.fl_step_host(self.h, _f32p(parts_in), _f32p(parts_out), n, substeps))

    def set_profiling(self, on=True):
        self._c(self.lib.fl_set_profiling(self.h, 1 if on else 0))

    def stage_times(self):
        """({stage: ms total}, substeps timed)."""
        ms = (ctypes.c_double * len(STAGES))()
        n = ctypes.c_uint64()
        self._c(self.lib.fl_get_stage_times(self.h, ms, ctypes.byref(n)))
        return {k: ms[i] for i, k in enumerate(STAGES)}, n.value

    def reset_stage_times(self):
        self._c(self.lib.fl_reset_stage_times(self.h))

    def coarse_times(self):
        """({'prep', 'pressure', 'finish': ms total}, substeps timed): the
        reference's coarse rollup of the stage totals (fl_get_coarse_times)."""
        ms = (ctypes.c_double * 3)()
        n = ctypes.c_uint64()
        self._c(self.lib.fl_get_coarse_times(self.h, ms, ctypes.byref(n)))
        return {"prep": ms[0], "pressure": ms[1], "finish": ms[2]}, n.value

    def sync(self):
        self._c(self.lib.fl_sync(self.h))

    def set_stream(self, stream_ptr):
        self._c(self.lib.fl_set_stream(self.h, ctypes.c_void_p(stream_ptr)))

    def set_wait_timeout(self, ns):
        """Limit of the device-side waits in ns (0 = the default 2 s)."""
        self._c(self.lib.fl_set_wait_timeout(self.h, int(ns)))

    def apply_impulse(self, dv):
        v = (ctypes.c_float * 3)(*dv)
        self._c(self.lib.fl_apply_impulse(self.h, v))

    def reset(self):
        self._c(self.lib.fl_reset(self.h))

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
            setattr(v, k, _f32p(g[k]))
        v.cell_type = g["cell_type"].ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
        v.counts = _u32p(g["counts"])
        v.offsets = _u32p(g["offsets"])
        self._c(self.lib.fl_get_grid(self.h, ctypes.byref(v)))
        return g

    def get_divergence(self):
        """nx*ny*nz float32: the last substep's divergence (0 off liquid cells)."""
        out = np.empty(self.C, np.float32)
        self._c(self.lib.fl_get_divergence(self.h, _f32p(out)))
        return out

    def seed(self, blocks, particle_count):
        """generate_particles on the device into this handle; returns the count."""
        arr = (FlBlock * len(blocks))(*blocks)
        n = c_u32()
        self._c(self.lib.fl_seed_particles(self.h, arr, len(blocks), particle_count, ctypes.byref(n)))
        return n.value

    def grid_slice(self, mode=0, k=None):
        """(ny, nx, 4) float32 image {r, g, b, visible} of the XY slice at k
        (default nz/2), the reference slice renderer's per-cell colours."""
        nx, ny, _ = self.params.grid
        out = np.empty((ny, nx, 4), np.float32)
        self._c(self.lib.fl_grid_slice(self.h, mode, 0xFFFFFFFF if k is None else k, _f32p(out)))
        return out

    def get_bins(self):
        n = self.particle_count()
        counts = np.empty(self.C, np.uint32)
        offsets = np.empty(self.C, np.uint32)
        perm = np.empty(n, np.uint32)
        self._c(self.lib.fl_get_bins(self.h, _u32p(counts), _u32p(offsets), _u32p(perm)))
        return counts, offsets, perm

    def stats(self):
        s = FlStats()
        self._c(self.lib.fl_get_stats(self.h, ctypes.byref(s)))
        return s.as_dict()

    def get_particles_device(self, ptr, ids_ptr=None):
        self._c(self.lib.fl_get_particles_device(self.h, ctypes.c_void_p(ptr), ctypes.c_void_p(ids_ptr)))

    def set_particles_device(self, ptr, n):
        self._c(self.lib.fl_set_particles_device(self.h, ctypes.c_void_p(ptr), n))

    def tape(self, max_steps):
        return Tape(self, max_steps)

    def save_state(self):
        size = ctypes.c_size_t(0)
        self._c(self.lib.fl_save_state(self.h, None, ctypes.byref(size)))
        buf = ctypes.create_string_buffer(size.value)
        self._c(self.lib.fl_save_state(self.h, buf, ctypes.byref(size)))
        return bytes(buf.raw[: size.value])

    def load_state(self, blob):
        buf = ctypes.create_string_buffer(blob, len(blob))
        self._c(self.lib.fl_load_state(self.h, buf, len(blob)))

    def state_size(self):
        size = ctypes.c_size_t(0)
        self._c(self.lib.fl_save_state(self.h, None, ctypes.byref(size)))
        return size.value

    def copy_pressure_device(self, ptr):
        """Pressure of the last substep (nx*ny*nz float32) into device memory at ptr."""
        self._c(self.lib.fl_copy_pressure_device(self.h, ctypes.c_void_p(ptr)))

    def step_replay(self, pressure_ptr, tape=None):
        """One substep with the pressure solve replaced by the field at pressure_ptr
        (recorded on `tape` when given)."""
        self._c(self.lib.fl_step_replay(self.h, ctypes.c_void_p(pressure_ptr), tape.t if tape is not None else None))

    def save_state_device(self, ptr, size):
        sz = ctypes.c_size_t(size)
        self._c(self.lib.fl_save_state_device(self.h, ctypes.c_void_p(ptr), ctypes.byref(sz)))
        return sz.value

    def load_state_device(self, ptr, size):
        self._c(self.lib.fl_load_state_device(self.h, ctypes.c_void_p(ptr), size))


def solve_pressure(cell_type, div, dims, h, rho, dt, max_iters, warm_start=False, pressure_in=None,
                   tolerance=0.0, precision=FL_CG_F32, lib=None):
    """GPU CG on host arrays (fl_solve_pressure).  Returns (pressure, stats)."""
    lib = lib or load_library()
    nx, ny, nz = dims
    ct = np.ascontiguousarray(cell_type, dtype=np.uint8)
    dv = np.ascontiguousarray(div, dtype=np.float32)
    pin = np.ascontiguousarray(pressure_in if pressure_in is not None else np.zeros_like(dv), dtype=np.float32)
    pout = np.empty_like(dv)
    st = FlStats()
    _check(lib, lib.fl_solve_pressure(nx, ny, nz, ct.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), _f32p(dv),
                                      _f32p(pin), _f32p(pout), h, rho, dt, max_iters, 1 if warm_start else 0,
                                      tolerance, precision, ctypes.byref(st)))
    return pout, st.as_dict()


def relax_pressure(cell_type, div, dims, h, rho, dt, method, iters, lib=None):
    """The reference's Jacobi (FL_RELAX_JACOBI) or red-black Gauss-Seidel
    (FL_RELAX_RBGS) solve from zero on the GPU (fl_relax_pressure)."""
    lib = lib or load_library()
    nx, ny, nz = dims
    ct = np.ascontiguousarray(cell_type, dtype=np.uint8)
    dv = np.ascontiguousarray(div, dtype=np.float32)
    pout = np.empty_like(dv)
    _check(lib, lib.fl_relax_pressure(nx, ny, nz, ct.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), _f32p(dv), h,
                                      rho, dt, method, iters, _f32p(pout)))
    return pout


class Tape:
    """Recorded substeps of a handle, for the adjoint (fl_tape_*)."""

    def __init__(self, fluid, max_steps):
        self.fluid = fluid
        t = ctypes.c_void_p()
        fluid._c(fluid.lib.fl_tape_create(fluid.h, max_steps, ctypes.byref(t)))
        self.t = t

    def close(self):
        if self.t:
            self.fluid.lib.fl_tape_free(self.t)
            self.t = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def clear(self):
        self.fluid._c(self.fluid.lib.fl_tape_clear(self.t))

    def set_adjoint_warm_start(self, enable):
        """Start each adjoint solve from the previous one's lambda (resets lambda to zero)."""
        self.fluid._c(self.fluid.lib.fl_tape_set_adjoint_warm_start(self.t, 1 if enable else 0))

    def set_adjoint_solver(self, solver):
        """FL_SOLVER_CG, FL_SOLVER_MGPCG or FL_SOLVER_FOLLOW (the handle's)."""
        self.fluid._c(self.fluid.lib.fl_tape_set_adjoint_solver(self.t, solver))

    def __len__(self):
        n = c_u32()
        self.fluid._c(self.fluid.lib.fl_tape_count(self.t, ctypes.byref(n)))
        return n.value

    def record(self):
        self.fluid._c(self.fluid.lib.fl_step_record(self.fluid.h, self.t))

    def last_stats(self):
        st = FlStats()
        self.fluid._c(self.fluid.lib.fl_tape_last_stats(self.t, ctypes.byref(st)))
        return st.as_dict()

    def adjoint(self, g_out_ptr, g_in_ptr, cg_iters=1000, cg_tol=1e-6):
        """Pop one step: dL/dout (device ptr) -> dL/din (device ptr); returns dL/dgravity."""
        gg = (ctypes.c_float * 3)(0.0, 0.0, 0.0)
        self.fluid._c(self.fluid.lib.fl_step_adjoint(self.fluid.h, self.t, ctypes.c_void_p(g_out_ptr),
                                                     ctypes.c_void_p(g_in_ptr), gg, cg_iters, cg_tol))
        return [gg[0], gg[1], gg[2]]


class Timestep:
    """Fixed-timestep accumulator (the reference's TimestepController,
    timestep.rs:64-233) through the C ABI; host only."""

    def __init__(self, fixed_dt, max_substeps, lib=None):
        self.lib = lib or load_library()
        h = ctypes.c_void_p()
        _check(self.lib, self.lib.fl_timestep_create(c_f32(fixed_dt), max_substeps, ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.fl_timestep_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def steps_for_frame(self, render_dt_s, sim_time_scale=1.0):
        n = c_u32()
        _check(self.lib, self.lib.fl_timestep_steps_for_frame(self.h, render_dt_s, sim_time_scale, ctypes.byref(n)))
        return n.value

    def record_manual_steps(self, render_dt_s, substeps, sim_time_scale=1.0):
        _check(self.lib, self.lib.fl_timestep_record_manual_steps(self.h, render_dt_s, substeps, sim_time_scale))

    def record_export_steps(self, sim_dt_s, substeps):
        _check(self.lib, self.lib.fl_timestep_record_export_steps(self.h, sim_dt_s, substeps))

    def record_idle_frame(self, render_dt_s, sim_time_scale=1.0):
        _check(self.lib, self.lib.fl_timestep_record_idle_frame(self.h, render_dt_s, sim_time_scale))

    def reset(self):
        _check(self.lib, self.lib.fl_timestep_reset(self.h))

    def last_stats(self):
        s = FlTimestepStats()
        _check(self.lib, self.lib.fl_timestep_last_stats(self.h, ctypes.byref(s)))
        d = s.as_dict()
        d["policy_label"] = self.lib.fl_timestep_policy_label(s.policy).decode()
        return d

    def total_dropped(self):
        v = c_f32()
        _check(self.lib, self.lib.fl_timestep_total_dropped(self.h, ctypes.byref(v)))
        return v.value

    def accumulator(self):
        v = c_f32()
        _check(self.lib, self.lib.fl_timestep_accumulator(self.h, ctypes.byref(v)))
        return v.value

    def frame(self, fluid, render_dt_ms, sim_speed=1.0, paused=False, pending_steps=0):
        """FluidApp::frame on `fluid`: returns (substeps run, pending steps left)."""
        pend = c_u32(pending_steps)
        n = c_u32()
        _check(self.lib, self.lib.fl_frame(fluid.h, self.h, render_dt_ms, sim_speed, 1 if paused else 0,
                                           ctypes.byref(pend), ctypes.byref(n)))
        return n.value, pend.value

    def export_frame(self, fluid, substeps, sim_dt_s):
        _check(self.lib, self.lib.fl_export_frame(fluid.h, self.h, substeps, sim_dt_s))


def scene_blocks(preset, drop_height=0.72, fill_level=0.2, lib=None):
    """preset_blocks (scene/mod.rs:204-236) as a list of FlBlock."""
    lib = lib or load_library()
    out = (FlBlock * 2)()
    n = c_u32()
    _check(lib, lib.fl_scene_blocks(preset, drop_height, fill_level, out, ctypes.byref(n)))
    return [out[i] for i in range(n.value)]


def seeded_fraction(blocks, lib=None):
    lib = lib or load_library()
    arr = (FlBlock * max(len(blocks), 1))(*blocks)
    v = c_f32()
    _check(lib, lib.fl_scene_seeded_fraction(arr, len(blocks), ctypes.byref(v)))
    return v.value


def scene_particle_count(dims, blocks, density, override_count=0, lib=None):
    lib = lib or load_library()
    arr = (FlBlock * max(len(blocks), 1))(*blocks)
    v = c_u32()
    _check(lib, lib.fl_scene_particle_count(dims[0], dims[1], dims[2], arr, len(blocks), density, override_count,
                                            ctypes.byref(v)))
    return v.value


def seed_count(params, blocks, particle_count, lib=None):
    lib = lib or load_library()
    arr = (FlBlock * len(blocks))(*blocks)
    v = c_u32()
    _check(lib, lib.fl_seed_count(ctypes.byref(params), arr, len(blocks), particle_count, ctypes.byref(v)))
    return v.value

