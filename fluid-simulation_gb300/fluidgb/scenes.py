"""Seeded synthetic scenes for the step's benchmark and parity workloads.

All scenes live in a unit box: an n^3 grid of cell size h = 1/n with origin 0;
the outer cell layer is solid (classify.wgsl:35-40).  A fluid cell is an
interior cell whose centre lies in the scene's liquid region; it receives 8
particles, one per 2x2x2 sub-cell, uniformly jittered inside its sub-cell, from
a splitmix64 stream (seed stated per run, default 0x5EED).  Positions and
velocities are f32, w = 0, in the reference's 32-byte particle layout
(gpu/fluid.rs:116-123).  The particle counts are those of the stated geometry.
"""
import ctypes

import numpy as np

from ._abi import FL_CG_F32, FlParams

DEFAULT_SEED = 0x5EED
_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed, count):
    """`count` successive outputs of splitmix64 seeded with `seed`."""
    with np.errstate(over="ignore"):
        k = np.arange(1, count + 1, dtype=np.uint64)
        z = np.uint64(seed) + k * _GOLDEN
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        z = z ^ (z >> np.uint64(31))
    return z


def uniform01(seed, count):
    return (splitmix64(seed, count) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def params_for(n, flip=0.95, iters=200, tol=1e-5, precision=FL_CG_F32, dt=1.0 / 120.0, gravity=-9.81,
               stiffness=0.45, warm_start=True, advect_order=1, ny=None, nz=None, rest=8.0):
    """Settings for an n^3 (or n x ny x nz) unit-cell-size-1/n box with origin 0.

    Registry defaults (settings/mod.rs:498-724) except the values a workload
    states.  Built in Python with the same fields as fl_params_default.
    """
    ny = n if ny is None else ny
    nz = n if nz is None else nz
    h = np.float32(1.0) / np.float32(n)
    p = FlParams()
    p.dims[:] = [n, 0, iters, 1 if warm_start else 0]
    p.geom[:] = [float(h), float(np.float32(1.0) / h), float(np.float32(dt)), 65536.0]
    p.phys[:] = [gravity, 1000.0, flip, 0.0]
    p.origin[:] = [0.0, 0.0, 0.0, 0.0]
    p.grav[:] = [0.0, gravity, 0.0, 0.0]
    p.spc[:] = [rest, stiffness, 0.5, 0.0]
    p.cls[:] = [1.0, 0.0, 2.0, 0.0]
    p.gdim[:] = [n, ny, nz, 0]
    p.pressure_tolerance = tol
    p.cg_precision = precision
    p.advect_order = advect_order
    p.sort_period = 1
    return p


def fluid_cells(n, region, ny=None, nz=None):
    """Indices (k, j, i order) of interior cells whose centre satisfies region(x, y, z)."""
    ny = n if ny is None else ny
    nz = n if nz is None else nz
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(n), indexing="ij")
    x, y, z = (i + 0.5) / n, (j + 0.5) / ny, (k + 0.5) / nz
    interior = (i > 0) & (j > 0) & (k > 0) & (i < n - 1) & (j < ny - 1) & (k < nz - 1)
    m = interior & region(x, y, z)
    return i[m], j[m], k[m]


def seed_particles(n, region, seed=DEFAULT_SEED, vel_sigma=0.0, ny=None, nz=None):
    """8 jittered particles per fluid cell; returns an (N, 8) float32 array."""
    ny = n if ny is None else ny
    nz = n if nz is None else nz
    ci, cj, ck = fluid_cells(n, region, ny, nz)
    ncell = ci.size
    sub = np.array([[sx, sy, sz] for sz in (0, 1) for sy in (0, 1) for sx in (0, 1)], dtype=np.float64)
    N = ncell * 8
    u = uniform01(seed, 3 * N).reshape(N, 3)
    cells = np.stack([ci, cj, ck], axis=1).astype(np.float64)
    cells = np.repeat(cells, 8, axis=0)
    subs = np.tile(sub, (ncell, 1))
    h = np.array([1.0 / n, 1.0 / ny, 1.0 / nz])
    pos = (cells + (subs + u) * 0.5) * h
    out = np.zeros((N, 8), np.float32)
    out[:, 0:3] = pos.astype(np.float32)
    if vel_sigma > 0.0:
        g = uniform01(seed ^ 0xA5A5A5A5, 6 * N).reshape(N, 6)
        r = np.sqrt(-2.0 * np.log(np.maximum(g[:, 0:3], 1e-300)))
        out[:, 4:7] = (vel_sigma * r * np.cos(2.0 * np.pi * g[:, 3:6])).astype(np.float32)
    return out


def box(xmax=1.0, ymax=1.0, zmax=1.0):
    return lambda x, y, z: (x < xmax) & (y < ymax) & (z < zmax)


def sphere_pool(center=(0.5, 0.75, 0.5), radius=0.12, depth=0.3):
    cx, cy, cz = center
    return lambda x, y, z: (y < depth) | ((x - cx) ** 2 + (y - cy) ** 2 + (z - cz) ** 2 < radius ** 2)


# Workloads of the benchmark configurations (name -> settings).
WORKLOADS = {
    # 32^3 dam break, fluid x<0.4, y<0.6; CG <= 40 iterations at 1e-4; 120 steps.
    "dam32": dict(n=32, region=box(0.4, 0.6), iters=40, tol=1e-4, steps=120),
    # 128^3, fluid x<0.5, y<0.5 (full depth); CG <= 200 at 1e-5; 300 steps.
    "dam128": dict(n=128, region=box(0.5, 0.5), iters=200, tol=1e-5, steps=300),
    # 128^3, fluid x<0.5, y<0.5, z<0.5: the ~2M-particle headline.
    "dam128_2m": dict(n=128, region=box(0.5, 0.5, 0.5), iters=200, tol=1e-5, steps=300),
    # 128^3 sphere r=0.12 at (0.5,0.75,0.5) above a pool of depth 0.3; 200 steps.
    "sphere_pool128": dict(n=128, region=sphere_pool(), iters=200, tol=1e-5, steps=200),
    # 64^3 block x<0.5, y<0.4; initial velocity N(0, 0.1^2); 60 steps.
    "block64": dict(n=64, region=box(0.5, 0.4), iters=200, tol=1e-5, steps=60, vel_sigma=0.1),
    # 256^3 block x<0.4, y<0.35; 120 steps.
    "block256": dict(n=256, region=box(0.4, 0.35), iters=200, tol=1e-5, steps=120),
}


def workload(name, seed=DEFAULT_SEED, precision=FL_CG_F32, **overrides):
    """(params, particles, spec) of a named workload."""
    spec = dict(WORKLOADS[name])
    spec.update(overrides)
    p = params_for(spec["n"], iters=spec["iters"], tol=spec["tol"], precision=precision,
                   flip=spec.get("flip", 0.95), stiffness=spec.get("stiffness", 0.45))
    parts = seed_particles(spec["n"], spec["region"], seed=seed, vel_sigma=spec.get("vel_sigma", 0.0))
    return p, parts, spec


def params_bytes(p):
    return ctypes.string_at(ctypes.byref(p), ctypes.sizeof(p))
