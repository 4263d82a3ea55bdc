// fl_mg.cu — multigrid-preconditioned CG, an opt-in pressure solver
// (fl_params.pressure_solver = FL_SOLVER_MGPCG).
//
// The reference solves the pressure system with plain CG (cg_*.wgsl) and
// ships a red-black Gauss-Seidel smoother (pressure.wgsl:26-61, built but not
// dispatched: gpu/fluid.rs:564-627) and a CPU Jacobi solver
// (sim/pressure.rs:68-136).  Here red-black Gauss-Seidel is the smoother of a
// multigrid V-cycle that preconditions CG.  Operator, right-hand side, warm
// start, iteration cap and stopping test (r.r <= tol^2 * r0.r0, tested after
// each update like cg_beta.wgsl:25-30) are the CG's; the iterates are not, so
// the pressure matches the CG's to the tolerance, not bit for bit.
//
// Hierarchy: level l+1 aggregates 2x2x2 cells of level l (the last aggregate
// of an odd extent has fewer).  Prolongation P is piecewise-constant
// injection, restriction is P^T (sum over the children) and the coarse
// operator is the exact Galerkin product P^T A P, which stays a 7-point
// stencil with integer weights: the weight between two aggregates is the
// number of liquid-liquid fine faces across their interface, the diagonal is
// the children's diagonals minus twice their internal couplings.  Stored as
// float4 {diag, weight to +x, +y, +z}; a cell is an unknown when diag > 0.
// V-cycle: one red-then-black sweep down, black-then-red up, symmetric
// Gauss-Seidel sweeps on the coarsest level (<= 64 cells, in shared memory of
// block 0), all from zero: a symmetric positive-definite preconditioner.
//
// One cooperative persistent kernel per solve, one 1024-thread block per SM.
// Level-0 cells are owned per block through the CG's plan of active chunks
// (k_cg_plan); coarser levels are grid-strided.  A pass boundary is a counter
// barrier (bounded wait, as in k_cg); a dot product is a per-block
// float-float partial, a barrier and a fixed-order sum, so results repeat
// bit for bit.  Each smoothing pass computes what it needs of the other
// colour on the fly (the red values of the pre-smoothing sweep are b/D; the
// corrected red values of the post-smoothing sweep are x + e(parent)), so a
// level costs four passes: pre-smooth, residual + restriction, correction +
// black sweep, red sweep.
#include "fl_device.cuh"

// Vectors written during the solve (r, z, d, the coarse b and x) are read
// through plain pointers, never const __restrict__: a read-only (non-coherent)
// load could return a value cached before another block's write.  The
// stencils and masks are fixed for the whole kernel.

namespace fl {

namespace {

constexpr int MG_THREADS = 1024;
constexpr int MG_PART = 1024;       // block partial slots per exchange parity
constexpr int MG_KCH = 2048;        // level-0 plan entries cached in shared memory
constexpr int MG_COARSE_SWEEPS = 8;  // symmetric Gauss-Seidel sweeps on the coarsest level

struct MgShared {
    uint32_t chunk[MG_KCH];
    float2 red[MG_THREADS / 32];
    float2 res;
    int ok;
    float4 cst[MG_COARSE_CELLS];
    float cb[MG_COARSE_CELLS], cx[MG_COARSE_CELLS];
};

__device__ __forceinline__ bool red_cell(uint32_t c, uint32_t nx, uint32_t ny) {
    const uint32_t i = c % nx, j = (c / nx) % ny, k = c / (nx * ny);
    return ((i + j + k) & 1u) == 0u;
}

// Level-0 operator from the CG's stencil mask: bit 0 liquid, bit s+1 the
// neighbour s (-x,+x,-y,+y,-z,+z) is liquid, bits 7-9 the non-solid count.
__device__ __forceinline__ float diag0(uint32_t info) { return (float)(info >> 7); }

// Sum over the liquid neighbours of v(nb).
template <class F>
__device__ __forceinline__ float nbsum0(uint32_t info, uint32_t c, uint32_t nx, uint32_t nxy, F v) {
    float s = 0.0f;
    if (info & (1u << 1)) s += v(c - 1);
    if (info & (1u << 2)) s += v(c + 1);
    if (info & (1u << 3)) s += v(c - nx);
    if (info & (1u << 4)) s += v(c + nx);
    if (info & (1u << 5)) s += v(c - nxy);
    if (info & (1u << 6)) s += v(c + nxy);
    return s;
}

// Coarse level: sum over the neighbours of w(nb) * v(nb) (a neighbour with a
// nonzero weight is an unknown).
template <class F>
__device__ __forceinline__ float nbsum(const float4* st, float4 sc, uint32_t c, uint32_t i, uint32_t j, uint32_t k,
                                       const MgLevel& lv, F v) {
    const uint32_t nxy = lv.nx * lv.ny;
    float s = 0.0f;
    if (sc.y != 0.0f) s += sc.y * v(c + 1);
    if (sc.z != 0.0f) s += sc.z * v(c + lv.nx);
    if (sc.w != 0.0f) s += sc.w * v(c + nxy);
    if (i > 0) {
        const float w = st[c - 1].y;
        if (w != 0.0f) s += w * v(c - 1);
    }
    if (j > 0) {
        const float w = st[c - lv.nx].z;
        if (w != 0.0f) s += w * v(c - lv.nx);
    }
    if (k > 0) {
        const float w = st[c - nxy].w;
        if (w != 0.0f) s += w * v(c - nxy);
    }
    return s;
}

__device__ __forceinline__ uint32_t parent_of(uint32_t c, uint32_t nx, uint32_t ny, const MgLevel& up) {
    const uint32_t i = c % nx, j = (c / nx) % ny, k = c / (nx * ny);
    return (i >> 1) + up.nx * ((j >> 1) + up.ny * (k >> 1));
}

struct Ctx {
    MgShared& sh;
    const DevBufs& b;
    const MgBufs& m;
    uint32_t nown;      // level-0 plan entries of this block
    uint32_t e0;        // first one (when not cached)
    uint32_t epoch;     // barrier target
    uint32_t parity;    // exchange slot parity
};

__device__ bool mg_barrier(Ctx& x) {
    __syncthreads();
    if (threadIdx.x == 0) {
        x.epoch += gridDim.x;
        __threadfence();
        red_release_add(x.m.bar, 1u);
        bool ok = true;
        const uint64_t t0 = global_ns();
        uint32_t spins = 0;
        while (ld_acquire(x.m.bar) < x.epoch) {
            if ((++spins & 63u) == 0u) {
                if (*(volatile uint32_t*)&x.b.st->status != 0u) {
                    ok = false;
                    break;
                }
                if (global_ns() - t0 > 2000000000ull) {
                    atomicCAS(&x.b.st->status, 0u, 5u /* FL_TIMEOUT */);
                    ok = false;
                    break;
                }
            }
        }
        x.sh.ok = ok;
    } else {
        x.epoch += gridDim.x;
    }
    __syncthreads();
    return x.sh.ok != 0;
}

// Sum of v over all threads of all blocks, in a fixed order; false on abort.
__device__ bool mg_allreduce(Ctx& x, Df v, Df& out) {
    v = warp_sum_df(v);
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (lane == 0) x.sh.red[warp] = make_float2(v.hi, v.lo);
    __syncthreads();
    float2* part = x.m.part + (size_t)x.parity * MG_PART;
    x.parity ^= 1u;
    if (threadIdx.x == 0) {
        Df s = {0.0f, 0.0f};
        for (uint32_t w = 0; w < MG_THREADS / 32; w++) s = df_add(s, Df{x.sh.red[w].x, x.sh.red[w].y});
        part[blockIdx.x] = make_float2(s.hi, s.lo);
    }
    if (!mg_barrier(x)) return false;
    if (warp == 0) {
        Df s = {0.0f, 0.0f};
        for (uint32_t g = lane; g < gridDim.x; g += 32) {
            const float2 p = part[g];
            s = df_add(s, Df{p.x, p.y});
        }
        s = warp_allsum_df(s);
        if (lane == 0) x.sh.res = make_float2(s.hi, s.lo);
    }
    __syncthreads();
    out = Df{x.sh.res.x, x.sh.res.y};
    return true;
}

// Calls f(c, info) for every liquid cell of this block's level-0 plan entries.
template <class F>
__device__ __forceinline__ void for_own(const Ctx& x, F f) {
    const DevParams& P = *x.b.prm;
    const uint32_t C = P.C, lo = threadIdx.x & (CHUNK - 1);
    for (uint32_t e = threadIdx.x / CHUNK; e < x.nown; e += MG_THREADS / CHUNK) {
        const uint32_t chunk = x.nown <= (uint32_t)MG_KCH ? x.sh.chunk[e] : x.b.cg_chunk[x.e0 + e];
        const uint32_t c = chunk * CHUNK + lo;
        if (c >= C) continue;
        const uint32_t info = x.b.cinfo[c];
        if (info >= (1u << 7)) f(c, info);  // liquid with a nonzero diagonal
    }
}

// Calls f(c, i, j, k, st) for every unknown of coarse level lv, grid-strided.
template <class F>
__device__ __forceinline__ void for_level(const MgLevel& lv, F f) {
    for (uint32_t c = blockIdx.x * MG_THREADS + threadIdx.x; c < lv.C; c += gridDim.x * MG_THREADS) {
        const float4 sc = lv.st[c];
        if (sc.x > 0.0f) {
            const uint32_t i = c % lv.nx, j = (c / lv.nx) % lv.ny, k = c / (lv.nx * lv.ny);
            f(c, i, j, k, sc);
        }
    }
}

// ---- level 0 passes (b = r, x = z) ----

__device__ void pre0(const Ctx& x) {
    const DevParams& P = *x.b.prm;
    const uint32_t nx = P.nx, ny = P.ny, nxy = nx * ny;
    const float* r = x.b.r;
    const uint16_t* __restrict__ ci = x.b.cinfo;
    float* z = x.m.lv[0].x;
    for_own(x, [&](uint32_t c, uint32_t info) {
        const float D = diag0(info);
        float v = r[c];
        if (!red_cell(c, nx, ny))
            v += nbsum0(info, c, nx, nxy, [&](uint32_t n) { return r[n] / diag0(ci[n]); });
        z[c] = v / D;
    });
}

// b1 = P^T (r - A z)
__device__ void restrict0(const Ctx& x) {
    const DevParams& P = *x.b.prm;
    const uint32_t nx = P.nx, ny = P.ny, nz = P.nz, nxy = nx * ny;
    const float* r = x.b.r;
    const uint16_t* __restrict__ ci = x.b.cinfo;
    const float* z = x.m.lv[0].x;
    const MgLevel& up = x.m.lv[1];
    for_level(up, [&](uint32_t I, uint32_t ii, uint32_t jj, uint32_t kk, float4) {
        float s = 0.0f;
        for (uint32_t d = 0; d < 8; d++) {
            const uint32_t i = 2 * ii + (d & 1), j = 2 * jj + ((d >> 1) & 1), k = 2 * kk + (d >> 2);
            if (i >= nx || j >= ny || k >= nz) continue;
            const uint32_t c = i + nx * (j + ny * k);
            const uint32_t info = ci[c];
            if (info < (1u << 7)) continue;
            const float az = diag0(info) * z[c] - nbsum0(info, c, nx, nxy, [&](uint32_t n) { return z[n]; });
            s += r[c] - az;
        }
        up.b[I] = s;
    });
}

// correction + black sweep: z_black = (r + sum (z_red + e(parent))) / D
__device__ void post0_black(const Ctx& x) {
    const DevParams& P = *x.b.prm;
    const uint32_t nx = P.nx, ny = P.ny, nxy = nx * ny;
    const float* r = x.b.r;
    float* z = x.m.lv[0].x;
    const MgLevel& up = x.m.lv[1];
    const float* e = up.x;
    for_own(x, [&](uint32_t c, uint32_t info) {
        if (red_cell(c, nx, ny)) return;
        const float s = nbsum0(info, c, nx, nxy, [&](uint32_t n) { return z[n] + e[parent_of(n, nx, ny, up)]; });
        z[c] = (r[c] + s) / diag0(info);
    });
}

// red sweep; returns this thread's share of r.z
__device__ Df post0_red(const Ctx& x) {
    const DevParams& P = *x.b.prm;
    const uint32_t nx = P.nx, ny = P.ny, nxy = nx * ny;
    const float* r = x.b.r;
    float* z = x.m.lv[0].x;
    Df acc = {0.0f, 0.0f};
    for_own(x, [&](uint32_t c, uint32_t info) {
        float zc;
        const float rc = r[c];
        if (red_cell(c, nx, ny)) {
            zc = (rc + nbsum0(info, c, nx, nxy, [&](uint32_t n) { return z[n]; })) / diag0(info);
            z[c] = zc;
        } else {
            zc = z[c];
        }
        acc = df_add(acc, df_prod(rc, zc));
    });
    return acc;
}

// ---- coarse level passes ----

__device__ void pre_l(const MgLevel& lv) {
    const float4* __restrict__ st = lv.st;
    for_level(lv, [&](uint32_t c, uint32_t i, uint32_t j, uint32_t k, float4 sc) {
        float v = lv.b[c];
        if (((i + j + k) & 1u) != 0u)
            v += nbsum(st, sc, c, i, j, k, lv, [&](uint32_t n) { return lv.b[n] / st[n].x; });
        lv.x[c] = v / sc.x;
    });
}

__device__ void restrict_l(const MgLevel& lv, const MgLevel& up) {
    const float4* __restrict__ st = lv.st;
    for_level(up, [&](uint32_t I, uint32_t ii, uint32_t jj, uint32_t kk, float4) {
        float s = 0.0f;
        for (uint32_t d = 0; d < 8; d++) {
            const uint32_t i = 2 * ii + (d & 1), j = 2 * jj + ((d >> 1) & 1), k = 2 * kk + (d >> 2);
            if (i >= lv.nx || j >= lv.ny || k >= lv.nz) continue;
            const uint32_t c = i + lv.nx * (j + lv.ny * k);
            const float4 sc = st[c];
            if (!(sc.x > 0.0f)) continue;
            const float ax = sc.x * lv.x[c] - nbsum(st, sc, c, i, j, k, lv, [&](uint32_t n) { return lv.x[n]; });
            s += lv.b[c] - ax;
        }
        up.b[I] = s;
    });
}

__device__ void post_black_l(const MgLevel& lv, const MgLevel& up) {
    const float4* __restrict__ st = lv.st;
    for_level(lv, [&](uint32_t c, uint32_t i, uint32_t j, uint32_t k, float4 sc) {
        if (((i + j + k) & 1u) == 0u) return;
        const float s = nbsum(st, sc, c, i, j, k, lv,
                              [&](uint32_t n) { return lv.x[n] + up.x[parent_of(n, lv.nx, lv.ny, up)]; });
        lv.x[c] = (lv.b[c] + s) / sc.x;
    });
}

__device__ void post_red_l(const MgLevel& lv) {
    const float4* __restrict__ st = lv.st;
    for_level(lv, [&](uint32_t c, uint32_t i, uint32_t j, uint32_t k, float4 sc) {
        if (((i + j + k) & 1u) != 0u) return;
        lv.x[c] = (lv.b[c] + nbsum(st, sc, c, i, j, k, lv, [&](uint32_t n) { return lv.x[n]; })) / sc.x;
    });
}

// Coarsest level: symmetric Gauss-Seidel sweeps from zero in shared memory
// (block 0 only; the other blocks go on to the next barrier).
__device__ void coarse_solve(MgShared& sh, const MgLevel& lv) {
    const uint32_t t = threadIdx.x, C = lv.C, nx = lv.nx, ny = lv.ny, nxy = nx * ny;
    if (t < C) {
        sh.cst[t] = lv.st[t];
        sh.cb[t] = lv.b[t];
        sh.cx[t] = 0.0f;
    }
    __syncthreads();
    uint32_t i = 0, j = 0, k = 0, col = 0;
    float4 sc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    if (t < C) {
        i = t % nx; j = (t / nx) % ny; k = t / nxy;
        col = (i + j + k) & 1u;
        sc = sh.cst[t];
    }
    for (int h = 0; h < 4 * MG_COARSE_SWEEPS; h++) {
        // forward sweeps red, black; backward sweeps black, red
        const uint32_t want = h < 2 * MG_COARSE_SWEEPS ? (uint32_t)(h & 1) : (uint32_t)((h & 1) ^ 1);
        if (t < C && sc.x > 0.0f && col == want) {
            float s = 0.0f;
            if (sc.y != 0.0f) s += sc.y * sh.cx[t + 1];
            if (sc.z != 0.0f) s += sc.z * sh.cx[t + nx];
            if (sc.w != 0.0f) s += sc.w * sh.cx[t + nxy];
            if (i > 0 && sh.cst[t - 1].y != 0.0f) s += sh.cst[t - 1].y * sh.cx[t - 1];
            if (j > 0 && sh.cst[t - nx].z != 0.0f) s += sh.cst[t - nx].z * sh.cx[t - nx];
            if (k > 0 && sh.cst[t - nxy].w != 0.0f) s += sh.cst[t - nxy].w * sh.cx[t - nxy];
            sh.cx[t] = (sh.cb[t] + s) / sc.x;
        }
        __syncthreads();
    }
    if (t < C) lv.x[t] = sh.cx[t];
}

// z = M^-1 r, then the r.z all-reduce (whose barrier ends the cycle).
__device__ bool vcycle(Ctx& x, Df& rz) {
    const MgBufs& m = x.m;
    const uint32_t L = m.L;
    pre0(x);
    if (!mg_barrier(x)) return false;
    restrict0(x);
    if (!mg_barrier(x)) return false;
    for (uint32_t l = 1; l + 1 < L; l++) {
        pre_l(m.lv[l]);
        if (!mg_barrier(x)) return false;
        restrict_l(m.lv[l], m.lv[l + 1]);
        if (!mg_barrier(x)) return false;
    }
    if (blockIdx.x == 0) coarse_solve(x.sh, m.lv[L - 1]);
    if (!mg_barrier(x)) return false;
    for (uint32_t l = L - 2; l >= 1; l--) {
        post_black_l(m.lv[l], m.lv[l + 1]);
        if (!mg_barrier(x)) return false;
        post_red_l(m.lv[l]);
        if (!mg_barrier(x)) return false;
    }
    post0_black(x);
    if (!mg_barrier(x)) return false;
    return mg_allreduce(x, post0_red(x), rz);
}

__global__ void __launch_bounds__(MG_THREADS, 1) k_mgpcg(DevBufs b, MgBufs m) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    MgShared& sh = *reinterpret_cast<MgShared*>(smem_raw);
    const DevParams& P = *b.prm;
    const uint32_t G = gridDim.x, tid = threadIdx.x;
    const uint32_t* start = b.cg_off + CHUNK + 3;
    const uint32_t e0 = start[blockIdx.x], e1 = start[blockIdx.x + 1];
    Ctx x{sh, b, m, e1 - e0, e0, 0u, 0u};
    if (x.nown <= (uint32_t)MG_KCH)
        for (uint32_t e = tid; e < x.nown; e += MG_THREADS) sh.chunk[e] = b.cg_chunk[e0 + e];
    __syncthreads();
    (void)G;
    const uint32_t nx = P.nx, nxy = P.nx * P.ny;
    const uint32_t iters = P.iters;
    const bool stop_on = P.tol_sq > 0.0f;
    float* p = b.p;
    float* r = b.r;
    float* q = b.q;
    const float* z = m.lv[0].x;
    DevStats* st = b.st;

    // r0.r0 (grid_prep left r = rhs - A p0)
    Df acc = {0.0f, 0.0f};
    for_own(x, [&](uint32_t c, uint32_t) {
        const float rc = r[c];
        acc = df_add(acc, df_prod(rc, rc));
    });
    Df rs0;
    if (!mg_allreduce(x, acc, rs0)) return;
    const double thr = (double)P.tol_sq_d * df_to_double(rs0);
    Df thr_d;
    thr_d.hi = (float)thr;
    thr_d.lo = (float)(thr - (double)thr_d.hi);
    Df rz, rs = rs0;
    if (!vcycle(x, rz)) return;
    float beta = 0.0f;
    uint32_t k = 0;
    for (uint32_t it = 0; it < iters; it++) {
        float* d_cur = (it & 1u) ? b.dB : b.dA;
        const float* d_prev = (it & 1u) ? b.dA : b.dB;
        const bool first = it == 0;
        // direction d = z + beta d_prev and q = A d (neighbours' d on the fly)
        acc = Df{0.0f, 0.0f};
        for_own(x, [&](uint32_t c, uint32_t info) {
            auto dv = [&](uint32_t n) { return first ? z[n] : z[n] + beta * d_prev[n]; };
            const float dc = dv(c);
            const float qc = diag0(info) * dc - nbsum0(info, c, nx, nxy, dv);
            d_cur[c] = dc;
            q[c] = qc;
            acc = df_add(acc, df_prod(dc, qc));
        });
        Df dq;
        if (!mg_allreduce(x, acc, dq)) return;
        // cg_alpha.wgsl:16-22: alpha = 0 when |d.q| <= 1e-30
        const float alpha = fabsf(dq.hi) > 1e-30f ? df_div(rz, dq) : 0.0f;
        acc = Df{0.0f, 0.0f};
        for_own(x, [&](uint32_t c, uint32_t) {
            p[c] += alpha * d_cur[c];
            const float rc = r[c] - alpha * q[c];
            r[c] = rc;
            acc = df_add(acc, df_prod(rc, rc));
        });
        if (!mg_allreduce(x, acc, rs)) return;
        k = it + 1;
        if (stop_on && df_le(rs, thr_d)) break;
        if (it + 1 == iters) break;
        Df rz_new;
        if (!vcycle(x, rz_new)) return;
        beta = rz.hi > 1e-30f ? df_div(rz_new, rz) : 0.0f;  // cg_beta.wgsl:16-23
        rz = rz_new;
    }
    if (blockIdx.x == 0 && tid == 0) {
        st->cg_iters = k;
        st->rs_init = df_to_double(rs0);
        st->rs_final = df_to_double(rs);
    }
}

// Level 1 from the grid's stencil masks.
__global__ void __launch_bounds__(256) k_mg_agg0(DevBufs b, MgBufs m) {
    const DevParams& P = *b.prm;
    const uint32_t nx = P.nx, ny = P.ny, nz = P.nz;
    const MgLevel& up = m.lv[1];
    for (uint32_t I = blockIdx.x * blockDim.x + threadIdx.x; I < up.C; I += gridDim.x * blockDim.x) {
        const uint32_t ii = I % up.nx, jj = (I / up.nx) % up.ny, kk = I / (up.nx * up.ny);
        float D = 0.0f, wx = 0.0f, wy = 0.0f, wz = 0.0f;
        for (uint32_t d = 0; d < 8; d++) {
            const uint32_t dx = d & 1, dy = (d >> 1) & 1, dz = d >> 2;
            const uint32_t i = 2 * ii + dx, j = 2 * jj + dy, k = 2 * kk + dz;
            if (i >= nx || j >= ny || k >= nz) continue;
            const uint32_t info = b.cinfo[i + nx * (j + ny * k)];
            if (info < (1u << 7)) continue;
            D += diag0(info);
            if (info & (1u << 2)) { if (dx == 0) D -= 2.0f; else wx += 1.0f; }
            if (info & (1u << 4)) { if (dy == 0) D -= 2.0f; else wy += 1.0f; }
            if (info & (1u << 6)) { if (dz == 0) D -= 2.0f; else wz += 1.0f; }
        }
        up.st[I] = make_float4(D, wx, wy, wz);
    }
}

// Level l+1 from level l (l >= 1).
__global__ void __launch_bounds__(256) k_mg_agg(MgBufs m, uint32_t l) {
    const MgLevel& lv = m.lv[l];
    const MgLevel& up = m.lv[l + 1];
    for (uint32_t I = blockIdx.x * blockDim.x + threadIdx.x; I < up.C; I += gridDim.x * blockDim.x) {
        const uint32_t ii = I % up.nx, jj = (I / up.nx) % up.ny, kk = I / (up.nx * up.ny);
        float D = 0.0f, wx = 0.0f, wy = 0.0f, wz = 0.0f;
        for (uint32_t d = 0; d < 8; d++) {
            const uint32_t dx = d & 1, dy = (d >> 1) & 1, dz = d >> 2;
            const uint32_t i = 2 * ii + dx, j = 2 * jj + dy, k = 2 * kk + dz;
            if (i >= lv.nx || j >= lv.ny || k >= lv.nz) continue;
            const float4 s = lv.st[i + lv.nx * (j + lv.ny * k)];
            if (!(s.x > 0.0f)) continue;
            D += s.x;
            if (dx == 0) D -= 2.0f * s.y; else wx += s.y;
            if (dy == 0) D -= 2.0f * s.z; else wy += s.z;
            if (dz == 0) D -= 2.0f * s.w; else wz += s.w;
        }
        up.st[I] = make_float4(D, wx, wy, wz);
    }
}

}  // namespace

int mg_max_blocks_per_sm() {
    int n = 0;
    if (cudaFuncSetAttribute(k_mgpcg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(MgShared)) !=
        cudaSuccess)
        return 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_mgpcg, MG_THREADS, sizeof(MgShared)) != cudaSuccess)
        return 0;
    return n;
}

// The caller has run k_grid_prep (r, p, cinfo, chunk_flag) and zeroed
// nothing: the plan, the barrier counter and the coarse operators are
// prepared here.  L.cg_blocks blocks (<= MG_PART), at most one per SM.
cudaError_t launch_mgpcg(const DevBufs& b, const MgBufs& m, const LaunchCfg& L, cudaStream_t s) {
    if (L.cg_blocks < 1 || L.cg_blocks > MG_PART || m.L < 2) return cudaErrorInvalidValue;
    cudaError_t e = launch_cg_plan(b, (uint32_t)L.cg_blocks, s);
    if (e != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(m.bar, 0, sizeof(uint32_t), s)) != cudaSuccess) return e;
    const int gb = L.num_sms * 8;
    k_mg_agg0<<<gb, 256, 0, s>>>(b, m);
    for (uint32_t l = 1; l + 1 < m.L; l++) k_mg_agg<<<gb, 256, 0, s>>>(m, l);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(L.cg_blocks);
    cfg.blockDim = dim3(MG_THREADS);
    cfg.dynamicSmemBytes = sizeof(MgShared);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_mgpcg, b, m);
}

}  // namespace fl
