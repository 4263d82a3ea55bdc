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
// Gauss-Seidel sweeps on the coarsest level (<= 64 cells), all from zero: a
// symmetric positive-definite preconditioner.
//
// One cooperative persistent kernel per solve, one 1024-thread block per SM.
// Level-0 cells are owned through the CG's plan of active chunks (k_cg_plan,
// split over blocks 1..G-1 when G > 1) and listed in shared memory with their
// stencil masks; level 1's unknowns are listed per block; other grid levels
// are split into one cell range per block.  The levels of at most
// MG_BLOCK0_CELLS cells run inside block 0 alone, with block barriers and
// their b, x and stencils in shared memory (the stencils in the cell-list
// space that block 0 does not need when it owns no level-0 cells).  A
// grid pass boundary is a counter barrier (bounded wait, as in k_cg); a dot
// product is a per-block float-float partial, a barrier and a fixed-order
// sum, so results repeat bit for bit.  Each smoothing pass computes what it
// needs of the other colour on the fly (the red values of the pre-smoothing
// sweep are b/D; the corrected red values of the post-smoothing sweep are
// x + e(parent)), so a level costs four passes: pre-smooth, residual +
// restriction (eight lanes per coarse cell), correction + black sweep, red
// sweep; on level 0 the CG update is fused with the pre-smoothing.
#include "fl_device.cuh"

// Vectors written during the solve (r, z, d, the coarse b and x) are read
// through plain pointers, never const __restrict__: a read-only (non-coherent)
// load could return a value cached before another block's write.  The
// stencils and masks are fixed for the whole kernel.

namespace fl {

namespace {

constexpr int MG_THREADS = 1024;
constexpr int MG_PART = 1024;             // block partial slots per exchange parity
constexpr int MG_CELLS = 20480;           // level-0 unknowns listed per block
constexpr int MG_L1 = 4096;               // level-1 unknowns listed per block
constexpr int MG_COARSE_SWEEPS = 2;       // symmetric Gauss-Seidel sweeps on the coarsest level
constexpr int MG_BATCH = 1;               // level-0 cells per thread whose loads are issued together
                                          // (2 measured slower: register pressure)

// Level-0 cell metadata: bits 0-9 the CG's stencil mask (bit 0 liquid, bit
// s+1 neighbour s of -x,+x,-y,+y,-z,+z liquid, bits 7-9 the non-solid count),
// bits 10-12 the parities of i, j, k, bit 13 the colour (i+j+k)&1 (0 = red).
constexpr uint32_t META_IODD = 1u << 10, META_JODD = 1u << 11, META_KODD = 1u << 12, META_BLACK = 1u << 13;

struct MgShared {
    uint32_t cell[MG_CELLS];
    uint16_t meta[MG_CELLS];
    uint32_t l1[MG_L1];
    float lb[MG_LOCAL_TOTAL], lx[MG_LOCAL_TOTAL];  // b and x of the levels block 0 runs alone
    float2 red[MG_THREADS / 32];
    uint32_t wc[MG_THREADS / 32];
    float2 res;
    int ok;
    uint32_t ncell, nl1, list0, list1;
    // solve scalars kept here rather than in registers through the loop
    float2 rs0, thr, rz;
};

__device__ __forceinline__ uint32_t make_meta(uint32_t info, uint32_t c, uint32_t nx, uint32_t ny) {
    const uint32_t i = c % nx, j = (c / nx) % ny, k = c / (nx * ny);
    return info | ((i & 1u) ? META_IODD : 0u) | ((j & 1u) ? META_JODD : 0u) | ((k & 1u) ? META_KODD : 0u) |
           (((i + j + k) & 1u) ? META_BLACK : 0u);
}

__device__ __forceinline__ float diag0(uint32_t meta) { return (float)((meta >> 7) & 7u); }

// Stencils and masks do not change during the solve: read-only cache; the
// levels block 0 runs alone read their stencils from its shared-memory copy.
__device__ __forceinline__ float4 ld_st(const float4* st, uint32_t c) {
    return __isShared(st) ? st[c] : __ldg(st + c);
}
__device__ __forceinline__ uint32_t ld_ci(const uint16_t* ci, uint32_t c) { return __ldg(ci + c); }

// Sum over the liquid neighbours of v(nb, side) (side 0..5 = -x,+x,-y,+y,-z,+z).
template <class F>
__device__ __forceinline__ float nbsum0(uint32_t meta, uint32_t c, uint32_t nx, uint32_t nxy, F v) {
    float s = 0.0f;
    if (meta & (1u << 1)) s += v(c - 1, 0);
    if (meta & (1u << 2)) s += v(c + 1, 1);
    if (meta & (1u << 3)) s += v(c - nx, 2);
    if (meta & (1u << 4)) s += v(c + nx, 3);
    if (meta & (1u << 5)) s += v(c - nxy, 4);
    if (meta & (1u << 6)) s += v(c + nxy, 5);
    return s;
}

// Coarse level: sum over the neighbours of w(nb) * v(nb, i, j, k of nb) (a
// neighbour with a nonzero weight is an unknown).
template <class F>
__device__ __forceinline__ float nbsum(const float4* st, float4 sc, uint32_t c, uint32_t i, uint32_t j, uint32_t k,
                                       const MgLevel& lv, F v) {
    const uint32_t nxy = lv.nx * lv.ny;
    float s = 0.0f;
    if (sc.y != 0.0f) s += sc.y * v(c + 1, i + 1, j, k);
    if (sc.z != 0.0f) s += sc.z * v(c + lv.nx, i, j + 1, k);
    if (sc.w != 0.0f) s += sc.w * v(c + nxy, i, j, k + 1);
    if (i > 0) {
        const float w = ld_st(st, c - 1).y;
        if (w != 0.0f) s += w * v(c - 1, i - 1, j, k);
    }
    if (j > 0) {
        const float w = ld_st(st, c - lv.nx).z;
        if (w != 0.0f) s += w * v(c - lv.nx, i, j - 1, k);
    }
    if (k > 0) {
        const float w = ld_st(st, c - nxy).w;
        if (w != 0.0f) s += w * v(c - nxy, i, j, k - 1);
    }
    return s;
}
// v(nb) = x[nb], the neighbour's coordinates unused
#define MG_X_OF(lv) [&](uint32_t n, uint32_t, uint32_t, uint32_t) { return (lv).x[n]; }

// The coarse cell (aggregate) holding the cell at (i, j, k), or cell c.
__device__ __forceinline__ uint32_t parent_at(uint32_t i, uint32_t j, uint32_t k, const MgLevel& up) {
    return (i >> 1) + up.nx * ((j >> 1) + up.ny * (k >> 1));
}
__device__ __forceinline__ uint32_t parent_of(uint32_t c, uint32_t nx, uint32_t ny, const MgLevel& up) {
    return parent_at(c % nx, (c / nx) % ny, c / (nx * ny), up);
}

struct Ctx {
    MgShared& sh;
    const DevBufs& b;
    const MgBufs& m;
    uint32_t e0, nown;  // this block's level-0 plan entries
    uint32_t Lg;        // first level run inside block 0 alone (>= 1)
    const float* r;     // the current residual (level 0's b)
    uint32_t epoch;     // barrier target
    uint32_t parity;    // exchange slot parity
    float4* lst;        // block 0: shared-memory copy of the stencils of levels Lg.. (nullptr: global)
};

__device__ bool mg_barrier(Ctx& x) {
    __syncthreads();
    x.epoch += gridDim.x;
    if (threadIdx.x == 0) {
        // the release add orders the block's writes (before the barrier
        // above) ahead of the arrival; a separate fence only added its wait
        red_release_add(x.m.bar, 1u);
        bool ok = true;
        const uint64_t t0 = global_ns(), limit = wait_limit_ns(x.b.prm);
        uint32_t spins = 0;
        while (ld_acquire(x.m.bar) < x.epoch) {
            // clock on the first re-poll and every 64 polls, status every 64
            ++spins;
            const bool slow = (spins & 63u) == 0u;
            if (slow && *(volatile uint32_t*)&x.b.st->status != 0u) {
                ok = false;
                break;
            }
            if ((slow || spins == 1u) && global_ns() - t0 > limit) {
                atomicCAS(&x.b.st->status, 0u, 5u /* FL_TIMEOUT */);
                ok = false;
                break;
            }
        }
        x.sh.ok = ok;
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
        for (uint32_t g0 = 0; g0 < gridDim.x; g0 += 8 * 32) {
            float2 p[8];
#pragma unroll
            for (int k = 0; k < 8; k++) {
                const uint32_t g = g0 + lane + 32u * k;
                p[k] = g < gridDim.x ? part[g] : make_float2(0.0f, 0.0f);
            }
#pragma unroll
            for (int k = 0; k < 8; k++) s = df_add(s, Df{p[k].x, p[k].y});
        }
        s = warp_allsum_df(s);
        if (lane == 0) x.sh.res = make_float2(s.hi, s.lo);
    }
    __syncthreads();
    out = Df{x.sh.res.x, x.sh.res.y};
    return true;
}

// Position of this thread's item among the flagged items of the block (in
// thread order) and their total; uses sh.wc.
__device__ __forceinline__ uint32_t block_rank(MgShared& sh, bool flag, uint32_t& total) {
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    const uint32_t ball = __ballot_sync(0xffffffffu, flag);
    if (lane == 0) sh.wc[warp] = __popc(ball);
    __syncthreads();
    uint32_t off = 0, tot = 0;
    for (uint32_t w = 0; w < MG_THREADS / 32; w++) {
        const uint32_t v = sh.wc[w];
        off += w < warp ? v : 0u;
        tot += v;
    }
    __syncthreads();
    total = tot;
    return off + __popc(ball & ((1u << lane) - 1u));
}

// Level-l cell range of this block (levels >= 1 outside block 0's share).
__device__ __forceinline__ void block_range(uint32_t C, uint32_t& lo, uint32_t& hi) {
    lo = (uint32_t)(((uint64_t)C * blockIdx.x) / gridDim.x);
    hi = (uint32_t)(((uint64_t)C * (blockIdx.x + 1)) / gridDim.x);
}

// Lists this block's level-0 unknowns (plan order) and level-1 unknowns.
__device__ void build_lists(Ctx& x) {
    MgShared& sh = x.sh;
    const DevParams& P = *x.b.prm;
    const uint32_t C = P.C, nx = P.nx, ny = P.ny, lo = threadIdx.x & (CHUNK - 1);
    uint32_t n = 0;
    for (uint32_t base = 0; base < x.nown; base += MG_THREADS / CHUNK) {
        const uint32_t e = base + threadIdx.x / CHUNK;
        uint32_t c = 0, info = 0;
        if (e < x.nown) {
            c = x.b.cg_chunk[x.e0 + e] * CHUNK + lo;
            if (c < C) info = ld_ci(x.b.cinfo, c);
        }
        const bool u = info >= (1u << 7);
        uint32_t tot;
        const uint32_t pos = n + block_rank(sh, u, tot);
        if (u && pos < (uint32_t)MG_CELLS) {
            sh.cell[pos] = c;
            sh.meta[pos] = (uint16_t)make_meta(info, c, nx, ny);
        }
        n += tot;
    }
    const MgLevel& l1 = x.m.lv[1];
    uint32_t n1 = 0, I0, I1;
    block_range(l1.C, I0, I1);
    for (uint32_t base = I0; base < I1; base += MG_THREADS) {
        const uint32_t I = base + threadIdx.x;
        const bool u = I < I1 && ld_st(l1.st, I).x > 0.0f;
        uint32_t tot;
        const uint32_t pos = n1 + block_rank(sh, u, tot);
        if (u && pos < (uint32_t)MG_L1) sh.l1[pos] = I;
        n1 += tot;
    }
    if (threadIdx.x == 0) {
        sh.ncell = n;
        sh.list0 = n <= (uint32_t)MG_CELLS;
        sh.nl1 = n1;
        sh.list1 = n1 <= (uint32_t)MG_L1;
    }
    __syncthreads();
}

// f(c, meta) for every level-0 unknown of this block.
template <class F>
__device__ __forceinline__ void for_own(const Ctx& x, F f) {
    const MgShared& sh = x.sh;
    if (sh.list0) {
        for (uint32_t e = threadIdx.x; e < sh.ncell; e += MG_THREADS) f(sh.cell[e], (uint32_t)sh.meta[e]);
        return;
    }
    const DevParams& P = *x.b.prm;
    const uint32_t C = P.C, lo = threadIdx.x & (CHUNK - 1);
    for (uint32_t e = threadIdx.x / CHUNK; e < x.nown; e += MG_THREADS / CHUNK) {
        const uint32_t c = x.b.cg_chunk[x.e0 + e] * CHUNK + lo;
        if (c >= C) continue;
        const uint32_t info = ld_ci(x.b.cinfo, c);
        if (info >= (1u << 7)) f(c, make_meta(info, c, P.nx, P.ny));
    }
}

// The same cells with loads and stores in two phases: ld(c, meta) (loads
// only) for MG_BATCH cells of the thread, then st(c, meta, value) for each,
// so that the batch's loads are in flight together.
template <int K = MG_BATCH, class Ld, class Stf>
__device__ __forceinline__ void for_own_batched(const Ctx& x, Ld ld, Stf stf) {
    const MgShared& sh = x.sh;
    if (!sh.list0) {
        for_own(x, [&](uint32_t c, uint32_t meta) { stf(c, meta, ld(c, meta)); });
        return;
    }
    const uint32_t n = sh.ncell;
    for (uint32_t e = threadIdx.x; e < n; e += K * MG_THREADS) {
        decltype(ld(0u, 0u)) v[K];
        uint32_t c[K], mt[K];
#pragma unroll
        for (int k = 0; k < K; k++) {
            const uint32_t ek = e + k * MG_THREADS;
            if (ek < n) {
                c[k] = sh.cell[ek];
                mt[k] = sh.meta[ek];
                v[k] = ld(c[k], mt[k]);
            }
        }
#pragma unroll
        for (int k = 0; k < K; k++)
            if (e + k * MG_THREADS < n) stf(c[k], mt[k], v[k]);
    }
}

// f(c, i, j, k, st) for every unknown of coarse level l: level 1 from this
// block's list, other grid levels over this block's range, local levels
// (block 0 alone, shared memory) over all cells.
// (i, j, k) of cell c of a level of at most MG_BLOCK0_CELLS cells by
// multiply-high with rounded-up reciprocals ceil(2^32 / d): exact because
// c * d stays below 2^32 (integer division by a runtime divisor is a long
// instruction sequence, and the levels block 0 runs alone are issue-bound).
// A divisor of 1 is stored as 0.
struct SmallDiv {
    uint32_t nx, nxy, mx, mxy;
    __device__ __forceinline__ static uint32_t recip(uint32_t d) { return d > 1u ? 0xffffffffu / d + 1u : 0u; }
    __device__ __forceinline__ explicit SmallDiv(const MgLevel& lv)
        : nx(lv.nx), nxy(lv.nx * lv.ny), mx(recip(lv.nx)), mxy(recip(lv.nx * lv.ny)) {}
    __device__ __forceinline__ void ijk(uint32_t c, uint32_t& i, uint32_t& j, uint32_t& k) const {
        k = mxy ? __umulhi(c, mxy) : c;
        const uint32_t rem = c - k * nxy;
        j = mx ? __umulhi(rem, mx) : rem;
        i = rem - j * nx;
    }
};
static_assert((uint64_t)MG_BLOCK0_CELLS * MG_BLOCK0_CELLS < (1ull << 32), "SmallDiv needs c * divisor < 2^32");

template <class F>
__device__ __forceinline__ void for_level(const Ctx& x, uint32_t l, const MgLevel& lv, bool local, F f) {
    auto visit = [&](uint32_t c, float4 sc) {
        const uint32_t i = c % lv.nx, j = (c / lv.nx) % lv.ny, k = c / (lv.nx * lv.ny);
        f(c, i, j, k, sc);
    };
    if (local) {
        const SmallDiv dv(lv);
        for (uint32_t c = threadIdx.x; c < lv.C; c += MG_THREADS) {
            const float4 sc = ld_st(lv.st, c);
            if (sc.x > 0.0f) {
                uint32_t i, j, k;
                dv.ijk(c, i, j, k);
                f(c, i, j, k, sc);
            }
        }
        return;
    }
    if (l == 1 && x.sh.list1) {
        for (uint32_t e = threadIdx.x; e < x.sh.nl1; e += MG_THREADS) {
            const uint32_t c = x.sh.l1[e];
            visit(c, ld_st(lv.st, c));
        }
        return;
    }
    uint32_t lo, hi;
    block_range(lv.C, lo, hi);
    for (uint32_t c = lo + threadIdx.x; c < hi; c += MG_THREADS) {
        const float4 sc = ld_st(lv.st, c);
        if (sc.x > 0.0f) visit(c, sc);
    }
}

// ---- level 0 passes (b = r, x = z) ----

// pre-smoothing from zero: red z = r/D; black z = (r + sum r_nb/D_nb)/D
__device__ void pre0(const Ctx& x) {
    const DevParams& P = *x.b.prm;
    const uint32_t nx = P.nx, nxy = nx * P.ny;
    const float* r = x.r;
    const uint16_t* __restrict__ ci = x.b.cinfo;
    float* z = x.m.lv[0].x;
    for_own_batched(
        x,
        [&](uint32_t c, uint32_t meta) {
            float v = r[c];
            if (meta & META_BLACK)
                v += nbsum0(meta, c, nx, nxy, [&](uint32_t n, int) { return r[n] / (float)(ld_ci(ci, n) >> 7); });
            return v / diag0(meta);
        },
        [&](uint32_t c, uint32_t, float v) { z[c] = v; });
}

// The CG update fused with pre0: p += alpha d, r_next = r - alpha q, and the
// pre-smoothing of r_next (a black cell's red neighbours' r_next computed on
// the fly from their r and q, which this pass does not change).  Returns this
// thread's share of r_next . r_next.
__device__ Df update_pre0(const Ctx& x, float alpha, const float* d, float* r_next) {
    const DevParams& P = *x.b.prm;
    const uint32_t nx = P.nx, nxy = nx * P.ny;
    const float* r = x.r;
    const float* q = x.b.q;
    float* p = x.b.p;
    const uint16_t* __restrict__ ci = x.b.cinfo;
    float* z = x.m.lv[0].x;
    Df acc = {0.0f, 0.0f};
    for_own(x, [&](uint32_t c, uint32_t meta) {
        const float rn = r[c] - alpha * q[c];
        float v = rn;
        if (meta & META_BLACK)
            v += nbsum0(meta, c, nx, nxy,
                        [&](uint32_t n, int) { return (r[n] - alpha * q[n]) / (float)(ld_ci(ci, n) >> 7); });
        p[c] += alpha * d[c];
        r_next[c] = rn;
        z[c] = v / diag0(meta);
        acc = df_add(acc, df_prod(rn, rn));
    });
    return acc;
}

// Unknowns of level l (grid pass: this block's share; local: all), eight
// consecutive lanes per cell: f(I, ii, jj, kk, child d = lane & 7) returns the
// child's term, the eight terms are summed in a fixed shuffle order and
// g(I, sum) runs on the first lane.  A cell's children are visited together.
template <class F, class G>
__device__ __forceinline__ void for_level8(const Ctx& x, uint32_t l, const MgLevel& lv, bool local, F f, G g) {
    const uint32_t d = threadIdx.x & 7u, slot = threadIdx.x >> 3;
    constexpr uint32_t per = MG_THREADS / 8;
    const SmallDiv dv(lv);  // used for local levels only (at most MG_BLOCK0_CELLS cells)
    auto one = [&](bool valid, uint32_t I) {
        float t = 0.0f;
        if (valid) {
            uint32_t ii, jj, kk;
            if (local) {
                dv.ijk(I, ii, jj, kk);
            } else {
                ii = I % lv.nx;
                jj = (I / lv.nx) % lv.ny;
                kk = I / (lv.nx * lv.ny);
            }
            t = f(I, ii, jj, kk, d);
        }
        t += __shfl_xor_sync(0xffffffffu, t, 1);
        t += __shfl_xor_sync(0xffffffffu, t, 2);
        t += __shfl_xor_sync(0xffffffffu, t, 4);
        if (valid && d == 0) g(I, t);
    };
    if (!local && l == 1 && x.sh.list1) {
        const uint32_t n = x.sh.nl1;
        for (uint32_t e0 = 0; e0 < n; e0 += per) {
            const uint32_t e = e0 + slot;
            one(e < n, e < n ? x.sh.l1[e] : 0u);
        }
        return;
    }
    uint32_t lo = 0, hi = lv.C;
    if (!local) block_range(lv.C, lo, hi);
    for (uint32_t c0 = lo; c0 < hi; c0 += per) {
        const uint32_t I = c0 + slot;
        one(I < hi && ld_st(lv.st, I < hi ? I : lo).x > 0.0f, I);
    }
}

// b1 = P^T (r - A z)
__device__ void restrict0(const Ctx& x) {
    const DevParams& P = *x.b.prm;
    const uint32_t nx = P.nx, ny = P.ny, nz = P.nz, nxy = nx * ny;
    const float* r = x.r;
    const uint16_t* __restrict__ ci = x.b.cinfo;
    const float* z = x.m.lv[0].x;
    const MgLevel& up = x.m.lv[1];
    for_level8(
        x, 1, up, false,
        [&](uint32_t, uint32_t ii, uint32_t jj, uint32_t kk, uint32_t d) {
            const uint32_t i = 2 * ii + (d & 1), j = 2 * jj + ((d >> 1) & 1), k = 2 * kk + (d >> 2);
            if (i >= nx || j >= ny || k >= nz) return 0.0f;
            const uint32_t c = i + nx * (j + ny * k);
            const uint32_t info = ld_ci(ci, c);
            if (info < (1u << 7)) return 0.0f;
            return r[c] - (diag0(info) * z[c] - nbsum0(info, c, nx, nxy, [&](uint32_t n, int) { return z[n]; }));
        },
        [&](uint32_t I, float s) { up.b[I] = s; });
}

// correction + black sweep: z_black = (r + sum (z_red + e(parent))) / D
__device__ void post0_black(const Ctx& x) {
    const DevParams& P = *x.b.prm;
    const uint32_t nx = P.nx, ny = P.ny, nxy = nx * ny;
    const float* r = x.r;
    float* z = x.m.lv[0].x;
    const MgLevel& up = x.m.lv[1];
    const float* e = up.x;
    const uint32_t unx = up.nx, unxy = up.nx * up.ny;
    for_own_batched(
        x,
        [&](uint32_t c, uint32_t meta) {
            if (!(meta & META_BLACK)) return 0.0f;
            const uint32_t pc = parent_of(c, nx, ny, up);
            // parent of the neighbour on side s: the own parent, or the next
            // one when the step leaves the 2x2x2 aggregate
            auto pn = [&](int side) {
                switch (side) {
                    case 0: return (meta & META_IODD) ? pc : pc - 1;
                    case 1: return (meta & META_IODD) ? pc + 1 : pc;
                    case 2: return (meta & META_JODD) ? pc : pc - unx;
                    case 3: return (meta & META_JODD) ? pc + unx : pc;
                    case 4: return (meta & META_KODD) ? pc : pc - unxy;
                    default: return (meta & META_KODD) ? pc + unxy : pc;
                }
            };
            const float s = nbsum0(meta, c, nx, nxy, [&](uint32_t n, int side) { return z[n] + e[pn(side)]; });
            return (r[c] + s) / diag0(meta);
        },
        [&](uint32_t c, uint32_t meta, float v) {
            if (meta & META_BLACK) z[c] = v;
        });
}

// red sweep; returns this thread's share of r.z
__device__ Df post0_red(const Ctx& x) {
    const DevParams& P = *x.b.prm;
    const uint32_t nx = P.nx, nxy = nx * P.ny;
    const float* r = x.r;
    float* z = x.m.lv[0].x;
    Df acc = {0.0f, 0.0f};
    for_own_batched(
        x,
        [&](uint32_t c, uint32_t meta) {
            const float rc = r[c];
            const float zc = (meta & META_BLACK)
                                 ? z[c]
                                 : (rc + nbsum0(meta, c, nx, nxy, [&](uint32_t n, int) { return z[n]; })) / diag0(meta);
            return make_float2(rc, zc);
        },
        [&](uint32_t c, uint32_t meta, float2 v) {
            if (!(meta & META_BLACK)) z[c] = v.y;
            acc = df_add(acc, df_prod(v.x, v.y));
        });
    return acc;
}

// ---- coarse level passes (grid levels, or block 0's local levels) ----

__device__ void pre_l(const Ctx& x, uint32_t l, const MgLevel& lv, bool local) {
    const float4* st = lv.st;
    for_level(x, l, lv, local, [&](uint32_t c, uint32_t i, uint32_t j, uint32_t k, float4 sc) {
        float v = lv.b[c];
        if (((i + j + k) & 1u) != 0u)
            v += nbsum(st, sc, c, i, j, k, lv,
                       [&](uint32_t n, uint32_t, uint32_t, uint32_t) { return lv.b[n] / ld_st(st, n).x; });
        lv.x[c] = v / sc.x;
    });
}

__device__ void restrict_l(const Ctx& x, uint32_t l, const MgLevel& lv, const MgLevel& up, bool local) {
    const float4* st = lv.st;
    for_level8(
        x, l + 1, up, local,
        [&](uint32_t, uint32_t ii, uint32_t jj, uint32_t kk, uint32_t d) {
            const uint32_t i = 2 * ii + (d & 1), j = 2 * jj + ((d >> 1) & 1), k = 2 * kk + (d >> 2);
            if (i >= lv.nx || j >= lv.ny || k >= lv.nz) return 0.0f;
            const uint32_t c = i + lv.nx * (j + lv.ny * k);
            const float4 sc = ld_st(st, c);
            if (!(sc.x > 0.0f)) return 0.0f;
            return lv.b[c] - (sc.x * lv.x[c] - nbsum(st, sc, c, i, j, k, lv, MG_X_OF(lv)));
        },
        [&](uint32_t I, float s) { up.b[I] = s; });
}

__device__ void post_black_l(const Ctx& x, uint32_t l, const MgLevel& lv, const MgLevel& up, bool local) {
    const float4* st = lv.st;
    for_level(x, l, lv, local, [&](uint32_t c, uint32_t i, uint32_t j, uint32_t k, float4 sc) {
        if (((i + j + k) & 1u) == 0u) return;
        const float s = nbsum(st, sc, c, i, j, k, lv, [&](uint32_t n, uint32_t ni, uint32_t nj, uint32_t nk) {
            return lv.x[n] + up.x[parent_at(ni, nj, nk, up)];
        });
        lv.x[c] = (lv.b[c] + s) / sc.x;
    });
}

__device__ void post_red_l(const Ctx& x, uint32_t l, const MgLevel& lv, bool local) {
    const float4* st = lv.st;
    for_level(x, l, lv, local, [&](uint32_t c, uint32_t i, uint32_t j, uint32_t k, float4 sc) {
        if (((i + j + k) & 1u) != 0u) return;
        lv.x[c] = (lv.b[c] + nbsum(st, sc, c, i, j, k, lv, MG_X_OF(lv))) / sc.x;
    });
}

// Block 0's view of level l >= Lg: b, x and (with more than one block) the
// stencil in shared memory.
__device__ __forceinline__ MgLevel local_level(const Ctx& x, uint32_t l) {
    MgLevel v = x.m.lv[l];
    uint32_t off = 0;
    for (uint32_t k = x.Lg; k < l; k++) off += x.m.lv[k].C;
    v.b = x.sh.lb + off;
    v.x = x.sh.lx + off;
    if (x.lst) v.st = x.lst + off;
    return v;
}

// Levels Lg .. L-1 by block 0 alone (block barriers instead of grid
// barriers): V-cycle with symmetric Gauss-Seidel sweeps from zero on the
// coarsest level.
__device__ void local_cycle(const Ctx& x) {
    const uint32_t L = x.m.L, Lg = x.Lg;
    {
        const MgLevel g = x.m.lv[Lg], s = local_level(x, Lg);
        for (uint32_t c = threadIdx.x; c < g.C; c += MG_THREADS) s.b[c] = g.b[c];
        __syncthreads();
    }
    for (uint32_t l = Lg; l + 1 < L; l++) {
        const MgLevel lv = local_level(x, l), up = local_level(x, l + 1);
        pre_l(x, l, lv, true);
        __syncthreads();
        restrict_l(x, l, lv, up, true);
        __syncthreads();
    }
    {
        const MgLevel lv = local_level(x, L - 1);
        const uint32_t t = threadIdx.x, nx = lv.nx, ny = lv.ny, nxy = nx * ny;
        uint32_t i = 0, j = 0, k = 0, col = 0;
        float4 sc = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (t < lv.C) {
            i = t % nx; j = (t / nx) % ny; k = t / nxy;
            col = (i + j + k) & 1u;
            sc = ld_st(lv.st, t);
            lv.x[t] = 0.0f;
        }
        __syncthreads();
        for (int h = 0; h < 4 * MG_COARSE_SWEEPS; h++) {
            // forward sweeps red, black; backward sweeps black, red
            const uint32_t want = h < 2 * MG_COARSE_SWEEPS ? (uint32_t)(h & 1) : (uint32_t)((h & 1) ^ 1);
            if (t < lv.C && sc.x > 0.0f && col == want)
                lv.x[t] = (lv.b[t] + nbsum(lv.st, sc, t, i, j, k, lv, MG_X_OF(lv))) / sc.x;
            __syncthreads();
        }
    }
    for (uint32_t l = L - 1; l-- > Lg;) {
        const MgLevel lv = local_level(x, l), up = local_level(x, l + 1);
        post_black_l(x, l, lv, up, true);
        __syncthreads();
        post_red_l(x, l, lv, true);
        __syncthreads();
    }
    {
        const MgLevel g = x.m.lv[Lg], s = local_level(x, Lg);
        for (uint32_t c = threadIdx.x; c < g.C; c += MG_THREADS) g.x[c] = s.x[c];
    }
}

// z = M^-1 r, then the r.z all-reduce (whose barrier ends the cycle).  With
// presmoothed, pre0 and its barrier have already run (update_pre0).
__device__ bool vcycle(Ctx& x, Df& rz, bool presmoothed) {
    const MgBufs& m = x.m;
    const uint32_t Lg = x.Lg;
    if (!presmoothed) {
        pre0(x);
        if (!mg_barrier(x)) return false;
    }
    restrict0(x);
    if (!mg_barrier(x)) return false;
    for (uint32_t l = 1; l < Lg; l++) {
        pre_l(x, l, m.lv[l], false);
        if (!mg_barrier(x)) return false;
        restrict_l(x, l, m.lv[l], m.lv[l + 1], false);
        if (!mg_barrier(x)) return false;
    }
    if (blockIdx.x == 0) local_cycle(x);
    if (!mg_barrier(x)) return false;
    for (uint32_t l = Lg; l-- > 1;) {
        post_black_l(x, l, m.lv[l], m.lv[l + 1], false);
        if (!mg_barrier(x)) return false;
        post_red_l(x, l, m.lv[l], false);
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
    const uint32_t tid = threadIdx.x;
    const uint32_t* start = b.cg_off + CHUNK + 3;
    uint32_t Lg = 1;
    while (Lg + 1 < m.L && m.lv[Lg].C > MG_BLOCK0_CELLS) Lg++;
    // With more than one block, block 0 owns no level-0 cells (launch_mgpcg
    // splits the plan over blocks 1..G-1): it runs the coarse levels alone
    // while the others wait, and its cell list space holds their stencils, so
    // its sweeps read shared memory instead of chains of L2 loads.
    const bool b0_local = gridDim.x > 1;
    uint32_t e0 = 0, nown = 0;
    if (!b0_local || blockIdx.x > 0) {
        const uint32_t pb = b0_local ? blockIdx.x - 1 : 0u;
        e0 = start[pb];
        nown = start[pb + 1] - start[pb];
    }
    Ctx x{sh, b, m, e0, nown, Lg, b.r, 0u, 0u, nullptr};
    build_lists(x);
    if (b0_local && blockIdx.x == 0) {
        static_assert(sizeof(sh.cell) >= MG_LOCAL_TOTAL * sizeof(float4), "local stencils exceed the cell list");
        float4* lst = reinterpret_cast<float4*>(sh.cell);
        uint32_t off = 0;
        for (uint32_t l = Lg; l < m.L; l++) {
            for (uint32_t c = tid; c < m.lv[l].C; c += MG_THREADS) lst[off + c] = ld_st(m.lv[l].st, c);
            off += m.lv[l].C;
        }
        x.lst = lst;
        __syncthreads();
    }
    const uint32_t nx = P.nx, nxy = P.nx * P.ny;
    const uint32_t iters = P.iters;
    const bool stop_on = P.tol_sq > 0.0f;
    float* q = b.q;
    const float* z = m.lv[0].x;
    DevStats* st = b.st;

    // r0.r0 (grid_prep left r = rhs - A p0)
    Df acc = {0.0f, 0.0f};
    for_own_batched(
        x, [&](uint32_t c, uint32_t) { return x.r[c]; },
        [&](uint32_t, uint32_t, float rc) { acc = df_add(acc, df_prod(rc, rc)); });
    Df rs;
    if (!mg_allreduce(x, acc, rs)) return;
    if (tid == 0) {
        const double thr = P.thr_abs ? P.thr_abs_d : (double)P.tol_sq_d * df_to_double(rs);
        const float hi = (float)thr;
        sh.rs0 = make_float2(rs.hi, rs.lo);
        sh.thr = make_float2(hi, (float)(thr - (double)hi));
    }
    {
        Df rz;
        if (!vcycle(x, rz, false)) return;  // its barriers also publish rs0 and thr
        if (tid == 0) sh.rz = make_float2(rz.hi, rz.lo);
    }
    float beta = 0.0f;
    uint32_t k = 0;
    for (uint32_t it = 0; it < iters; it++) {
        float* d_cur = (it & 1u) ? b.dB : b.dA;
        const float* d_prev = (it & 1u) ? b.dA : b.dB;
        const bool first = it == 0;
        // direction d = z + beta d_prev and q = A d (neighbours' d on the fly)
        acc = Df{0.0f, 0.0f};
        for_own_batched(
            x,
            [&](uint32_t c, uint32_t meta) {
                auto dv = [&](uint32_t n, int) { return first ? z[n] : z[n] + beta * d_prev[n]; };
                const float dc = dv(c, 0);
                return make_float2(dc, diag0(meta) * dc - nbsum0(meta, c, nx, nxy, dv));
            },
            [&](uint32_t c, uint32_t, float2 v) {
                d_cur[c] = v.x;
                q[c] = v.y;
                acc = df_add(acc, df_prod(v.x, v.y));
            });
        Df dq;
        if (!mg_allreduce(x, acc, dq)) return;
        // cg_alpha.wgsl:16-22: alpha = 0 when |d.q| <= 1e-30
        const float alpha = fabsf(dq.hi) > 1e-30f ? df_div(Df{sh.rz.x, sh.rz.y}, dq) : 0.0f;
        // residuals alternate between r and r2: neighbours' old values are
        // read while the new ones are written
        float* r_next = x.r == b.r ? m.r2 : b.r;
        if (!mg_allreduce(x, update_pre0(x, alpha, d_cur, r_next), rs)) return;
        x.r = r_next;
        k = it + 1;
        if (stop_on && df_le(rs, Df{sh.thr.x, sh.thr.y})) break;
        if (it + 1 == iters) break;
        Df rz_new;
        if (!vcycle(x, rz_new, true)) return;
        const Df rz = {sh.rz.x, sh.rz.y};
        beta = rz.hi > 1e-30f ? df_div(rz_new, rz) : 0.0f;  // cg_beta.wgsl:16-23
        __syncthreads();
        if (tid == 0) sh.rz = make_float2(rz_new.hi, rz_new.lo);
    }
    if (blockIdx.x == 0 && tid == 0) {
        st->cg_iters = k;
        st->rs_init = df_to_double(Df{sh.rs0.x, sh.rs0.y});
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
    // level-0 cells go to blocks 1..G-1 (block 0 runs the coarse levels)
    cudaError_t e = launch_cg_plan(b, L.cg_blocks > 1 ? (uint32_t)L.cg_blocks - 1 : 1u, s);
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
