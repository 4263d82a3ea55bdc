// fl_cg.cu — persistent matrix-free CG for the MAC pressure Poisson system.
//
// One cooperative launch runs the whole solve that the reference issues as
// 9 dispatches per iteration (fluid.rs:1689-1701): cg_spmv, cg_reduce(d,q),
// cg_alpha, cg_update, cg_reduce(r,r), cg_beta, cg_dir.  Per iteration:
//
//   phase 1  d_new = r + beta*d_old (cg_dir.wgsl:30) fused with q = A d_new
//            (cg_spmv.wgsl:46-68); neighbours' d_new are recomputed from r and
//            d_old (same f32 ops, same bits), so no barrier is needed between
//            the direction update and the stencil.  d ping-pongs between two
//            buffers.  Partial d.q per 256-cell chunk.
//   barrier  alpha = rs_old/dq (cg_alpha.wgsl)
//   phase 2  p += alpha d, r -= alpha q (cg_update.wgsl); partial r.r
//   barrier  beta, convergence test (cg_beta.wgsl) — the loop really exits.
//
// Only 256-cell chunks holding a liquid cell are visited (the rest are zero in
// every vector).  k_cg_plan lists them once per solve, grouped by residue
// chunk mod 256 and ascending within a group: segment li holds exactly the
// nonzero terms that thread li of cg_reduce_final.wgsl adds in sequence (the
// skipped terms are +0, and acc + 0 == acc for an accumulator that starts at
// +0).  Partials are stored in plan order, so in FL_CG_F32 every block
// re-evaluates the reference's two-level tree from contiguous segments; all
// blocks hold identical scalars without a broadcast and the result is the
// reference's f32 arithmetic exactly.  Each group caches its plan entries and
// a list of its liquid cells with their stencil masks (k_grid_prep's cinfo) in
// shared memory for the whole solve: an iteration touches liquid cells only,
// issues no dependent loads for topology, scatters each product into its fixed
// slot of the chunk's tree, and reduces KB chunks at a time with one
// multi-tree.  FL_CG_F64: see Df below.
#include "fl_device.cuh"

namespace fl {

constexpr int KPLAN = 64;  // plan entries cached in shared memory per group
constexpr int KINFO = 24;  // chunks per group whose liquid cells are listed in shared memory
constexpr int KB = 4;      // chunks reduced together by one multi-tree
constexpr int NBATCH = KINFO / KB;
constexpr int KCELL = KINFO * CHUNK;  // listed cells per group

struct CgShared {
    uint32_t off[CHUNK + 1];
    uint32_t plan[CG_GROUPS][KPLAN];
    float tree[CG_GROUPS][KB][CHUNK];
    // Liquid cells of the group's first KINFO chunks, grouped by batch of KB
    // chunks: bits 0-9 stencil mask (cinfo), 10-17 cell in chunk, 18-23 chunk slot.
    uint32_t cell[CG_GROUPS][KCELL];
    uint32_t boff[CG_GROUPS][NBATCH + 1];
    uint32_t wcnt[CG_GROUPS][KINFO][CHUNK / 32];  // per (chunk slot, warp): count, then list offset
    double red64[CG_THREADS / 32];
    float scal_f;
    double scal_d;
    int abort_flag;
};

__device__ __forceinline__ void named_bar(int id, int count) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// cg_reduce.wgsl:38-49 over the 256 threads of one group.  Valid at lt == 0.
__device__ __forceinline__ float group_tree(float prod, float* s, int group, int lt) {
    s[lt] = prod;
    named_bar(1 + group, CHUNK);
    if (lt < 128) s[lt] = __fadd_rn(s[lt], s[lt + 128]);
    named_bar(1 + group, CHUNK);
    if (lt < 64) s[lt] = __fadd_rn(s[lt], s[lt + 64]);
    named_bar(1 + group, CHUNK);
    float v = 0.0f;
    if (lt < 32) {
        v = __fadd_rn(s[lt], s[lt + 32]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = __fadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
    }
    named_bar(1 + group, CHUNK);  // s is reused afterwards
    return v;
}

// The same tree over nb <= KB arrays at once (one barrier per level for all
// of them); warp w of the group finishes array w with shuffles and writes its
// partial to out[e0 + w*estride].
__device__ __forceinline__ void multi_tree(float (*s)[CHUNK], uint32_t nb, int group, int lt, float* out,
                                           uint32_t e0, uint32_t estride) {
    named_bar(1 + group, CHUNK);
    if (lt < 128)
        for (uint32_t k = 0; k < nb; k++) s[k][lt] = __fadd_rn(s[k][lt], s[k][lt + 128]);
    named_bar(1 + group, CHUNK);
    if (lt < 64)
        for (uint32_t k = 0; k < nb; k++) s[k][lt] = __fadd_rn(s[k][lt], s[k][lt + 64]);
    named_bar(1 + group, CHUNK);
    const uint32_t w = (uint32_t)lt >> 5, lane = (uint32_t)lt & 31u;
    if (w < nb) {
        float v = __fadd_rn(s[w][lane], s[w][lane + 32]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = __fadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
        if (lane == 0) out[e0 + w * estride] = v;
    }
    named_bar(1 + group, CHUNK);
}

// cg_reduce_final.wgsl:24-53: thread li sums the nonzero partials of chunks
// li, li+256, ... in order (its plan segment), then the 256-wide tree.
// Evaluated by group 0; the result goes to all threads.  With `chunk_ids`, the
// partials are indexed by chunk (the initial residual from k_grid_prep); else
// they are stored in plan order.
__device__ float final_reduce_f32(const float* part, const uint32_t* chunk_ids, CgShared& sh) {
    __syncthreads();
    if (threadIdx.x < CHUNK) {
        float acc = 0.0f;
        const uint32_t beg = sh.off[threadIdx.x], end = sh.off[threadIdx.x + 1];
        if (chunk_ids) {
            for (uint32_t e = beg; e < end; e++) acc = __fadd_rn(acc, part[chunk_ids[e]]);
        } else {
#pragma unroll 4
            for (uint32_t e = beg; e < end; e++) acc = __fadd_rn(acc, part[e]);
        }
        const float v = group_tree(acc, sh.tree[0][0], 0, threadIdx.x);
        if (threadIdx.x == 0) sh.scal_f = v;
    }
    __syncthreads();
    return sh.scal_f;
}

// Deterministic f64 sum of n values (lanes stride, then a fixed shuffle tree);
// with `ids`, value i is part[ids[i]].
__device__ double final_reduce_f64(const double* part, uint32_t n, CgShared& sh, const uint32_t* ids = nullptr) {
    __syncthreads();
    if (threadIdx.x < 32) {
        double acc = 0.0;
        for (uint32_t i = threadIdx.x; i < n; i += 32) acc += part[ids ? ids[i] : i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) sh.scal_d = acc;
    }
    __syncthreads();
    return sh.scal_d;
}

// FL_CG_F64 accumulation: exact f32 products (two-product with fmaf) summed in
// compensated float-float (two-sum) by each thread and across its warp, then
// in double across warps, blocks and the grid.  The FP64 pipe of this part is
// slow, so it is used where the error would otherwise grow: the ~1e5-term sums
// across warps/blocks, alpha, beta, the residual norm and the stopping test.
struct Df {
    float hi, lo;
};
__device__ __forceinline__ Df df_add(Df a, Df b) {
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    const float hi = __fadd_rn(s, e);
    return {hi, __fsub_rn(e, __fsub_rn(hi, s))};
}
__device__ __forceinline__ Df df_prod(float x, float y) {
    const float p = __fmul_rn(x, y);
    return {p, __fmaf_rn(x, y, -p)};
}

__device__ __forceinline__ Df warp_sum_df(Df v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        Df w;
        w.hi = __shfl_down_sync(0xffffffffu, v.hi, o);
        w.lo = __shfl_down_sync(0xffffffffu, v.lo, o);
        v = df_add(v, w);
    }
    return v;
}

// Block partial: float-float across lanes and then across the block's warps
// (in warp order), one conversion to double at the end.
__device__ void block_sum_df(Df v, double* out, CgShared& sh) {
    v = warp_sum_df(v);
    float* red = reinterpret_cast<float*>(sh.red64);
    if ((threadIdx.x & 31) == 0) {
        red[2 * (threadIdx.x >> 5)] = v.hi;
        red[2 * (threadIdx.x >> 5) + 1] = v.lo;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        Df w = {red[2 * threadIdx.x], red[2 * threadIdx.x + 1]};
        w = warp_sum_df(w);
        if (threadIdx.x == 0) *out = (double)w.hi + (double)w.lo;
    }
}

// Grid barrier with a bounded wait (see fl_device.cuh).  false = abort.
__device__ bool grid_barrier(DevStats* st, uint32_t target, CgShared& sh) {
    __syncthreads();
    if (threadIdx.x == 0) {
        red_release_add(&st->barrier, 1u);
        const uint64_t t0 = global_ns();
        int ab = 0;
        uint32_t spins = 0;
        while (ld_acquire(&st->barrier) < target) {
            if ((++spins & 255u) != 0u) continue;  // poll the counter; check the rest now and then
            if (*(volatile uint32_t*)&st->status != 0u) { ab = 1; break; }
            if (global_ns() - t0 > 2000000000ull) {
                atomicCAS(&st->status, 0u, 5u /* FL_TIMEOUT */);
                ab = 1;
                break;
            }
        }
        sh.abort_flag = ab;
    }
    __syncthreads();
    return sh.abort_flag == 0;
}

// The solve's plan: active chunks grouped by residue mod 256 (one block).
__global__ void __launch_bounds__(CHUNK) k_cg_plan(DevBufs b) {
    __shared__ uint32_t s_warp[CHUNK / 32];
    const uint32_t nchunks = b.prm->nchunks;
    const uint32_t li = threadIdx.x, lane = li & 31, warp = li >> 5;
    uint32_t cnt = 0;
    for (uint32_t c = li; c < nchunks; c += CHUNK) cnt += b.chunk_flag[c] ? 1u : 0u;
    uint32_t x = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= (uint32_t)o) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    uint32_t base = 0;
    for (uint32_t w = 0; w < warp; w++) base += s_warp[w];
    const uint32_t off = base + x - cnt;
    b.cg_off[li] = off;
    if (li == CHUNK - 1) b.cg_off[CHUNK] = off + cnt;
    uint32_t pos = off;
    for (uint32_t c = li; c < nchunks; c += CHUNK)
        if (b.chunk_flag[c]) b.cg_chunk[pos++] = c;
}

__global__ void __launch_bounds__(CG_THREADS, 1) k_cg(DevBufs b) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CgShared& sh = *reinterpret_cast<CgShared*>(smem_raw);
    const DevParams& P = *b.prm;
    const uint32_t C = P.C, iters = P.iters;
    const size_t nx = P.nx, nxy = (size_t)P.nx * P.ny;
    const int group = threadIdx.x >> 8, lt = threadIdx.x & (CHUNK - 1);
    const uint32_t G = gridDim.x;
    const bool f64 = P.precision == 1u;
    float* __restrict__ r = b.r;
    float* __restrict__ p = b.p;
    float* __restrict__ q = b.q;
    const uint16_t* __restrict__ cinfo = b.cinfo;
    double* cta64 = b.cta_part64;
    uint32_t target = 0;
    for (int i = threadIdx.x; i <= CHUNK; i += blockDim.x) sh.off[i] = b.cg_off[i];
    __syncthreads();
    const uint32_t A = sh.off[CHUNK];  // active chunks
    const uint32_t* __restrict__ plan = b.cg_chunk;
    // This group's plan entries are e_j = gid + j*gstride, j < nk.
    const uint32_t gid = blockIdx.x * CG_GROUPS + group, gstride = G * CG_GROUPS;
    const uint32_t nk = A > gid ? (A - 1 - gid) / gstride + 1 : 0u;
    // Cache the entries, and list the liquid cells of the first KINFO chunks
    // (with their stencil masks) per batch, for the whole solve.
    const uint32_t lane = (uint32_t)lt & 31u, lt_mask = (1u << lane) - 1u;
    for (uint32_t j = lt; j < nk && j < (uint32_t)KPLAN; j += CHUNK) sh.plan[group][j] = plan[gid + j * gstride];
    const uint32_t nkc = nk < (uint32_t)KINFO ? nk : (uint32_t)KINFO;
    const uint32_t nbt = (nkc + KB - 1) / KB;
    const uint32_t warp = (uint32_t)lt >> 5;
    named_bar(1 + group, CHUNK);
    for (uint32_t j = 0; j < nkc; j++) {
        const size_t c = (size_t)sh.plan[group][j] * CHUNK + lt;
        const bool liq = c < C && (cinfo[c] & 1u);
        const uint32_t m = __ballot_sync(0xffffffffu, liq);
        if (lane == 0) sh.wcnt[group][j][warp] = (uint32_t)__popc(m);
    }
    named_bar(1 + group, CHUNK);
    if (lt == 0) {  // list order: batch, chunk slot, warp, lane — fixed, so runs repeat bit for bit
        uint32_t acc = 0;
        for (uint32_t bt = 0; bt < nbt; bt++) {
            sh.boff[group][bt] = acc;
            for (uint32_t j = bt * KB; j < nkc && j < (bt + 1) * KB; j++)
                for (uint32_t w = 0; w < CHUNK / 32; w++) {
                    const uint32_t n = sh.wcnt[group][j][w];
                    sh.wcnt[group][j][w] = acc;
                    acc += n;
                }
        }
        sh.boff[group][nbt] = acc;
    }
    named_bar(1 + group, CHUNK);
    for (uint32_t j = 0; j < nkc; j++) {
        const size_t c = (size_t)sh.plan[group][j] * CHUNK + lt;
        const uint32_t info = c < C ? cinfo[c] : 0u;
        const bool liq = info & 1u;
        const uint32_t m = __ballot_sync(0xffffffffu, liq);
        if (liq) sh.cell[group][sh.wcnt[group][j][warp] + __popc(m & lt_mask)] = (j << 18) | ((uint32_t)lt << 10) | info;
    }
    named_bar(1 + group, CHUNK);

    float rs_old_f = 0.0f, rs_init_f = 0.0f;
    double rs_old_d = 0.0, rs_init_d = 0.0;
    if (f64) {
        rs_old_d = final_reduce_f64(b.chunk_rr64, A, sh, plan);
        rs_init_d = rs_old_d;
    } else {
        rs_old_f = final_reduce_f32(b.part_rr, plan, sh);
        rs_init_f = rs_old_f;
    }
    float beta = 0.0f;
    uint32_t k = 0;
    for (uint32_t it = 0; it < iters; it++) {
        float* __restrict__ d_cur = (it & 1u) ? b.dB : b.dA;
        const float* __restrict__ d_prev = (it & 1u) ? b.dA : b.dB;
        const bool first = it == 0;
        // ---------------- phase 1: direction + SpMV + d.q ----------------
        Df acc = {0.0f, 0.0f};
        // phase-1 work on one liquid cell c with stencil mask `info`
        auto spmv_cell = [&](size_t c, uint32_t info) -> float {
            float dc;
            if (first) {
                dc = d_cur[c];
            } else {
                dc = __fadd_rn(r[c], __fmul_rn(beta, d_prev[c]));  // cg_dir.wgsl:30
                d_cur[c] = dc;
            }
            // cg_spmv.wgsl:46-68: neighbours -x,+x,-y,+y,-z,+z
            const size_t nbr[6] = {c - 1, c + 1, c - nx, c + nx, c - nxy, c + nxy};
            float sum = 0.0f;
#pragma unroll
            for (int s = 0; s < 6; s++) {
                if (info & (2u << s)) {
                    const float dn = first ? d_cur[nbr[s]] : __fadd_rn(r[nbr[s]], __fmul_rn(beta, d_prev[nbr[s]]));
                    sum = __fadd_rn(sum, dn);
                }
            }
            const float cnt = (float)((info >> 7) & 7u);
            const float qc = __fsub_rn(__fmul_rn(cnt, dc), sum);
            q[c] = qc;
            if (f64) acc = df_add(acc, df_prod(dc, qc));
            return __fmul_rn(dc, qc);
        };
        for (uint32_t bt = 0; bt < nbt; bt++) {  // listed chunks: liquid cells only
            const uint32_t j0 = bt * KB, nb = nkc - j0 < (uint32_t)KB ? nkc - j0 : (uint32_t)KB;
            for (uint32_t k2 = 0; k2 < nb; k2++) sh.tree[group][k2][lt] = 0.0f;
            named_bar(1 + group, CHUNK);
            for (uint32_t t = sh.boff[group][bt] + lt; t < sh.boff[group][bt + 1]; t += CHUNK) {
                const uint32_t ent = sh.cell[group][t];
                const uint32_t j = ent >> 18, cl = (ent >> 10) & 255u;
                const size_t c = (size_t)sh.plan[group][j] * CHUNK + cl;
                sh.tree[group][j - j0][cl] = spmv_cell(c, ent & 1023u);
            }
            if (!f64) multi_tree(sh.tree[group], nb, group, lt, b.part_dq, gid + j0 * gstride, gstride);
            else named_bar(1 + group, CHUNK);
        }
        for (uint32_t j0 = nkc; j0 < nk; j0 += KB) {  // further chunks: one cell slot per thread
            const uint32_t nb = nk - j0 < (uint32_t)KB ? nk - j0 : (uint32_t)KB;
            for (uint32_t kb = 0; kb < nb; kb++) {
                const uint32_t j = j0 + kb;
                const uint32_t chunk = j < (uint32_t)KPLAN ? sh.plan[group][j] : plan[gid + j * gstride];
                const size_t c = (size_t)chunk * CHUNK + lt;
                const uint32_t info = c < C ? cinfo[c] : 0u;
                sh.tree[group][kb][lt] = (info & 1u) ? spmv_cell(c, info) : 0.0f;
            }
            if (!f64) multi_tree(sh.tree[group], nb, group, lt, b.part_dq, gid + j0 * gstride, gstride);
        }
        if (f64) {
            __syncthreads();
            block_sum_df(acc, &cta64[blockIdx.x], sh);
        }
        target += G;
        if (!grid_barrier(b.st, target, sh)) return;
        float alpha;
        if (f64) {
            const double dq = final_reduce_f64(cta64, G, sh);
            alpha = fabs(dq) > 1e-30 ? (float)(rs_old_d / dq) : 0.0f;
        } else {
            const float dq = final_reduce_f32(b.part_dq, nullptr, sh);
            alpha = fabsf(dq) > 1e-30f ? __fdiv_rn(rs_old_f, dq) : 0.0f;  // cg_alpha.wgsl:17-22
        }
        // ---------------- phase 2: update + r.r ----------------
        acc = {0.0f, 0.0f};
        auto update_cell = [&](size_t c) -> float {
            p[c] = __fadd_rn(p[c], __fmul_rn(alpha, d_cur[c]));      // cg_update.wgsl:33
            const float rc = __fsub_rn(r[c], __fmul_rn(alpha, q[c]));  // cg_update.wgsl:34
            r[c] = rc;
            if (f64) acc = df_add(acc, df_prod(rc, rc));
            return __fmul_rn(rc, rc);
        };
        for (uint32_t bt = 0; bt < nbt; bt++) {
            const uint32_t j0 = bt * KB, nb = nkc - j0 < (uint32_t)KB ? nkc - j0 : (uint32_t)KB;
            for (uint32_t k2 = 0; k2 < nb; k2++) sh.tree[group][k2][lt] = 0.0f;
            named_bar(1 + group, CHUNK);
            for (uint32_t t = sh.boff[group][bt] + lt; t < sh.boff[group][bt + 1]; t += CHUNK) {
                const uint32_t ent = sh.cell[group][t];
                const uint32_t j = ent >> 18, cl = (ent >> 10) & 255u;
                const size_t c = (size_t)sh.plan[group][j] * CHUNK + cl;
                sh.tree[group][j - j0][cl] = update_cell(c);
            }
            if (!f64) multi_tree(sh.tree[group], nb, group, lt, b.part_rr, gid + j0 * gstride, gstride);
            else named_bar(1 + group, CHUNK);
        }
        for (uint32_t j0 = nkc; j0 < nk; j0 += KB) {
            const uint32_t nb = nk - j0 < (uint32_t)KB ? nk - j0 : (uint32_t)KB;
            for (uint32_t kb = 0; kb < nb; kb++) {
                const uint32_t j = j0 + kb;
                const uint32_t chunk = j < (uint32_t)KPLAN ? sh.plan[group][j] : plan[gid + j * gstride];
                const size_t c = (size_t)chunk * CHUNK + lt;
                const uint32_t info = c < C ? cinfo[c] : 0u;
                sh.tree[group][kb][lt] = (info & 1u) ? update_cell(c) : 0.0f;
            }
            if (!f64) multi_tree(sh.tree[group], nb, group, lt, b.part_rr, gid + j0 * gstride, gstride);
        }
        if (f64) {
            __syncthreads();
            block_sum_df(acc, &cta64[G + blockIdx.x], sh);
        }
        target += G;
        if (!grid_barrier(b.st, target, sh)) return;
        k = it + 1;
        bool done;
        if (f64) {
            const double rs_new = final_reduce_f64(cta64 + G, G, sh);
            beta = rs_old_d > 1e-30 ? (float)(rs_new / rs_old_d) : 0.0f;
            rs_old_d = rs_new;
            done = P.tol_sq_d > 0.0 && rs_new <= P.tol_sq_d * rs_init_d;
        } else {
            const float rs_new = final_reduce_f32(b.part_rr, nullptr, sh);
            beta = rs_old_f > 1e-30f ? __fdiv_rn(rs_new, rs_old_f) : 0.0f;  // cg_beta.wgsl:16-23
            rs_old_f = rs_new;
            done = P.tol_sq > 0.0f && rs_new <= __fmul_rn(P.tol_sq, rs_init_f);  // cg_beta.wgsl:25-30
        }
        if (done) break;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        b.st->cg_iters = k;
        b.st->rs_init = f64 ? rs_init_d : (double)rs_init_f;
        b.st->rs_final = f64 ? rs_old_d : (double)rs_old_f;
    }
}

int cg_max_blocks_per_sm() {
    if (cudaFuncSetAttribute(k_cg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(CgShared)) != cudaSuccess)
        return 0;
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_cg, CG_THREADS, sizeof(CgShared)) != cudaSuccess) return 0;
    return n;
}

cudaError_t launch_cg(const DevBufs& b, const LaunchCfg& L, cudaStream_t s) {
    k_cg_plan<<<1, CHUNK, 0, s>>>(b);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(L.cg_blocks);
    cfg.blockDim = dim3(CG_THREADS);
    cfg.dynamicSmemBytes = sizeof(CgShared);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_cg, b);
}

}  // namespace fl
