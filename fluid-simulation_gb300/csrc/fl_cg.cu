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
// every vector).  In FL_CG_F32 every block re-evaluates the reference's
// two-level tree (cg_reduce.wgsl, cg_reduce_final.wgsl) over the per-chunk
// partials, so all blocks hold identical scalars without a broadcast and the
// result is the reference's f32 arithmetic exactly.  FL_CG_F64 accumulates the
// inner products in double (per thread, warp shuffles, blocks in index order).
#include "fl_device.cuh"

namespace fl {

struct CgShared {
    float tree[CG_GROUPS][CHUNK];
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
    named_bar(1 + group, CHUNK);  // s is reused by the next chunk of this group
    return v;
}

// cg_reduce_final.wgsl:24-53: thread li sums partials li, li+256, ... in
// order, then the 256-wide tree.  Evaluated by group 0; result to all threads.
__device__ float final_reduce_f32(const float* part, uint32_t nwg, CgShared& sh) {
    __syncthreads();
    if (threadIdx.x < CHUNK) {
        float acc = 0.0f;
        for (uint32_t idx = threadIdx.x; idx < nwg; idx += CHUNK) acc = __fadd_rn(acc, part[idx]);
        const float v = group_tree(acc, sh.tree[0], 0, threadIdx.x);
        if (threadIdx.x == 0) sh.scal_f = v;
    }
    __syncthreads();
    return sh.scal_f;
}

// Deterministic f64 sum of n values (lanes stride, then a fixed shuffle tree).
__device__ double final_reduce_f64(const double* part, uint32_t n, CgShared& sh) {
    __syncthreads();
    if (threadIdx.x < 32) {
        double acc = 0.0;
        for (uint32_t i = threadIdx.x; i < n; i += 32) acc += part[i];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (threadIdx.x == 0) sh.scal_d = acc;
    }
    __syncthreads();
    return sh.scal_d;
}

__device__ void block_sum_f64(double v, double* out, CgShared& sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh.red64[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0.0;
        for (int w = 0; w < CG_THREADS / 32; w++) a += sh.red64[w];
        *out = a;
    }
}

// Grid barrier with a bounded wait (see fl_device.cuh).  false = abort.
__device__ bool grid_barrier(DevStats* st, uint32_t target, CgShared& sh) {
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        red_release_add(&st->barrier, 1u);
        const uint64_t t0 = global_ns();
        int ab = 0;
        while (ld_acquire(&st->barrier) < target) {
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

__global__ void __launch_bounds__(CG_THREADS, 1) k_cg(DevBufs b) {
    __shared__ CgShared sh;
    const DevParams& P = *b.prm;
    const uint32_t C = P.C, nchunks = P.nchunks, iters = P.iters;
    const size_t nx = P.nx, nxy = (size_t)P.nx * P.ny;
    const int group = threadIdx.x >> 8, lt = threadIdx.x & (CHUNK - 1);
    const uint32_t G = gridDim.x;
    const bool f64 = P.precision == 1u;
    const uint8_t* __restrict__ ct = b.ct;
    float* r = b.r;
    float* p = b.p;
    float* q = b.q;
    double* cta64 = b.cta_part64;
    uint32_t target = 0;

    float rs_old_f = 0.0f, rs_init_f = 0.0f;
    double rs_old_d = 0.0, rs_init_d = 0.0;
    if (f64) {
        rs_old_d = final_reduce_f64(b.chunk_rr64, nchunks, sh);
        rs_init_d = rs_old_d;
    } else {
        rs_old_f = final_reduce_f32(b.part_rr, nchunks, sh);
        rs_init_f = rs_old_f;
    }
    float beta = 0.0f;
    uint32_t k = 0;
    for (uint32_t it = 0; it < iters; it++) {
        float* d_cur = (it & 1u) ? b.dB : b.dA;
        const float* d_prev = (it & 1u) ? b.dA : b.dB;
        const bool first = it == 0;
        // ---------------- phase 1: direction + SpMV + d.q ----------------
        double acc64 = 0.0;
        for (uint32_t base = blockIdx.x * CG_GROUPS; base < nchunks; base += G * CG_GROUPS) {
            const uint32_t chunk = base + group;
            if (chunk >= nchunks || !b.chunk_flag[chunk]) continue;
            const size_t c = (size_t)chunk * CHUNK + lt;
            float prod = 0.0f;
            if (c < C && ct[c] == CELL_LIQUID) {
                float dc;
                if (first) {
                    dc = d_cur[c];
                } else {
                    dc = __fadd_rn(r[c], __fmul_rn(beta, d_prev[c]));
                    d_cur[c] = dc;
                }
                float cnt = 0.0f, sum = 0.0f;
                const size_t nb[6] = {c - 1, c + 1, c - nx, c + nx, c - nxy, c + nxy};
#pragma unroll
                for (int s = 0; s < 6; s++) {
                    const uint8_t t = ct[nb[s]];
                    if (t != CELL_SOLID) {
                        cnt = __fadd_rn(cnt, 1.0f);
                        if (t == CELL_LIQUID) {
                            const float dn = first ? d_cur[nb[s]] : __fadd_rn(r[nb[s]], __fmul_rn(beta, d_prev[nb[s]]));
                            sum = __fadd_rn(sum, dn);
                        }
                    }
                }
                const float qc = __fsub_rn(__fmul_rn(cnt, dc), sum);
                q[c] = qc;
                prod = __fmul_rn(dc, qc);
                acc64 += (double)dc * (double)qc;
            }
            if (!f64) {
                const float v = group_tree(prod, sh.tree[group], group, lt);
                if (lt == 0) b.part_dq[chunk] = v;
            }
        }
        if (f64) {
            __syncthreads();
            block_sum_f64(acc64, &cta64[blockIdx.x], sh);
        }
        target += G;
        if (!grid_barrier(b.st, target, sh)) return;
        float alpha;
        if (f64) {
            const double dq = final_reduce_f64(cta64, G, sh);
            alpha = fabs(dq) > 1e-30 ? (float)(rs_old_d / dq) : 0.0f;
        } else {
            const float dq = final_reduce_f32(b.part_dq, nchunks, sh);
            alpha = fabsf(dq) > 1e-30f ? __fdiv_rn(rs_old_f, dq) : 0.0f;  // cg_alpha.wgsl:17-22
        }
        // ---------------- phase 2: update + r.r ----------------
        acc64 = 0.0;
        for (uint32_t base = blockIdx.x * CG_GROUPS; base < nchunks; base += G * CG_GROUPS) {
            const uint32_t chunk = base + group;
            if (chunk >= nchunks || !b.chunk_flag[chunk]) continue;
            const size_t c = (size_t)chunk * CHUNK + lt;
            float prod = 0.0f;
            if (c < C && ct[c] == CELL_LIQUID) {
                p[c] = __fadd_rn(p[c], __fmul_rn(alpha, d_cur[c]));   // cg_update.wgsl:33
                const float rc = __fsub_rn(r[c], __fmul_rn(alpha, q[c]));  // cg_update.wgsl:34
                r[c] = rc;
                prod = __fmul_rn(rc, rc);
                acc64 += (double)rc * (double)rc;
            }
            if (!f64) {
                const float v = group_tree(prod, sh.tree[group], group, lt);
                if (lt == 0) b.part_rr[chunk] = v;
            }
        }
        if (f64) {
            __syncthreads();
            block_sum_f64(acc64, &cta64[G + blockIdx.x], sh);
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
            const float rs_new = final_reduce_f32(b.part_rr, nchunks, sh);
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
    int n = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_cg, CG_THREADS, 0) != cudaSuccess) return 0;
    return n;
}

cudaError_t launch_cg(const DevBufs& b, const LaunchCfg& L, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(L.cg_blocks);
    cfg.blockDim = dim3(CG_THREADS);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k_cg, b);
}

}  // namespace fl
