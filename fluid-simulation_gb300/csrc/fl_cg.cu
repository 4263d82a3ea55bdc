// fl_cg.cu — persistent matrix-free CG for the MAC pressure Poisson system.
//
// One cooperative launch runs the whole solve that the reference issues as
// 9 dispatches per iteration (fluid.rs:1689-1701): cg_spmv, cg_reduce(d,q),
// cg_alpha, cg_update, cg_reduce(r,r), cg_beta, cg_dir.  Per iteration:
//
//   phase 1   d_new = r + beta*d_old (cg_dir.wgsl:30) fused with q = A d_new
//             (cg_spmv.wgsl:46-68); neighbours' d_new are recomputed from r and
//             d_old (same f32 ops, same bits), so no grid-wide step separates
//             the direction update from the stencil.  d ping-pongs between two
//             buffers.  One d.q partial per 256-cell chunk.
//   exchange  alpha = rs_old/dq (cg_alpha.wgsl)
//   phase 2   p += alpha d, r -= alpha q (cg_update.wgsl); r.r partials
//   exchange  beta and the convergence test (cg_beta.wgsl); the loop exits.
//
// Exchange = grid barrier and reduction in one step.  Every partial is
// published as one 64-bit word {tag, value}, a block's words stored together
// by one warp (on the block's own 128-byte lines in the line layouts); each
// block polls all partials until every word carries the exchange's tag, then
// reduces them itself.  No counter, no second read of the partials, no
// broadcast: seeing the tags is the barrier, and all blocks
// evaluate the same reduction in the same order.  Tags are unique per solve
// (a per-area epoch advanced by k_cg_plan), so words left by earlier solves
// never match.  Exchange B publishes with release semantics and polls with
// acquire loads: a block's release covers all of its vector writes of the
// update phase and the phase before, which is what the next direction +
// SpMV phase's neighbour loads need.  Exchange A carries only its partials
// (relaxed).
//
// Only 256-cell chunks holding a liquid cell are visited (the rest are zero in
// every vector).  k_cg_plan lists them once per solve, grouped by residue
// chunk mod 256 and ascending within a group: segment li holds exactly the
// nonzero terms that thread li of cg_reduce_final.wgsl adds in sequence (the
// skipped terms are +0, and acc + 0 == acc for an accumulator that starts at
// +0).  It also splits the plan into one contiguous range per block with equal
// liquid-cell weight.  FL_CG_F32: a warp evaluates a chunk's 256-wide
// cg_reduce.wgsl tree (same pairing, same order); every block stages all chunk
// partials, sums its segments and evaluates the cg_reduce_final.wgsl tree, so
// the scalars are the reference's f32 arithmetic exactly.  FL_CG_F64: see Df.
// Each block lists its liquid cells with their stencil masks (k_grid_prep's
// cinfo) in shared memory once per solve; an iteration then touches liquid
// cells only and issues no dependent loads for topology.
#include <cstddef>

#include "fl_device.cuh"

namespace fl {

constexpr int CG_WARPS = CG_THREADS / 32;
constexpr uint32_t KT = 2 * CG_WARPS;    // chunks per tree pass: two chunk trees per warp
constexpr uint32_t CELL_CAP = 16384;     // liquid cells listed per block
constexpr uint32_t QCAP = CELL_CAP / 2;  // quads listed per block (8 bytes each, in the same array)
constexpr uint32_t KCH = 2048;           // chunk ids cached per block
constexpr uint32_t VAL_CAP = 16384;      // chunk partials staged per window
constexpr uint32_t MAX_PASS = KCH / KT;  // cached tree passes
// Resident operands: when a block's listed cells fit one pass of at most two
// cells per thread and the exchange window needs at most half of `vals`, each
// listed cell keeps {d, r, q, p} in the upper half of `vals` for the whole
// solve (16 B per cell; the half holds 2 * CG_THREADS cells).
constexpr uint32_t VALS_HALF = (VAL_CAP + VAL_CAP / 32) / 2;
constexpr uint32_t RES_MAX_A = VALS_HALF - VALS_HALF / 33;  // vpos(A - 1) < VALS_HALF
constexpr uint32_t TAG_SPAN_MAX = 1u << 30;
constexpr int STAGE_BATCH = 8;
// Words in flight per thread when staging the blocks' slot lines (one window:
// at 128^3 about 2.4 words per thread, so a smaller batch frees registers).
constexpr int LINE_BATCH = 4;
constexpr uint32_t MAX_CG_BLOCKS = 1024;
// Per-chunk cost in liquid-cell units for the block split (each chunk adds a
// tree and, when sparsely filled, cells that share few cache lines).  Kept
// small: a block above 2 * CG_THREADS listed cells needs a second, serial
// round of the cell loop, which costs more than the chunk overhead (measured
// on the 128^3 dam break; 128 pushed dense blocks past that threshold).
constexpr uint32_t CHUNK_WEIGHT = 32;

struct CgShared {
    float tree[KT][CHUNK];     // per-chunk products of one pass, tree slot = cell in chunk
    float vals[VAL_CAP + VAL_CAP / 32];  // staged partials of one exchange window (positions vpos)
    uint32_t cell[CELL_CAP];   // listed liquid cells: bits 0-9 stencil mask, 10-17 cell in chunk, 18-31 chunk
    uint32_t chunk[KCH];       // this block's chunk ids (plan order)
    uint32_t off[CHUNK + 1];   // plan segment offsets
    uint32_t pass_off[MAX_PASS + 1];
    float seg[CHUNK];          // segment sums (cg_reduce_final.wgsl thread accumulators)
    float red[2 * CG_WARPS];   // F64: float-float warp partials; F32: one pass of chunk trees
    uint32_t wcnt[CG_WARPS];
    float scal[4];             // scalars of an exchange, broadcast by warp 0
    uint32_t layout, nslot;              // exchange slot layout (0 plan order, 1 lines, 2 one line per block), slots used
    float thr_f;                         // f32 stopping threshold on r.r
    float thr_dh, thr_dl;                // FL_CG_F64 stopping threshold on r.r (float-float)
    double rs_d, thr_d;                  // FL_CG_F64_IEEE: r.r of the last exchange, stopping threshold
    float rs_hi, rs_lo;                  // r.r of the last exchange (rs_old); FL_CG_F32 uses rs_hi
    // Block-uniform loop bounds, read from shared memory where used (the cell
    // loops sit at the 64-register limit of a 1024-thread block).
    uint32_t u_s0, u_m, u_mc, u_npc, u_ncell, u_res, u_quad, u_lb;
    uint32_t bstart[MAX_CG_BLOCKS + 1];  // first plan entry of every block
    uint32_t spos[MAX_CG_BLOCKS + 1];    // first exchange slot of every block
    uint16_t lineblk[VAL_CAP / 16 + MAX_CG_BLOCKS];  // line of the slot area -> owning block
};
static_assert(sizeof(CgShared) <= 227 * 1024, "CG shared memory exceeds the 227 KB per-block limit");
static_assert(offsetof(CgShared, vals) % 16 == 0 && (VALS_HALF * 4) % 16 == 0, "resident operands are float4");
static_assert(offsetof(CgShared, tree) % 16 == 0 && offsetof(CgShared, cell) % 8 == 0,
              "quad layout: float4 tree slots, 8-byte quad entries");
static_assert(offsetof(CgShared, tree) % 8 == 0 && sizeof(CgShared::tree) >= 8 * CG_THREADS,
              "the IEEE-double form stages its thread partials in the tree buffer");
static_assert(VALS_HALF + 4 * 2 * CG_THREADS <= VAL_CAP + VAL_CAP / 32, "resident operands fit the upper half");

// ---------------------------------------------------------------------------
// Tagged words

__device__ __forceinline__ void st_release_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
// The polling loads carry no "memory" clobber, so the compiler may compute
// all of a batch's addresses (shared-memory lookups) before issuing the
// loads; what follows a poll is ordered by data dependence or a barrier.
__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p));
    return v;
}
__device__ __forceinline__ void st_relaxed_u64(unsigned long long* p, unsigned long long v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ unsigned long long ld_relaxed_u64(const unsigned long long* p) {
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p));
    return v;
}
// `rel`: release store, for the exchange after which other blocks read this
// block's vector writes; the other exchange carries only its partials.
__device__ __forceinline__ void publish(unsigned long long* p, uint32_t tag, float v, bool rel) {
    const unsigned long long w = ((unsigned long long)tag << 32) | (unsigned long long)__float_as_uint(v);
    if (rel) st_release_u64(p, w);
    else st_relaxed_u64(p, w);
}
// Polls of an exchange after which the reader loads other blocks' vector
// writes are acquire loads (measured faster than relaxed polls followed by an
// acquire fence in every thread); the other exchange polls relaxed.
__device__ __forceinline__ unsigned long long ld_tag(const unsigned long long* p, bool acq) {
    return acq ? ld_acquire_u64(p) : ld_relaxed_u64(p);
}

// Polls *p until it carries `tag` and returns the word.  Bounded: after the
// settings' wait limit (2 s by default), or once another block recorded an
// error, it records FL_TIMEOUT and returns a word without the tag.
__device__ __noinline__ unsigned long long wait_tag(const unsigned long long* p, uint32_t tag, DevStats* st, bool acq,
                                                    const DevParams* prm) {
    const uint64_t t0 = global_ns(), limit = wait_limit_ns(prm);
    uint32_t spins = 0;
    unsigned long long w = ld_tag(p, acq);
    while ((uint32_t)(w >> 32) != tag) {
        // The clock is read on the first re-poll and then every 64 polls (so
        // a limit below one poll's latency expires at the first miss); the
        // status word, a global load, every 64 polls only.
        ++spins;
        const bool slow = (spins & 63u) == 0u;
        if (slow && *(volatile uint32_t*)&st->status != 0u) return 0ull;
        if ((slow || spins == 1u) && global_ns() - t0 > limit) {
            atomicCAS(&st->status, 0u, 5u /* FL_TIMEOUT */);
            return 0ull;
        }
        w = ld_tag(p, acq);
    }
    return w;
}

// Stages tagged words: for each virtual index v < nvirt, addr(v) is the word
// (nullptr: unused index) and dst(v) its slot in vals.  A thread issues up to
// STAGE_BATCH loads at once, then waits for its unpublished words one at a
// time (one poll in flight per thread keeps the traffic on the shared lines
// low; measured faster than re-polling all pending words together).
// Returns false on abort.
template <class AddrF, class DstF>
__device__ __forceinline__ bool stage_words(uint32_t nvirt, uint32_t tag, bool acq, DevStats* st,
                                            const DevParams* prm, float* vals, AddrF addr, DstF dst) {
    bool ok = true;
    for (uint32_t v0 = threadIdx.x; v0 < nvirt; v0 += STAGE_BATCH * CG_THREADS) {
        unsigned long long w[STAGE_BATCH];
#pragma unroll
        for (int k = 0; k < STAGE_BATCH; k++) {
            const uint32_t v = v0 + k * CG_THREADS;
            const unsigned long long* a = v < nvirt ? addr(v) : nullptr;
            w[k] = a ? ld_tag(a, acq) : 0ull;
        }
#pragma unroll
        for (int k = 0; k < STAGE_BATCH; k++) {
            const uint32_t v = v0 + k * CG_THREADS;
            const unsigned long long* a = v < nvirt ? addr(v) : nullptr;
            if (a && ok) {
                if ((uint32_t)(w[k] >> 32) != tag) {
                    w[k] = wait_tag(a, tag, st, acq, prm);
                    ok = (uint32_t)(w[k] >> 32) == tag;
                }
                vals[dst(v)] = __uint_as_float((uint32_t)w[k]);
            }
        }
    }
    return ok;
}

// ---------------------------------------------------------------------------
// Reductions

// Staging position of entry e of an exchange window: one pad word every 32
// entries.  Thread li sums its segment's entries in sequence; segments of
// equal length 16 (a common case) would start on two banks only, so
// without the pad the segment sums ran 16-way bank conflicted (0.85 vs
// 0.47 us per exchange at 128^3).
__device__ __forceinline__ uint32_t vpos(uint32_t e) { return e + (e >> 5); }

// float4 access to the CG vectors in the quad layout (16-byte aligned quads)
__device__ __forceinline__ float4 ld_f4(const float* a) { return *reinterpret_cast<const float4*>(a); }
__device__ __forceinline__ void st_f4(float* a, float4 v) { *reinterpret_cast<float4*>(a) = v; }
__device__ __forceinline__ float f4_at(const float4& v, int k) { return k == 0 ? v.x : k == 1 ? v.y : k == 2 ? v.z : v.w; }
__device__ __forceinline__ void f4_set(float4& v, int k, float x) {
    if (k == 0) v.x = x;
    else if (k == 1) v.y = x;
    else if (k == 2) v.z = x;
    else v.w = x;
}

// A block-uniform value read from shared memory at its use (not kept in a register).
__device__ __forceinline__ uint32_t vld(const uint32_t& x) { return *(const volatile uint32_t*)&x; }

// cg_reduce.wgsl:38-49 over s[0..255], evaluated by one warp: lane l forms the
// level-128 sums of indices l, l+32, l+64, l+96, the level-64 sums of l and
// l+32, the level-32 sum of l, then the same shuffle steps 16..1.  Operand
// order and pairing equal the 256-thread tree's.  Valid in lane 0.
__device__ __forceinline__ float chunk_tree(const float* s, uint32_t lane) {
    const float a0 = __fadd_rn(s[lane], s[lane + 128]);
    const float a1 = __fadd_rn(s[lane + 32], s[lane + 160]);
    const float a2 = __fadd_rn(s[lane + 64], s[lane + 192]);
    const float a3 = __fadd_rn(s[lane + 96], s[lane + 224]);
    float v = __fadd_rn(__fadd_rn(a0, a2), __fadd_rn(a1, a3));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = __fadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// Per-thread inner-product accumulator of the extended-precision forms:
// float-float (FL_CG_F64: exact products by two-product, sums by two-sum on
// the FP32 pipe) or IEEE double (FL_CG_F64_IEEE: f32 x f32 products are
// exact in double; sums, trees and combines in double).
template <int PREC>
struct AccT {
    using type = Df;
};
template <>
struct AccT<FL_CG_F64_IEEE> {
    using type = double;
};
__device__ __forceinline__ void acc_add(Df& a, float x, float y) { a = df_add(a, df_prod(x, y)); }
// f32 x f32 is exact in double, so one fma = the exact product added with one rounding
__device__ __forceinline__ void acc_add(double& a, float x, float y) { a = __fma_rn((double)x, (double)y, a); }
__device__ __forceinline__ double warp_sum_d(double v) {  // result in lane 0
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_allsum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
// a double's bits in two f32 slots (shared-memory staging and tagged words)
__device__ __forceinline__ float d_lo(double v) { return __int_as_float(__double2loint(v)); }
__device__ __forceinline__ float d_hi(double v) { return __int_as_float(__double2hiint(v)); }
__device__ __forceinline__ double d_of(float lo, float hi) { return __hiloint2double(__float_as_int(hi), __float_as_int(lo)); }

// FL_CG_F64: inner products accumulated in float-float (fl_device.cuh) by each
// thread, across its block and across blocks; alpha and beta are float-float
// quotients rounded to f32, and the stopping test compares float-float values.

// a / b rounded to f32: the f32 quotient plus one float-float correction.

// ---------------------------------------------------------------------------
// Plan

// One block of 256 threads.  Lists the active chunks by residue (segment li =
// chunks li, li+256, ... ascending), splits the list into G contiguous ranges
// of equal weight (liquid cells + CHUNK_WEIGHT per chunk), and reserves this solve's
// tag range.  When the 32-bit epoch would wrap, the exchange words are
// cleared first, so no stale word can carry a tag of a later solve.
__global__ void __launch_bounds__(CHUNK) k_cg_plan(DevBufs b, uint32_t G) {
    __shared__ uint32_t s_wc[CHUNK / 32], s_ww[CHUNK / 32];
    __shared__ int s_wrap;
    const DevParams& P = *b.prm;
    const uint32_t nchunks = P.nchunks;
    const uint32_t li = threadIdx.x, lane = li & 31, warp = li >> 5;
    uint32_t* hdr = b.cg_off;
    uint32_t* start = hdr + CHUNK + 3;
    uint32_t* spos = start + G + 1;
    uint32_t cnt = 0, wsum = 0;
    for (uint32_t c = li; c < nchunks; c += CHUNK) {
        const uint32_t f = b.chunk_flag[c];
        if (f) {
            cnt++;
            wsum += f + CHUNK_WEIGHT;
        }
    }
    uint32_t x = cnt, y = wsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t xa = __shfl_up_sync(0xffffffffu, x, o), ya = __shfl_up_sync(0xffffffffu, y, o);
        if (lane >= (uint32_t)o) {
            x += xa;
            y += ya;
        }
    }
    if (lane == 31) {
        s_wc[warp] = x;
        s_ww[warp] = y;
    }
    __syncthreads();
    uint32_t base = 0, wbase = 0, A = 0, W = 0;
    for (uint32_t w = 0; w < CHUNK / 32; w++) {
        if (w < warp) {
            base += s_wc[w];
            wbase += s_ww[w];
        }
        A += s_wc[w];
        W += s_ww[w];
    }
    const uint32_t off = base + x - cnt;
    hdr[li] = off;
    if (li == CHUNK - 1) hdr[CHUNK] = off + cnt;
    uint32_t pos = off;
    uint64_t XG = (uint64_t)(wbase + y - wsum) * G;  // G x the weight of all plan entries before `pos`
    // Blocks bb with X*G < bb*W <= X1*G start after the entry spanning
    // weights [X, X1).  X only grows along this thread's entries, so the
    // next such block is tracked incrementally from one division.
    uint64_t bb_next = W ? XG / W + 1 : 0, bbW = bb_next * W;
    for (uint32_t c = li; c < nchunks; c += CHUNK) {
        const uint32_t f = b.chunk_flag[c];
        if (!f) continue;
        b.cg_chunk[pos] = c;
        XG += (uint64_t)(f + CHUNK_WEIGHT) * G;
        for (; bbW <= XG; bb_next++, bbW += W) start[bb_next] = pos + 1;
        pos++;
    }
    if (A == 0)
        for (uint32_t bb = li; bb <= G; bb += CHUNK) start[bb] = 0;
    else if (li == 0)
        start[0] = 0;
    __syncthreads();
    // Slot layout: block bb's chunk partials at spos[bb] + j, each block's
    // range rounded up to whole 128-byte lines (16 words) and packed in block
    // order (a reader maps a line back to its block); used when all chunk
    // partials fit one staging window.  Else densely at plan entry s_bb + j
    // (spos[bb] = s_bb).  hdr[CHUNK + 2] = 1 for the line layout.
    const bool lines = A > 0 && A <= VAL_CAP;
    {
        const uint32_t per = (G + CHUNK - 1) / CHUNK;
        const uint32_t b0 = li * per < G ? li * per : G, b1 = b0 + per < G ? b0 + per : G;
        uint32_t mine = 0;
        for (uint32_t bb = b0; bb < b1; bb++) {
            const uint32_t mb = start[bb + 1] - start[bb];
            mine += lines ? (mb + 15u) & ~15u : mb;
        }
        uint32_t xs = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, xs, o);
            if (lane >= (uint32_t)o) xs += t;
        }
        if (lane == 31) s_wc[warp] = xs;
        __syncthreads();
        uint32_t run = xs - mine;
        for (uint32_t w = 0; w < warp; w++) run += s_wc[w];
        for (uint32_t bb = b0; bb < b1; bb++) {
            spos[bb] = run;
            const uint32_t mb = start[bb + 1] - start[bb];
            run += lines ? (mb + 15u) & ~15u : mb;
        }
        if (b0 < b1 && b1 == G) spos[G] = run;
        if (G == 0 && li == 0) spos[0] = 0;
    }
    // 2: every block owns 1..16 chunks, so block bb's line is simply line bb
    uint32_t mmin = 0xffffffffu, mmax = 0;
    for (uint32_t bb = li; bb < G; bb += CHUNK) {
        const uint32_t mb = start[bb + 1] - start[bb];
        mmin = mb < mmin ? mb : mmin;
        mmax = mb > mmax ? mb : mmax;
    }
    const int one_line = __syncthreads_and(mmin >= 1u && mmax <= 16u);
    if (li == 0) hdr[CHUNK + 2] = lines ? (one_line ? 2u : 1u) : 0u;
    if (li == 0) {
        const uint32_t span = 2u * (P.iters < TAG_SPAN_MAX ? P.iters : TAG_SPAN_MAX) + 4u;
        uint32_t e0 = (uint32_t)b.cg_x[0];
        int wrap = 0;
        if (e0 > 0xffffffffu - span) {
            wrap = 1;
            e0 = 0;
        }
        b.cg_x[0] = (unsigned long long)(e0 + span);
        hdr[CHUNK + 1] = e0;
        s_wrap = wrap;
    }
    __syncthreads();
    if (s_wrap) {
        const size_t n = cg_x_words(nchunks, G);
        for (size_t i = 1 + li; i < n; i += CHUNK) b.cg_x[i] = 0ull;
    }
}

// ---------------------------------------------------------------------------
// The solve

template <int PREC>
__global__ void __launch_bounds__(CG_THREADS, 1) k_cg(DevBufs b) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    CgShared& sh = *reinterpret_cast<CgShared*>(smem_raw);
    // Settings in registers: the L1 is invalidated at every exchange.
    const DevParams& P = *b.prm;
    const uint32_t C = P.C, iters = P.iters < TAG_SPAN_MAX ? P.iters : TAG_SPAN_MAX, nchunks = P.nchunks;
    const uint32_t nx = P.nx, nxy = P.nx * P.ny;  // grids hold at most 2^30 cells
    constexpr bool f64 = PREC != FL_CG_F32;       // no chunk trees: per-thread accumulators
    constexpr bool ieee = PREC == FL_CG_F64_IEEE;
    using Acc = typename AccT<PREC>::type;
    const float tol_sq = P.tol_sq;
    const double tol_sq_d = P.tol_sq_d;
    // Stopping test enabled: evaluated once (a double compare in the loop
    // would run on the FP64 pipe in every warp of every iteration).
    const bool stop_on = f64 ? P.tol_sq_d > 0.0 : P.tol_sq > 0.0f;
    DevStats* st = b.st;
    const uint32_t G = gridDim.x, tid = threadIdx.x, lane = tid & 31u, warp = tid >> 5;
    float* __restrict__ r = b.r;
    float* __restrict__ p = b.p;
    float* __restrict__ q = b.q;
    const uint16_t* __restrict__ cinfo = b.cinfo;
    const uint32_t* __restrict__ plan = b.cg_chunk;
    const uint32_t* hdr = b.cg_off;
    for (uint32_t i = tid; i <= CHUNK; i += CG_THREADS) sh.off[i] = hdr[i];
    const uint32_t tag_base = hdr[CHUNK + 1];
    // Block-uniform values read only by the exchanges live in shared memory
    // (sh.layout, sh.nslot, sh.off[CHUNK]) rather than in registers: the cell
    // loops are at the 64-register limit of a 1024-thread block.
    if (tid == 0) sh.layout = hdr[CHUNK + 2];
    const uint32_t* bstart = hdr + CHUNK + 3;
    const uint32_t* spos = bstart + G + 1;
    for (uint32_t i = tid; i <= G; i += CG_THREADS) {
        sh.bstart[i] = bstart[i];
        sh.spos[i] = spos[i];
    }
    const uint32_t s0 = bstart[blockIdx.x], s1 = bstart[blockIdx.x + 1];
    const uint32_t m = s1 - s0;  // this block's chunks: plan entries [s0, s1)
    if (tid == 0) sh.nslot = spos[G];
    __syncthreads();
    if (sh.layout != 0u)  // line -> owning block
        for (uint32_t bb = tid; bb < G; bb += CG_THREADS)
            for (uint32_t L = sh.spos[bb] >> 4; L < sh.spos[bb + 1] >> 4; L++) sh.lineblk[L] = (uint16_t)bb;
    // Every exchange area starts on a 128-byte line (the pool is 256-byte
    // aligned): a block's slot line must not share a physical line with a
    // neighbour's (measured 8-11 % of the solve at 128^3 when it did).
    const size_t nslot = (((size_t)nchunks + 15) & ~(size_t)15) + 16 * (size_t)G;
    unsigned long long* slotA = b.cg_x + 16;       // d.q chunk partials
    unsigned long long* slotB = slotA + nslot;     // r.r chunk partials
    unsigned long long* wordA = slotB + nslot;     // FL_CG_F64: {hi, lo} of block b at 16*b
    unsigned long long* wordB = wordA + 16 * (size_t)G;
    unsigned long long* segA = wordB + 16 * (size_t)G;  // two-hop exchanges: 256 segment sums each
    unsigned long long* segB = segA + CHUNK;
    const uint32_t mch = m < KCH ? m : KCH;
    for (uint32_t j = tid; j < mch; j += CG_THREADS) sh.chunk[j] = plan[s0 + j];
    for (uint32_t i = tid; i < KT * CHUNK; i += CG_THREADS) (&sh.tree[0][0])[i] = 0.0f;
    __syncthreads();
    const uint32_t A = sh.off[CHUNK];

    // Quad layout: when rows are a multiple of four cells and the vectors are
    // 16-byte aligned, every aligned run of four cells (a quad) and its +-y
    // and +-z rows load as float4, so the cell loops issue one load per four
    // cells per vector instead of one per cell.  The listing then holds the
    // quads with a liquid cell (QCAP of them), each with its four cells'
    // stencil words; otherwise the liquid cells one by one (CELL_CAP).
    //
    // A block whose cells qualify for the resident operands (one pass, at
    // most 2 * CG_THREADS liquid cells: chunk_flag counts them, saturated at
    // 255, so 256 bounds a full chunk) lists cells: with every operand in
    // shared memory the cell form was faster (CG stage at 128^3 1.69 vs
    // 1.75 ms per substep); larger blocks take quads (256^3 8.01 vs 8.72 ms).
    uint32_t liq_bound = 0;
    if (warp == 0 && m <= KT) {
        for (uint32_t j = lane; j < m; j += 32) {
            const uint32_t f = b.chunk_flag[sh.chunk[j]];
            liq_bound += f == 255u ? 256u : f;
        }
        liq_bound = __reduce_add_sync(0xffffffffu, liq_bound);
        if (lane == 0) sh.u_lb = liq_bound;
    }
    __syncthreads();
    const bool res_fit = m <= KT && sh.u_lb <= 2u * CG_THREADS && A <= RES_MAX_A;
    __syncthreads();
    const bool quads = !res_fit && (nx & 3u) == 0u &&
                       (((uintptr_t)p | (uintptr_t)r | (uintptr_t)q | (uintptr_t)b.dA | (uintptr_t)b.dB) & 15u) == 0u &&
                       ((uintptr_t)cinfo & 7u) == 0u;
    uint2* const qlist = reinterpret_cast<uint2*>(sh.cell);
    uint32_t ncell = 0, mc = 0;
    if (quads) {
        // 16 chunks (64 quads each) per round, in (chunk, quad) order; entry
        // x = stencil words of cells 0..2 (10 bits each), y = cell 3's word |
        // quad << 10 | chunk slot << 16.
        const uint32_t lt_mask = (1u << lane) - 1u;
        for (uint32_t j0 = 0; j0 < mch; j0 += 16) {
            if ((j0 % KT) == 0 && tid == 0) sh.pass_off[j0 / KT] = ncell;
            const uint32_t j = j0 + (tid >> 6), qd = tid & 63u;
            uint2 info = make_uint2(0u, 0u);
            if (j < mch) {
                const uint32_t c0 = sh.chunk[j] * CHUNK + 4u * qd;
                if (c0 < C) info = *reinterpret_cast<const uint2*>(cinfo + c0);  // C is a multiple of 4
            }
            const uint32_t w0 = info.x & 1023u, w1 = (info.x >> 16) & 1023u, w2 = info.y & 1023u,
                           w3 = (info.y >> 16) & 1023u;
            const bool liq = ((w0 | w1 | w2 | w3) & 1u) != 0u;
            const uint32_t bal = __ballot_sync(0xffffffffu, liq);
            if (lane == 0) sh.wcnt[warp] = (uint32_t)__popc(bal);
            __syncthreads();
            uint32_t before = 0, total = 0;
            for (uint32_t w = 0; w < (uint32_t)CG_WARPS; w++) {
                const uint32_t n = sh.wcnt[w];
                if (w < warp) before += n;
                total += n;
            }
            __syncthreads();
            if (ncell + total > QCAP) break;  // uniform: every thread sees the same totals
            if (liq) qlist[ncell + before + __popc(bal & lt_mask)] = make_uint2(w0 | (w1 << 10) | (w2 << 20), w3 | (qd << 10) | (j << 16));
            ncell += total;
            mc = j0 + 16 < mch ? j0 + 16 : mch;
        }
    } else {
        // List the liquid cells of chunks [0, mc), four chunks per round, in
        // (chunk, cell) order; stop before CELL_CAP would be exceeded.
        const uint32_t lt_mask = (1u << lane) - 1u;
        for (uint32_t j0 = 0; j0 < mch; j0 += 4) {
            if ((j0 % KT) == 0 && tid == 0) sh.pass_off[j0 / KT] = ncell;
            const uint32_t j = j0 + (tid >> 8), cl = tid & (CHUNK - 1);
            uint32_t info = 0;
            if (j < mch) {
                const uint32_t c = sh.chunk[j] * CHUNK + cl;
                if (c < C) info = cinfo[c];
            }
            const bool liq = info & 1u;
            const uint32_t bal = __ballot_sync(0xffffffffu, liq);
            if (lane == 0) sh.wcnt[warp] = (uint32_t)__popc(bal);
            __syncthreads();
            uint32_t before = 0, total = 0;
            for (uint32_t w = 0; w < (uint32_t)CG_WARPS; w++) {
                const uint32_t n = sh.wcnt[w];
                if (w < warp) before += n;
                total += n;
            }
            __syncthreads();
            if (ncell + total > CELL_CAP) break;  // uniform: every thread sees the same totals
            if (liq) sh.cell[ncell + before + __popc(bal & lt_mask)] = info | (cl << 10) | (j << 18);
            ncell += total;
            mc = j0 + 4 < mch ? j0 + 4 : mch;
        }
    }
    const uint32_t npc = (mc + KT - 1) / KT;  // cached passes
    if (tid == 0) sh.pass_off[npc] = ncell;
    // One pass in all: non-liquid tree slots stay zero for the whole solve.
    const bool multi = npc > 1 || mc < m;
    __syncthreads();
    // Resident operands: thread t owns listed cells t and t + CG_THREADS in
    // both phases, so their {d, r, q, p} stay in shared memory for the whole
    // solve.  Phase 2 then loads nothing from global memory, q is never
    // written there, and p is written once at the end; d (phase 1) and r
    // (phase 2) are still stored for the neighbours in other blocks.  At 128^3
    // this took the update phase from 2300 to 1640 cycles per iteration.
    const bool res = !quads && !multi && ncell <= 2u * CG_THREADS && A <= RES_MAX_A;
    float4* const rv4 = reinterpret_cast<float4*>(sh.vals + VALS_HALF);
    if (tid == 0) {
        sh.u_s0 = s0;
        sh.u_m = m;
        sh.u_mc = mc;
        sh.u_npc = npc;
        sh.u_ncell = ncell;
        sh.u_res = res ? 1u : 0u;
        sh.u_quad = quads ? 1u : 0u;
    }
    if (res)
        for (uint32_t tu = tid; tu < ncell; tu += CG_THREADS) {
            const uint32_t e = sh.cell[tu];
            const uint32_t c = sh.chunk[e >> 18] * CHUNK + ((e >> 10) & 255u);
            rv4[tu] = make_float4(b.dA[c], r[c], 0.0f, p[c]);
        }

    // The scalars that follow an exchange, from its sum v: post 1 alpha
    // (cg_alpha.wgsl:17-22, sc = rs_old / v), post 2 beta and the stopping test
    // (cg_beta.wgsl:16-30, sc = v / rs_old, dn).  Evaluated once, by lane 0 of
    // warp 0, and broadcast through sh.scal.
    auto post_f32 = [&](int post, float v) {
        const float rs_old = sh.rs_hi;
        float sc = 0.0f;
        bool dn = false;
        if (post == 1) sc = fabsf(v) > 1e-30f ? __fdiv_rn(rs_old, v) : 0.0f;
        if (post != 1) sh.rs_hi = v;  // the initial r.r, or rs_new
        if (post == 2) {
            sc = rs_old > 1e-30f ? __fdiv_rn(v, rs_old) : 0.0f;
            dn = stop_on && v <= sh.thr_f;
        }
        sh.scal[0] = v;
        sh.scal[1] = sc;
        sh.scal[2] = dn ? 1.0f : 0.0f;
    };
    // FL_CG_F32 scalar: the segment sums of cg_reduce_final.wgsl, then its
    // 256-wide tree, evaluated by warp 0 (32 warps evaluating it redundantly
    // competed for issue slots: 0.3 us per exchange at 128^3).  Every thread
    // receives the sum (out) and the post scalars (sc, dn).  Returns false on
    // abort.  Three ways to the segment sums:
    //  * line layouts (all partials fit one window): every block stages every
    //    block's slot line and sums all 256 segments itself (one hop);
    //  * plan-order layout (more active chunks than one window: every block
    //    reading every partial cost 6-9 us per exchange at 256^3): two hops.
    //    Block bb owns segments bb, bb + G, ...; one warp per owned segment
    //    polls its partials (plan entries off[li]..off[li+1]), sums them in
    //    order in lane 0 and publishes the segment sum as a tagged word in
    //    `segw` (release on the exchange after which vector writes are read:
    //    the owners' acquires and releases carry every block's writes on);
    //    then every block polls the 256 segment words;
    //  * `x` == nullptr: the initial residual partials part_rr, indexed by
    //    chunk, staged in windows.
    auto reduce_f32 = [&](const unsigned long long* x, unsigned long long* segw, uint32_t tag, bool acq, int post,
                          float& out, float& sc, bool& dn) -> bool {
        float acc = 0.0f;
        bool ok = true;
        const uint32_t A = sh.off[CHUNK];
        if (x && sh.layout == 0u) {
            float* buf = sh.vals + warp * 256u;  // per-warp staging of 256 partials
            for (uint32_t li = blockIdx.x + warp * G; li < (uint32_t)CHUNK; li += CG_WARPS * G) {
                const uint32_t lo = sh.off[li], hi = sh.off[li + 1];
                float s = 0.0f;
                for (uint32_t e0 = lo; e0 < hi; e0 += 256u) {
                    // all eight polls of a lane in flight, then the waits (the
                    // wait after each load serialised them: one round trip per word)
                    unsigned long long w[8];
#pragma unroll
                    for (int k2 = 0; k2 < 8; k2++) {
                        const uint32_t e = e0 + lane + 32u * k2;
                        w[k2] = e < hi ? ld_tag(x + e, acq) : 0ull;
                    }
#pragma unroll
                    for (int k2 = 0; k2 < 8; k2++) {
                        const uint32_t e = e0 + lane + 32u * k2;
                        if (e < hi && (uint32_t)(w[k2] >> 32) != tag && ok) {
                            w[k2] = wait_tag(x + e, tag, st, acq, b.prm);
                            ok = (uint32_t)(w[k2] >> 32) == tag;
                        }
                        buf[lane + 32u * k2] = e < hi ? __uint_as_float((uint32_t)w[k2]) : 0.0f;
                    }
                    __syncwarp();
                    if (lane == 0) {  // cg_reduce_final.wgsl:29-36: in plan order, from +0
                        // entries past the segment's end were staged as +0,
                        // which leaves s (never -0) unchanged
                        const uint32_t n = hi - e0 < 256u ? hi - e0 : 256u;
                        for (uint32_t j = 0; j < n; j += 16) {
                            float t16[16];
#pragma unroll
                            for (int k2 = 0; k2 < 16; k2++) t16[k2] = buf[j + k2];
#pragma unroll
                            for (int k2 = 0; k2 < 16; k2++) s = __fadd_rn(s, t16[k2]);
                        }
                    }
                    __syncwarp();
                }
                // a segment whose partials did not all arrive is not published
                if (__all_sync(0xffffffffu, ok) && lane == 0) publish(segw + li, tag, s, acq);
            }
            if (tid < (uint32_t)CHUNK) {
                unsigned long long w = ld_tag(segw + tid, acq);
                if ((uint32_t)(w >> 32) != tag && ok) {
                    w = wait_tag(segw + tid, tag, st, acq, b.prm);
                    ok = (uint32_t)(w >> 32) == tag;
                }
                sh.seg[tid] = __uint_as_float((uint32_t)w);
            }
            if (__syncthreads_or(!ok)) return false;
        } else {
        for (uint32_t w0 = 0; w0 < A; w0 += VAL_CAP) {
            const uint32_t wn = A - w0 < VAL_CAP ? A - w0 : VAL_CAP;
            if (x && sh.layout != 0u) {  // one window (A <= VAL_CAP): walk the blocks' lines.  Written
                                         // out rather than through stage_words: measured 0.5 ms/step faster.
                const uint32_t nslot_used = sh.nslot;
                const bool one_line = sh.layout == 2u;
                for (uint32_t v0 = tid; v0 < nslot_used; v0 += LINE_BATCH * CG_THREADS) {
                    unsigned long long w[LINE_BATCH];
                    uint32_t dst[LINE_BATCH];
#pragma unroll
                    for (int k2 = 0; k2 < LINE_BATCH; k2++) {
                        const uint32_t v = v0 + k2 * CG_THREADS;
                        const uint32_t bb = v < nslot_used ? (one_line ? v >> 4 : (uint32_t)sh.lineblk[v >> 4]) : 0u;
                        const uint32_t j = v - sh.spos[bb];
                        const bool use = v < nslot_used && j < sh.bstart[bb + 1] - sh.bstart[bb];
                        dst[k2] = use ? sh.bstart[bb] + j : 0xffffffffu;
                        w[k2] = use ? ld_tag(x + v, acq) : 0ull;
                    }
#pragma unroll
                    for (int k2 = 0; k2 < LINE_BATCH; k2++) {
                        if (dst[k2] != 0xffffffffu && ok) {
                            if ((uint32_t)(w[k2] >> 32) != tag) {
                                w[k2] = wait_tag(x + v0 + k2 * CG_THREADS, tag, st, acq, b.prm);
                                ok = (uint32_t)(w[k2] >> 32) == tag;
                            }
                            sh.vals[vpos(dst[k2])] = __uint_as_float((uint32_t)w[k2]);
                        }
                    }
                }
            } else {
                for (uint32_t i = tid; i < wn; i += CG_THREADS) sh.vals[vpos(i)] = b.part_rr[plan[w0 + i]];
            }
            if (__syncthreads_or(!ok)) return false;
            if (tid < (uint32_t)CHUNK) {
                // 16 loads first (past the segment's end: +0), then the
                // sequential adds.  acc starts at +0 and a sum of floats is
                // -0 only when both terms are, so acc is never -0 and adding
                // +0 leaves it unchanged: the fold equals the loop over
                // [lo, hi) exactly, with no per-lane tail loop.
                const uint32_t lo = sh.off[tid] > w0 ? sh.off[tid] : w0;
                const uint32_t hi = sh.off[tid + 1] < w0 + wn ? sh.off[tid + 1] : w0 + wn;
                for (uint32_t e = lo; e < hi; e += 16) {
                    float v[16];
#pragma unroll
                    for (int k2 = 0; k2 < 16; k2++) v[k2] = e + k2 < hi ? sh.vals[vpos(e - w0 + k2)] : 0.0f;
#pragma unroll
                    for (int k2 = 0; k2 < 16; k2++) acc = __fadd_rn(acc, v[k2]);
                }
            }
            if (w0 + wn < A) __syncthreads();
        }
        if (tid < (uint32_t)CHUNK) sh.seg[tid] = acc;
        __syncthreads();
        }
        if (warp == 0) {
            const float v = chunk_tree(sh.seg, lane);
            if (lane == 0) post_f32(post, v);
        }
        __syncthreads();
        out = sh.scal[0];
        sc = sh.scal[1];
        dn = sh.scal[2] != 0.0f;
        return true;
    };
    // FL_CG_F64 scalar: the blocks' float-float partials (two words of block b
    // at 16*b), summed by warp 0 in a fixed order (lanes stride over blocks,
    // then a shuffle tree); lane 0 evaluates the post scalars (alpha, or beta
    // and the stopping test, from rs_old) and broadcasts them with the sum.
    auto reduce_df = [&](const unsigned long long* words, uint32_t tag, bool acq, int post, float& sc,
                         bool& dn) -> bool {
        const bool ok = stage_words(
            2 * G, tag, acq, st, b.prm, sh.vals,
            [&](uint32_t v) -> const unsigned long long* { return words + (v >> 1) * 16u + (v & 1u); },
            [&](uint32_t v) -> uint32_t { return v; });
        if (__syncthreads_or(!ok)) return false;
        if (ieee && warp == 0) {  // the blocks' doubles, in the same fixed order
            double v = 0.0;
            for (uint32_t bb = lane; bb < G; bb += 32) v += d_of(sh.vals[2 * bb], sh.vals[2 * bb + 1]);
            v = warp_sum_d(v);
            if (lane == 0) {
                const double rs_old = sh.rs_d;
                float scv = 0.0f;
                bool d2 = false;
                if (post == 1) scv = fabs(v) > 1e-30 ? (float)(rs_old / v) : 0.0f;
                if (post == 2) {
                    scv = rs_old > 1e-30 ? (float)(v / rs_old) : 0.0f;
                    d2 = stop_on && v <= sh.thr_d;
                    sh.rs_d = v;
                }
                sh.scal[2] = scv;
                sh.scal[3] = d2 ? 1.0f : 0.0f;
            }
        } else if (warp == 0) {
            Df acc = {0.0f, 0.0f};
            for (uint32_t bb = lane; bb < G; bb += 32) acc = df_add(acc, Df{sh.vals[2 * bb], sh.vals[2 * bb + 1]});
            acc = warp_sum_df(acc);
            if (lane == 0) {
                const Df rs_old = {sh.rs_hi, sh.rs_lo};
                float scv = 0.0f;
                bool d2 = false;
                if (post == 1) scv = fabsf(acc.hi) > 1e-30f ? df_div(rs_old, acc) : 0.0f;
                if (post == 2) {
                    scv = rs_old.hi > 1e-30f ? df_div(acc, rs_old) : 0.0f;
                    d2 = stop_on && df_le(acc, Df{sh.thr_dh, sh.thr_dl});
                    sh.rs_hi = acc.hi;
                    sh.rs_lo = acc.lo;
                }
                sh.scal[0] = acc.hi;
                sh.scal[1] = acc.lo;
                sh.scal[2] = scv;
                sh.scal[3] = d2 ? 1.0f : 0.0f;
            }
        }
        __syncthreads();
        sc = sh.scal[2];
        dn = sh.scal[3] != 0.0f;
        return true;
    };
    // Block partial published as two tagged words on the block's line: the
    // float-float {hi, lo}, or a double's low and high 32 bits.
    auto publish_df = [&](Acc acc, unsigned long long* words, uint32_t tag, bool rel) {
        if constexpr (ieee) {
            // The FP64 pipe (about 2 lane-operations per clock per SM) is the
            // bound: warp 0 sums the 1024 thread partials (lane l: partials l,
            // l + 32, ... in sequence, then a 5-level tree) instead of a tree
            // in every warp (36 double adds per block instead of 160).  The
            // partials are staged in the chunk-tree buffer, which the
            // extended-precision forms do not use (the exchange window is
            // written by the other warps' polls while warp 0 reads).
            double* part = reinterpret_cast<double*>(&sh.tree[0][0]);
            part[tid] = acc;
            __syncthreads();
            if (warp == 0) {
                double s = 0.0;
                for (uint32_t t2 = lane; t2 < (uint32_t)CG_THREADS; t2 += 32) s += part[t2];
                const double v = warp_sum_d(s);
                const float lo = __shfl_sync(0xffffffffu, d_lo(v), 0), hi = __shfl_sync(0xffffffffu, d_hi(v), 0);
                if (lane < 2) publish(words + 16 * blockIdx.x + lane, tag, lane ? hi : lo, rel);
            }
        } else {
            acc = warp_sum_df(acc);
            if (lane == 0) {
                sh.red[2 * warp] = acc.hi;
                sh.red[2 * warp + 1] = acc.lo;
            }
            __syncthreads();
            if (warp == 0) {
                Df v = {sh.red[2 * lane], sh.red[2 * lane + 1]};
                v = warp_sum_df(v);
                // lanes 0 and 1 store {hi, lo} in one instruction (the FP64-reduction
                // CG stage measured 1.96-1.98 vs 2.10-2.13 ms per substep at 128^3
                // against two stores by lane 0: readers saw hi before lo)
                const float lo = __shfl_sync(0xffffffffu, v.lo, 0);
                if (lane < 2) publish(words + 16 * blockIdx.x + lane, tag, lane ? lo : v.hi, rel);
            }
        }
    };
    // Warp w evaluates the trees of chunks j0 + w and j0 + w + 32 of the pass
    // into shared memory (sh.red, KT floats); warp 0 then publishes them
    // together, one store instruction per 32 words, so a polling block finds
    // a block's slot line complete in one read instead of filling in word by
    // word (the CG stage measured 2.06 vs 2.21-2.26 ms per substep at 128^3
    // against one store per tree warp).
    // With `rel`, warp 0 issues the release fence (after the barrier that
    // orders the block's vector writes before it) while warps 1.. evaluate the
    // trees, and then stores the words relaxed: fence + strong store in one
    // thread is a release pattern, and the fence's wait for the block's
    // stores overlaps the trees (1-2 % of the CG stage at 128^3 against a
    // release store after the trees).
    static_assert(2 * CG_WARPS == KT, "sh.red stages one pass of chunk trees");
    // With `zero` (passes that share the tree rows), the tree warps clear
    // the rows they read, so the next pass starts on zeroed rows without a
    // clearing loop and barrier of its own; the next pass's first barrier
    // orders this pass's publication before its trees rewrite sh.red.
    auto publish_trees = [&](uint32_t j0, uint32_t nb, unsigned long long* slots, uint32_t tag, bool rel, bool zero) {
        __syncthreads();
        if (rel && warp == 0) {
            asm volatile("fence.acq_rel.gpu;" ::: "memory");
        } else {
            const uint32_t w0 = rel ? warp - 1 : warp, nw = rel ? CG_WARPS - 1 : CG_WARPS;
            for (uint32_t j = w0; j < nb; j += nw) {
                const float v = chunk_tree(sh.tree[j], lane);
                if (lane == 0) sh.red[j] = v;
                if (zero) {
                    __syncwarp();
                    float4* row = reinterpret_cast<float4*>(sh.tree[j]);
                    row[lane] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                    row[lane + 32] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                }
            }
        }
        __syncthreads();
        if (warp == 0)
            for (uint32_t j = lane; j < nb; j += 32) publish(slots + sh.spos[blockIdx.x] + j0 + j, tag, sh.red[j], false);
    };

    // Initial residual norm (cg_init.wgsl + cg_reduce of r.r).
    float rs_init_f = 0.0f;
    Df rs_init_d = {0.0f, 0.0f};
    if (ieee) {  // the chunks' float-float partials (exact in double), summed in double
        double acc = 0.0;
        for (uint32_t e = tid; e < A; e += CG_THREADS) {
            const float2 v = b.chunk_rr_df[plan[e]];
            acc += (double)v.x + (double)v.y;
        }
        acc = warp_allsum_d(acc);
        if (lane == 0) {
            sh.red[2 * warp] = d_lo(acc);
            sh.red[2 * warp + 1] = d_hi(acc);
        }
        __syncthreads();
        const double rs0 = warp_allsum_d(d_of(sh.red[2 * lane], sh.red[2 * lane + 1]));
        if (tid == 0) {
            sh.rs_d = rs0;
            sh.thr_d = P.thr_abs ? P.thr_abs_d : tol_sq_d * rs0;
            if (blockIdx.x == 0) st->rs_init = rs0;
        }
        __syncthreads();  // sh.red is reused
    } else if (f64) {
        Df acc = {0.0f, 0.0f};
        for (uint32_t e = tid; e < A; e += CG_THREADS) {
            const float2 v = b.chunk_rr_df[plan[e]];
            acc = df_add(acc, Df{v.x, v.y});
        }
        acc = warp_allsum_df(acc);
        if (lane == 0) {
            sh.red[2 * warp] = acc.hi;
            sh.red[2 * warp + 1] = acc.lo;
        }
        __syncthreads();
        rs_init_d = warp_allsum_df(Df{sh.red[2 * lane], sh.red[2 * lane + 1]});
        // stopping threshold tol^2 * rs_init (or the absolute one), once per solve
        if (tid == 0) {
            sh.rs_hi = rs_init_d.hi;
            sh.rs_lo = rs_init_d.lo;
            const double thr = P.thr_abs ? P.thr_abs_d : tol_sq_d * df_to_double(rs_init_d);
            sh.thr_dh = (float)thr;
            sh.thr_dl = (float)(thr - (double)sh.thr_dh);
        }
        __syncthreads();  // sh.red is reused
    } else {
        float sc0;
        bool dn0;
        reduce_f32(nullptr, nullptr, 0u, false, 0, rs_init_f, sc0, dn0);  // also sets sh.rs_hi
    }
    // Thresholds and rs_init are stored once here, not held in registers
    // through the loop.  f32: tol^2 * rs_init (cg_beta.wgsl:25-30) or the
    // absolute threshold.
    if (tid == 0) {
        if (!f64) sh.thr_f = P.thr_abs ? P.thr_abs_f : __fmul_rn(tol_sq, rs_init_f);
        if (blockIdx.x == 0 && !ieee) st->rs_init = f64 ? df_to_double(rs_init_d) : (double)rs_init_f;
    }
    __syncthreads();

    float beta = 0.0f;
    uint32_t k = 0, tag = tag_base;
    for (uint32_t it = 0; it < iters; it++) {
        float* __restrict__ d_cur = (it & 1u) ? b.dB : b.dA;
        const float* __restrict__ d_prev = (it & 1u) ? b.dA : b.dB;
        const bool first = it == 0;
        const float* __restrict__ d_src = first ? d_cur : d_prev;
        // ---------------- phase 1: direction + SpMV + d.q ----------------
        Acc acc{};
        tag++;
        if (vld(sh.u_res)) {  // resident operands: own d, r from shared memory, neighbours' from global
            uint32_t ent[2], cc[2];
            float rv[2][7], dv[2][7];
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const uint32_t tu = tid + u * CG_THREADS;
                const bool ok = tu < vld(sh.u_ncell);
                ent[u] = ok ? sh.cell[tu] : 0u;
                cc[u] = sh.chunk[ent[u] >> 18] * CHUNK + ((ent[u] >> 10) & 255u);
                const uint32_t c = cc[u];
                const float2 own = ok ? *reinterpret_cast<const float2*>(&rv4[tu]) : make_float2(0.0f, 0.0f);
                dv[u][0] = own.x;
                rv[u][0] = own.y;
                const uint32_t nb6[6] = {c - 1, c + 1, c - nx, c + nx, c - nxy, c + nxy};
#pragma unroll
                for (int s = 1; s < 7; s++) {
                    const bool need = ok && ((ent[u] >> s) & 1u);
                    dv[u][s] = need ? d_src[nb6[s - 1]] : 0.0f;
                    rv[u][s] = (need && !first) ? r[nb6[s - 1]] : 0.0f;
                }
            }
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const uint32_t tu = tid + u * CG_THREADS;
                if (tu >= vld(sh.u_ncell)) continue;
                const uint32_t info = ent[u];
                const float dc = first ? dv[u][0] : __fadd_rn(rv[u][0], __fmul_rn(beta, dv[u][0]));  // cg_dir.wgsl:30
                float sum = 0.0f;
#pragma unroll
                for (int s = 1; s < 7; s++) {
                    if ((info >> s) & 1u) {
                        const float dn = first ? dv[u][s] : __fadd_rn(rv[u][s], __fmul_rn(beta, dv[u][s]));
                        sum = __fadd_rn(sum, dn);
                    }
                }
                const float qc = __fsub_rn(__fmul_rn((float)((info >> 7) & 7u), dc), sum);  // cg_spmv.wgsl:46-68
                if (!first) d_cur[cc[u]] = dc;
                rv4[tu].x = dc;
                rv4[tu].z = qc;
                if (f64) acc_add(acc, dc, qc);
                else sh.tree[info >> 18][(info >> 10) & 255u] = __fmul_rn(dc, qc);
            }
            if (!f64) publish_trees(0, vld(sh.u_mc), slotA, tag, false, false);
        } else {
            uint32_t j0 = 0;
            for (uint32_t ps = 0; ps < vld(sh.u_npc); ps++, j0 += KT) {
                const uint32_t nb = vld(sh.u_mc) - j0 < KT ? vld(sh.u_mc) - j0 : KT;
                const uint32_t beg = sh.pass_off[ps], end = sh.pass_off[ps + 1];
                if (vld(sh.u_quad)) {
                    for (uint32_t t = beg + tid; t < end; t += CG_THREADS) {
                        // One quad: cells c0..c0+3 of one row.  Its own d, r and
                        // its +-y, +-z rows as float4, the two x edges as scalars;
                        // the -x/+x neighbours inside the quad are its own cells.
                        const uint2 e = qlist[t];
                        const uint32_t w[4] = {e.x & 1023u, (e.x >> 10) & 1023u, (e.x >> 20) & 1023u, e.y & 1023u};
                        const uint32_t jq = e.y >> 16, qd = (e.y >> 10) & 63u;
                        const uint32_t c0 = sh.chunk[jq] * CHUNK + 4u * qd;
                        const uint32_t any = w[0] | w[1] | w[2] | w[3];
                        const float4 z4 = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
                        const float4 dc4 = ld_f4(d_src + c0);
                        const float4 rc4 = first ? z4 : ld_f4(r + c0);
                        const bool xm = (w[0] & 2u) != 0u, xp = (w[3] & 4u) != 0u;
                        const float dxm = xm ? d_src[c0 - 1] : 0.0f, rxm = (xm && !first) ? r[c0 - 1] : 0.0f;
                        const float dxp = xp ? d_src[c0 + 4] : 0.0f, rxp = (xp && !first) ? r[c0 + 4] : 0.0f;
                        float4 dn4[4], rn4[4];  // -y, +y, -z, +z rows
                        const uint32_t off4[4] = {c0 - nx, c0 + nx, c0 - nxy, c0 + nxy};
#pragma unroll
                        for (int s = 0; s < 4; s++) {
                            const bool need = (any >> (3 + s)) & 1u;
                            dn4[s] = need ? ld_f4(d_src + off4[s]) : z4;
                            rn4[s] = (need && !first) ? ld_f4(r + off4[s]) : z4;
                        }
                        // cg_dir.wgsl:30 for the quad, the edges and the rows,
                        // then cg_spmv.wgsl:46-68 per cell (order -x,+x,-y,+y,-z,+z)
                        auto dir = [&](float dv, float rv) { return first ? dv : __fadd_rn(rv, __fmul_rn(beta, dv)); };
                        const float dq[4] = {dir(dc4.x, rc4.x), dir(dc4.y, rc4.y), dir(dc4.z, rc4.z), dir(dc4.w, rc4.w)};
                        const float dm = dir(dxm, rxm), dp = dir(dxp, rxp);
                        float ov[4], oq[4], op[4];
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            const uint32_t wk = w[k];
                            float sum = 0.0f;
                            if (wk & 2u) sum = __fadd_rn(sum, k == 0 ? dm : dq[k > 0 ? k - 1 : 0]);
                            if (wk & 4u) sum = __fadd_rn(sum, k == 3 ? dp : dq[k < 3 ? k + 1 : 3]);
#pragma unroll
                            for (int s = 0; s < 4; s++)
                                if ((wk >> (3 + s)) & 1u) sum = __fadd_rn(sum, dir(f4_at(dn4[s], k), f4_at(rn4[s], k)));
                            const bool liq = (wk & 1u) != 0u;
                            const float qc = __fsub_rn(__fmul_rn((float)((wk >> 7) & 7u), dq[k]), sum);
                            ov[k] = liq ? dq[k] : 0.0f;
                            oq[k] = liq ? qc : 0.0f;
                            op[k] = liq ? __fmul_rn(dq[k], qc) : 0.0f;
                            if (f64 && liq) acc_add(acc, dq[k], qc);
                        }
                        if (!first) st_f4(d_cur + c0, make_float4(ov[0], ov[1], ov[2], ov[3]));
                        st_f4(q + c0, make_float4(oq[0], oq[1], oq[2], oq[3]));
                        if (!f64) *reinterpret_cast<float4*>(&sh.tree[jq - j0][4u * qd]) = make_float4(op[0], op[1], op[2], op[3]);
                    }
                } else
                for (uint32_t t = beg + tid; t < end; t += 2 * CG_THREADS) {
                    // two cells in flight: all loads first
                    uint32_t ent[2], cc[2];
                    float rv[2][7], dv[2][7];
#pragma unroll
                    for (int u = 0; u < 2; u++) {
                        const uint32_t tu = t + u * CG_THREADS;
                        const bool ok = tu < end;
                        ent[u] = ok ? sh.cell[tu] : 0u;
                        cc[u] = sh.chunk[ent[u] >> 18] * CHUNK + ((ent[u] >> 10) & 255u);
                        const uint32_t c = cc[u];
                        const uint32_t nb7[7] = {c, c - 1, c + 1, c - nx, c + nx, c - nxy, c + nxy};
#pragma unroll
                        for (int s = 0; s < 7; s++) {
                            const bool need = ok && (s == 0 || ((ent[u] >> s) & 1u));
                            dv[u][s] = need ? d_src[nb7[s]] : 0.0f;
                            rv[u][s] = (need && !first) ? r[nb7[s]] : 0.0f;
                        }
                    }
#pragma unroll
                    for (int u = 0; u < 2; u++) {
                        if (t + u * CG_THREADS >= end) continue;
                        const uint32_t info = ent[u];
                        // cg_dir.wgsl:30 for the cell and its liquid neighbours,
                        // then cg_spmv.wgsl:46-68 (order -x,+x,-y,+y,-z,+z)
                        const float dc = first ? dv[u][0] : __fadd_rn(rv[u][0], __fmul_rn(beta, dv[u][0]));
                        float sum = 0.0f;
#pragma unroll
                        for (int s = 1; s < 7; s++) {
                            if ((info >> s) & 1u) {
                                const float dn = first ? dv[u][s] : __fadd_rn(rv[u][s], __fmul_rn(beta, dv[u][s]));
                                sum = __fadd_rn(sum, dn);
                            }
                        }
                        const float cnt = (float)((info >> 7) & 7u);
                        const float qc = __fsub_rn(__fmul_rn(cnt, dc), sum);
                        const uint32_t c = cc[u];
                        if (!first) d_cur[c] = dc;
                        q[c] = qc;
                        if (f64) acc_add(acc, dc, qc);
                        else sh.tree[(info >> 18) - j0][(info >> 10) & 255u] = __fmul_rn(dc, qc);
                    }
                }
                if (!f64) publish_trees(j0, nb, slotA, tag, false, multi);
            }
            for (j0 = vld(sh.u_mc); j0 < vld(sh.u_m); j0 += KT) {  // chunks beyond the list: one cell slot per thread
                const uint32_t nb = vld(sh.u_m) - j0 < KT ? vld(sh.u_m) - j0 : KT;
                for (uint32_t t = tid; t < nb * CHUNK; t += CG_THREADS) {
                    const uint32_t j = j0 + t / CHUNK, cl = t & (CHUNK - 1);
                    const uint32_t chunk = j < KCH ? sh.chunk[j] : plan[vld(sh.u_s0) + j];
                    const uint32_t c = chunk * CHUNK + cl;
                    const uint32_t info = c < C ? cinfo[c] : 0u;
                    float prod = 0.0f;
                    if (info & 1u) {
                        const uint32_t nb7[7] = {c, c - 1, c + 1, c - nx, c + nx, c - nxy, c + nxy};
                        float dc = 0.0f, sum = 0.0f;
#pragma unroll
                        for (int s = 0; s < 7; s++) {
                            if (s == 0 || ((info >> s) & 1u)) {
                                const float dn = first ? d_src[nb7[s]]
                                                       : __fadd_rn(r[nb7[s]], __fmul_rn(beta, d_src[nb7[s]]));
                                if (s == 0) dc = dn;
                                else sum = __fadd_rn(sum, dn);
                            }
                        }
                        const float qc = __fsub_rn(__fmul_rn((float)((info >> 7) & 7u), dc), sum);
                        if (!first) d_cur[c] = dc;
                        q[c] = qc;
                        if (f64) acc_add(acc, dc, qc);
                        prod = __fmul_rn(dc, qc);
                    }
                    if (!f64) sh.tree[t / CHUNK][cl] = prod;
                }
                if (!f64) {
                    publish_trees(j0, nb, slotA, tag, false, true);  // clears its rows for the next phase's passes
                    __syncthreads();
                }
            }
        }
        float alpha;
        {
            bool dn_unused;
            if (f64) {
                publish_df(acc, wordA, tag, false);
                if (!reduce_df(wordA, tag, false, 1, alpha, dn_unused)) return;
            } else {
                float dq;
                if (!reduce_f32(slotA, segA, tag, false, 1, dq, alpha, dn_unused)) return;
            }
        }
        // ---------------- phase 2: update + r.r ----------------
        acc = Acc{};
        tag++;
        if (vld(sh.u_res)) {  // every operand in shared memory; r also to global for the neighbours
#pragma unroll
            for (int u = 0; u < 2; u++) {
                const uint32_t tu = tid + u * CG_THREADS;
                if (tu >= vld(sh.u_ncell)) continue;
                const uint32_t e = sh.cell[tu];
                const float4 o = rv4[tu];
                const float pn = __fadd_rn(o.w, __fmul_rn(alpha, o.x));  // cg_update.wgsl:33
                const float rc = __fsub_rn(o.y, __fmul_rn(alpha, o.z));  // cg_update.wgsl:34
                r[sh.chunk[e >> 18] * CHUNK + ((e >> 10) & 255u)] = rc;
                rv4[tu].y = rc;
                rv4[tu].w = pn;
                if (f64) acc_add(acc, rc, rc);
                else sh.tree[e >> 18][(e >> 10) & 255u] = __fmul_rn(rc, rc);
            }
            if (!f64) publish_trees(0, vld(sh.u_mc), slotB, tag, true, false);
        } else {
            uint32_t j0 = 0;
            for (uint32_t ps = 0; ps < vld(sh.u_npc); ps++, j0 += KT) {
                const uint32_t nb = vld(sh.u_mc) - j0 < KT ? vld(sh.u_mc) - j0 : KT;
                const uint32_t beg = sh.pass_off[ps], end = sh.pass_off[ps + 1];
                if (vld(sh.u_quad)) {
                    for (uint32_t t = beg + tid; t < end; t += CG_THREADS) {
                        // cg_update.wgsl:33-34 for the quad's liquid cells; the
                        // others keep their p and r (written back unchanged)
                        const uint2 e = qlist[t];
                        const uint32_t w[4] = {e.x & 1u, (e.x >> 10) & 1u, (e.x >> 20) & 1u, e.y & 1u};
                        const uint32_t jq = e.y >> 16, qd = (e.y >> 10) & 63u;
                        const uint32_t c0 = sh.chunk[jq] * CHUNK + 4u * qd;
                        float4 p4 = ld_f4(p + c0), r4 = ld_f4(r + c0);
                        const float4 d4 = ld_f4(d_cur + c0), q4 = ld_f4(q + c0);
                        float op[4];
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            const float pn = __fadd_rn(f4_at(p4, k), __fmul_rn(alpha, f4_at(d4, k)));
                            const float rc = __fsub_rn(f4_at(r4, k), __fmul_rn(alpha, f4_at(q4, k)));
                            const bool liq = w[k] != 0u;
                            if (liq) {
                                f4_set(p4, k, pn);
                                f4_set(r4, k, rc);
                            }
                            op[k] = liq ? __fmul_rn(rc, rc) : 0.0f;
                            if (f64 && liq) acc_add(acc, rc, rc);
                        }
                        st_f4(p + c0, p4);
                        st_f4(r + c0, r4);
                        if (!f64) *reinterpret_cast<float4*>(&sh.tree[jq - j0][4u * qd]) = make_float4(op[0], op[1], op[2], op[3]);
                    }
                } else
                for (uint32_t t = beg + tid; t < end; t += 2 * CG_THREADS) {
                    uint32_t ent[2], cc[2];
                    float pv[2], dv[2], rv[2], qv[2];
#pragma unroll
                    for (int u = 0; u < 2; u++) {
                        const uint32_t tu = t + u * CG_THREADS;
                        const bool ok = tu < end;
                        ent[u] = ok ? sh.cell[tu] : 0u;
                        cc[u] = sh.chunk[ent[u] >> 18] * CHUNK + ((ent[u] >> 10) & 255u);
                        pv[u] = ok ? p[cc[u]] : 0.0f;
                        dv[u] = ok ? d_cur[cc[u]] : 0.0f;
                        rv[u] = ok ? r[cc[u]] : 0.0f;
                        qv[u] = ok ? q[cc[u]] : 0.0f;
                    }
#pragma unroll
                    for (int u = 0; u < 2; u++) {
                        if (t + u * CG_THREADS >= end) continue;
                        const uint32_t c = cc[u];
                        p[c] = __fadd_rn(pv[u], __fmul_rn(alpha, dv[u]));       // cg_update.wgsl:33
                        const float rc = __fsub_rn(rv[u], __fmul_rn(alpha, qv[u]));  // cg_update.wgsl:34
                        r[c] = rc;
                        if (f64) acc_add(acc, rc, rc);
                        else sh.tree[(ent[u] >> 18) - j0][(ent[u] >> 10) & 255u] = __fmul_rn(rc, rc);
                    }
                }
                if (!f64) publish_trees(j0, nb, slotB, tag, true, multi);
            }
            for (j0 = vld(sh.u_mc); j0 < vld(sh.u_m); j0 += KT) {
                const uint32_t nb = vld(sh.u_m) - j0 < KT ? vld(sh.u_m) - j0 : KT;
                for (uint32_t t = tid; t < nb * CHUNK; t += CG_THREADS) {
                    const uint32_t j = j0 + t / CHUNK, cl = t & (CHUNK - 1);
                    const uint32_t chunk = j < KCH ? sh.chunk[j] : plan[vld(sh.u_s0) + j];
                    const uint32_t c = chunk * CHUNK + cl;
                    const uint32_t info = c < C ? cinfo[c] : 0u;
                    float prod = 0.0f;
                    if (info & 1u) {
                        p[c] = __fadd_rn(p[c], __fmul_rn(alpha, d_cur[c]));
                        const float rc = __fsub_rn(r[c], __fmul_rn(alpha, q[c]));
                        r[c] = rc;
                        if (f64) acc_add(acc, rc, rc);
                        prod = __fmul_rn(rc, rc);
                    }
                    if (!f64) sh.tree[t / CHUNK][cl] = prod;
                }
                if (!f64) {
                    publish_trees(j0, nb, slotB, tag, true, true);  // clears its rows for the next phase's passes
                    __syncthreads();
                }
            }
        }
        k = it + 1;
        bool done;
        if (f64) {
            publish_df(acc, wordB, tag, true);
            if (!reduce_df(wordB, tag, true, 2, beta, done)) return;
        } else {
            float rs_new;
            if (!reduce_f32(slotB, segB, tag, true, 2, rs_new, beta, done)) return;
        }
        if (done) break;
    }
    if (res)  // the resident pressure, once
        for (uint32_t tu = tid; tu < ncell; tu += CG_THREADS) {
            const uint32_t e = sh.cell[tu];
            p[sh.chunk[e >> 18] * CHUNK + ((e >> 10) & 255u)] = rv4[tu].w;
        }
    if (blockIdx.x == 0 && tid == 0) {
        st->cg_iters = k;
        st->rs_final = ieee ? sh.rs_d : (f64 ? df_to_double(Df{sh.rs_hi, sh.rs_lo}) : (double)sh.rs_hi);
    }
}

int cg_max_blocks_per_sm() {
    const void* fs[3] = {(const void*)k_cg<FL_CG_F32>, (const void*)k_cg<FL_CG_F64>, (const void*)k_cg<FL_CG_F64_IEEE>};
    int lo = 1 << 30;
    for (int i = 0; i < 3; i++) {
        int n = 0;
        if (cudaFuncSetAttribute(fs[i], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(CgShared)) !=
            cudaSuccess)
            return 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fs[i], CG_THREADS, sizeof(CgShared)) != cudaSuccess) return 0;
        lo = n < lo ? n : lo;
    }
    return lo;
}

cudaError_t launch_cg_plan(const DevBufs& b, uint32_t G, cudaStream_t s) {
    if (G < 1 || G > MAX_CG_BLOCKS) return cudaErrorInvalidValue;
    k_cg_plan<<<1, CHUNK, 0, s>>>(b, G);
    return cudaGetLastError();
}

cudaError_t launch_cg(const DevBufs& b, const LaunchCfg& L, cudaStream_t s, uint32_t precision) {
    if (precision > FL_CG_F64_IEEE) return cudaErrorInvalidValue;
    if (L.cg_blocks < 1 || (uint32_t)L.cg_blocks > MAX_CG_BLOCKS) return cudaErrorInvalidValue;
    k_cg_plan<<<1, CHUNK, 0, s>>>(b, (uint32_t)L.cg_blocks);
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
    if (precision == FL_CG_F64_IEEE) return cudaLaunchKernelEx(&cfg, k_cg<FL_CG_F64_IEEE>, b);
    return precision == FL_CG_F64 ? cudaLaunchKernelEx(&cfg, k_cg<FL_CG_F64>, b) : cudaLaunchKernelEx(&cfg, k_cg<FL_CG_F32>, b);
}

}  // namespace fl
