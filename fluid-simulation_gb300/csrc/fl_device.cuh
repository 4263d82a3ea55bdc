// fl_device.cuh — device-side layout and helpers of the FLIP/PIC substep.
//
// Arithmetic follows the reference's WGSL shaders expression by expression,
// written with explicit round-to-nearest intrinsics (__fadd_rn, __fmul_rn, ...)
// so that nvcc cannot contract a*b+c into an FMA: the f32 path then produces the
// same bits as the reference arithmetic evaluated op by op.
// SH/ below = app/crates/fluid-lab/src/gpu/shaders/ of the reference project.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fluidgb.h"

namespace fl {

constexpr uint8_t CELL_SOLID = 0, CELL_LIQUID = 1, CELL_AIR = 2;
constexpr int CHUNK = 256;        // cells per reduction chunk (the 256-wide workgroup of cg_reduce.wgsl)
constexpr int CG_GROUPS = 4;      // 256-thread chunk groups per CG block
constexpr int CG_THREADS = CHUNK * CG_GROUPS;
constexpr int SCAN_ITEMS = 4;     // counts per thread in the bin scan
constexpr int SCAN_THREADS = 1024;
constexpr int SCAN_TILE = SCAN_ITEMS * SCAN_THREADS;
constexpr int BIG_BUCKET_SMEM = 4096;  // larger buckets use the global-memory rank pass
constexpr int TILE = 8;           // P2G tile edge (cells)

// Device copy of the step settings.  Derived scalars are computed once on the
// host with the same f32 operations the shaders use (see fl_host.cpp).
struct DevParams {
    uint32_t nx, ny, nz, C;
    uint32_t F3[3], n;
    float h, inv_h, dt, fixed_scale;
    float rho, flip, friction, maxs;     // maxs = max(cfl,1)*h/dt (g2p.wgsl:159-160)
    float origin[3], scale_rhs;          // rho*h*h/dt (cg_init.wgsl:68)
    float grav[3], coeff_grad;           // (dt/rho)/h (gradient.wgsl:65)
    float rest, stiff, drift_clamp, tol_sq;  // spc; clamp(tol,0,0.1)^2 in f32
    float lo[3], half_dt;                // origin + h*1.05 (g2p.wgsl:166)
    float hi[3], pad0;                   // origin + extent - h*1.05 (g2p.wgsl:167)
    uint32_t thresh, dilation, warm, iters;
    uint32_t precision, advect_order, nchunks, solver;  // solver: FL_SOLVER_*
    double tol_sq_d;
    // Absolute stopping threshold on r.r, used instead of tol^2 * (r0.r0) when
    // thr_abs is 1 (the warm-started adjoint solve: tol^2 * |rhs|^2, written
    // on the device by k_adj_thr before the solve).
    double thr_abs_d;
    float thr_abs_f;
    uint32_t thr_abs;
    // Bound on every device-side wait (CG exchange polls, multigrid barrier)
    // in ns; 0 = the default of 2 s.  On expiry the kernel records FL_TIMEOUT
    // and every block returns.
    uint64_t wait_ns;
};

// Per-step device counters and results.
struct DevStats {
    // zeroed at the start of every substep (first 32 bytes)
    uint32_t liquid;
    uint32_t strays;
    uint32_t big_buckets;
    uint32_t cg_iters;
    uint32_t barrier;     // CG grid-barrier arrival counter
    uint32_t pad0[3];
    // kept until the host reads it
    uint32_t status;      // 0 or an fl_status code recorded by a kernel
    uint32_t pad1[3];
    double rs_init, rs_final;
};
constexpr size_t DEVSTATS_STEP_BYTES = 32;

// All device buffers of one handle.  Particles are 2 float4 per particle
// (pos.xyzw, vel.xyzw) exactly like the reference buffer (fluid.rs:116-123).
struct DevBufs {
    const DevParams* prm;
    DevStats* st;
    float4* part_in;       // particles at step start (read by binning, written by G2P)
    float4* part_sorted;   // bin-ordered copy; pos.w = 1 marks a stray particle
    float4* part_out;      // G2P destination (== part_in for the handle path)
    uint32_t* ids_in;      // may be null
    uint32_t* ids_sorted;
    uint32_t* keys;
    uint32_t* perm;
    uint32_t* scratch_u32; // capacity-sized scratch (big-bucket rank pass)
    uint32_t* stray_list;
    uint32_t* counts;
    uint32_t* offsets;
    uint32_t* cursor;
    uint32_t* spine;
    uint32_t* big_list;
    uint8_t* ct;
    uint16_t* cinfo;       // per liquid cell: bit0 liquid, bits1-6 liquid neighbours (-x,+x,-y,+y,-z,+z),
                           // bits 7-9 count of non-solid neighbours (cg_spmv.wgsl:46-66); 0 elsewhere
    uint8_t* chunk_flag;   // liquid cells of each 256-cell chunk, saturated at 255 (0: none)
    int32_t* num[3];
    int32_t* den[3];
    float* vel[3];
    float* sav[3];
    float *p, *r, *dA, *dB, *q;
    float* div;            // divergence of the last substep (divergence.wgsl, drift included); 0 off
                           // liquid cells; null where no one reads it (the stand-alone solves)
    float* part_rr;        // per-chunk f32 tree partials of the initial residual
    float2* chunk_rr_df;   // per-chunk float-float partials {hi, lo} of the initial residual
    uint32_t* cg_chunk;    // CG plan: active chunks grouped by (chunk mod 256), ascending
    uint32_t* cg_off;      // CG plan header, cg_plan_words(max blocks) words: 257 segment
                           // offsets into cg_chunk, the launch's tag base, the slot
                           // layout, the first plan entry of every block and the
                           // first exchange slot of every block (blocks + 1 each)
    unsigned long long* cg_x;  // CG exchange words, cg_x_words(nchunks, max blocks): [0] tag
                               // epoch (persists across solves), then tagged partials
};

// Sizes of the CG plan header and exchange area (fl_cg.cu).
#if defined(__CUDACC__)
#define FL_HD __host__ __device__
#else
#define FL_HD
#endif
FL_HD constexpr size_t cg_plan_words(size_t max_blocks) { return (size_t)CHUNK + 3 + 2 * (max_blocks + 1); }
FL_HD constexpr size_t cg_x_words(size_t nchunks, size_t max_blocks) {
    return 16 + 2 * ((nchunks + 15) & ~(size_t)15) + 64 * max_blocks + 2 * 256;
}

// Buffers of one adjoint step (fl_adjoint.cu).
struct AdjBufs {
    const DevParams* prm;
    // recorded step
    const float4* part;      // bin-ordered particles at step start (pos, vel)
    const uint32_t* perm;    // perm[d] = input slot of sorted particle d
    const uint8_t* ct;
    const float* sav[3];     // normalised P2G face velocity (pre-force)
    const float* fin[3];     // final face velocity (post-projection)
    // gradients
    const float4* g_out;     // dL/d(output particle d), bin order, 2 float4 each
    float4* g_sorted;        // dL/d(input particle in bin order), 2 float4 each
    float4* g_in;            // dL/d(input particle), input order
    float2* g_fs[3];         // {dL/d final face velocity, dL/d saved face velocity} per face
    float* g_norm[3];
    // Unquantised P2G sums {sum w, sum w v} of the recorded step.
    float2* wsum[3];
    float* lam;              // adjoint pressure (the solve's x)
    float* rhs;              // dL/dp
    float2* rhs_part;        // per-chunk float-float partials of rhs.rhs (null: not needed)
    double* g_grav;          // 3 sums of the block partials
    double* grav_part[3];    // per k_adj_faces block: its partial of dL/dgravity
    // Deterministic face gradients (gathered per face in a fixed order).
    float4* coef;            // per particle (bin order), 3 float4: {q, v_x}, {v_y, v_z, gpic_x/W, gpic_y/W},
                             // {gpic_z/W, gsaved/W per axis}
    const uint32_t* cell_first;  // first bin-ordered particle of every cell (the step's bin offsets)
    uint32_t* flags;         // [0] the step has stray particles, [1] max |midpoint coefficient| (float bits)
    float4* mid;             // midpoint step: per particle {qm.xyz, _}, {gfin/W at qm per axis, _}
    unsigned long long* gmid[3];  // midpoint-stencil face gradients, 64-bit fixed point
};

// ---------------------------------------------------------------------------
// helpers (device code only; fl_host.cpp sees the layout above)
#if defined(__CUDACC__)

// Float-float ("double-single") arithmetic: a value is hi + lo with two f32,
// |lo| <= ulp(hi)/2, about 48 significand bits.  GB300's FP64 pipe has a
// dependent-op latency of ~64 cycles for one warp and ~600 with a full SM
// issuing (DDIV ~640 for one warp), so the FL_CG_F64 inner products, residual
// norms and stopping test are carried in float-float on the FP32 pipe
// (df_add: ~32 cycles dependent latency) and converted to double only for the
// statistics.  Products use the exact two-product (fmaf), sums the two-sum.
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
__device__ __forceinline__ Df warp_sum_df(Df v) {  // result in lane 0
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        Df w;
        w.hi = __shfl_down_sync(0xffffffffu, v.hi, o);
        w.lo = __shfl_down_sync(0xffffffffu, v.lo, o);
        v = df_add(v, w);
    }
    return v;
}
__device__ __forceinline__ Df warp_allsum_df(Df v) {  // result in every lane
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        Df w;
        w.hi = __shfl_xor_sync(0xffffffffu, v.hi, o);
        w.lo = __shfl_xor_sync(0xffffffffu, v.lo, o);
        v = df_add(v, w);
    }
    return v;
}

// a/b to f32 precision from float-float operands (one Newton correction).
__device__ __forceinline__ float df_div(Df a, Df b) {
    const float q1 = __fdiv_rn(a.hi, b.hi);
    const float p = __fmul_rn(q1, b.hi);
    const float pe = __fmaf_rn(q1, b.hi, -p);  // q1*b.hi - p, exact
    const float r = __fadd_rn(__fsub_rn(__fsub_rn(__fsub_rn(a.hi, p), pe), __fmul_rn(q1, b.lo)), a.lo);
    return __fadd_rn(q1, __fdiv_rn(r, b.hi));
}
__device__ __forceinline__ bool df_le(Df a, Df b) { return a.hi < b.hi || (a.hi == b.hi && a.lo <= b.lo); }
__device__ __forceinline__ double df_to_double(Df a) { return (double)a.hi + (double)a.lo; }

__device__ __forceinline__ uint32_t face_dim(const DevParams& P, int axis, int b) {
    uint32_t n = b == 0 ? P.nx : (b == 1 ? P.ny : P.nz);
    return n + (axis == b ? 1u : 0u);
}

// mark.wgsl:39-43: clamp(floor((p - o)/h), 0, n-1).  fmaxf returns the other
// operand for NaN, so a NaN coordinate lands in cell 0.
__device__ __forceinline__ uint32_t key_coord(float pos, float origin, float h, uint32_t n) {
    float g = __fdiv_rn(__fsub_rn(pos, origin), h);
    float f = floorf(g);
    float c = fminf(fmaxf(f, 0.0f), (float)(n - 1u));
    return (uint32_t)c;
}

__device__ __forceinline__ uint32_t cell_key(const DevParams& P, float4 pos, uint32_t* kc) {
    kc[0] = key_coord(pos.x, P.origin[0], P.h, P.nx);
    kc[1] = key_coord(pos.y, P.origin[1], P.h, P.ny);
    kc[2] = key_coord(pos.z, P.origin[2], P.h, P.nz);
    return kc[0] + P.nx * (kc[1] + P.ny * kc[2]);
}

// True when the multiply-form cell coordinate (p-o)*inv_h of scatter.wgsl:94
// disagrees with the division-form bin on some axis (an ulp tie or a clamped
// bin).  Such particles are scattered by the separate stray pass.
__device__ __forceinline__ bool is_stray(const DevParams& P, float4 pos, const uint32_t* kc) {
    float q0 = __fmul_rn(__fsub_rn(pos.x, P.origin[0]), P.inv_h);
    float q1 = __fmul_rn(__fsub_rn(pos.y, P.origin[1]), P.inv_h);
    float q2 = __fmul_rn(__fsub_rn(pos.z, P.origin[2]), P.inv_h);
    return floorf(q0) != (float)kc[0] || floorf(q1) != (float)kc[1] || floorf(q2) != (float)kc[2];
}

__device__ __forceinline__ int32_t floor_to_i32(float x) { return __float2int_rz(floorf(x)); }

// SH/scatter.wgsl:71-72: i32(round(x)) — round half to even, saturating.
__device__ __forceinline__ int32_t fixed_round(float x) { return __float2int_rn(x); }

// The reference's weight ordering w = wx * wy * wz with the loop order
// dk (outer), dj, di (inner) of scatter.wgsl:55-67.
__device__ __forceinline__ float tent(float t, int d) { return d == 1 ? t : __fsub_rn(1.0f, t); }

// Grid barrier over all blocks of a cooperative launch.  Arrival is a
// release-add on a counter that only grows within one launch; waiting is an
// acquire-load spin bounded by %globaltimer (about 2 s).  On expiry, or when
// another block has recorded an error, it records FL_TIMEOUT and returns false.
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ uint64_t wait_limit_ns(const DevParams* P) {
    const uint64_t w = P->wait_ns;
    return w ? w : 2000000000ull;
}
__device__ __forceinline__ uint32_t ld_acquire(const uint32_t* p) {
    uint32_t v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void red_release_add(uint32_t* p, uint32_t v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

#endif  // __CUDACC__
}  // namespace fl

// Launchers (defined in the .cu files); all enqueue on `s` and return the
// launch error.
namespace fl {
struct LaunchCfg {
    int num_sms;
    int cg_blocks;         // cooperative grid size for the CG kernel
    int particle_blocks;   // grid-stride particle kernels
};
cudaError_t launch_bin(const DevBufs& b, const LaunchCfg& L, uint32_t C, uint32_t cap, cudaStream_t s);
cudaError_t launch_classify(const DevBufs& b, uint32_t C, cudaStream_t s);
// clear: zero the face accumulators first (unless the caller's memset covers them).
cudaError_t launch_p2g(const DevBufs& b, const LaunchCfg& L, uint32_t nx, uint32_t ny, uint32_t nz,
                       cudaStream_t s, bool clear);
cudaError_t launch_grid_prep(const DevBufs& b, uint32_t C, cudaStream_t s);
// precision: FL_CG_F32, FL_CG_F64 or FL_CG_F64_IEEE (the kernel is specialised per precision).
cudaError_t launch_cg(const DevBufs& b, const LaunchCfg& L, cudaStream_t s, uint32_t precision);
cudaError_t launch_project(const DevBufs& b, uint32_t C, cudaStream_t s);
cudaError_t launch_g2p(const DevBufs& b, const LaunchCfg& L, cudaStream_t s);
cudaError_t launch_iota(uint32_t* ids, uint32_t n, cudaStream_t s);
cudaError_t launch_impulse(float4* part, const DevParams* prm, float dx, float dy, float dz,
                           const LaunchCfg& L, cudaStream_t s);
int cg_max_blocks_per_sm();
cudaError_t launch_slice(const DevBufs& b, uint32_t nx, uint32_t ny, uint32_t mode, uint32_t k, float4* out,
                         cudaStream_t s);
// Particle seeding (fl_scene.cu): one liquid block of the jittered lattice.
struct SeedBlock {
    float wmin[3];      // world position of the block's min corner
    float spacing;      // lattice spacing
    int32_t counts[3];  // lattice points per axis
    uint32_t first;     // index of the block's first particle
};
struct SeedArgs {
    SeedBlock blk[16];  // FL_SCENE_MAX_BLOCKS
    uint32_t nblocks, n;
    float lo[3], hi[3];  // wall clamp of the positions
};
// Layout of generate_particles for the settings' tank; the total count, or -1.
long long seed_layout(const fl_params& prm, const fl_block* blocks, uint32_t nblocks, uint32_t particle_count,
                      SeedArgs* out);
cudaError_t launch_seed(const SeedArgs& a, float4* part, cudaStream_t s);
// Multigrid hierarchy of the MGPCG solver (fl_mg.cu).  Level 0 is the grid
// (its operator comes from cinfo; b = the CG residual r, x = z = M^-1 r);
// level l+1 aggregates 2x2x2 cells of level l.
constexpr int MG_MAX_LEVELS = 12;
constexpr uint32_t MG_COARSE_CELLS = 64;  // the coarsest level holds at most this many cells
constexpr uint32_t MG_BLOCK0_CELLS = 4096;  // levels this small run inside one block (block barriers)
constexpr uint32_t MG_LOCAL_TOTAL = 4800;   // cells of all those levels together (b, x in shared memory)
struct MgLevel {
    uint32_t nx, ny, nz, C;
    float4* st;  // {diag, weight to +x, +y, +z} (levels >= 1)
    float* b;
    float* x;
};
struct MgBufs {
    uint32_t L;         // number of levels (>= 2)
    MgLevel lv[MG_MAX_LEVELS];
    float* r2;          // second residual buffer (level-0 size)
    float2* part;       // 2 x MAX_CG_BLOCKS float-float block partials
    uint32_t* bar;      // barrier counter, zeroed before each solve
};
// Level sizes of an nx x ny x nz grid; returns L.
FL_HD inline uint32_t mg_levels(uint32_t nx, uint32_t ny, uint32_t nz, uint32_t dims[MG_MAX_LEVELS][3]) {
    uint32_t L = 0;
    for (;;) {
        dims[L][0] = nx; dims[L][1] = ny; dims[L][2] = nz;
        L++;
        if ((size_t)nx * ny * nz <= MG_COARSE_CELLS || L == MG_MAX_LEVELS) break;
        nx = (nx + 1) / 2; ny = (ny + 1) / 2; nz = (nz + 1) / 2;
    }
    return L;
}
// Relaxation solves from zero (fl_relax.cu): method 0 Jacobi (ping-pong
// between pa and pb), 1 red-black Gauss-Seidel (in place in pa); *result is
// the buffer that holds the answer.
cudaError_t launch_relax(const uint8_t* ct, const float* div, float scale, float* pa, float* pb, uint32_t nx,
                         uint32_t ny, uint32_t nz, uint32_t method, uint32_t iters, cudaStream_t s, float** result);
// The CG's plan of active chunks split over G blocks (fl_cg.cu).
cudaError_t launch_cg_plan(const DevBufs& b, uint32_t G, cudaStream_t s);
cudaError_t launch_mgpcg(const DevBufs& b, const MgBufs& m, const LaunchCfg& L, cudaStream_t s);
int mg_max_blocks_per_sm();

struct AdjBufs;
cudaError_t launch_adj_g2p(const AdjBufs& a, const LaunchCfg& L, cudaStream_t s);
cudaError_t launch_adj_prhs(const AdjBufs& a, uint32_t C, cudaStream_t s);
// tol^2 * (rhs.rhs) into cg_prm's absolute threshold (rhs_part of a block-per-chunk k_adj_prhs)
cudaError_t launch_adj_thr(const AdjBufs& a, uint32_t nchunks, double tol_sq, DevParams* cg_prm, cudaStream_t s);
cudaError_t launch_adj_faces(const AdjBufs& a, const uint32_t F3[3], cudaStream_t s);
// the midpoint step's face gradients into gmid (zeroed by the caller)
cudaError_t launch_adj_mid(const AdjBufs& a, const LaunchCfg& L, cudaStream_t s);
// g_fs and wsum of every face, gathered per cell in a fixed order
cudaError_t launch_adj_gather(const AdjBufs& a, uint32_t C, bool midpoint, cudaStream_t s);
cudaError_t launch_adj_p2g(const AdjBufs& a, const LaunchCfg& L, cudaStream_t s);
cudaError_t launch_adj_unsort(const AdjBufs& a, const LaunchCfg& L, cudaStream_t s);
// Stand-alone CG on prepared cell arrays (used by fl_solve_pressure).
cudaError_t launch_solve_init(const DevBufs& b, uint32_t C, const float* div, cudaStream_t s);
}  // namespace fl
