// fl_host.cpp — C ABI of the FLIP/PIC substep (include/fluidgb.h).
//
// A handle owns one device pool holding every buffer of the step, a stream,
// and a CUDA graph of one substep (the reference records one command encoder
// per substep, gpu/mod.rs:973-982; here the whole substep replays as one graph
// launch).  Settings live in device memory, so live parameter changes
// (fluid.rs:1294-1371) never invalidate the graph.
//
// This file is compiled with -ffp-contract=off: the derived scalars below are
// evaluated in f32 in the shaders' operation order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "../../include/fluidgb.h"
#include "fl_device.cuh"

using fl::DevBufs;
using fl::DevParams;
using fl::DevStats;

struct fl_handle {
    fl_params prm;
    uint32_t nx = 0, ny = 0, nz = 0, C = 0, F3[3] = {0, 0, 0}, nchunks = 0;
    uint32_t cap = 0, n = 0;
    int device = 0;
    fl::LaunchCfg L{};
    DevParams hp{};
    DevBufs b{};
    void* pool = nullptr;
    size_t pool_bytes = 0;
    size_t clear_bytes = 0;  // counts .. den[2]: cleared at the start of every substep
    float4* partA = nullptr;
    uint32_t* idsA = nullptr;
    DevParams* dprm = nullptr;
    DevStats* dst = nullptr;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t graph = nullptr;
    bool graph_failed = false;
    bool profiling = false;
    cudaEvent_t ev[FL_STAGE_COUNT + 1] = {};
    double stage_ms[FL_STAGE_COUNT] = {};
    uint64_t stage_steps = 0;
    std::vector<float> init_part;
    uint32_t init_n = 0;
    uint64_t substeps = 0;
    float4* slice_buf = nullptr;  // device staging of fl_grid_slice (nx*ny float4), allocated on first use
    fl::MgBufs mg{};              // MGPCG hierarchy, allocated when that solver is first selected
    void* mg_pool = nullptr;
    uint64_t wait_ns = 0;         // device-side wait limit (fl_set_wait_timeout; 0 = default)
    std::string err;
};

namespace {

thread_local std::string g_err;

fl_status set_err(fl_handle* h, fl_status s, const std::string& msg) {
    if (h)
        h->err = msg;
    else
        g_err = msg;
    return s;
}

fl_status cuda_err(fl_handle* h, cudaError_t e, const char* what) {
    return set_err(h, FL_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
}

}  // namespace

// The message slot fl_last_error(NULL) reads, for entry points in other
// translation units (fl_noalloc.cu).
void fl_record_global_error(const std::string& msg) { g_err = msg; }

namespace {

#define FL_CUDA(h, call)                                        \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return cuda_err((h), e_, #call); \
    } while (0)

uint32_t f2u_sat(float x) {
    if (!(x > 0.0f)) return 0u;
    if (x >= 4294967296.0f) return 0xffffffffu;
    return (uint32_t)x;
}

fl_status validate(const fl_params* p, std::string* why) {
    if (!p) { *why = "params is NULL"; return FL_INVALID_ARG; }
    if (p->gdim[0] < 3 || p->gdim[1] < 3 || p->gdim[2] < 3) { *why = "each grid dimension must be >= 3"; return FL_INVALID_ARG; }
    if (p->gdim[0] > 2048 || p->gdim[1] > 2048 || p->gdim[2] > 2048) { *why = "grid dimension > 2048"; return FL_INVALID_ARG; }
    if ((uint64_t)p->gdim[0] * p->gdim[1] * p->gdim[2] > (1ull << 30)) { *why = "more than 2^30 cells"; return FL_INVALID_ARG; }
    if (!(p->geom[0] > 0.0f) || !(p->geom[1] > 0.0f)) { *why = "h and inv_h must be > 0"; return FL_INVALID_ARG; }
    if (!(p->geom[2] > 0.0f)) { *why = "dt must be > 0"; return FL_INVALID_ARG; }
    if (!(p->phys[1] > 0.0f)) { *why = "rho must be > 0"; return FL_INVALID_ARG; }
    if (p->cg_precision > FL_CG_F64_IEEE) {
        *why = "cg_precision must be FL_CG_F32, FL_CG_F64 or FL_CG_F64_IEEE";
        return FL_INVALID_ARG;
    }
    if (p->advect_order > 2u) { *why = "advect_order must be 1 or 2"; return FL_INVALID_ARG; }
    if (p->pressure_solver > 1u) { *why = "pressure_solver must be FL_SOLVER_CG or FL_SOLVER_MGPCG"; return FL_INVALID_ARG; }
    for (int i = 0; i < 3; i++)
        if (p->reserved[i]) { *why = "reserved fields must be zero"; return FL_INVALID_ARG; }
    return FL_OK;
}

// Derived settings, in the shaders' f32 operation order.
void derive(const fl_params& p, uint32_t n, DevParams& d) {
    d = DevParams{};
    d.nx = p.gdim[0]; d.ny = p.gdim[1]; d.nz = p.gdim[2];
    d.C = d.nx * d.ny * d.nz;
    d.F3[0] = (d.nx + 1) * d.ny * d.nz;
    d.F3[1] = d.nx * (d.ny + 1) * d.nz;
    d.F3[2] = d.nx * d.ny * (d.nz + 1);
    d.n = n;
    d.h = p.geom[0]; d.inv_h = p.geom[1]; d.dt = p.geom[2]; d.fixed_scale = p.geom[3];
    d.rho = p.phys[1]; d.flip = p.phys[2]; d.friction = p.phys[3];
    const float cfl = std::fmax(p.cls[2], 1.0f);                 // g2p.wgsl:159
    d.maxs = cfl * d.h / d.dt;                                    // g2p.wgsl:160
    for (int a = 0; a < 3; a++) { d.origin[a] = p.origin[a]; d.grav[a] = p.grav[a]; }
    d.scale_rhs = d.rho * d.h * d.h / d.dt;                       // cg_init.wgsl:68
    d.coeff_grad = (d.dt / d.rho) / d.h;                          // gradient.wgsl:65
    d.rest = p.spc[0]; d.stiff = p.spc[1]; d.drift_clamp = p.spc[2];
    const float tolc = std::fmin(std::fmax(p.pressure_tolerance, 0.0f), 0.1f);  // fluid.rs:47-50
    d.tol_sq = tolc * tolc;
    d.tol_sq_d = (double)tolc * (double)tolc;
    const uint32_t nn[3] = {d.nx, d.ny, d.nz};
    for (int a = 0; a < 3; a++) {
        const float extent = (float)nn[a] * d.h;                  // g2p.wgsl:165
        d.lo[a] = d.origin[a] + d.h * 1.05f;                      // g2p.wgsl:166
        d.hi[a] = d.origin[a] + extent - d.h * 1.05f;             // g2p.wgsl:167
    }
    d.half_dt = 0.5f * d.dt;
    d.thresh = std::max(f2u_sat(p.cls[0]), 1u);                   // classify.wgsl:42
    d.dilation = f2u_sat(p.cls[1]) >= 1u ? 1u : 0u;               // classify.wgsl:48
    d.warm = p.dims[3] != 0u ? 1u : 0u;
    d.iters = p.dims[2] ? p.dims[2] : 1u;                          // fluid.rs:286
    d.precision = p.cg_precision;
    d.advect_order = p.advect_order == 2u ? 2u : 1u;
    d.nchunks = (d.C + fl::CHUNK - 1) / fl::CHUNK;
    d.solver = p.pressure_solver;
}

struct PoolPlan {
    size_t off = 0;
    template <class T>
    size_t take(size_t count) {
        off = (off + 255) & ~size_t(255);
        const size_t o = off;
        off += sizeof(T) * std::max<size_t>(count, 1);
        return o;
    }
};

int g_num_sms = -1;
int g_cg_per_sm = 0;

// Multigrid hierarchy of an nx x ny x nz grid in one device pool: per level
// l >= 1 the float4 stencil, b and x; z of level 0; the block partials and the
// barrier counter.  Level 0's b is the solve's residual r.
fl_status mg_alloc(fl_handle* h, uint32_t nx, uint32_t ny, uint32_t nz, float* r, fl::MgBufs* m, void** pool) {
    if (*pool) return FL_OK;
    uint32_t dims[fl::MG_MAX_LEVELS][3];
    const uint32_t L = fl::mg_levels(nx, ny, nz, dims);
    if (L < 2 || (size_t)dims[L - 1][0] * dims[L - 1][1] * dims[L - 1][2] > fl::MG_COARSE_CELLS)
        return set_err(h, FL_INVALID_ARG, "grid too small or too large for the multigrid hierarchy");
    {
        // the levels from the first one of at most MG_BLOCK0_CELLS cells on run
        // in one block, their vectors in its shared memory
        auto cells = [&](uint32_t l) { return (size_t)dims[l][0] * dims[l][1] * dims[l][2]; };
        uint32_t Lg = 1;
        while (Lg + 1 < L && cells(Lg) > fl::MG_BLOCK0_CELLS) Lg++;
        size_t local = 0;
        for (uint32_t l = Lg; l < L; l++) local += cells(l);
        if (local > fl::MG_LOCAL_TOTAL)
            return set_err(h, FL_INVALID_ARG, "grid shape unsupported by the multigrid solver (coarse levels too elongated)");
    }
    if (fl::mg_max_blocks_per_sm() < 1) return set_err(h, FL_INTERNAL, "MGPCG kernel cannot be resident");
    PoolPlan pl;
    size_t o_st[fl::MG_MAX_LEVELS] = {}, o_b[fl::MG_MAX_LEVELS] = {}, o_x[fl::MG_MAX_LEVELS] = {};
    for (uint32_t l = 0; l < L; l++) {
        const size_t C = (size_t)dims[l][0] * dims[l][1] * dims[l][2];
        if (l > 0) {
            o_st[l] = pl.take<float4>(C);
            o_b[l] = pl.take<float>(C);
        }
        o_x[l] = pl.take<float>(C);
    }
    const size_t o_r2 = pl.take<float>((size_t)nx * ny * nz);
    const size_t o_part = pl.take<float2>(2 * 1024), o_bar = pl.take<uint32_t>(1);
    void* base = nullptr;
    cudaError_t e = cudaMalloc(&base, pl.off);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return set_err(h, FL_OOM, "multigrid allocation of " + std::to_string(pl.off) + " bytes failed");
    }
    char* c = (char*)base;
    *m = fl::MgBufs{};
    m->L = L;
    for (uint32_t l = 0; l < L; l++) {
        fl::MgLevel& lv = m->lv[l];
        lv.nx = dims[l][0]; lv.ny = dims[l][1]; lv.nz = dims[l][2];
        lv.C = lv.nx * lv.ny * lv.nz;
        lv.st = l ? (float4*)(c + o_st[l]) : nullptr;
        lv.b = l ? (float*)(c + o_b[l]) : r;
        lv.x = (float*)(c + o_x[l]);
    }
    m->r2 = (float*)(c + o_r2);
    m->part = (float2*)(c + o_part);
    m->bar = (uint32_t*)(c + o_bar);
    *pool = base;
    return FL_OK;
}

fl_status device_check(fl_handle* h) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_err(h, FL_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, dev);
    if (e != cudaSuccess) return set_err(h, FL_NO_DEVICE, std::string("cudaGetDeviceProperties: ") + cudaGetErrorString(e));
    if (!(prop.major == 10 && prop.minor == 3))
        return set_err(h, FL_NO_DEVICE, "this build targets sm_103a (GB300); found sm_" + std::to_string(prop.major) +
                                            std::to_string(prop.minor));
    if (!prop.cooperativeLaunch) return set_err(h, FL_NO_DEVICE, "device does not support cooperative launch");
    g_num_sms = prop.multiProcessorCount;
    g_cg_per_sm = fl::cg_max_blocks_per_sm();
    if (g_cg_per_sm < 1) return set_err(h, FL_INTERNAL, "CG kernel cannot be resident (occupancy 0)");
    return FL_OK;
}

fl::LaunchCfg make_cfg(uint32_t nchunks) {
    fl::LaunchCfg L;
    L.num_sms = g_num_sms;
    const int max_cg = g_num_sms * g_cg_per_sm;
    const int want = (int)((nchunks + fl::CG_GROUPS - 1) / fl::CG_GROUPS);
    L.cg_blocks = std::max(1, std::min(max_cg, want));
    L.particle_blocks = g_num_sms * 8;
    return L;
}

// Enqueue one substep.  The caller set b.part_in/out/ids.  With `ev`, an
// event is recorded before the first stage and after every stage.  With
// `p_replay`, the pressure solve is replaced by a copy of that pressure field
// (C floats): the substep that produced it is reproduced without its CG.
cudaError_t enqueue_step(fl_handle* h, const DevBufs& b, cudaStream_t s, cudaEvent_t* ev = nullptr,
                         const float* p_replay = nullptr) {
    cudaError_t e;
    auto mark = [&](int i) { return ev ? cudaEventRecord(ev[i], s) : cudaSuccess; };
    if ((e = mark(0)) != cudaSuccess) return e;
    if ((e = cudaMemsetAsync(h->dst, 0, fl::DEVSTATS_STEP_BYTES, s)) != cudaSuccess) return e;
    // the histogram and the P2G accumulators (scatter.wgsl's sums start at
    // zero: the reference's clear pass), one contiguous span of the pool,
    // timed with the binning stage
    if ((e = cudaMemsetAsync(b.counts, 0, h->clear_bytes, s)) != cudaSuccess) return e;
    if ((e = fl::launch_bin(b, h->L, h->C, h->cap, s)) != cudaSuccess) return e;
    if ((e = mark(1)) != cudaSuccess) return e;
    if ((e = fl::launch_classify(b, h->C, s)) != cudaSuccess) return e;
    if ((e = mark(2)) != cudaSuccess) return e;
    if ((e = fl::launch_p2g(b, h->L, h->nx, h->ny, h->nz, s, false)) != cudaSuccess) return e;
    if ((e = mark(3)) != cudaSuccess) return e;
    if ((e = fl::launch_grid_prep(b, h->C, s)) != cudaSuccess) return e;
    if ((e = mark(4)) != cudaSuccess) return e;
    if (p_replay) {
        if ((e = cudaMemcpyAsync(b.p, p_replay, sizeof(float) * (size_t)h->C, cudaMemcpyDeviceToDevice, s)) !=
            cudaSuccess)
            return e;
    } else if (h->prm.pressure_solver == FL_SOLVER_MGPCG) {
        if ((e = fl::launch_mgpcg(b, h->mg, h->L, s)) != cudaSuccess) return e;
    } else if ((e = fl::launch_cg(b, h->L, s, h->prm.cg_precision)) != cudaSuccess) {
        return e;
    }
    if ((e = mark(5)) != cudaSuccess) return e;
    if ((e = fl::launch_project(b, h->C, s)) != cudaSuccess) return e;
    if ((e = mark(6)) != cudaSuccess) return e;
    if ((e = fl::launch_g2p(b, h->L, s)) != cudaSuccess) return e;
    if ((e = mark(7)) != cudaSuccess) return e;
    return cudaSuccess;
}

fl_status upload_params(fl_handle* h) {
    derive(h->prm, h->n, h->hp);
    h->hp.wait_ns = h->wait_ns;
    FL_CUDA(h, cudaMemcpyAsync(h->dprm, &h->hp, sizeof(DevParams), cudaMemcpyHostToDevice, h->stream));
    return FL_OK;
}

fl_status read_status(fl_handle* h) {
    uint32_t st = 0;
    FL_CUDA(h, cudaMemcpyAsync(&st, &h->dst->status, 4, cudaMemcpyDeviceToHost, h->stream));
    FL_CUDA(h, cudaStreamSynchronize(h->stream));
    if (st != 0u) {
        const uint32_t zero = 0;
        FL_CUDA(h, cudaMemcpyAsync(&h->dst->status, &zero, 4, cudaMemcpyHostToDevice, h->stream));
        FL_CUDA(h, cudaStreamSynchronize(h->stream));
        return set_err(h, (fl_status)st, "a device-side wait expired (status " + std::to_string(st) + ")");
    }
    return FL_OK;
}

fl_status build_graph(fl_handle* h) {
    if (h->graph || h->graph_failed) return FL_OK;
    DevBufs b = h->b;
    b.part_in = h->partA;
    b.part_out = h->partA;
    b.ids_in = h->idsA;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(h->own_stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t le = enqueue_step(h, b, h->own_stream);
        e = cudaStreamEndCapture(h->own_stream, &g);
        if (le != cudaSuccess) e = le;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&h->graph, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        // Fall back to direct launches; clear the sticky capture error.
        h->graph = nullptr;
        h->graph_failed = true;
        (void)cudaGetLastError();
    }
    return FL_OK;
}

}  // namespace

extern "C" {

uint32_t fl_abi_version(void) { return FL_ABI_VERSION; }

const char* fl_status_string(fl_status s) {
    switch (s) {
        case FL_OK: return "FL_OK";
        case FL_INVALID_ARG: return "FL_INVALID_ARG";
        case FL_OOM: return "FL_OOM";
        case FL_CUDA_ERROR: return "FL_CUDA_ERROR";
        case FL_NOT_CONVERGED: return "FL_NOT_CONVERGED";
        case FL_TIMEOUT: return "FL_TIMEOUT";
        case FL_NO_DEVICE: return "FL_NO_DEVICE";
        case FL_INTERNAL: return "FL_INTERNAL";
    }
    return "FL_UNKNOWN";
}

fl_status fl_params_default(fl_params* out, uint32_t nx, uint32_t ny, uint32_t nz, float h, const float* origin) {
    if (!out) return set_err(nullptr, FL_INVALID_ARG, "out is NULL");
    if (!(h > 0.0f)) return set_err(nullptr, FL_INVALID_ARG, "h must be > 0");
    std::memset(out, 0, sizeof(*out));
    // Registry defaults, app/crates/fluid-lab/src/settings/mod.rs:498-724.
    out->dims[0] = nx;
    out->dims[1] = 0;
    out->dims[2] = 30;   // solver.pressure_iterations
    out->dims[3] = 1;    // solver.pressure_warm_start
    out->geom[0] = h;
    out->geom[1] = 1.0f / h;
    out->geom[2] = 1.0f / 120.0f;  // physics.fixed_dt
    out->geom[3] = 65536.0f;       // FIXED_SCALE (fluid.rs:41)
    out->phys[0] = -9.81f;         // physics.gravity
    out->phys[1] = 1000.0f;        // rho (fluid.rs:299)
    out->phys[2] = 0.9f;           // physics.flip_blend
    out->phys[3] = 0.0f;           // physics.wall_friction
    const uint32_t nn[3] = {nx, ny, nz};
    for (int a = 0; a < 3; a++) out->origin[a] = origin ? origin[a] : -(float)nn[a] * h / 2.0f;  // fluid.rs:262-266
    out->grav[1] = -9.81f;
    out->spc[0] = 8.0f;            // effective rest density at the reference particle density
    out->spc[1] = 0.45f;           // physics.volume_stiffness
    out->spc[2] = 0.5f;            // physics.drift_clamp
    out->cls[0] = 1.0f;            // classify.liquid_threshold
    out->cls[1] = 0.0f;            // classify.surface_dilation
    out->cls[2] = 2.0f;            // physics.cfl
    out->gdim[0] = nx; out->gdim[1] = ny; out->gdim[2] = nz;
    out->pressure_tolerance = 0.0f;  // solver.pressure_residual_tolerance
    out->cg_precision = FL_CG_F32;
    out->advect_order = 1;
    out->sort_period = 4;            // dev.particle_sort_period
    return FL_OK;
}

fl_status fl_create(const fl_params* params, uint32_t capacity, fl_handle** out) {
    if (!out) return set_err(nullptr, FL_INVALID_ARG, "out is NULL");
    *out = nullptr;
    std::string why;
    if (validate(params, &why) != FL_OK) return set_err(nullptr, FL_INVALID_ARG, why);
    fl_status s = device_check(nullptr);
    if (s != FL_OK) return s;
    fl_handle* h = new (std::nothrow) fl_handle();
    if (!h) return set_err(nullptr, FL_OOM, "host allocation failed");
    h->prm = *params;
    h->nx = params->gdim[0]; h->ny = params->gdim[1]; h->nz = params->gdim[2];
    h->C = h->nx * h->ny * h->nz;
    h->F3[0] = (h->nx + 1) * h->ny * h->nz;
    h->F3[1] = h->nx * (h->ny + 1) * h->nz;
    h->F3[2] = h->nx * h->ny * (h->nz + 1);
    h->nchunks = (h->C + fl::CHUNK - 1) / fl::CHUNK;
    h->cap = capacity;
    cudaGetDevice(&h->device);
    h->L = make_cfg(h->nchunks);

    const size_t cap = std::max<uint32_t>(capacity, 1);
    const size_t C = h->C;
    const uint32_t nb = (h->C + fl::SCAN_TILE - 1) / fl::SCAN_TILE;
    PoolPlan pl;
    size_t o_partA = pl.take<float4>(2 * cap), o_partB = pl.take<float4>(2 * cap);
    size_t o_idsA = pl.take<uint32_t>(cap), o_idsB = pl.take<uint32_t>(cap);
    size_t o_keys = pl.take<uint32_t>(cap), o_perm = pl.take<uint32_t>(cap);
    size_t o_scr = pl.take<uint32_t>(cap), o_stray = pl.take<uint32_t>(cap);
    // The per-substep accumulators (the histogram and P2G's fixed-point
    // sums) are contiguous, so one memset clears them all (enqueue_step).
    size_t o_num[3], o_den[3], o_vel[3], o_sav[3];
    size_t o_counts = pl.take<uint32_t>(C);
    for (int a = 0; a < 3; a++) {
        o_num[a] = pl.take<int32_t>(h->F3[a]);
        o_den[a] = pl.take<int32_t>(h->F3[a]);
    }
    h->clear_bytes = pl.off - o_counts;
    size_t o_offs = pl.take<uint32_t>(C), o_cur = pl.take<uint32_t>(C);
    size_t o_spine = pl.take<uint32_t>(nb), o_big = pl.take<uint32_t>(C);
    size_t o_ct = pl.take<uint8_t>(C), o_flag = pl.take<uint8_t>(h->nchunks), o_cinfo = pl.take<uint16_t>(C);
    for (int a = 0; a < 3; a++) {
        o_vel[a] = pl.take<float>(h->F3[a]);
        o_sav[a] = pl.take<float>(h->F3[a]);
    }
    size_t o_p = pl.take<float>(C), o_r = pl.take<float>(C), o_dA = pl.take<float>(C), o_dB = pl.take<float>(C),
           o_q = pl.take<float>(C), o_div = pl.take<float>(C);
    const size_t gmax = (size_t)g_num_sms * g_cg_per_sm;
    size_t o_prr = pl.take<float>(h->nchunks), o_c64 = pl.take<float2>(h->nchunks);
    size_t o_plan = pl.take<uint32_t>(h->nchunks), o_poff = pl.take<uint32_t>(fl::cg_plan_words(gmax));
    size_t o_cgx = pl.take<unsigned long long>(fl::cg_x_words(h->nchunks, gmax));
    size_t o_prm = pl.take<DevParams>(1), o_st = pl.take<DevStats>(1);
    h->pool_bytes = pl.off;

    cudaError_t e = cudaMalloc(&h->pool, h->pool_bytes);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        const size_t bytes = h->pool_bytes;
        delete h;
        return set_err(nullptr, FL_OOM, "cudaMalloc of " + std::to_string(bytes) + " bytes failed");
    }
    char* base = (char*)h->pool;
    if ((e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking)) != cudaSuccess) {
        cudaFree(h->pool);
        delete h;
        return cuda_err(nullptr, e, "cudaStreamCreate");
    }
    h->stream = h->own_stream;
    if ((e = cudaMemsetAsync(h->pool, 0, h->pool_bytes, h->stream)) != cudaSuccess) {
        fl_destroy(h);
        return cuda_err(nullptr, e, "cudaMemset");
    }
    DevBufs& b = h->b;
    h->partA = (float4*)(base + o_partA);
    h->idsA = (uint32_t*)(base + o_idsA);
    h->dprm = (DevParams*)(base + o_prm);
    h->dst = (DevStats*)(base + o_st);
    b.prm = h->dprm;
    b.st = h->dst;
    b.part_in = h->partA;
    b.part_sorted = (float4*)(base + o_partB);
    b.part_out = h->partA;
    b.ids_in = h->idsA;
    b.ids_sorted = (uint32_t*)(base + o_idsB);
    b.keys = (uint32_t*)(base + o_keys);
    b.perm = (uint32_t*)(base + o_perm);
    b.scratch_u32 = (uint32_t*)(base + o_scr);
    b.stray_list = (uint32_t*)(base + o_stray);
    b.counts = (uint32_t*)(base + o_counts);
    b.offsets = (uint32_t*)(base + o_offs);
    b.cursor = (uint32_t*)(base + o_cur);
    b.spine = (uint32_t*)(base + o_spine);
    b.big_list = (uint32_t*)(base + o_big);
    b.ct = (uint8_t*)(base + o_ct);
    b.cinfo = (uint16_t*)(base + o_cinfo);
    b.chunk_flag = (uint8_t*)(base + o_flag);
    for (int a = 0; a < 3; a++) {
        b.num[a] = (int32_t*)(base + o_num[a]);
        b.den[a] = (int32_t*)(base + o_den[a]);
        b.vel[a] = (float*)(base + o_vel[a]);
        b.sav[a] = (float*)(base + o_sav[a]);
    }
    b.p = (float*)(base + o_p);
    b.r = (float*)(base + o_r);
    b.dA = (float*)(base + o_dA);
    b.dB = (float*)(base + o_dB);
    b.q = (float*)(base + o_q);
    b.div = (float*)(base + o_div);
    b.part_rr = (float*)(base + o_prr);
    b.chunk_rr_df = (float2*)(base + o_c64);
    b.cg_chunk = (uint32_t*)(base + o_plan);
    b.cg_off = (uint32_t*)(base + o_poff);
    b.cg_x = (unsigned long long*)(base + o_cgx);
    if (params->pressure_solver == FL_SOLVER_MGPCG &&
        (s = mg_alloc(h, h->nx, h->ny, h->nz, b.r, &h->mg, &h->mg_pool)) != FL_OK) {
        std::string m = h->err;
        fl_destroy(h);
        return set_err(nullptr, s, m);
    }
    if ((s = upload_params(h)) != FL_OK) {
        std::string m = h->err;
        fl_destroy(h);
        return set_err(nullptr, s, m);
    }
    *out = h;
    return FL_OK;
}

fl_status fl_destroy(fl_handle* h) {
    if (!h) return FL_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->graph) cudaGraphExecDestroy(h->graph);
    for (int k = 0; k <= FL_STAGE_COUNT; k++)
        if (h->ev[k]) cudaEventDestroy(h->ev[k]);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
    if (h->pool) cudaFree(h->pool);
    if (h->slice_buf) cudaFree(h->slice_buf);
    if (h->mg_pool) cudaFree(h->mg_pool);
    delete h;
    return FL_OK;
}

fl_status fl_set_params(fl_handle* h, const fl_params* params) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    std::string why;
    if (validate(params, &why) != FL_OK) return set_err(h, FL_INVALID_ARG, why);
    if (params->gdim[0] != h->nx || params->gdim[1] != h->ny || params->gdim[2] != h->nz)
        return set_err(h, FL_INVALID_ARG, "grid dimensions cannot change on a live handle; create a new one");
    if (params->pressure_solver == FL_SOLVER_MGPCG) {
        fl_status s = mg_alloc(h, h->nx, h->ny, h->nz, h->b.r, &h->mg, &h->mg_pool);
        if (s != FL_OK) return s;
    }
    if ((params->cg_precision != h->prm.cg_precision || params->pressure_solver != h->prm.pressure_solver) &&
        h->graph) {
        // the solver kernels differ per precision and solver: capture the step again
        FL_CUDA(h, cudaStreamSynchronize(h->stream));
        cudaGraphExecDestroy(h->graph);
        h->graph = nullptr;
    }
    h->prm = *params;
    return upload_params(h);
}

fl_status fl_get_params(const fl_handle* h, fl_params* out) {
    if (!h || !out) return set_err(nullptr, FL_INVALID_ARG, "NULL argument");
    *out = h->prm;
    out->dims[1] = h->n;
    return FL_OK;
}

fl_status fl_set_particles(fl_handle* h, const float* aos, uint32_t n) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    if (n > h->cap) return set_err(h, FL_INVALID_ARG, "n exceeds the handle capacity");
    if (n && !aos) return set_err(h, FL_INVALID_ARG, "particles is NULL");
    h->init_part.assign(aos, aos + (size_t)n * 8);
    h->init_n = n;
    return fl_reset(h);
}

fl_status fl_get_particles(fl_handle* h, float* out, uint32_t* ids) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    if (out && h->n)
        FL_CUDA(h, cudaMemcpyAsync(out, h->partA, (size_t)h->n * 32, cudaMemcpyDeviceToHost, h->stream));
    if (ids && h->n) FL_CUDA(h, cudaMemcpyAsync(ids, h->idsA, (size_t)h->n * 4, cudaMemcpyDeviceToHost, h->stream));
    return read_status(h);
}

fl_status fl_particle_count(const fl_handle* h, uint32_t* n_out) {
    if (!h || !n_out) return set_err(nullptr, FL_INVALID_ARG, "NULL argument");
    *n_out = h->n;
    return FL_OK;
}

fl_status fl_step(fl_handle* h, uint32_t substeps) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    if (substeps == 0) return FL_OK;
    build_graph(h);
    for (uint32_t i = 0; i < substeps; i++) {
        if (h->profiling) {
            DevBufs b = h->b;
            b.part_in = h->partA;
            b.part_out = h->partA;
            b.ids_in = h->idsA;
            FL_CUDA(h, enqueue_step(h, b, h->stream, h->ev));
            FL_CUDA(h, cudaEventSynchronize(h->ev[FL_STAGE_COUNT]));
            for (int k = 0; k < FL_STAGE_COUNT; k++) {
                float ms = 0.0f;
                FL_CUDA(h, cudaEventElapsedTime(&ms, h->ev[k], h->ev[k + 1]));
                h->stage_ms[k] += ms;
            }
            h->stage_steps++;
        } else if (h->graph) {
            FL_CUDA(h, cudaGraphLaunch(h->graph, h->stream));
        } else {
            DevBufs b = h->b;
            b.part_in = h->partA;
            b.part_out = h->partA;
            b.ids_in = h->idsA;
            FL_CUDA(h, enqueue_step(h, b, h->stream));
        }
        h->substeps++;
    }
    return FL_OK;
}

fl_status fl_step_device(fl_handle* h, void* particles_dev, uint32_t n) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    if (n > h->cap) return set_err(h, FL_INVALID_ARG, "n exceeds the handle capacity");
    if (n && !particles_dev) return set_err(h, FL_INVALID_ARG, "particles_dev is NULL");
    if (((uintptr_t)particles_dev & 15u) != 0) return set_err(h, FL_INVALID_ARG, "particles_dev must be 16-byte aligned");
    cudaPointerAttributes attr;
    cudaError_t e = cudaPointerGetAttributes(&attr, particles_dev);
    if (e != cudaSuccess || (attr.type != cudaMemoryTypeDevice && attr.type != cudaMemoryTypeManaged)) {
        (void)cudaGetLastError();
        return set_err(h, FL_INVALID_ARG, "particles_dev is not a device pointer");
    }
    if (n != h->n) {
        h->n = n;
        fl_status s = upload_params(h);
        if (s != FL_OK) return s;
    }
    DevBufs b = h->b;
    b.part_in = (float4*)particles_dev;
    b.part_out = (float4*)particles_dev;
    b.ids_in = nullptr;
    FL_CUDA(h, enqueue_step(h, b, h->stream));
    h->substeps++;
    return FL_OK;
}

fl_status fl_step_host(fl_handle* h, const float* in, float* out, uint32_t n, uint32_t substeps) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    if (n > h->cap) return set_err(h, FL_INVALID_ARG, "n exceeds the handle capacity");
    if (n && (!in || !out)) return set_err(h, FL_INVALID_ARG, "particle buffer is NULL");
    if (n) FL_CUDA(h, cudaMemcpyAsync(h->partA, in, (size_t)n * 32, cudaMemcpyHostToDevice, h->stream));
    if (n != h->n) {
        h->n = n;
        fl_status s = upload_params(h);
        if (s != FL_OK) return s;
    }
    fl_status s = fl_step(h, substeps);
    if (s != FL_OK) return s;
    if (n) FL_CUDA(h, cudaMemcpyAsync(out, h->partA, (size_t)n * 32, cudaMemcpyDeviceToHost, h->stream));
    FL_CUDA(h, cudaStreamSynchronize(h->stream));
    return read_status(h);
}

fl_status fl_set_profiling(fl_handle* h, int enable) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    if (enable && !h->ev[0]) {
        for (int k = 0; k <= FL_STAGE_COUNT; k++) FL_CUDA(h, cudaEventCreate(&h->ev[k]));
    }
    h->profiling = enable != 0;
    return FL_OK;
}

fl_status fl_get_stage_times(fl_handle* h, double* ms_out, uint64_t* substeps_out) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    if (ms_out)
        for (int k = 0; k < FL_STAGE_COUNT; k++) ms_out[k] = h->stage_ms[k];
    if (substeps_out) *substeps_out = h->stage_steps;
    return FL_OK;
}

namespace {
// gpu/timing.rs:32-59 (FINE_SECTIONS) and :93 (CG_CATS), with the stage that times each.
struct SectionRow {
    const char* name;
    int stage;
};
constexpr SectionRow kSections[FL_SECTION_COUNT] = {
    {"clear", FL_STAGE_SORT},          {"mark", FL_STAGE_SORT},          {"sort", FL_STAGE_SORT},
    {"classify", FL_STAGE_CLASSIFY},   {"scatter", FL_STAGE_SCATTER},    {"normalize_u", FL_STAGE_PREP},
    {"normalize_v", FL_STAGE_PREP},    {"normalize_w", FL_STAGE_PREP},   {"savevel_u", FL_STAGE_PREP},
    {"savevel_v", FL_STAGE_PREP},      {"savevel_w", FL_STAGE_PREP},     {"forces_u", FL_STAGE_PREP},
    {"forces_v", FL_STAGE_PREP},       {"forces_w", FL_STAGE_PREP},      {"bound_pre_u", FL_STAGE_PREP},
    {"bound_pre_v", FL_STAGE_PREP},    {"bound_pre_w", FL_STAGE_PREP},   {"divergence", FL_STAGE_PREP},
    {"cg_init", FL_STAGE_PREP},        {"gradient_u", FL_STAGE_GRADIENT}, {"gradient_v", FL_STAGE_GRADIENT},
    {"gradient_w", FL_STAGE_GRADIENT}, {"bound_post_u", FL_STAGE_GRADIENT}, {"bound_post_v", FL_STAGE_GRADIENT},
    {"bound_post_w", FL_STAGE_GRADIENT}, {"g2p", FL_STAGE_G2P},         {"cg_spmv", FL_STAGE_CG},
    {"cg_reduce", FL_STAGE_CG},        {"cg_update", FL_STAGE_CG},       {"cg_scalars", FL_STAGE_CG},
};
}  // namespace

const char* fl_section_name(uint32_t i) { return i < FL_SECTION_COUNT ? kSections[i].name : nullptr; }

int fl_section_stage(uint32_t i) { return i < FL_SECTION_COUNT ? kSections[i].stage : -1; }

fl_status fl_get_coarse_times(fl_handle* h, double* ms_out, uint64_t* substeps_out) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    if (ms_out) {
        const double* t = h->stage_ms;
        ms_out[0] = t[FL_STAGE_SORT] + t[FL_STAGE_CLASSIFY] + t[FL_STAGE_SCATTER] + t[FL_STAGE_PREP];
        ms_out[1] = t[FL_STAGE_CG];
        ms_out[2] = t[FL_STAGE_GRADIENT] + t[FL_STAGE_G2P];
    }
    if (substeps_out) *substeps_out = h->stage_steps;
    return FL_OK;
}

fl_status fl_reset_stage_times(fl_handle* h) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    for (int k = 0; k < FL_STAGE_COUNT; k++) h->stage_ms[k] = 0.0;
    h->stage_steps = 0;
    return FL_OK;
}

fl_status fl_sync(fl_handle* h) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    FL_CUDA(h, cudaStreamSynchronize(h->stream));
    return read_status(h);
}

fl_status fl_set_stream(fl_handle* h, void* cuda_stream) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    FL_CUDA(h, cudaStreamSynchronize(h->stream));
    h->stream = cuda_stream ? (cudaStream_t)cuda_stream : h->own_stream;
    return FL_OK;
}

fl_status fl_set_wait_timeout(fl_handle* h, uint64_t ns) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    h->wait_ns = ns;
    return upload_params(h);
}

fl_status fl_apply_impulse(fl_handle* h, const float dv[3]) {
    if (!h || !dv) return set_err(h, FL_INVALID_ARG, "NULL argument");
    FL_CUDA(h, fl::launch_impulse(h->partA, h->dprm, dv[0], dv[1], dv[2], h->L, h->stream));
    return FL_OK;
}

fl_status fl_reset(fl_handle* h) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    h->n = h->init_n;
    if (h->n) {
        FL_CUDA(h, cudaMemcpyAsync(h->partA, h->init_part.data(), (size_t)h->n * 32, cudaMemcpyHostToDevice, h->stream));
        std::vector<uint32_t> ids(h->n);
        for (uint32_t i = 0; i < h->n; i++) ids[i] = i;
        FL_CUDA(h, cudaMemcpyAsync(h->idsA, ids.data(), (size_t)h->n * 4, cudaMemcpyHostToDevice, h->stream));
        FL_CUDA(h, cudaStreamSynchronize(h->stream));  // `ids` is a local
    }
    FL_CUDA(h, cudaMemsetAsync(h->b.p, 0, sizeof(float) * (size_t)h->C, h->stream));
    h->substeps = 0;
    return upload_params(h);
}

fl_status fl_get_grid(fl_handle* h, const fl_grid_view* v) {
    if (!h || !v) return set_err(h, FL_INVALID_ARG, "NULL argument");
    float* fd[6] = {v->u, v->v, v->w, v->u_saved, v->v_saved, v->w_saved};
    for (int a = 0; a < 6; a++) {
        if (!fd[a]) continue;
        const float* src = a < 3 ? h->b.vel[a] : h->b.sav[a - 3];
        FL_CUDA(h, cudaMemcpyAsync(fd[a], src, sizeof(float) * (size_t)h->F3[a % 3], cudaMemcpyDeviceToHost, h->stream));
    }
    const size_t C = h->C;
    if (v->pressure) FL_CUDA(h, cudaMemcpyAsync(v->pressure, h->b.p, 4 * C, cudaMemcpyDeviceToHost, h->stream));
    if (v->cell_type) FL_CUDA(h, cudaMemcpyAsync(v->cell_type, h->b.ct, C, cudaMemcpyDeviceToHost, h->stream));
    if (v->counts) FL_CUDA(h, cudaMemcpyAsync(v->counts, h->b.counts, 4 * C, cudaMemcpyDeviceToHost, h->stream));
    if (v->offsets) FL_CUDA(h, cudaMemcpyAsync(v->offsets, h->b.offsets, 4 * C, cudaMemcpyDeviceToHost, h->stream));
    return read_status(h);
}

fl_status fl_get_divergence(fl_handle* h, float* out) {
    if (!h || !out) return set_err(h, FL_INVALID_ARG, "NULL argument");
    FL_CUDA(h, cudaMemcpyAsync(out, h->b.div, sizeof(float) * (size_t)h->C, cudaMemcpyDeviceToHost, h->stream));
    return read_status(h);
}

fl_status fl_get_bins(fl_handle* h, uint32_t* counts, uint32_t* offsets, uint32_t* perm) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    const size_t C = h->C;
    if (counts) FL_CUDA(h, cudaMemcpyAsync(counts, h->b.counts, 4 * C, cudaMemcpyDeviceToHost, h->stream));
    if (offsets) FL_CUDA(h, cudaMemcpyAsync(offsets, h->b.offsets, 4 * C, cudaMemcpyDeviceToHost, h->stream));
    if (perm && h->n) FL_CUDA(h, cudaMemcpyAsync(perm, h->b.perm, 4 * (size_t)h->n, cudaMemcpyDeviceToHost, h->stream));
    return read_status(h);
}

fl_status fl_get_stats(fl_handle* h, fl_stats* out) {
    if (!h || !out) return set_err(h, FL_INVALID_ARG, "NULL argument");
    DevStats ds;
    FL_CUDA(h, cudaMemcpyAsync(&ds, h->dst, sizeof(ds), cudaMemcpyDeviceToHost, h->stream));
    FL_CUDA(h, cudaStreamSynchronize(h->stream));
    std::memset(out, 0, sizeof(*out));
    out->liquid_cells = ds.liquid;
    out->cg_iterations = ds.cg_iters;
    out->stray_particles = ds.strays;
    out->device_status = ds.status;
    out->substeps = h->substeps;
    out->rs_initial = ds.rs_init;
    out->rs_final = ds.rs_final;
    return FL_OK;
}

// State blob: header, particles (n*32 B), ids (n*4 B), pressure (C*4 B).
struct StateHeader {
    char magic[8];
    uint32_t version, nx, ny, nz, n, pad;
    uint64_t substeps;
};

fl_status fl_save_state(fl_handle* h, void* buf, size_t* size_inout) {
    if (!h || !size_inout) return set_err(h, FL_INVALID_ARG, "NULL argument");
    const size_t need = sizeof(StateHeader) + (size_t)h->n * 36 + 4 * (size_t)h->C;
    if (!buf) {
        *size_inout = need;
        return FL_OK;
    }
    if (*size_inout < need) return set_err(h, FL_INVALID_ARG, "buffer too small");
    StateHeader hd{};
    std::memcpy(hd.magic, "FLGBSTAT", 8);
    hd.version = 1; hd.nx = h->nx; hd.ny = h->ny; hd.nz = h->nz; hd.n = h->n; hd.substeps = h->substeps;
    char* p = (char*)buf;
    std::memcpy(p, &hd, sizeof(hd));
    p += sizeof(hd);
    if (h->n) {
        FL_CUDA(h, cudaMemcpyAsync(p, h->partA, (size_t)h->n * 32, cudaMemcpyDeviceToHost, h->stream));
        p += (size_t)h->n * 32;
        FL_CUDA(h, cudaMemcpyAsync(p, h->idsA, (size_t)h->n * 4, cudaMemcpyDeviceToHost, h->stream));
        p += (size_t)h->n * 4;
    }
    FL_CUDA(h, cudaMemcpyAsync(p, h->b.p, 4 * (size_t)h->C, cudaMemcpyDeviceToHost, h->stream));
    *size_inout = need;
    return read_status(h);
}

fl_status fl_load_state(fl_handle* h, const void* buf, size_t size) {
    if (!h || !buf) return set_err(h, FL_INVALID_ARG, "NULL argument");
    if (size < sizeof(StateHeader)) return set_err(h, FL_INVALID_ARG, "state blob too small");
    StateHeader hd;
    std::memcpy(&hd, buf, sizeof(hd));
    if (std::memcmp(hd.magic, "FLGBSTAT", 8) != 0 || hd.version != 1)
        return set_err(h, FL_INVALID_ARG, "not a state blob of this library");
    if (hd.nx != h->nx || hd.ny != h->ny || hd.nz != h->nz) return set_err(h, FL_INVALID_ARG, "grid mismatch");
    if (hd.n > h->cap) return set_err(h, FL_INVALID_ARG, "particle count exceeds capacity");
    const size_t need = sizeof(StateHeader) + (size_t)hd.n * 36 + 4 * (size_t)h->C;
    if (size < need) return set_err(h, FL_INVALID_ARG, "state blob truncated");
    const char* p = (const char*)buf + sizeof(hd);
    h->n = hd.n;
    if (h->n) {
        FL_CUDA(h, cudaMemcpyAsync(h->partA, p, (size_t)h->n * 32, cudaMemcpyHostToDevice, h->stream));
        p += (size_t)h->n * 32;
        FL_CUDA(h, cudaMemcpyAsync(h->idsA, p, (size_t)h->n * 4, cudaMemcpyHostToDevice, h->stream));
        p += (size_t)h->n * 4;
    }
    FL_CUDA(h, cudaMemcpyAsync(h->b.p, p, 4 * (size_t)h->C, cudaMemcpyHostToDevice, h->stream));
    h->substeps = hd.substeps;
    fl_status s = upload_params(h);
    if (s != FL_OK) return s;
    FL_CUDA(h, cudaStreamSynchronize(h->stream));
    return FL_OK;
}

fl_status fl_save_state_device(fl_handle* h, void* dst_dev, size_t* size_inout) {
    if (!h || !size_inout) return set_err(h, FL_INVALID_ARG, "NULL argument");
    const size_t need = sizeof(StateHeader) + (size_t)h->n * 36 + 4 * (size_t)h->C;
    if (!dst_dev) {
        *size_inout = need;
        return FL_OK;
    }
    if (*size_inout < need) return set_err(h, FL_INVALID_ARG, "buffer too small");
    if ((uintptr_t)dst_dev & 15u) return set_err(h, FL_INVALID_ARG, "device state buffer must be 16-byte aligned");
    StateHeader hd{};
    std::memcpy(hd.magic, "FLGBSTAT", 8);
    hd.version = 1; hd.nx = h->nx; hd.ny = h->ny; hd.nz = h->nz; hd.n = h->n; hd.substeps = h->substeps;
    char* p = (char*)dst_dev;
    // pageable source: the call returns once `hd` has been staged
    FL_CUDA(h, cudaMemcpyAsync(p, &hd, sizeof(hd), cudaMemcpyHostToDevice, h->stream));
    p += sizeof(hd);
    if (h->n) {
        FL_CUDA(h, cudaMemcpyAsync(p, h->partA, (size_t)h->n * 32, cudaMemcpyDeviceToDevice, h->stream));
        p += (size_t)h->n * 32;
        FL_CUDA(h, cudaMemcpyAsync(p, h->idsA, (size_t)h->n * 4, cudaMemcpyDeviceToDevice, h->stream));
        p += (size_t)h->n * 4;
    }
    FL_CUDA(h, cudaMemcpyAsync(p, h->b.p, 4 * (size_t)h->C, cudaMemcpyDeviceToDevice, h->stream));
    *size_inout = need;
    return FL_OK;
}

fl_status fl_load_state_device(fl_handle* h, const void* src_dev, size_t size) {
    if (!h || !src_dev) return set_err(h, FL_INVALID_ARG, "NULL argument");
    if (size < sizeof(StateHeader)) return set_err(h, FL_INVALID_ARG, "state blob too small");
    StateHeader hd;
    FL_CUDA(h, cudaMemcpyAsync(&hd, src_dev, sizeof(hd), cudaMemcpyDeviceToHost, h->stream));
    FL_CUDA(h, cudaStreamSynchronize(h->stream));
    if (std::memcmp(hd.magic, "FLGBSTAT", 8) != 0 || hd.version != 1)
        return set_err(h, FL_INVALID_ARG, "not a state blob of this library");
    if (hd.nx != h->nx || hd.ny != h->ny || hd.nz != h->nz) return set_err(h, FL_INVALID_ARG, "grid mismatch");
    if (hd.n > h->cap) return set_err(h, FL_INVALID_ARG, "particle count exceeds capacity");
    const size_t need = sizeof(StateHeader) + (size_t)hd.n * 36 + 4 * (size_t)h->C;
    if (size < need) return set_err(h, FL_INVALID_ARG, "state blob truncated");
    const char* p = (const char*)src_dev + sizeof(hd);
    h->n = hd.n;
    if (h->n) {
        FL_CUDA(h, cudaMemcpyAsync(h->partA, p, (size_t)h->n * 32, cudaMemcpyDeviceToDevice, h->stream));
        p += (size_t)h->n * 32;
        FL_CUDA(h, cudaMemcpyAsync(h->idsA, p, (size_t)h->n * 4, cudaMemcpyDeviceToDevice, h->stream));
        p += (size_t)h->n * 4;
    }
    FL_CUDA(h, cudaMemcpyAsync(h->b.p, p, 4 * (size_t)h->C, cudaMemcpyDeviceToDevice, h->stream));
    h->substeps = hd.substeps;
    return upload_params(h);
}

fl_status fl_solve_pressure(uint32_t nx, uint32_t ny, uint32_t nz, const uint8_t* cell_type, const float* divergence,
                            const float* pressure_in, float* pressure_out, float h, float rho, float dt,
                            uint32_t max_iters, uint32_t warm_start, float tolerance, uint32_t cg_precision,
                            fl_stats* stats_out) {
    if (!cell_type || !divergence || !pressure_out) return set_err(nullptr, FL_INVALID_ARG, "NULL argument");
    if (warm_start && !pressure_in) return set_err(nullptr, FL_INVALID_ARG, "warm start needs pressure_in");
    if (nx < 3 || ny < 3 || nz < 3 || (uint64_t)nx * ny * nz > (1ull << 30))
        return set_err(nullptr, FL_INVALID_ARG, "bad grid size");
    if (!(h > 0.0f) || !(rho > 0.0f) || !(dt > 0.0f)) return set_err(nullptr, FL_INVALID_ARG, "h, rho, dt must be > 0");
    if (cg_precision > FL_CG_F64_IEEE) return set_err(nullptr, FL_INVALID_ARG, "bad cg_precision");
    fl_status s = device_check(nullptr);
    if (s != FL_OK) return s;
    fl_params prm;
    std::memset(&prm, 0, sizeof(prm));
    prm.gdim[0] = nx; prm.gdim[1] = ny; prm.gdim[2] = nz;
    prm.geom[0] = h; prm.geom[1] = 1.0f / h; prm.geom[2] = dt; prm.geom[3] = 65536.0f;
    prm.phys[1] = rho;
    prm.dims[2] = max_iters;
    prm.dims[3] = warm_start ? 1u : 0u;
    prm.pressure_tolerance = tolerance;
    prm.cg_precision = cg_precision;
    DevParams hp;
    derive(prm, 0, hp);
    const size_t C = hp.C;
    const uint32_t nchunks = hp.nchunks;
    fl::LaunchCfg L = make_cfg(nchunks);
    PoolPlan pl;
    size_t o_ct = pl.take<uint8_t>(C), o_div = pl.take<float>(C), o_p = pl.take<float>(C), o_r = pl.take<float>(C),
           o_dA = pl.take<float>(C), o_dB = pl.take<float>(C), o_q = pl.take<float>(C);
    size_t o_flag = pl.take<uint8_t>(nchunks), o_prr = pl.take<float>(nchunks);
    size_t o_cinfo = pl.take<uint16_t>(C);
    size_t o_c64 = pl.take<float2>(nchunks);
    size_t o_plan = pl.take<uint32_t>(nchunks), o_poff = pl.take<uint32_t>(fl::cg_plan_words(L.cg_blocks));
    size_t o_cgx = pl.take<unsigned long long>(fl::cg_x_words(nchunks, L.cg_blocks));
    size_t o_prm = pl.take<DevParams>(1), o_st = pl.take<DevStats>(1);
    void* pool = nullptr;
    cudaError_t e = cudaMalloc(&pool, pl.off);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return set_err(nullptr, FL_OOM, "cudaMalloc failed");
    }
    char* base = (char*)pool;
    DevBufs b{};
    b.prm = (DevParams*)(base + o_prm);
    b.st = (DevStats*)(base + o_st);
    b.ct = (uint8_t*)(base + o_ct);
    b.p = (float*)(base + o_p);
    b.r = (float*)(base + o_r);
    b.dA = (float*)(base + o_dA);
    b.dB = (float*)(base + o_dB);
    b.q = (float*)(base + o_q);
    b.chunk_flag = (uint8_t*)(base + o_flag);
    b.cinfo = (uint16_t*)(base + o_cinfo);
    b.part_rr = (float*)(base + o_prr);
    b.chunk_rr_df = (float2*)(base + o_c64);
    b.cg_chunk = (uint32_t*)(base + o_plan);
    b.cg_off = (uint32_t*)(base + o_poff);
    b.cg_x = (unsigned long long*)(base + o_cgx);
    float* ddiv = (float*)(base + o_div);
    cudaStream_t st = nullptr;
    fl_status rs = FL_OK;
    DevStats ds{};
    do {
        if ((e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(pool, 0, pl.off, st)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync((void*)b.prm, &hp, sizeof(hp), cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(b.ct, cell_type, C, cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(ddiv, divergence, 4 * C, cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
        if (warm_start && (e = cudaMemcpyAsync(b.p, pressure_in, 4 * C, cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
        if ((e = fl::launch_solve_init(b, (uint32_t)C, ddiv, st)) != cudaSuccess) break;
        if ((e = fl::launch_cg(b, L, st, cg_precision)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(pressure_out, b.p, 4 * C, cudaMemcpyDeviceToHost, st)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(&ds, b.st, sizeof(ds), cudaMemcpyDeviceToHost, st)) != cudaSuccess) break;
        e = cudaStreamSynchronize(st);
    } while (0);
    if (e != cudaSuccess) rs = cuda_err(nullptr, e, "fl_solve_pressure");
    if (st) cudaStreamDestroy(st);
    cudaFree(pool);
    if (rs != FL_OK) return rs;
    if (ds.status) return set_err(nullptr, (fl_status)ds.status, "a device-side wait expired");
    if (stats_out) {
        std::memset(stats_out, 0, sizeof(*stats_out));
        stats_out->cg_iterations = ds.cg_iters;
        stats_out->rs_initial = ds.rs_init;
        stats_out->rs_final = ds.rs_final;
    }
    return FL_OK;
}

fl_status fl_relax_pressure(uint32_t nx, uint32_t ny, uint32_t nz, const uint8_t* cell_type, const float* divergence,
                            float h, float rho, float dt, uint32_t method, uint32_t iters, float* pressure_out) {
    if (!cell_type || !divergence || !pressure_out) return set_err(nullptr, FL_INVALID_ARG, "NULL argument");
    if (nx < 3 || ny < 3 || nz < 3 || (uint64_t)nx * ny * nz > (1ull << 30))
        return set_err(nullptr, FL_INVALID_ARG, "bad grid size");
    if (!(h > 0.0f) || !(rho > 0.0f) || !(dt > 0.0f)) return set_err(nullptr, FL_INVALID_ARG, "h, rho, dt must be > 0");
    if (method > 1u) return set_err(nullptr, FL_INVALID_ARG, "method must be FL_RELAX_JACOBI or FL_RELAX_RBGS");
    fl_status s = device_check(nullptr);
    if (s != FL_OK) return s;
    const size_t C = (size_t)nx * ny * nz;
    const float scale = rho * h * h / dt;  // ProjectionParams::rhs_scale (sim/pressure.rs:31-33)
    PoolPlan pl;
    const size_t o_ct = pl.take<uint8_t>(C), o_div = pl.take<float>(C), o_a = pl.take<float>(C),
                 o_b = pl.take<float>(C);
    void* pool = nullptr;
    cudaError_t e = cudaMalloc(&pool, pl.off);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        return set_err(nullptr, FL_OOM, "cudaMalloc failed");
    }
    char* base = (char*)pool;
    uint8_t* dct = (uint8_t*)(base + o_ct);
    float* ddiv = (float*)(base + o_div);
    float* pa = (float*)(base + o_a);
    float* pb = (float*)(base + o_b);
    float* res = pa;
    cudaStream_t st = nullptr;
    do {
        if ((e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking)) != cudaSuccess) break;
        if ((e = cudaMemsetAsync(pool, 0, pl.off, st)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(dct, cell_type, C, cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
        if ((e = cudaMemcpyAsync(ddiv, divergence, 4 * C, cudaMemcpyHostToDevice, st)) != cudaSuccess) break;
        if ((e = fl::launch_relax(dct, ddiv, scale, pa, pb, nx, ny, nz, method, iters, st, &res)) != cudaSuccess)
            break;
        if ((e = cudaMemcpyAsync(pressure_out, res, 4 * C, cudaMemcpyDeviceToHost, st)) != cudaSuccess) break;
        e = cudaStreamSynchronize(st);
    } while (0);
    fl_status rs = e != cudaSuccess ? cuda_err(nullptr, e, "fl_relax_pressure") : FL_OK;
    if (st) cudaStreamDestroy(st);
    cudaFree(pool);
    return rs;
}

fl_status fl_get_particles_device(fl_handle* h, void* dst_dev, uint32_t* ids_dev) {
    if (!h || (!dst_dev && h->n)) return set_err(h, FL_INVALID_ARG, "NULL argument");
    if (h->n) FL_CUDA(h, cudaMemcpyAsync(dst_dev, h->partA, (size_t)h->n * 32, cudaMemcpyDeviceToDevice, h->stream));
    if (h->n && ids_dev)
        FL_CUDA(h, cudaMemcpyAsync(ids_dev, h->idsA, (size_t)h->n * 4, cudaMemcpyDeviceToDevice, h->stream));
    FL_CUDA(h, cudaStreamSynchronize(h->stream));
    return read_status(h);
}

fl_status fl_set_particles_device(fl_handle* h, const void* src_dev, uint32_t n) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    if (n > h->cap) return set_err(h, FL_INVALID_ARG, "n exceeds the handle capacity");
    if (n && !src_dev) return set_err(h, FL_INVALID_ARG, "src_dev is NULL");
    if (n) FL_CUDA(h, cudaMemcpyAsync(h->partA, src_dev, (size_t)n * 32, cudaMemcpyDeviceToDevice, h->stream));
    FL_CUDA(h, fl::launch_iota(h->idsA, n, h->stream));
    if (n != h->n) {
        h->n = n;
        fl_status s = upload_params(h);
        if (s != FL_OK) return s;
    }
    FL_CUDA(h, cudaStreamSynchronize(h->stream));
    return FL_OK;
}

fl_status fl_seed_count(const fl_params* params, const fl_block* blocks, uint32_t nblocks, uint32_t particle_count,
                        uint32_t* n_out) {
    if (!params || !n_out) return set_err(nullptr, FL_INVALID_ARG, "NULL argument");
    fl::SeedArgs a;
    const long long n = fl::seed_layout(*params, blocks, nblocks, particle_count, &a);
    if (n < 0) return set_err(nullptr, FL_INVALID_ARG, "need 1..FL_SCENE_MAX_BLOCKS blocks");
    *n_out = (uint32_t)n;
    return FL_OK;
}

// generate_particles (fluid.rs:1838-1913) on the device: the lattice is laid
// out on the host, every particle is computed by its own thread.
fl_status fl_seed_particles(fl_handle* h, const fl_block* blocks, uint32_t nblocks, uint32_t particle_count,
                            uint32_t* n_out) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    fl::SeedArgs a;
    const long long n = fl::seed_layout(h->prm, blocks, nblocks, particle_count, &a);
    if (n < 0) return set_err(h, FL_INVALID_ARG, "need 1..FL_SCENE_MAX_BLOCKS blocks");
    if (n_out) *n_out = (uint32_t)n;
    if ((unsigned long long)n > h->cap)
        return set_err(h, FL_INVALID_ARG, "the layout has " + std::to_string(n) + " particles, above the capacity");
    FL_CUDA(h, fl::launch_seed(a, h->partA, h->stream));
    // the seeded particles become the state fl_reset restores
    h->init_part.resize((size_t)n * 8);
    if (n) FL_CUDA(h, cudaMemcpyAsync(h->init_part.data(), h->partA, (size_t)n * 32, cudaMemcpyDeviceToHost, h->stream));
    FL_CUDA(h, cudaStreamSynchronize(h->stream));
    h->init_n = (uint32_t)n;
    return fl_reset(h);
}

// Headless grid slice (slice.wgsl:69-141): one float4 {r, g, b, visible} per
// cell of the XY cross-section at k.
fl_status fl_grid_slice_device(fl_handle* h, uint32_t mode, uint32_t slice_k, void* rgba_dev) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    if (!rgba_dev || ((uintptr_t)rgba_dev & 15u)) return set_err(h, FL_INVALID_ARG, "rgba_dev must be 16-byte aligned");
    const uint32_t k = slice_k == FL_SLICE_MIDDLE ? h->nz / 2 : slice_k;
    if (k >= h->nz) return set_err(h, FL_INVALID_ARG, "slice_k out of range");
    FL_CUDA(h, fl::launch_slice(h->b, h->nx, h->ny, mode, k, (float4*)rgba_dev, h->stream));
    return FL_OK;
}

fl_status fl_grid_slice(fl_handle* h, uint32_t mode, uint32_t slice_k, float* rgba_out) {
    if (!h) return set_err(nullptr, FL_INVALID_ARG, "handle is NULL");
    if (!rgba_out) return set_err(h, FL_INVALID_ARG, "rgba_out is NULL");
    const size_t bytes = sizeof(float4) * (size_t)h->nx * h->ny;
    if (!h->slice_buf) {
        cudaError_t e = cudaMalloc(&h->slice_buf, bytes);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            h->slice_buf = nullptr;
            return set_err(h, FL_OOM, "slice buffer allocation failed");
        }
    }
    fl_status s = fl_grid_slice_device(h, mode, slice_k, h->slice_buf);
    if (s != FL_OK) return s;
    FL_CUDA(h, cudaMemcpyAsync(rgba_out, h->slice_buf, bytes, cudaMemcpyDeviceToHost, h->stream));
    FL_CUDA(h, cudaStreamSynchronize(h->stream));
    return FL_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// tapes and the adjoint step

struct fl_tape {
    fl_handle* h = nullptr;
    uint32_t max_steps = 0, count = 0;
    void* pool = nullptr;
    char* slots = nullptr;
    size_t slot_bytes = 0, o_part = 0, o_perm = 0, o_ct = 0, o_off = 0, o_sav[3] = {}, o_fin[3] = {};
    float4* g_sorted = nullptr;
    float2* g_fs[3] = {};
    float* g_norm[3] = {};
    float2* wsum[3] = {};
    unsigned long long* gmid[3] = {};
    double* grav_part[3] = {};
    float4* coef = nullptr;
    float4* mid = nullptr;
    uint32_t* flags = nullptr;
    float* rhs = nullptr;
    double* g_grav = nullptr;
    DevBufs cg{};        // buffers of the adjoint pressure solve (cg.p holds lambda)
    DevParams hp_cg{};
    fl_stats last{};     // of the last adjoint pressure solve
    bool adj_warm = false;  // start each adjoint solve from the previous lambda
    fl::MgBufs mg{};        // multigrid hierarchy of the adjoint solve (FL_SOLVER_MGPCG)
    void* mg_pool = nullptr;
    uint32_t adj_solver = 0xffffffffu;  // FL_SOLVER_*, or the handle's pressure_solver
};

extern "C" {

fl_status fl_tape_create(fl_handle* h, uint32_t max_steps, fl_tape** out) {
    if (!h || !out || max_steps == 0) return set_err(h, FL_INVALID_ARG, "bad argument");
    *out = nullptr;
    fl_tape* t = new (std::nothrow) fl_tape();
    if (!t) return set_err(h, FL_OOM, "host allocation failed");
    t->h = h;
    t->max_steps = max_steps;
    const size_t cap = std::max<uint32_t>(h->cap, 1), C = h->C, nch = h->nchunks;
    const size_t gmax = (size_t)g_num_sms * g_cg_per_sm;
    PoolPlan slot;
    t->o_part = slot.take<float4>(2 * cap);
    t->o_perm = slot.take<uint32_t>(cap);
    t->o_ct = slot.take<uint8_t>(C);
    t->o_off = slot.take<uint32_t>(C);  // the step's bin offsets (first particle of every cell)
    for (int a = 0; a < 3; a++) {
        t->o_sav[a] = slot.take<float>(h->F3[a]);
        t->o_fin[a] = slot.take<float>(h->F3[a]);
    }
    t->slot_bytes = (slot.off + 255) & ~size_t(255);
    PoolPlan pl;
    pl.off = t->slot_bytes * max_steps;
    size_t o_gs = pl.take<float4>(2 * cap), o_gf[3], o_gn[3], o_ws[3], o_gm[3], o_gp[3];
    for (int a = 0; a < 3; a++) {
        o_gf[a] = pl.take<float2>(h->F3[a]);
        o_gn[a] = pl.take<float>(h->F3[a]);
        o_ws[a] = pl.take<float2>(h->F3[a]);
        o_gm[a] = pl.take<unsigned long long>(h->F3[a]);
        o_gp[a] = pl.take<double>((h->F3[a] + 255) / 256);
    }
    const size_t o_coef = pl.take<float4>(3 * cap), o_mid = pl.take<float4>(2 * cap), o_flags = pl.take<uint32_t>(2);
    size_t o_rhs = pl.take<float>(C), o_lam = pl.take<float>(C), o_r = pl.take<float>(C), o_dA = pl.take<float>(C),
           o_dB = pl.take<float>(C), o_q = pl.take<float>(C), o_ci = pl.take<uint16_t>(C), o_fl = pl.take<uint8_t>(nch),
           o_prr = pl.take<float>(nch), o_c64 = pl.take<float2>(nch), o_plan = pl.take<uint32_t>(nch),
           o_poff = pl.take<uint32_t>(fl::cg_plan_words(gmax)), o_gg = pl.take<double>(3),
           o_prm = pl.take<DevParams>(1), o_st = pl.take<DevStats>(1);
    const size_t cgx_words = fl::cg_x_words(nch, gmax);
    const size_t o_cgx = pl.take<unsigned long long>(cgx_words);
    cudaError_t e = cudaMalloc(&t->pool, pl.off);
    if (e != cudaSuccess) {
        (void)cudaGetLastError();
        delete t;
        return set_err(h, FL_OOM, "tape allocation of " + std::to_string(pl.off) + " bytes failed");
    }
    char* base = (char*)t->pool;
    t->slots = base;
    t->g_sorted = (float4*)(base + o_gs);
    for (int a = 0; a < 3; a++) {
        t->g_fs[a] = (float2*)(base + o_gf[a]);
        t->g_norm[a] = (float*)(base + o_gn[a]);
        t->wsum[a] = (float2*)(base + o_ws[a]);
        t->gmid[a] = (unsigned long long*)(base + o_gm[a]);
        t->grav_part[a] = (double*)(base + o_gp[a]);
    }
    t->coef = (float4*)(base + o_coef);
    t->mid = (float4*)(base + o_mid);
    t->flags = (uint32_t*)(base + o_flags);
    t->rhs = (float*)(base + o_rhs);
    t->g_grav = (double*)(base + o_gg);
    DevBufs& b = t->cg;
    b.prm = (DevParams*)(base + o_prm);
    b.st = (DevStats*)(base + o_st);
    b.p = (float*)(base + o_lam);
    b.r = (float*)(base + o_r);
    b.dA = (float*)(base + o_dA);
    b.dB = (float*)(base + o_dB);
    b.q = (float*)(base + o_q);
    b.cinfo = (uint16_t*)(base + o_ci);
    b.chunk_flag = (uint8_t*)(base + o_fl);
    b.part_rr = (float*)(base + o_prr);
    b.chunk_rr_df = (float2*)(base + o_c64);
    b.cg_chunk = (uint32_t*)(base + o_plan);
    b.cg_off = (uint32_t*)(base + o_poff);
    b.cg_x = (unsigned long long*)(base + o_cgx);
    // The exchange words start cleared (tags of an earlier owner of this
    // memory must not match); lambda starts at zero for a warm start.
    if ((e = cudaMemsetAsync(b.cg_x, 0, cgx_words * sizeof(unsigned long long), h->stream)) != cudaSuccess ||
        (e = cudaMemsetAsync(b.p, 0, sizeof(float) * C, h->stream)) != cudaSuccess ||
        (e = cudaStreamSynchronize(h->stream)) != cudaSuccess) {
        cudaFree(t->pool);
        delete t;
        return cuda_err(h, e, "tape exchange-area clear");
    }
    *out = t;
    return FL_OK;
}

fl_status fl_tape_free(fl_tape* t) {
    if (!t) return FL_OK;
    if (t->h && t->h->stream) cudaStreamSynchronize(t->h->stream);
    if (t->pool) cudaFree(t->pool);
    if (t->mg_pool) cudaFree(t->mg_pool);
    delete t;
    return FL_OK;
}

fl_status fl_tape_clear(fl_tape* t) {
    if (!t) return set_err(nullptr, FL_INVALID_ARG, "tape is NULL");
    t->count = 0;
    return FL_OK;
}

fl_status fl_tape_set_adjoint_warm_start(fl_tape* t, int enable) {
    if (!t) return set_err(nullptr, FL_INVALID_ARG, "tape is NULL");
    fl_handle* h = t->h;
    t->adj_warm = enable != 0;
    FL_CUDA(h, cudaMemsetAsync(t->cg.p, 0, sizeof(float) * (size_t)h->C, h->stream));
    return FL_OK;
}

fl_status fl_tape_set_adjoint_solver(fl_tape* t, uint32_t solver) {
    if (!t) return set_err(nullptr, FL_INVALID_ARG, "tape is NULL");
    if (solver > FL_SOLVER_MGPCG && solver != FL_SOLVER_FOLLOW)
        return set_err(t->h, FL_INVALID_ARG, "solver must be FL_SOLVER_CG, FL_SOLVER_MGPCG or FL_SOLVER_FOLLOW");
    t->adj_solver = solver;
    return FL_OK;
}

fl_status fl_tape_count(const fl_tape* t, uint32_t* n_out) {
    if (!t || !n_out) return set_err(nullptr, FL_INVALID_ARG, "NULL argument");
    *n_out = t->count;
    return FL_OK;
}

fl_status fl_tape_last_stats(const fl_tape* t, fl_stats* out) {
    if (!t || !out) return set_err(nullptr, FL_INVALID_ARG, "NULL argument");
    *out = t->last;
    return FL_OK;
}

}  // extern "C"

namespace {

// Append the step just enqueued on the handle to the tape.
fl_status tape_append(fl_handle* h, fl_tape* t) {
    char* slot = t->slots + (size_t)t->count * t->slot_bytes;
    const size_t n = h->n;
    cudaStream_t st = h->stream;
    if (n) {
        FL_CUDA(h, cudaMemcpyAsync(slot + t->o_part, h->b.part_sorted, 32 * n, cudaMemcpyDeviceToDevice, st));
        FL_CUDA(h, cudaMemcpyAsync(slot + t->o_perm, h->b.perm, 4 * n, cudaMemcpyDeviceToDevice, st));
    }
    FL_CUDA(h, cudaMemcpyAsync(slot + t->o_ct, h->b.ct, h->C, cudaMemcpyDeviceToDevice, st));
    FL_CUDA(h, cudaMemcpyAsync(slot + t->o_off, h->b.offsets, 4 * (size_t)h->C, cudaMemcpyDeviceToDevice, st));
    for (int a = 0; a < 3; a++) {
        const size_t fb = 4 * (size_t)h->F3[a];
        FL_CUDA(h, cudaMemcpyAsync(slot + t->o_sav[a], h->b.sav[a], fb, cudaMemcpyDeviceToDevice, st));
        FL_CUDA(h, cudaMemcpyAsync(slot + t->o_fin[a], h->b.vel[a], fb, cudaMemcpyDeviceToDevice, st));
    }
    t->count++;
    return FL_OK;
}

}  // namespace

extern "C" {

fl_status fl_step_record(fl_handle* h, fl_tape* t) {
    if (!h || !t || t->h != h) return set_err(h, FL_INVALID_ARG, "tape does not belong to this handle");
    if (t->count >= t->max_steps) return set_err(h, FL_INVALID_ARG, "tape is full");
    fl_status s = fl_step(h, 1);
    if (s != FL_OK) return s;
    return tape_append(h, t);
}

fl_status fl_copy_pressure_device(fl_handle* h, void* dst_dev) {
    if (!h || !dst_dev) return set_err(h, FL_INVALID_ARG, "NULL argument");
    FL_CUDA(h, cudaMemcpyAsync(dst_dev, h->b.p, sizeof(float) * (size_t)h->C, cudaMemcpyDeviceToDevice, h->stream));
    return FL_OK;
}

fl_status fl_step_replay(fl_handle* h, const void* pressure_dev, fl_tape* t) {
    if (!h || !pressure_dev) return set_err(h, FL_INVALID_ARG, "NULL argument");
    if (t && t->h != h) return set_err(h, FL_INVALID_ARG, "tape does not belong to this handle");
    if (t && t->count >= t->max_steps) return set_err(h, FL_INVALID_ARG, "tape is full");
    DevBufs b = h->b;
    b.part_in = h->partA;
    b.part_out = h->partA;
    b.ids_in = h->idsA;
    FL_CUDA(h, enqueue_step(h, b, h->stream, nullptr, (const float*)pressure_dev));
    h->substeps++;
    return t ? tape_append(h, t) : FL_OK;
}

fl_status fl_step_adjoint(fl_handle* h, fl_tape* t, const void* dL_dout_dev, void* dL_din_dev, float* dL_dgrav,
                          uint32_t adj_cg_iters, float adj_cg_tol) {
    if (!h || !t || t->h != h) return set_err(h, FL_INVALID_ARG, "tape does not belong to this handle");
    if (t->count == 0) return set_err(h, FL_INVALID_ARG, "tape is empty");
    if (h->n && (!dL_dout_dev || !dL_din_dev)) return set_err(h, FL_INVALID_ARG, "gradient buffer is NULL");
    const uint32_t k = t->count - 1;
    char* slot = t->slots + (size_t)k * t->slot_bytes;
    cudaStream_t st = h->stream;
    fl::AdjBufs a{};
    a.prm = h->dprm;
    a.part = (const float4*)(slot + t->o_part);
    a.perm = (const uint32_t*)(slot + t->o_perm);
    a.ct = (const uint8_t*)(slot + t->o_ct);
    a.cell_first = (const uint32_t*)(slot + t->o_off);
    const bool midpoint = h->prm.advect_order == 2u;
    for (int ax = 0; ax < 3; ax++) {
        a.sav[ax] = (const float*)(slot + t->o_sav[ax]);
        a.fin[ax] = (const float*)(slot + t->o_fin[ax]);
        a.g_fs[ax] = t->g_fs[ax];
        a.g_norm[ax] = t->g_norm[ax];
        a.wsum[ax] = t->wsum[ax];
        a.gmid[ax] = t->gmid[ax];
        a.grav_part[ax] = t->grav_part[ax];
        if (midpoint) FL_CUDA(h, cudaMemsetAsync(t->gmid[ax], 0, 8 * (size_t)h->F3[ax], st));
    }
    a.coef = t->coef;
    a.mid = t->mid;
    a.flags = t->flags;
    FL_CUDA(h, cudaMemsetAsync(t->flags, 0, 2 * sizeof(uint32_t), st));
    a.g_out = (const float4*)dL_dout_dev;
    a.g_sorted = t->g_sorted;
    a.g_in = (float4*)dL_din_dev;
    a.lam = t->cg.p;
    a.rhs = t->rhs;
    a.rhs_part = t->adj_warm ? t->cg.chunk_rr_df : nullptr;  // free until k_solve_init
    a.g_grav = t->g_grav;
    FL_CUDA(h, fl::launch_adj_g2p(a, h->L, st));
    if (midpoint) FL_CUDA(h, fl::launch_adj_mid(a, h->L, st));
    FL_CUDA(h, fl::launch_adj_gather(a, h->C, midpoint, st));
    FL_CUDA(h, fl::launch_adj_prhs(a, h->C, st));
    // adjoint pressure solve: A lambda = dL/dp (k_solve_init's rhs is
    // -scale*div, so scale = -1 passes dL/dp through unchanged).  Cold start:
    // stop at |r| <= tol |r0| = tol |dL/dp|.  Warm start from the previous
    // step's lambda: the same bound, as an absolute threshold from k_adj_thr.
    fl_params q;
    std::memset(&q, 0, sizeof(q));
    q.gdim[0] = h->nx; q.gdim[1] = h->ny; q.gdim[2] = h->nz;
    q.geom[0] = h->prm.geom[0]; q.geom[1] = h->prm.geom[1]; q.geom[2] = h->prm.geom[2]; q.geom[3] = h->prm.geom[3];
    q.phys[1] = h->prm.phys[1];
    q.dims[2] = adj_cg_iters ? adj_cg_iters : 1u;
    q.dims[3] = t->adj_warm ? 1u : 0u;
    q.pressure_tolerance = adj_cg_tol;
    q.cg_precision = h->prm.cg_precision;
    derive(q, h->n, t->hp_cg);
    t->hp_cg.scale_rhs = -1.0f;
    t->hp_cg.wait_ns = h->wait_ns;
    DevBufs cg = t->cg;
    cg.ct = const_cast<uint8_t*>(a.ct);
    FL_CUDA(h, cudaMemcpyAsync((void*)cg.prm, &t->hp_cg, sizeof(DevParams), cudaMemcpyHostToDevice, st));
    FL_CUDA(h, cudaMemsetAsync(cg.st, 0, sizeof(DevStats), st));
    if (t->adj_warm) FL_CUDA(h, fl::launch_adj_thr(a, h->nchunks, t->hp_cg.tol_sq_d, (DevParams*)cg.prm, st));
    FL_CUDA(h, fl::launch_solve_init(cg, h->C, t->rhs, st));
    const uint32_t solver = t->adj_solver == FL_SOLVER_FOLLOW ? h->prm.pressure_solver : t->adj_solver;
    if (solver == FL_SOLVER_MGPCG) {
        // the same system through the multigrid preconditioner
        fl_status ms = mg_alloc(h, h->nx, h->ny, h->nz, t->cg.r, &t->mg, &t->mg_pool);
        if (ms != FL_OK) return ms;
        FL_CUDA(h, fl::launch_mgpcg(cg, t->mg, h->L, st));
    } else {
        FL_CUDA(h, fl::launch_cg(cg, h->L, st, h->prm.cg_precision));
    }
    FL_CUDA(h, fl::launch_adj_faces(a, h->F3, st));
    FL_CUDA(h, fl::launch_adj_p2g(a, h->L, st));
    FL_CUDA(h, fl::launch_adj_unsort(a, h->L, st));
    double gg[3];
    DevStats ds;
    FL_CUDA(h, cudaMemcpyAsync(gg, t->g_grav, sizeof(gg), cudaMemcpyDeviceToHost, st));
    FL_CUDA(h, cudaMemcpyAsync(&ds, cg.st, sizeof(ds), cudaMemcpyDeviceToHost, st));
    FL_CUDA(h, cudaStreamSynchronize(st));
    t->last = fl_stats{};
    t->last.liquid_cells = ds.liquid;
    t->last.cg_iterations = ds.cg_iters;
    t->last.device_status = ds.status;
    t->last.rs_initial = ds.rs_init;
    t->last.rs_final = ds.rs_final;
    if (ds.status) return set_err(h, (fl_status)ds.status, "adjoint pressure solve: a device-side wait expired");
    if (dL_dgrav)
        for (int i = 0; i < 3; i++) dL_dgrav[i] += (float)gg[i];
    t->count--;
    return FL_OK;
}

const char* fl_last_error(const fl_handle* h) {
    if (h) return h->err.c_str();
    return g_err.c_str();
}

}  // extern "C"
