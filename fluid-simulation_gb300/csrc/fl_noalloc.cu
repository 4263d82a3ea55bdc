// fl_noalloc.cu — fl_solve_pressure_noalloc: the pressure CG with its scratch
// in a fixed, file-scope device array instead of device memory allocated per
// call.
//
// Who needs this: callers that must not (or cannot) call cudaMalloc around
// the solve — code running between the steps of a frame loop that has a
// no-allocation rule for latency, plugins embedded in a host application that
// owns every device allocation through its own pool, and tools that must not
// grow the device footprint after start-up.  They pass the inputs and the
// output as device pointers; this entry point allocates nothing.
//
// The scratch (CG vectors r, d (two copies), q, the stencil masks, per-chunk
// partials, the solve plan, the exchange words, the settings block and the
// device counters) lives in `g_noalloc_scratch`, sized for at most
// FL_NOALLOC_MAX_CELLS cells (~4.6 MB).  Every GPU that loads this library
// holds that array until the process exits.  All calls share it: a call keeps
// the previous call's contents, so the set-up kernel clears what must start at
// zero (the counters and the status word; the exchange words carry tags that
// are unique per solve and need no clearing), and calls that overlap on the
// GPU (different streams, or different host threads) race on it.
//
// In host code `g_noalloc_scratch` is a host-side stand-in, not a device
// address.  The device address is obtained once per device, with that device
// current, by cudaGetSymbolAddress on the first call on that device.  Every
// call copies the solve's statistics back and synchronizes the caller's
// stream, so the entry point cannot be called while that stream is being
// captured into a CUDA graph.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/fluidgb.h"
#include "fl_device.cuh"

void fl_record_global_error(const std::string& msg);  // fl_host.cpp

namespace {

constexpr size_t kMaxCtas = 1024;  // cooperative blocks the plan header and exchange area are sized for
constexpr size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// Scratch layout (byte offsets), sized for FL_NOALLOC_MAX_CELLS cells.
constexpr size_t kCells = FL_NOALLOC_MAX_CELLS;
constexpr size_t kChunks = (kCells + fl::CHUNK - 1) / fl::CHUNK;
constexpr size_t kOffParams = 0;
constexpr size_t kOffStats = align256(kOffParams + sizeof(fl::DevParams));
constexpr size_t kOffR = align256(kOffStats + sizeof(fl::DevStats));
constexpr size_t kOffDA = align256(kOffR + 4 * kCells);
constexpr size_t kOffDB = align256(kOffDA + 4 * kCells);
constexpr size_t kOffQ = align256(kOffDB + 4 * kCells);
constexpr size_t kOffFlag = align256(kOffQ + 4 * kCells);
constexpr size_t kOffPrr = align256(kOffFlag + kChunks);
constexpr size_t kOffC64 = align256(kOffPrr + 4 * kChunks);
constexpr size_t kOffPlan = align256(kOffC64 + 8 * kChunks);
constexpr size_t kOffPlanOff = align256(kOffPlan + 4 * kChunks);
constexpr size_t kOffInfo = align256(kOffPlanOff + 4 * fl::cg_plan_words(kMaxCtas));
constexpr size_t kOffX = align256(kOffInfo + 2 * kCells);
constexpr size_t kScratchBytes = align256(kOffX + 8 * fl::cg_x_words(kChunks, kMaxCtas));

constexpr int kMaxDevices = 64;

}  // namespace

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {

std::mutex g_mu;
void* g_scratch_dev[kMaxDevices] = {};
int g_sms[kMaxDevices] = {};
int g_cg_per_sm[kMaxDevices] = {};
// Failures return their fl_status and leave the message where
// fl_last_error(NULL) reads it (the slot fl_solve_pressure uses).
fl_status fail(fl_status s, const std::string& m) {
    fl_record_global_error("fl_solve_pressure_noalloc: " + m);
    return s;
}

// True when byte ranges [a, a + na) and [b, b + nb) share a byte.
bool overlaps(const void* a, size_t na, const void* b, size_t nb) {
    const uintptr_t x = (uintptr_t)a, y = (uintptr_t)b;
    return x < y + nb && y < x + na;
}

// Writes the settings block and clears the counters the CG relies on.
__global__ void k_noalloc_setup(fl::DevParams prm, fl::DevParams* dst, fl::DevStats* st) {
    if (threadIdx.x == 0) {
        *dst = prm;
        memset(st, 0, sizeof(fl::DevStats));
    }
}

// Once per device, with the device current: the device address of the array.
fl_status device_setup(int dev) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (g_scratch_dev[dev]) return FL_OK;
    int major = 0, minor = 0, coop = 0, sms = 0;
    cudaError_t e = cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return fail(FL_NO_DEVICE, std::string("device query: ") + cudaGetErrorString(e));
    if (!(major == 10 && minor == 3)) return fail(FL_NO_DEVICE, "this build targets sm_103a (GB300)");
    if (!coop) return fail(FL_NO_DEVICE, "device does not support cooperative launch");
    void* ptr = nullptr;
    e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (e != cudaSuccess || ptr == nullptr)
        return fail(FL_CUDA_ERROR, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
    const int per_sm = fl::cg_max_blocks_per_sm();
    if (per_sm < 1) return fail(FL_INTERNAL, "CG kernel cannot be resident (occupancy 0)");
    g_sms[dev] = sms;
    g_cg_per_sm[dev] = per_sm;
    g_scratch_dev[dev] = ptr;
    return FL_OK;
}

}  // namespace

extern "C" fl_status fl_solve_pressure_noalloc(uint32_t nx, uint32_t ny, uint32_t nz, const uint8_t* cell_type_dev,
                                               const float* divergence_dev, float* pressure_dev, float h,
                                               float rho, float dt, uint32_t max_iters, uint32_t warm_start,
                                               float tolerance, uint32_t cg_precision, void* cuda_stream,
                                               fl_stats* stats_out) {
    if (!cell_type_dev || !divergence_dev || !pressure_dev) return fail(FL_INVALID_ARG, "NULL device pointer");
    if (nx < 3 || ny < 3 || nz < 3) return fail(FL_INVALID_ARG, "each grid dimension must be >= 3");
    const uint64_t cells = (uint64_t)nx * ny * nz;
    if (cells > FL_NOALLOC_MAX_CELLS)
        return fail(FL_INVALID_ARG, "grid of " + std::to_string(cells) + " cells exceeds the no-allocation limit of " +
                                        std::to_string((unsigned long long)FL_NOALLOC_MAX_CELLS) +
                                        " cells; use fl_solve_pressure");
    // The warm-start residual reads neighbouring pressures while other threads
    // overwrite pressure; the solve reads divergence and cell types throughout.
    if (overlaps(pressure_dev, 4 * cells, divergence_dev, 4 * cells) ||
        overlaps(pressure_dev, 4 * cells, cell_type_dev, cells))
        return fail(FL_INVALID_ARG, "pressure_dev must not overlap divergence_dev or cell_type_dev");
    if (!(h > 0.0f) || !(rho > 0.0f) || !(dt > 0.0f)) return fail(FL_INVALID_ARG, "h, rho, dt must be > 0");
    if (cg_precision > 1u) return fail(FL_INVALID_ARG, "cg_precision must be FL_CG_F32 or FL_CG_F64");
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return fail(FL_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
    if (dev < 0 || dev >= kMaxDevices) return fail(FL_NO_DEVICE, "device ordinal out of range");
    fl_status s = device_setup(dev);
    if (s != FL_OK) return s;
    char* base = (char*)g_scratch_dev[dev];

    // Settings, with the same f32 operations as fl_solve_pressure.
    fl::DevParams d{};
    d.nx = nx; d.ny = ny; d.nz = nz;
    d.C = (uint32_t)cells;
    d.h = h; d.inv_h = 1.0f / h; d.dt = dt; d.fixed_scale = 65536.0f;
    d.rho = rho;
    d.scale_rhs = d.rho * d.h * d.h / d.dt;
    const float tolc = std::fmin(std::fmax(tolerance, 0.0f), 0.1f);
    d.tol_sq = tolc * tolc;
    d.tol_sq_d = (double)tolc * (double)tolc;
    d.warm = warm_start ? 1u : 0u;
    d.iters = max_iters ? max_iters : 1u;
    d.precision = cg_precision;
    d.advect_order = 1;
    d.nchunks = (d.C + fl::CHUNK - 1) / fl::CHUNK;

    fl::LaunchCfg L{};
    L.num_sms = g_sms[dev];
    const int want = (int)((d.nchunks + fl::CG_GROUPS - 1) / fl::CG_GROUPS);
    L.cg_blocks = want < g_sms[dev] * g_cg_per_sm[dev] ? want : g_sms[dev] * g_cg_per_sm[dev];
    if (L.cg_blocks < 1) L.cg_blocks = 1;
    if ((size_t)L.cg_blocks > kMaxCtas) return fail(FL_INTERNAL, "cooperative grid exceeds the scratch reservation");
    L.particle_blocks = g_sms[dev];

    fl::DevBufs b{};
    b.prm = (const fl::DevParams*)(base + kOffParams);
    b.st = (fl::DevStats*)(base + kOffStats);
    b.ct = const_cast<uint8_t*>(cell_type_dev);
    b.p = pressure_dev;
    b.r = (float*)(base + kOffR);
    b.dA = (float*)(base + kOffDA);
    b.dB = (float*)(base + kOffDB);
    b.q = (float*)(base + kOffQ);
    b.chunk_flag = (uint8_t*)(base + kOffFlag);
    b.part_rr = (float*)(base + kOffPrr);
    b.chunk_rr_df = (float2*)(base + kOffC64);
    b.cg_chunk = (uint32_t*)(base + kOffPlan);
    b.cg_off = (uint32_t*)(base + kOffPlanOff);
    b.cinfo = (uint16_t*)(base + kOffInfo);
    b.cg_x = (unsigned long long*)(base + kOffX);

    cudaStream_t st = (cudaStream_t)cuda_stream;
    k_noalloc_setup<<<1, 32, 0, st>>>(d, (fl::DevParams*)(base + kOffParams), b.st);
    if ((e = cudaGetLastError()) != cudaSuccess) return fail(FL_CUDA_ERROR, std::string("setup: ") + cudaGetErrorString(e));
    if ((e = fl::launch_solve_init(b, d.C, divergence_dev, st)) != cudaSuccess)
        return fail(FL_CUDA_ERROR, std::string("init: ") + cudaGetErrorString(e));
    if ((e = fl::launch_cg(b, L, st, cg_precision)) != cudaSuccess)
        return fail(FL_CUDA_ERROR, std::string("cg: ") + cudaGetErrorString(e));
    fl::DevStats ds;
    if ((e = cudaMemcpyAsync(&ds, b.st, sizeof(ds), cudaMemcpyDeviceToHost, st)) != cudaSuccess)
        return fail(FL_CUDA_ERROR, std::string("stats: ") + cudaGetErrorString(e));
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess)
        return fail(FL_CUDA_ERROR, std::string("sync: ") + cudaGetErrorString(e));
    if (ds.status != 0u) return fail((fl_status)ds.status, "a device-side wait expired");
    if (stats_out) {
        std::memset(stats_out, 0, sizeof(*stats_out));
        stats_out->cg_iterations = ds.cg_iters;
        stats_out->rs_initial = ds.rs_init;
        stats_out->rs_final = ds.rs_final;
    }
    return FL_OK;
}
