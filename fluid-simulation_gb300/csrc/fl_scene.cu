// fl_scene.cu — scene presets and particle seeding on the device.
//
// Host side (f32 arithmetic in the reference's order; -ffp-contract=off):
//   fl_scene_blocks            preset_blocks (app/crates/fluid-lab/src/scene/mod.rs:204-236)
//                              with shift_block_y / scale_block_* (:238-266)
//   fl_scene_seeded_fraction   seeded_volume_fraction (scene/mod.rs:155-165)
//   fl_scene_particle_count    resolved_particle_count (scene/mod.rs:178-192)
// Device side:
//   fl_seed_particles          generate_particles (app/crates/fluid-lab/src/gpu/fluid.rs:1838-1913):
//                              a jittered lattice per liquid block, the particle
//                              budget split by block volume.  The reference draws
//                              three LCG numbers per particle in one sequential
//                              loop; here particle p is computed by its own thread,
//                              which jumps the LCG to draw 3p by affine-map squaring
//                              (O(log p)), so the output equals the sequential loop.
#include <cmath>
#include <cstring>

#include "../../include/fluidgb.h"
#include "fl_device.cuh"

namespace {

constexpr float kDefaultDropHeight = 0.72f;  // scene/mod.rs:10
constexpr float kDefaultFill = 0.2f;          // scene/mod.rs:22
constexpr uint32_t kLcgA = 1664525u, kLcgC = 1013904223u, kLcgSeed = 0x12345678u;  // fluid.rs:1878-1882

// Rust's f32::clamp (NaN passes through).
float clampf(float x, float lo, float hi) {
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}
// glam's Vec3::clamp per component: max then min (a NaN operand yields the other).
float gclamp(float x, float lo, float hi) { return std::fmin(std::fmax(x, lo), hi); }

struct Blk {
    float mn[3], mx[3];
};

// shift_block_y (scene/mod.rs:243-248)
Blk shift_block_y(Blk b, float delta) {
    const float shift = clampf(delta, -b.mn[1], 1.0f - b.mx[1]);
    b.mn[1] += shift;
    b.mx[1] += shift;
    return b;
}

// scale_block_axes (scene/mod.rs:254-266)
Blk scale_block_axes(Blk b, const float factor[3]) {
    Blk o = b;
    for (int a = 0; a < 3; a++) {
        const float center = 0.5f * (b.mn[a] + b.mx[a]);
        const float half = 0.5f * (b.mx[a] - b.mn[a]);
        const float scaled = half * std::fmax(factor[a], 1.0e-3f);
        o.mn[a] = gclamp(center - scaled, 0.0f, 1.0f);
        o.mx[a] = gclamp(center + scaled, o.mn[a] + 1.0e-3f, 1.0f);
        o.mn[a] = std::fmax(std::fmin(o.mn[a], o.mx[a] - 1.0e-3f), 0.0f);
    }
    return o;
}

// scale_block_about_center (scene/mod.rs:238-241)
Blk scale_block_about_center(Blk b, float fill) {
    const float f = std::pow(std::fmax(fill, 1.0e-4f) / kDefaultFill, 1.0f / 3.0f);
    const float factor[3] = {f, f, f};
    return scale_block_axes(b, factor);
}

// scale_suspended_drop (scene/mod.rs:250-252)
Blk scale_suspended_drop(Blk b, float fill) {
    const float factor[3] = {1.0f, fill / kDefaultFill, 1.0f};
    return scale_block_axes(b, factor);
}

Blk make(float x0, float y0, float z0, float x1, float y1, float z1) {
    Blk b;
    b.mn[0] = x0; b.mn[1] = y0; b.mn[2] = z0;
    b.mx[0] = x1; b.mx[1] = y1; b.mx[2] = z1;
    return b;
}

}  // namespace

namespace fl {

// State after `k` LCG steps from the seed: the affine map x -> A x + C
// composed k times, by squaring.
__device__ __forceinline__ uint32_t lcg_jump(uint64_t k) {
    uint32_t am = 1u, ac = 0u;        // accumulated map
    uint32_t cm = kLcgA, cc = kLcgC;  // map of 2^i steps
    while (k) {
        if (k & 1u) {
            am = am * cm;
            ac = ac * cm + cc;
        }
        cc = (cm + 1u) * cc;
        cm = cm * cm;
        k >>= 1;
    }
    return am * kLcgSeed + ac;
}
__device__ __forceinline__ float rand01_of(uint32_t st) {  // fluid.rs:1881
    return __fdiv_rn((float)(st >> 8), 16777216.0f);
}

__global__ void __launch_bounds__(256) k_seed(SeedArgs a, float4* __restrict__ part) {
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    uint32_t b = 0;
    while (b + 1 < a.nblocks && p >= a.blk[b + 1].first) b++;
    const SeedBlock& B = a.blk[b];
    const uint32_t l = p - B.first;
    const uint32_t cyz = (uint32_t)B.counts[1] * (uint32_t)B.counts[2];
    const uint32_t idx[3] = {l / cyz, (l / (uint32_t)B.counts[2]) % (uint32_t)B.counts[1], l % (uint32_t)B.counts[2]};
    uint32_t st = lcg_jump(3ull * p + 1ull);  // the state the reference's draw 3p reads
    float pos[3];
#pragma unroll
    for (int ax = 0; ax < 3; ax++) {
        if (ax) st = st * kLcgA + kLcgC;
        // jx = (rand01() - 0.5) * spacing * 0.5  (fluid.rs:1897-1899)
        const float j = __fmul_rn(__fmul_rn(__fsub_rn(rand01_of(st), 0.5f), B.spacing), 0.5f);
        // (wmin + (i + 0.5) * spacing + j).clamp(lo, hi)  (fluid.rs:1901-1903)
        const float x = __fadd_rn(__fadd_rn(B.wmin[ax], __fmul_rn(__fadd_rn((float)idx[ax], 0.5f), B.spacing)), j);
        pos[ax] = fminf(fmaxf(x, a.lo[ax]), a.hi[ax]);
    }
    part[2 * (size_t)p] = make_float4(pos[0], pos[1], pos[2], 0.0f);
    part[2 * (size_t)p + 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
}

// generate_particles' block layout (fluid.rs:1863-1893) in f32: per-block
// lattice counts and spacing from the volume-proportional budget.  Returns the
// total particle count (saturated at 2^32-1) or -1 for invalid input.
long long seed_layout(const fl_params& prm, const fl_block* blocks, uint32_t nblocks, uint32_t particle_count,
                      SeedArgs* out) {
    if (!blocks || nblocks == 0 || nblocks > FL_SCENE_MAX_BLOCKS) return -1;
    const float h = prm.geom[0];
    float origin[3], extent[3];
    for (int a = 0; a < 3; a++) {
        origin[a] = prm.origin[a];
        extent[a] = (float)prm.gdim[a] * h;
    }
    SeedArgs s;
    std::memset(&s, 0, sizeof(s));
    for (int a = 0; a < 3; a++) {
        s.lo[a] = origin[a] + h * 1.05f;
        s.hi[a] = origin[a] + extent[a] - h * 1.05f;
    }
    float wmin[FL_SCENE_MAX_BLOCKS][3], ext[FL_SCENE_MAX_BLOCKS][3], vol[FL_SCENE_MAX_BLOCKS];
    float total_vol = 0.0f;
    for (uint32_t b = 0; b < nblocks; b++) {
        for (int a = 0; a < 3; a++) {
            wmin[b][a] = origin[a] + blocks[b].min[a] * extent[a];
            const float wmax = origin[a] + blocks[b].max[a] * extent[a];
            ext[b][a] = wmax - wmin[b][a];
        }
        vol[b] = std::fmax(ext[b][0] * ext[b][1] * ext[b][2], 1e-6f);
        total_vol += vol[b];
    }
    total_vol = std::fmax(total_vol, 1e-6f);
    const float total_target = (float)(particle_count > 1u ? particle_count : 1u);
    unsigned long long n = 0;
    for (uint32_t b = 0; b < nblocks; b++) {
        const float target = std::fmax(total_target * (vol[b] / total_vol), 1.0f);
        const float spacing = std::fmax(std::cbrt(vol[b] / target), 1e-4f);
        SeedBlock& B = s.blk[b];
        B.spacing = spacing;
        unsigned long long c = 1;
        for (int a = 0; a < 3; a++) {
            B.wmin[a] = wmin[b][a];
            const float q = std::floor(ext[b][a] / spacing);  // `as i32` saturates; max(1)
            int32_t ci = !(q == q) ? 0 : (q >= 2147483647.0f ? 2147483647 : (q <= -2147483648.0f ? INT32_MIN : (int32_t)q));
            B.counts[a] = ci > 1 ? ci : 1;
            c *= (unsigned long long)B.counts[a];
        }
        B.first = (uint32_t)(n < 0xffffffffull ? n : 0xffffffffull);
        n += c;
    }
    s.nblocks = nblocks;
    s.n = (uint32_t)(n < 0xffffffffull ? n : 0xffffffffull);
    *out = s;
    return (long long)(n < 0xffffffffull ? n : 0xffffffffull);
}

cudaError_t launch_seed(const SeedArgs& a, float4* part, cudaStream_t s) {
    if (a.n) k_seed<<<(a.n + 255) / 256, 256, 0, s>>>(a, part);
    return cudaGetLastError();
}

}  // namespace fl

extern "C" {

fl_status fl_scene_blocks(uint32_t preset, float drop_height, float fill_level, fl_block* out, uint32_t* n_out) {
    if (!out || !n_out) return FL_INVALID_ARG;
    const float fill = clampf(fill_level, 0.0f, 1.0f);
    Blk bl[2];
    uint32_t n = 0;
    if (preset == FL_PRESET_DAM_BREAK) {  // scene/mod.rs:218-222
        const float kCeiling = 0.98f;
        const float top = clampf(fill * kCeiling, 1.0e-3f, kCeiling);
        bl[n++] = make(0.05f, 0.0f, 0.05f, 0.42f, top, 0.95f);
    } else if (preset == FL_PRESET_DOUBLE_SPLASH) {  // scene/mod.rs:223-234
        const float delta = clampf(drop_height, 0.0f, 1.0f) - kDefaultDropHeight;
        bl[n++] = scale_suspended_drop(shift_block_y(make(0.1f, 0.45f, 0.3f, 0.34f, 0.92f, 0.7f), delta), fill);
        bl[n++] = scale_suspended_drop(shift_block_y(make(0.66f, 0.45f, 0.3f, 0.9f, 0.92f, 0.7f), delta), fill);
    } else {  // FallingBlob and any other value (ScenePreset::from_u32), scene/mod.rs:213-217
        const float delta = clampf(drop_height, 0.0f, 1.0f) - kDefaultDropHeight;
        bl[n++] = scale_block_about_center(shift_block_y(make(0.19f, 0.2f, 0.19f, 0.81f, 0.72f, 0.81f), delta), fill);
    }
    for (uint32_t b = 0; b < n; b++)
        for (int a = 0; a < 3; a++) {
            out[b].min[a] = bl[b].mn[a];
            out[b].max[a] = bl[b].mx[a];
        }
    *n_out = n;
    return FL_OK;
}

fl_status fl_scene_seeded_fraction(const fl_block* blocks, uint32_t nblocks, float* out) {
    if ((!blocks && nblocks) || !out) return FL_INVALID_ARG;
    float sum = 0.0f;
    for (uint32_t b = 0; b < nblocks; b++) {
        float v[3];
        for (int a = 0; a < 3; a++) v[a] = std::fmax(blocks[b].max[a] - blocks[b].min[a], 0.0f);
        sum += std::fmax(v[0] * v[1] * v[2], 0.0f);
    }
    *out = clampf(sum, 0.0f, 1.0f);
    return FL_OK;
}

fl_status fl_scene_particle_count(uint32_t nx, uint32_t ny, uint32_t nz, const fl_block* blocks, uint32_t nblocks,
                                  float density, uint32_t override_count, uint32_t* out) {
    if (!out) return FL_INVALID_ARG;
    if (override_count > 0) {
        *out = override_count;
        return FL_OK;
    }
    float frac = 0.0f;
    fl_status s = fl_scene_seeded_fraction(blocks, nblocks, &frac);
    if (s != FL_OK) return s;
    const double cells = (double)nx * (double)ny * (double)nz * (double)frac;
    if (cells <= 0.0) {
        *out = 0;
        return FL_OK;
    }
    const double d = density > 0.0f ? (double)density : 0.0;
    const double c = std::round(cells * d);
    const uint32_t ci = !(c == c) || c <= 0.0 ? 0u : (c >= 4294967295.0 ? 0xffffffffu : (uint32_t)c);
    *out = ci > 1024u ? ci : 1024u;
    return FL_OK;
}

}  // extern "C"
