// fl_slice.cu — headless grid-slice extraction.
//
// Restates the per-cell arithmetic of the reference's slice debug renderer
// (app/crates/fluid-lab/src/gpu/shaders/slice.wgsl:69-141) as a CUDA kernel:
// for every cell (i, j) of the XY cross-section at k it writes one float4
// {r, g, b, visible} instead of a screen-space quad (visible = 0 where the
// shader makes the quad degenerate: air cells in mode 0, non-liquid cells in
// modes 1 and 2).  Modes: 0 cell type, 1 pressure, 2 (and above) speed.
// `mix` is the WGSL definition e1*(1-e3) + e2*e3 and `length` is
// sqrt(x*x + y*y + z*z), in f32 without contraction.
#include "fl_device.cuh"

namespace fl {

struct Rgb {
    float r, g, b;
};

__device__ __forceinline__ float mixf(float a, float b, float s) {
    return __fadd_rn(__fmul_rn(a, __fsub_rn(1.0f, s)), __fmul_rn(b, s));
}
__device__ __forceinline__ Rgb mix3(Rgb a, Rgb b, float s) { return {mixf(a.r, b.r, s), mixf(a.g, b.g, s), mixf(a.b, b.b, s)}; }
__device__ __forceinline__ float clamp01(float t) { return fminf(fmaxf(t, 0.0f), 1.0f); }

// slice.wgsl:41-52
__device__ __forceinline__ Rgb colormap_diverging(float t) {
    const float tc = clamp01(t);
    if (tc < 0.5f) return mix3({0.0f, 0.2f, 0.9f}, {1.0f, 1.0f, 1.0f}, __fmul_rn(tc, 2.0f));
    return mix3({1.0f, 1.0f, 1.0f}, {0.9f, 0.05f, 0.05f}, __fmul_rn(__fsub_rn(tc, 0.5f), 2.0f));
}

// slice.wgsl:55-67
__device__ __forceinline__ Rgb colormap_speed(float t) {
    const float tc = clamp01(t);
    if (tc < 0.333f) return mix3({0.0f, 0.0f, 0.8f}, {0.0f, 0.9f, 0.9f}, __fdiv_rn(tc, 0.333f));
    if (tc < 0.667f) return mix3({0.0f, 0.9f, 0.9f}, {1.0f, 1.0f, 0.0f}, __fdiv_rn(__fsub_rn(tc, 0.333f), 0.333f));
    return mix3({1.0f, 1.0f, 0.0f}, {0.9f, 0.0f, 0.0f}, __fdiv_rn(__fsub_rn(tc, 0.667f), 0.333f));
}

__global__ void __launch_bounds__(256) k_slice(DevBufs b, uint32_t mode, uint32_t k, float4* __restrict__ out) {
    const DevParams& P = *b.prm;
    const uint32_t nx = P.nx, ny = P.ny;
    const uint32_t ii = blockIdx.x * blockDim.x + threadIdx.x;
    if (ii >= nx * ny) return;
    const uint32_t i = ii % nx, j = ii / nx;
    const size_t idx = (size_t)i + nx * ((size_t)j + (size_t)ny * k);
    const uint8_t ct = b.ct[idx];
    Rgb c = {0.0f, 0.0f, 0.0f};
    bool visible;
    if (mode == 0u) {  // slice.wgsl:94-103
        visible = ct != CELL_AIR;
        c = ct == CELL_SOLID ? Rgb{0.40f, 0.40f, 0.46f} : Rgb{0.20f, 0.55f, 1.00f};
    } else if (mode == 1u) {  // slice.wgsl:104-116
        visible = ct == CELL_LIQUID;
        if (visible) {
            const float p = b.p[idx];
            c = colormap_diverging(clamp01(__fadd_rn(__fmul_rn(__fdiv_rn(p, 2000.0f), 0.5f), 0.5f)));
        }
    } else {  // slice.wgsl:117-141
        visible = ct == CELL_LIQUID;
        if (visible) {
            const float u0 = b.vel[0][i + (size_t)(nx + 1) * (j + (size_t)ny * k)];
            const float u1 = b.vel[0][(i + 1) + (size_t)(nx + 1) * (j + (size_t)ny * k)];
            const float v0 = b.vel[1][i + (size_t)nx * (j + (size_t)(ny + 1) * k)];
            const float v1 = b.vel[1][i + (size_t)nx * ((j + 1) + (size_t)(ny + 1) * k)];
            const float w0 = b.vel[2][i + (size_t)nx * (j + (size_t)ny * k)];
            const float w1 = b.vel[2][i + (size_t)nx * (j + (size_t)ny * (k + 1))];
            const float au = __fmul_rn(__fadd_rn(u0, u1), 0.5f);
            const float av = __fmul_rn(__fadd_rn(v0, v1), 0.5f);
            const float aw = __fmul_rn(__fadd_rn(w0, w1), 0.5f);
            const float spd = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(au, au), __fmul_rn(av, av)), __fmul_rn(aw, aw)));
            c = colormap_speed(clamp01(__fdiv_rn(spd, 4.0f)));
        }
    }
    out[ii] = make_float4(c.r, c.g, c.b, visible ? 1.0f : 0.0f);
}

cudaError_t launch_slice(const DevBufs& b, uint32_t nx, uint32_t ny, uint32_t mode, uint32_t k, float4* out,
                         cudaStream_t s) {
    const uint32_t n = nx * ny;
    k_slice<<<(n + 255) / 256, 256, 0, s>>>(b, mode, k, out);
    return cudaGetLastError();
}

}  // namespace fl
