// fl_relax.cu — the reference's relaxation solvers for the pressure system,
// as CUDA kernels (fl_relax_pressure):
//
//   k_jacobi  sim/pressure.rs:72-117 jacobi_iteration: one sweep from p_in to
//             p_out over all cells; non-liquid cells get 0; air neighbours
//             count toward n (Dirichlet p = 0), solid ones are excluded
//             (Neumann).  jacobi_solve (:120-136) ping-pongs from zero.
//   k_rbgs    pressure.wgsl:26-61: the same update in place for the cells of
//             one colour (i+j+k)&1; non-liquid cells are not written (zero
//             from the start).  One iteration = red phase, then black.
//
// Both evaluate (sum - scale*div) / n in f32 with the neighbours in the order
// -x, +x, -y, +y, -z, +z, like the reference (no contraction: --fmad=false).
#include "fl_device.cuh"

namespace fl {

namespace {

__device__ __forceinline__ float relax_cell(const uint8_t* ct, const float* div, float scale, const float* p,
                                            uint32_t c, uint32_t nx, uint32_t nxy) {
    const uint32_t nb[6] = {c - 1, c + 1, c - nx, c + nx, c - nxy, c + nxy};
    float sum = 0.0f, n = 0.0f;
#pragma unroll
    for (int s = 0; s < 6; s++) {
        const uint8_t t = ct[nb[s]];
        if (t == CELL_SOLID) continue;
        if (t == CELL_LIQUID) sum = __fadd_rn(sum, p[nb[s]]);
        n = __fadd_rn(n, 1.0f);
    }
    return n > 0.0f ? __fdiv_rn(__fsub_rn(sum, __fmul_rn(scale, div[c])), n) : 0.0f;
}

__global__ void __launch_bounds__(256) k_jacobi(const uint8_t* __restrict__ ct, const float* __restrict__ div,
                                                float scale, const float* __restrict__ p_in,
                                                float* __restrict__ p_out, uint32_t nx, uint32_t ny, uint32_t C) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    // liquid cells are interior (the boundary layer is solid): neighbours exist
    p_out[c] = ct[c] == CELL_LIQUID ? relax_cell(ct, div, scale, p_in, c, nx, nx * ny) : 0.0f;
}

__global__ void __launch_bounds__(256) k_rbgs(const uint8_t* __restrict__ ct, const float* __restrict__ div,
                                              float scale, float* p, uint32_t nx, uint32_t ny, uint32_t C,
                                              uint32_t phase) {
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C || ct[c] != CELL_LIQUID) return;
    const uint32_t i = c % nx, j = (c / nx) % ny, k = c / (nx * ny);
    if (((i + j + k) & 1u) != phase) return;
    p[c] = relax_cell(ct, div, scale, p, c, nx, nx * ny);
}

}  // namespace

cudaError_t launch_relax(const uint8_t* ct, const float* div, float scale, float* pa, float* pb, uint32_t nx,
                         uint32_t ny, uint32_t nz, uint32_t method, uint32_t iters, cudaStream_t s, float** result) {
    const uint32_t C = nx * ny * nz, grid = (C + 255) / 256;
    float* cur = pa;
    for (uint32_t it = 0; it < iters; it++) {
        if (method == 0u) {
            float* nxt = cur == pa ? pb : pa;
            k_jacobi<<<grid, 256, 0, s>>>(ct, div, scale, cur, nxt, nx, ny, C);
            cur = nxt;
        } else {
            k_rbgs<<<grid, 256, 0, s>>>(ct, div, scale, cur, nx, ny, C, 0u);
            k_rbgs<<<grid, 256, 0, s>>>(ct, div, scale, cur, nx, ny, C, 1u);
        }
    }
    *result = cur;
    return cudaGetLastError();
}

}  // namespace fl
