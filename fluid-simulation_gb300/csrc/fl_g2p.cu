// fl_g2p.cu — grid-to-particle transfer, FLIP/PIC blend, advection, wall push-out.
//
// k_g2p restates g2p.wgsl:131-198 per particle in bin order (sorted input, so
// neighbouring threads gather neighbouring faces).  advect_order == 2 adds a
// midpoint step through the final grid velocity (an extension; the reference
// advects with forward Euler, g2p.wgsl:186).
#include <algorithm>

#include "fl_device.cuh"

namespace fl {

// g2p.wgsl:35-54
__device__ __forceinline__ bool touches_static(int axis, int ii, int jj, int kk, int nx, int ny, int nz) {
    if (axis == 0) return ii <= 1 || ii >= nx - 1 || jj <= 0 || jj >= ny - 1 || kk <= 0 || kk >= nz - 1;
    if (axis == 1) return ii <= 0 || ii >= nx - 1 || jj <= 1 || jj >= ny - 1 || kk <= 0 || kk >= nz - 1;
    return ii <= 0 || ii >= nx - 1 || jj <= 0 || jj >= ny - 1 || kk <= 1 || kk >= nz - 1;
}

// g2p.wgsl:56-129 sample_u / sample_v / sample_w.  with_saved=false skips the
// saved gather (midpoint sample).
template <bool WITH_SAVED>
__device__ __forceinline__ void sample(const DevBufs& b, const DevParams& P, int axis, float px, float py, float pz,
                                       float& out_fin, float& out_sav) {
    const int nx = (int)P.nx, ny = (int)P.ny, nz = (int)P.nz;
    const int dim0 = nx + (axis == 0), dim1 = ny + (axis == 1), dim2 = nz + (axis == 2);
    const float g0 = __fadd_rn(__fmul_rn(__fsub_rn(px, P.origin[0]), P.inv_h), axis == 0 ? 0.0f : -0.5f);
    const float g1 = __fadd_rn(__fmul_rn(__fsub_rn(py, P.origin[1]), P.inv_h), axis == 1 ? 0.0f : -0.5f);
    const float g2 = __fadd_rn(__fmul_rn(__fsub_rn(pz, P.origin[2]), P.inv_h), axis == 2 ? 0.0f : -0.5f);
    const int b0 = floor_to_i32(g0), b1 = floor_to_i32(g1), b2 = floor_to_i32(g2);
    const float t0 = __fsub_rn(g0, (float)b0), t1 = __fsub_rn(g1, (float)b1), t2 = __fsub_rn(g2, (float)b2);
    const float* __restrict__ fv = b.vel[axis];
    const float* __restrict__ sv = b.sav[axis];
    float fin = 0.0f, sav = 0.0f, wsum = 0.0f;
    // All eight taps in range and off the static walls (the common case away
    // from the walls): the same sums in the same order, without the per-tap
    // tests.
    const int lo0 = axis == 0 ? 2 : 1, lo1 = axis == 1 ? 2 : 1, lo2 = axis == 2 ? 2 : 1;
    if (b0 >= lo0 && b0 + 1 <= nx - 2 && b1 >= lo1 && b1 + 1 <= ny - 2 && b2 >= lo2 && b2 + 1 <= nz - 2) {
#pragma unroll
        for (int dk = 0; dk < 2; dk++) {
            const float wz = tent(t2, dk);
#pragma unroll
            for (int dj = 0; dj < 2; dj++) {
                const float wy = tent(t1, dj);
                const size_t row = (size_t)b0 + (size_t)dim0 * ((size_t)(b1 + dj) + (size_t)dim1 * (b2 + dk));
#pragma unroll
                for (int di = 0; di < 2; di++) {
                    const float w = __fmul_rn(__fmul_rn(tent(t0, di), wy), wz);
                    fin = __fadd_rn(fin, __fmul_rn(w, __ldg(fv + row + di)));
                    if (WITH_SAVED) sav = __fadd_rn(sav, __fmul_rn(w, __ldg(sv + row + di)));
                    wsum = __fadd_rn(wsum, w);
                }
            }
        }
        out_fin = __fdiv_rn(fin, wsum);
        out_sav = WITH_SAVED ? __fdiv_rn(sav, wsum) : 0.0f;
        return;
    }
#pragma unroll
    for (int dk = 0; dk < 2; dk++) {
        const int kk = b2 + dk;
        if (kk < 0 || kk >= dim2) continue;
        const float wz = tent(t2, dk);
#pragma unroll
        for (int dj = 0; dj < 2; dj++) {
            const int jj = b1 + dj;
            if (jj < 0 || jj >= dim1) continue;
            const float wy = tent(t1, dj);
#pragma unroll
            for (int di = 0; di < 2; di++) {
                const int ii = b0 + di;
                if (ii < 0 || ii >= dim0) continue;
                if (touches_static(axis, ii, jj, kk, nx, ny, nz)) continue;
                const float wx = tent(t0, di);
                const float w = __fmul_rn(__fmul_rn(wx, wy), wz);
                const size_t idx = (size_t)ii + (size_t)dim0 * ((size_t)jj + (size_t)dim1 * kk);
                fin = __fadd_rn(fin, __fmul_rn(w, __ldg(fv + idx)));
                if (WITH_SAVED) sav = __fadd_rn(sav, __fmul_rn(w, __ldg(sv + idx)));
                wsum = __fadd_rn(wsum, w);
            }
        }
    }
    if (wsum > 0.0f) {
        out_fin = __fdiv_rn(fin, wsum);
        out_sav = WITH_SAVED ? __fdiv_rn(sav, wsum) : 0.0f;
    } else {
        out_fin = 0.0f;
        out_sav = 0.0f;
    }
}

// g2p.wgsl:159-162
__device__ __forceinline__ void speed_clamp(float& x, float& y, float& z, float maxs) {
    const float sp = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
    if (sp > maxs && sp > 0.0f) {
        const float s = __fdiv_rn(maxs, sp);
        x = __fmul_rn(x, s);
        y = __fmul_rn(y, s);
        z = __fmul_rn(z, s);
    }
}

__global__ void __launch_bounds__(256) k_g2p(DevBufs b) {
    const DevParams& P = *b.prm;
    const uint32_t n = P.n;
    const float alpha = P.flip, dt = P.dt, maxs = P.maxs, friction = P.friction;
    const float one_minus_alpha = __fsub_rn(1.0f, alpha);
    const bool rk2 = P.advect_order == 2u;
    for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d < n; d += gridDim.x * blockDim.x) {
        const float4 pos = b.part_sorted[2 * (size_t)d];
        const float4 pvel = b.part_sorted[2 * (size_t)d + 1];
        float pic[3], saved[3];
        sample<true>(b, P, 0, pos.x, pos.y, pos.z, pic[0], saved[0]);
        sample<true>(b, P, 1, pos.x, pos.y, pos.z, pic[1], saved[1]);
        sample<true>(b, P, 2, pos.x, pos.y, pos.z, pic[2], saved[2]);
        const float pv[3] = {pvel.x, pvel.y, pvel.z};
        float nv[3];
#pragma unroll
        for (int a = 0; a < 3; a++) {
            const float flip = __fadd_rn(pv[a], __fsub_rn(pic[a], saved[a]));        // g2p.wgsl:151
            nv[a] = __fadd_rn(__fmul_rn(pic[a], one_minus_alpha), __fmul_rn(flip, alpha));  // mix, :152
        }
        speed_clamp(nv[0], nv[1], nv[2], maxs);
        const float P3[3] = {pos.x, pos.y, pos.z};
        if (friction > 0.0f) {  // g2p.wgsl:173-184
            const float band = __fmul_rn(P.h, 2.5f);
            float nr[3];
#pragma unroll
            for (int a = 0; a < 3; a++) {
                const float dlo = __fdiv_rn(__fsub_rn(P3[a], P.lo[a]), band);
                const float dhi = __fdiv_rn(__fsub_rn(P.hi[a], P3[a]), band);
                nr[a] = fminf(fmaxf(__fsub_rn(1.0f, fminf(dlo, dhi)), 0.0f), 1.0f);
            }
            nv[0] = __fmul_rn(nv[0], __fsub_rn(1.0f, __fmul_rn(friction, fmaxf(nr[1], nr[2]))));
            nv[1] = __fmul_rn(nv[1], __fsub_rn(1.0f, __fmul_rn(friction, fmaxf(nr[0], nr[2]))));
            nv[2] = __fmul_rn(nv[2], __fsub_rn(1.0f, __fmul_rn(friction, fmaxf(nr[0], nr[1]))));
        }
        float np[3];
        if (rk2) {
            float k1[3] = {pic[0], pic[1], pic[2]};
            speed_clamp(k1[0], k1[1], k1[2], maxs);
            float pm[3];
#pragma unroll
            for (int a = 0; a < 3; a++) pm[a] = __fadd_rn(P3[a], __fmul_rn(k1[a], P.half_dt));
            float k2[3], unused;
            sample<false>(b, P, 0, pm[0], pm[1], pm[2], k2[0], unused);
            sample<false>(b, P, 1, pm[0], pm[1], pm[2], k2[1], unused);
            sample<false>(b, P, 2, pm[0], pm[1], pm[2], k2[2], unused);
            speed_clamp(k2[0], k2[1], k2[2], maxs);
#pragma unroll
            for (int a = 0; a < 3; a++) np[a] = __fadd_rn(P3[a], __fmul_rn(k2[a], dt));
        } else {
#pragma unroll
            for (int a = 0; a < 3; a++) np[a] = __fadd_rn(P3[a], __fmul_rn(nv[a], dt));  // :186
        }
#pragma unroll
        for (int a = 0; a < 3; a++) {  // :189-194
            if (np[a] < P.lo[a]) { np[a] = P.lo[a]; nv[a] = 0.0f; }
            if (np[a] > P.hi[a]) { np[a] = P.hi[a]; nv[a] = 0.0f; }
        }
        b.part_out[2 * (size_t)d] = make_float4(np[0], np[1], np[2], 0.0f);
        b.part_out[2 * (size_t)d + 1] = make_float4(nv[0], nv[1], nv[2], 0.0f);
        if (b.ids_in) b.ids_in[d] = b.ids_sorted[d];
    }
}

// impulse.wgsl:26-35
__global__ void __launch_bounds__(256) k_impulse(float4* part, const DevParams* prm, float dx, float dy, float dz) {
    const uint32_t n = prm->n;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        float4 v = part[2 * (size_t)p + 1];
        v.x = __fadd_rn(v.x, dx);
        v.y = __fadd_rn(v.y, dy);
        v.z = __fadd_rn(v.z, dz);
        v.w = __fadd_rn(v.w, 0.0f);
        part[2 * (size_t)p + 1] = v;
    }
}

__global__ void __launch_bounds__(256) k_iota(uint32_t* ids, uint32_t n) {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) ids[i] = i;
}

cudaError_t launch_iota(uint32_t* ids, uint32_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    const uint32_t blocks = std::min<uint32_t>((n + 255) / 256, 4096u);
    k_iota<<<blocks, 256, 0, s>>>(ids, n);
    return cudaGetLastError();
}

cudaError_t launch_g2p(const DevBufs& b, const LaunchCfg& L, cudaStream_t s) {
    k_g2p<<<L.particle_blocks, 256, 0, s>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_impulse(float4* part, const DevParams* prm, float dx, float dy, float dz, const LaunchCfg& L,
                           cudaStream_t s) {
    k_impulse<<<L.particle_blocks, 256, 0, s>>>(part, prm, dx, dy, dz);
    return cudaGetLastError();
}

}  // namespace fl
