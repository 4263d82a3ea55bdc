// fl_adjoint.cu — hand-written adjoint of one substep.
//
// The forward substep (fl_bin/fl_grid/fl_cg/fl_g2p) is differentiated with its
// discrete choices held fixed from the recorded step: the bin permutation, the
// cell types (and therefore the wet / solid / gradient-face masks), the CFL
// and wall clamps.  The fixed-point P2G is differentiated as the real-valued
// weighted mean it approximates (vel_f = sum w v / sum w), linearised at the
// unquantised sums: where sum w is small (faces at the liquid surface) the
// 2^-16 quantum of the fixed-point sums is a large fraction of vel_f, and the
// position derivative dw (v_p - vel_f) / sum w would amplify it.  The pressure
// solve as the exact linear solve A p = b (A symmetric), so its adjoint is a
// second CG solve with the same operator.  Stages, in reverse order:
//
//   k_adj_g2p       g2p.wgsl:131-198 (friction band, speed clamp, forward Euler
//                   or the midpoint step, wall clamp): particle gradients
//                   w.r.t. position and velocity, and per particle the face
//                   coefficients of its gathers (gradient / weight sum)
//   k_adj_mid       (midpoint step) the midpoint gather's face gradients as
//                   64-bit fixed-point integer atomics (order-free)
//   k_adj_gather    per face, in a fixed order over the particles of the
//                   cells around it: the face gradients of the final and
//                   saved velocities (the trilinear gather transposed) and
//                   scatter.wgsl's sums {sum w, sum w v} without the
//                   fixed-point rounding.  No float atomics anywhere: two
//                   backward passes give the same bits
//   k_adj_prhs      gradient.wgsl transposed: dL/dp per liquid cell, the RHS
//                   of the adjoint pressure solve A lambda = dL/dp
//   k_adj_thr       (warm start only) the solve's absolute stopping threshold
//   (k_solve_init + k_cg with the RHS: the adjoint solve)
//   k_adj_faces     divergence.wgsl and gradient.wgsl transposed, then
//                   boundaries.wgsl / forces.wgsl / save_vel.wgsl: gradient of
//                   the normalised P2G face velocity; dL/dgravity as block
//                   partials, summed in order by k_adj_grav
//   k_adj_p2g       scatter.wgsl transposed: a gather from faces to particles
//                   (velocity and position gradients)
//   k_adj_unsort    sort_scatter.wgsl transposed: back to the step's input order
#include "fl_device.cuh"

namespace fl {

__device__ __forceinline__ bool touches_static_a(int axis, int ii, int jj, int kk, int nx, int ny, int nz) {
    if (axis == 0) return ii <= 1 || ii >= nx - 1 || jj <= 0 || jj >= ny - 1 || kk <= 0 || kk >= nz - 1;
    if (axis == 1) return ii <= 0 || ii >= nx - 1 || jj <= 1 || jj >= ny - 1 || kk <= 0 || kk >= nz - 1;
    return ii <= 0 || ii >= nx - 1 || jj <= 0 || jj >= ny - 1 || kk <= 1 || kk >= nz - 1;
}

// Trilinear stencil of one axis at cell-space point q (forward: scatter.wgsl /
// g2p.wgsl).  Calls f(face index, w, dw/dq[3]) for each in-range tap.
template <class Fn>
__device__ __forceinline__ void stencil(const DevParams& P, int axis, const float q[3], bool wall_aware, Fn f) {
    const int n3[3] = {(int)P.nx, (int)P.ny, (int)P.nz};
    int dim[3], base[3];
    float t[3];
#pragma unroll
    for (int b = 0; b < 3; b++) {
        dim[b] = n3[b] + (axis == b ? 1 : 0);
        const float g = q[b] + (b == axis ? 0.0f : -0.5f);
        base[b] = __float2int_rz(floorf(g));
        t[b] = g - (float)base[b];
    }
    // All eight taps in range (and off the static walls when wall_aware): the
    // same taps in the same order without the per-tap tests.
    bool all_in = true;
#pragma unroll
    for (int b = 0; b < 3; b++) {
        const int lo = wall_aware ? (axis == b ? 2 : 1) : 0;
        const int hi = wall_aware ? n3[b] - 2 : dim[b] - 1;
        all_in = all_in && base[b] >= lo && base[b] + 1 <= hi;
    }
    if (all_in) {
#pragma unroll
        for (int dk = 0; dk < 2; dk++) {
            const float wz = dk ? t[2] : 1.0f - t[2], sz = dk ? 1.0f : -1.0f;
#pragma unroll
            for (int dj = 0; dj < 2; dj++) {
                const float wy = dj ? t[1] : 1.0f - t[1], sy = dj ? 1.0f : -1.0f;
                const size_t row = (size_t)base[0] + (size_t)dim[0] * ((size_t)(base[1] + dj) + (size_t)dim[1] * (base[2] + dk));
#pragma unroll
                for (int di = 0; di < 2; di++) {
                    const float wx = di ? t[0] : 1.0f - t[0], sx = di ? 1.0f : -1.0f;
                    const float dw[3] = {sx * wy * wz, wx * sy * wz, wx * wy * sz};
                    f(row + di, wx * wy * wz, dw);
                }
            }
        }
        return;
    }
#pragma unroll
    for (int dk = 0; dk < 2; dk++) {
        const int kk = base[2] + dk;
        if (kk < 0 || kk >= dim[2]) continue;
        const float wz = dk ? t[2] : 1.0f - t[2], sz = dk ? 1.0f : -1.0f;
#pragma unroll
        for (int dj = 0; dj < 2; dj++) {
            const int jj = base[1] + dj;
            if (jj < 0 || jj >= dim[1]) continue;
            const float wy = dj ? t[1] : 1.0f - t[1], sy = dj ? 1.0f : -1.0f;
#pragma unroll
            for (int di = 0; di < 2; di++) {
                const int ii = base[0] + di;
                if (ii < 0 || ii >= dim[0]) continue;
                if (wall_aware && touches_static_a(axis, ii, jj, kk, n3[0], n3[1], n3[2])) continue;
                const float wx = di ? t[0] : 1.0f - t[0], sx = di ? 1.0f : -1.0f;
                const float dw[3] = {sx * wy * wz, wx * sy * wz, wx * wy * sz};
                const size_t idx = (size_t)ii + (size_t)dim[0] * ((size_t)jj + (size_t)dim[1] * kk);
                f(idx, wx * wy * wz, dw);
            }
        }
    }
}

// ---------------------------------------------------------------------------
// G2P + advection adjoint.

// Wall-aware renormalised gather of the final (and saved) face velocities at
// cell-space point q (g2p.wgsl:56-129), with the position derivatives of the
// quotients per unit world coordinate.  W = sum of weights (0: no tap).
template <bool WITH_SAVED>
__device__ __forceinline__ void gather_d(const AdjBufs& a, const DevParams& P, const float q[3], float val[3],
                                         float dval[3][3], float sav[3], float dsav[3][3], float W[3]) {
    #pragma unroll
    for (int ax = 0; ax < 3; ax++) {
        float fsum = 0.0f, ssum = 0.0f, wsum = 0.0f, dws[3] = {0, 0, 0}, dfs[3] = {0, 0, 0}, dss[3] = {0, 0, 0};
        const float* fv = a.fin[ax];
        const float* svv = a.sav[ax];
        stencil(P, ax, q, true, [&](size_t idx, float w, const float* dw) {
            const float f = fv[idx];
            fsum += w * f;
            wsum += w;
            #pragma unroll
            for (int b = 0; b < 3; b++) {
                dws[b] += dw[b];
                dfs[b] += dw[b] * f;
            }
            if (WITH_SAVED) {
                const float s = svv[idx];
                ssum += w * s;
                #pragma unroll
                for (int b = 0; b < 3; b++) dss[b] += dw[b] * s;
            }
        });
        W[ax] = wsum;
        if (wsum > 0.0f) {
            val[ax] = fsum / wsum;
            if (WITH_SAVED) sav[ax] = ssum / wsum;
            #pragma unroll
            for (int b = 0; b < 3; b++) {  // d(F/W) = (dF - (F/W) dW)/W, per unit cell coordinate
                dval[ax][b] = (dfs[b] - val[ax] * dws[b]) / wsum * P.inv_h;
                if (WITH_SAVED) dsav[ax][b] = (dss[b] - sav[ax] * dws[b]) / wsum * P.inv_h;
            }
        } else {
            val[ax] = 0.0f;
            if (WITH_SAVED) sav[ax] = 0.0f;
            #pragma unroll
            for (int b = 0; b < 3; b++) {
                dval[ax][b] = 0.0f;
                if (WITH_SAVED) dsav[ax][b] = 0.0f;
            }
        }
    }
}

// The speed clamp v * maxs/|v| (g2p.wgsl:159-162): forward factor and the
// gradient of its input from the gradient g of its output.
struct Clamp {
    float sp, sc;
    bool on;
};
__device__ __forceinline__ Clamp clamp_fwd(const float v[3], float maxs) {
    Clamp c;
    c.sp = sqrtf(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    c.on = c.sp > maxs && c.sp > 0.0f;
    c.sc = c.on ? maxs / c.sp : 1.0f;
    return c;
}
__device__ __forceinline__ void clamp_bwd(const Clamp& c, const float v[3], const float g[3], float out[3]) {
    if (c.on) {
        const float inv = 1.0f / c.sp;
        const float dotp = (g[0] * v[0] + g[1] * v[1] + g[2] * v[2]) * inv * inv;
        #pragma unroll
        for (int b = 0; b < 3; b++) out[b] = c.sc * (g[b] - v[b] * dotp);
    } else {
        #pragma unroll
        for (int b = 0; b < 3; b++) out[b] = g[b];
    }
}

// g2p.wgsl:131-198 and the midpoint option, in reverse.  Forward recomputed
// per particle: PIC and saved gathers at X, mix, speed clamp, the friction
// band factors (g2p.wgsl:173-184), then forward Euler (g2p.wgsl:186) or the
// midpoint step (k1 = clamp(PIC(X)), Xm = X + k1 dt/2, k2 = clamp(fin(Xm)),
// X' = X + k2 dt) and the wall clamp (g2p.wgsl:189-194).  The discrete choices
// of the recorded step are held fixed: which clamps are active, which side of
// the band's min and which axis of the band's max are taken, which components
// are pinned to the walls.
__global__ void __launch_bounds__(256) k_adj_g2p(AdjBufs a) {
    const DevParams& P = *a.prm;
    const uint32_t n = P.n;
    const float alpha = P.flip, dt = P.dt, maxs = P.maxs, inv_h = P.inv_h, friction = P.friction;
    const bool rk2 = P.advect_order == 2u;
    for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d < n; d += gridDim.x * blockDim.x) {
        const float4 pos = a.part[2 * (size_t)d], pvel = a.part[2 * (size_t)d + 1];
        const float X[3] = {pos.x, pos.y, pos.z}, pv[3] = {pvel.x, pvel.y, pvel.z};
        const float q[3] = {(pos.x - P.origin[0]) * inv_h, (pos.y - P.origin[1]) * inv_h, (pos.z - P.origin[2]) * inv_h};
        float pic[3], sv[3], dpic[3][3], dsv[3][3], W[3];
        gather_d<true>(a, P, q, pic, dpic, sv, dsv, W);
        float mix[3];
        #pragma unroll
        for (int b = 0; b < 3; b++) mix[b] = pic[b] * (1.0f - alpha) + (pv[b] + (pic[b] - sv[b])) * alpha;
        const Clamp cm = clamp_fwd(mix, maxs);
        float nvc[3];  // after the speed clamp, before friction
        #pragma unroll
        for (int b = 0; b < 3; b++) nvc[b] = mix[b] * cm.sc;
        // friction: nv_b = nvc_b (1 - friction max(nr_c, nr_d)), nr_a = clamp(1 - min(dlo, dhi), 0, 1)
        float ff[3] = {1.0f, 1.0f, 1.0f}, dnr[3] = {0.0f, 0.0f, 0.0f};
        int fsel[3] = {-1, -1, -1};
        if (friction > 0.0f) {
            const float band = P.h * 2.5f;
            float nr[3];
            #pragma unroll
            for (int c = 0; c < 3; c++) {
                const float dlo = (X[c] - P.lo[c]) / band, dhi = (P.hi[c] - X[c]) / band;
                const float u = 1.0f - fminf(dlo, dhi);
                nr[c] = fminf(fmaxf(u, 0.0f), 1.0f);
                dnr[c] = (u > 0.0f && u < 1.0f) ? (dlo <= dhi ? -1.0f / band : 1.0f / band) : 0.0f;
            }
            #pragma unroll
            for (int b = 0; b < 3; b++) {
                const int c1 = b == 0 ? 1 : 0, c2 = b == 2 ? 1 : 2;
                const bool first_max = nr[c1] >= nr[c2];
                fsel[b] = first_max ? c1 : c2;
                ff[b] = 1.0f - friction * (first_max ? nr[c1] : nr[c2]);
            }
        }
        float nv[3], np[3];
        #pragma unroll
        for (int b = 0; b < 3; b++) nv[b] = nvc[b] * ff[b];
        // advection
        float qm[3], pic2[3], dpic2[3][3], W2[3], k1[3], k2[3];
        Clamp c1 = {0.0f, 1.0f, false}, c2 = {0.0f, 1.0f, false};
        if (rk2) {
            c1 = clamp_fwd(pic, maxs);
            float Xm[3];
            #pragma unroll
            for (int b = 0; b < 3; b++) {
                k1[b] = pic[b] * c1.sc;
                Xm[b] = X[b] + k1[b] * P.half_dt;
                qm[b] = (Xm[b] - P.origin[b]) * inv_h;
            }
            gather_d<false>(a, P, qm, pic2, dpic2, nullptr, nullptr, W2);
            c2 = clamp_fwd(pic2, maxs);
            #pragma unroll
            for (int b = 0; b < 3; b++) {
                k2[b] = pic2[b] * c2.sc;
                np[b] = X[b] + k2[b] * dt;
            }
        } else {
            #pragma unroll
            for (int b = 0; b < 3; b++) np[b] = X[b] + nv[b] * dt;
        }
        bool wall[3];
        #pragma unroll
        for (int b = 0; b < 3; b++) wall[b] = np[b] < P.lo[b] || np[b] > P.hi[b];
        // ---- backward
        const float4 g0 = a.g_out[2 * (size_t)d], g1 = a.g_out[2 * (size_t)d + 1];
        const float gnp_o[3] = {g0.x, g0.y, g0.z}, gnv_o[3] = {g1.x, g1.y, g1.z};
        float gX[3], gnp[3], gnv[3], gpic_k1[3] = {0.0f, 0.0f, 0.0f};
        #pragma unroll
        for (int b = 0; b < 3; b++) {  // a pinned component: position at the wall, velocity zero
            gnp[b] = wall[b] ? 0.0f : gnp_o[b];
            gX[b] = gnp[b];
            gnv[b] = (wall[b] ? 0.0f : gnv_o[b]) + (rk2 ? 0.0f : gnp[b] * dt);
        }
        if (rk2) {
            float gk2[3], gpic2[3], gk1[3];
            #pragma unroll
            for (int b = 0; b < 3; b++) gk2[b] = gnp[b] * dt;
            clamp_bwd(c2, pic2, gk2, gpic2);
            float gXm[3] = {0.0f, 0.0f, 0.0f};
            #pragma unroll
            for (int b = 0; b < 3; b++)
                #pragma unroll
                for (int ax = 0; ax < 3; ax++) gXm[b] += gpic2[ax] * dpic2[ax][b];
            // midpoint-stencil coefficients: gfin/W2 per axis, scattered by k_adj_mid
            float c2[3];
#pragma unroll
            for (int ax = 0; ax < 3; ax++) c2[ax] = W2[ax] > 0.0f ? gpic2[ax] / W2[ax] : 0.0f;
            a.mid[2 * (size_t)d] = make_float4(qm[0], qm[1], qm[2], 0.0f);
            a.mid[2 * (size_t)d + 1] = make_float4(c2[0], c2[1], c2[2], 0.0f);
            const float m2 = fmaxf(fmaxf(fabsf(c2[0]), fabsf(c2[1])), fabsf(c2[2]));
            if (m2 > 0.0f) atomicMax(&a.flags[1], __float_as_uint(m2));  // order-free
            #pragma unroll
            for (int b = 0; b < 3; b++) {
                gX[b] += gXm[b];
                gk1[b] = gXm[b] * P.half_dt;
            }
            clamp_bwd(c1, pic, gk1, gpic_k1);
        }
        float gnvc[3];
        #pragma unroll
        for (int b = 0; b < 3; b++) {
            gnvc[b] = gnv[b] * ff[b];
#pragma unroll
            #pragma unroll
            for (int c = 0; c < 3; c++)
                if (fsel[b] == c) gX[c] += gnv[b] * nvc[b] * (-friction) * dnr[c];
        }
        float gmix[3];
        clamp_bwd(cm, mix, gnvc, gmix);
        // mix = pic + alpha*(pv - saved)
        float gpv[3], gpic[3], gsv[3];
        #pragma unroll
        for (int b = 0; b < 3; b++) {
            gpic[b] = gmix[b] + gpic_k1[b];
            gpv[b] = alpha * gmix[b];
            gsv[b] = -alpha * gmix[b];
        }
        #pragma unroll
        for (int b = 0; b < 3; b++)
            #pragma unroll
            for (int ax = 0; ax < 3; ax++) gX[b] += gpic[ax] * dpic[ax][b] + gsv[ax] * dsv[ax][b];
        // face coefficients of the gathers at X, summed per face by k_adj_gather
        float cf[3], cs[3];
#pragma unroll
        for (int ax = 0; ax < 3; ax++) {
            cf[ax] = W[ax] > 0.0f ? gpic[ax] / W[ax] : 0.0f;
            cs[ax] = W[ax] > 0.0f ? gsv[ax] / W[ax] : 0.0f;
        }
        a.coef[3 * (size_t)d] = make_float4(q[0], q[1], q[2], pv[0]);
        a.coef[3 * (size_t)d + 1] = make_float4(pv[1], pv[2], cf[0], cf[1]);
        a.coef[3 * (size_t)d + 2] = make_float4(cf[2], cs[0], cs[1], cs[2]);
        if (pos.w != 0.0f) a.flags[0] = 1u;  // a stray particle (its P2G cell is not its bin)
        a.g_sorted[2 * (size_t)d] = make_float4(gX[0], gX[1], gX[2], 0.0f);
        a.g_sorted[2 * (size_t)d + 1] = make_float4(gpv[0], gpv[1], gpv[2], 0.0f);
    }
}

// Gradient faces: interior, neither side solid, at least one side liquid (gradient.wgsl:45-63).
__device__ __forceinline__ bool grad_face(uint8_t lt, uint8_t ht) {
    return lt != CELL_SOLID && ht != CELL_SOLID && (lt == CELL_LIQUID || ht == CELL_LIQUID);
}

// dL/dp_c = -coeff * (sum over gradient faces whose hi cell is c of g - ... whose lo cell is c).
// One block per 256-cell chunk; with rhs_part set it also writes the chunk's
// float-float sum of rhs^2 (fixed order: warp shuffles, then warps in order).
__global__ void __launch_bounds__(256) k_adj_prhs(AdjBufs a) {
    __shared__ float2 s_red[8];
    const DevParams& P = *a.prm;
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    float acc = 0.0f;
    if (c < P.C && a.ct[c] == CELL_LIQUID) {
        const uint32_t nx = P.nx, ny = P.ny;
        const uint32_t i = c % nx, j = (c / nx) % ny, k = c / (nx * ny);
        const uint32_t ijk[3] = {i, j, k};
        const size_t step[3] = {1, nx, (size_t)nx * ny};
        for (int ax = 0; ax < 3; ax++) {
            const uint32_t dx = face_dim(P, ax, 0), dy = face_dim(P, ax, 1);
            // face at the low side of c (c is its hi cell) and at the high side (c is its lo cell)
            for (int side = 0; side < 2; side++) {
                uint32_t f3[3] = {i, j, k};
                f3[ax] = ijk[ax] + side;
                const size_t fidx = (size_t)f3[0] + dx * ((size_t)f3[1] + (size_t)dy * f3[2]);
                const size_t other = side == 0 ? c - step[ax] : c + step[ax];
                if (!grad_face(a.ct[side == 0 ? other : c], a.ct[side == 0 ? c : other])) continue;
                const float g = a.g_fs[ax][fidx].x;
                acc += side == 0 ? g : -g;
            }
        }
        acc *= -P.coeff_grad;
    }
    if (c < P.C) a.rhs[c] = acc;
    if (a.rhs_part) {
        const Df sq = warp_sum_df(df_prod(acc, acc));
        if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = make_float2(sq.hi, sq.lo);
        __syncthreads();
        if (threadIdx.x == 0) {
            Df t = {0.0f, 0.0f};
            for (int w = 0; w < 8; w++) t = df_add(t, Df{s_red[w].x, s_red[w].y});
            a.rhs_part[blockIdx.x] = make_float2(t.hi, t.lo);
        }
    }
}

// Absolute stopping threshold of the warm-started adjoint solve: tol^2 times
// the squared norm of its right-hand side, the value the cold-start test
// tol^2 * (r0.r0) uses (r0 = rhs when the solve starts from zero).  One block;
// the chunk partials are summed in a fixed order.
__global__ void __launch_bounds__(1024) k_adj_thr(const float2* __restrict__ part, uint32_t nchunks, double tol_sq,
                                                  DevParams* __restrict__ cg_prm) {
    __shared__ float2 s_red[32];
    Df t = {0.0f, 0.0f};
    for (uint32_t i = threadIdx.x; i < nchunks; i += blockDim.x) t = df_add(t, Df{part[i].x, part[i].y});
    t = warp_sum_df(t);
    const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
    if (lane == 0) s_red[warp] = make_float2(t.hi, t.lo);
    __syncthreads();
    if (threadIdx.x == 0) {
        Df s = {0.0f, 0.0f};
        for (uint32_t w = 0; w < blockDim.x / 32; w++) s = df_add(s, Df{s_red[w].x, s_red[w].y});
        const double thr = tol_sq * ((double)s.hi + (double)s.lo);
        cg_prm->thr_abs_d = thr;
        cg_prm->thr_abs_f = (float)thr;
        cg_prm->thr_abs = 1u;
    }
}

// Face stage: projection (divergence transposed), boundaries, forces, save_vel.
__global__ void __launch_bounds__(256) k_adj_faces(AdjBufs a, int axis) {
    __shared__ double s_red[8];
    const DevParams& P = *a.prm;
    const uint32_t nf = P.F3[axis];
    const uint32_t f = blockIdx.x * blockDim.x + threadIdx.x;
    double gg = 0.0;
    if (f < nf) {
        const uint32_t dx = face_dim(P, axis, 0), dy = face_dim(P, axis, 1);
        const uint32_t i = f % dx, j = (f / dx) % dy, k = f / (dx * dy);
        const uint32_t comp = axis == 0 ? i : (axis == 1 ? j : k);
        const uint32_t nax = axis == 0 ? P.nx : (axis == 1 ? P.ny : P.nz);
        const size_t hi_c = (size_t)i + P.nx * ((size_t)j + (size_t)P.ny * k);
        const size_t step = axis == 0 ? 1 : (axis == 1 ? P.nx : (size_t)P.nx * P.ny);
        const uint8_t tl = comp > 0 ? a.ct[hi_c - step] : CELL_SOLID;
        const uint8_t th = comp < nax ? a.ct[hi_c] : CELL_SOLID;
        const bool solid = comp == 0 || comp == nax || tl == CELL_SOLID || th == CELL_SOLID;
        float gpre = 0.0f;
        if (!solid) {
            // vel_final = vel_pre - coeff*(p_hi - p_lo) on gradient faces; p = A^-1(-scale*div(vel_pre))
            const float2 gfs = a.g_fs[axis][f];
            float g = gfs.x;
            float dl = 0.0f;
            if (tl == CELL_LIQUID) dl += a.lam[hi_c - step];
            if (th == CELL_LIQUID) dl -= a.lam[hi_c];
            g += -P.scale_rhs * P.inv_h * dl;
            gpre = g;
            const bool wet = tl == CELL_LIQUID || th == CELL_LIQUID;
            if (wet) gg = (double)gpre * (double)P.dt;
        }
        a.g_norm[axis][f] = gpre + a.g_fs[axis][f].y;
    }
    // dL/dg_axis: the block's partial in a fixed order (k_adj_grav sums the
    // blocks' partials in order)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) gg += __shfl_down_sync(0xffffffffu, gg, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = gg;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < 8; w++) s += s_red[w];
        a.grav_part[axis][blockIdx.x] = s;
    }
}

// dL/dgravity: per axis (one block each) the k_adj_faces partials, thread t
// summing partials t, t + 1024, ... in sequence, then a fixed tree.
__global__ void __launch_bounds__(1024) k_adj_grav(AdjBufs a, uint32_t nb0, uint32_t nb1, uint32_t nb2) {
    __shared__ double s_red[32];
    const uint32_t axis = blockIdx.x, nb = axis == 0 ? nb0 : (axis == 1 ? nb1 : nb2);
    const double* part = a.grav_part[axis];
    double s = 0.0;
    for (uint32_t i = threadIdx.x; i < nb; i += blockDim.x) s += part[i];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x < 32) {
        double v = s_red[threadIdx.x];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (threadIdx.x == 0) a.g_grav[axis] = v;
    }
}

// ---------------------------------------------------------------------------
// Face gradients and P2G sums, gathered per face in a fixed order.

// Scale of the midpoint stencil's 64-bit fixed-point sums: with m the largest
// |coefficient| of the step (flags[1]), m < 2^e, and at most 2^24 terms per
// face, |sum| * 2^(38 - e) < 2^62.  Quantum about 7e-12 m.
__device__ __forceinline__ int mid_exponent(const AdjBufs& a) {
    const float m = __uint_as_float(a.flags[1]);
    int e = 0;
    frexpf(m, &e);
    return 38 - e;
}

// The midpoint step's face gradients: each particle's wall-aware stencil at
// its midpoint Xm, w * (gfin/W at Xm), added as 64-bit fixed-point integers
// (integer sums do not depend on the order of the atomics).
__global__ void __launch_bounds__(256) k_adj_mid(AdjBufs a) {
    const DevParams& P = *a.prm;
    const uint32_t n = P.n;
    if (a.flags[1] == 0u) return;
    const double scale = ldexp(1.0, mid_exponent(a));
    for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d < n; d += gridDim.x * blockDim.x) {
        const float4 qm4 = a.mid[2 * (size_t)d], c4 = a.mid[2 * (size_t)d + 1];
        const float qm[3] = {qm4.x, qm4.y, qm4.z}, c2[3] = {c4.x, c4.y, c4.z};
#pragma unroll
        for (int ax = 0; ax < 3; ax++) {
            if (c2[ax] == 0.0f) continue;
            unsigned long long* g = a.gmid[ax];
            stencil(P, ax, qm, true, [&](size_t idx, float w, const float*) {
                atomicAdd(g + idx, (unsigned long long)llrint((double)(w * c2[ax]) * scale));
            });
        }
    }
}

// One thread per cell (i, j, k): the low faces u(i,j,k), v(i,j,k), w(i,j,k)
// of the cell, and on the grid's high sides also u(nx,j,k), v(i,ny,k),
// w(i,j,nz).  Every particle whose trilinear stencil (at its cell-space
// position q, scatter.wgsl:44-117 / g2p.wgsl:56-129) reaches one of these
// faces lies in the cells i-1..i+1, j-1..j+1, k-1..k+1 (two cells on every
// side when the step has stray particles, whose P2G cell differs from their
// bin by one); each (y, z) row of them is one contiguous range of the
// bin-ordered particles.  The rows are visited in (z, y) order and their
// particles in bin order, so every face's sums come out the same on every run:
//   g_fs = {sum w gpic/W, sum w gsaved/W}  (0 on faces touching the static
//          walls, which the wall-aware gathers skip) + the midpoint stencil's sum,
//   wsum = {sum w, sum w v_axis}  (every in-range tap, like scatter.wgsl).
// Candidates read the compact record {q, v_x} (16 B); the rest of a
// particle's record only when it has a tap among the faces.
__global__ void __launch_bounds__(256) k_adj_gather(AdjBufs a, int midpoint) {
    const DevParams& P = *a.prm;
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= P.C) return;
    const int nx = (int)P.nx, ny = (int)P.ny, nz = (int)P.nz;
    const int i = (int)(c % (uint32_t)nx), j = (int)((c / (uint32_t)nx) % (uint32_t)ny), k = (int)(c / ((uint32_t)nx * ny));
    const int cc[3] = {i, j, k}, n3[3] = {nx, ny, nz};
    // faces: 0..2 the low faces of axis 0..2, 3..5 the high-side faces of axis 0..2
    bool has[6];
    int fc[6][3];
    bool wall[6];
#pragma unroll
    for (int e = 0; e < 6; e++) {
        const int ax = e % 3;
#pragma unroll
        for (int b = 0; b < 3; b++) fc[e][b] = cc[b] + (e >= 3 && b == ax ? 1 : 0);
        has[e] = e < 3 || cc[ax] == n3[ax] - 1;
        wall[e] = touches_static_a(ax, fc[e][0], fc[e][1], fc[e][2], nx, ny, nz);
    }
    const int rad = a.flags[0] ? 2 : 1;
    int lo[3], hi[3];
#pragma unroll
    for (int b = 0; b < 3; b++) {
        lo[b] = max(cc[b] - rad, 0);
        hi[b] = min(cc[b] + rad, n3[b] - 1);
    }
    const uint32_t n = P.n, C = P.C;
    float gf[6], gs[6], W[6], WV[6];
#pragma unroll
    for (int e = 0; e < 6; e++) gf[e] = gs[e] = W[e] = WV[e] = 0.0f;
    for (int ck = lo[2]; ck <= hi[2]; ck++) {
        for (int cj = lo[1]; cj <= hi[1]; cj++) {
            const uint32_t row = (uint32_t)nx * ((uint32_t)cj + (uint32_t)ny * (uint32_t)ck);
            const uint32_t d0 = a.cell_first[row + lo[0]];
            const uint32_t e1 = row + (uint32_t)hi[0] + 1u;
            const uint32_t d1 = e1 < C ? a.cell_first[e1] : n;
            for (uint32_t d = d0; d < d1; d++) {
                const float4 r0 = a.coef[3 * (size_t)d];
                const float q[3] = {r0.x, r0.y, r0.z};
                // per dimension, the stencil's weight for face coordinate cc (lo) and
                // cc + 1 (hi) along the face axis (g = q + 0), and for cc across it
                // (g = q - 0.5); 0 where the coordinate is not one of the two taps
                float wlo[3], whi[3], wx[3];
#pragma unroll
                for (int b = 0; b < 3; b++) {
                    const float g0 = q[b] + 0.0f, g1 = q[b] + -0.5f;
                    const int b0 = __float2int_rz(floorf(g0)), b1 = __float2int_rz(floorf(g1));
                    const float t0 = g0 - (float)b0, t1 = g1 - (float)b1;
                    const int o0 = cc[b] - b0, o1 = cc[b] - b1;
                    wlo[b] = o0 == 0 ? 1.0f - t0 : (o0 == 1 ? t0 : 0.0f);
                    whi[b] = o0 == -1 ? 1.0f - t0 : (o0 == 0 ? t0 : 0.0f);
                    wx[b] = o1 == 0 ? 1.0f - t1 : (o1 == 1 ? t1 : 0.0f);
                }
                float w[6];
                bool any = false;
#pragma unroll
                for (int e = 0; e < 6; e++) {
                    const int ax = e % 3;
                    const float f0 = ax == 0 ? (e >= 3 ? whi[0] : wlo[0]) : wx[0];
                    const float f1 = ax == 1 ? (e >= 3 ? whi[1] : wlo[1]) : wx[1];
                    const float f2 = ax == 2 ? (e >= 3 ? whi[2] : wlo[2]) : wx[2];
                    w[e] = has[e] ? f0 * f1 * f2 : 0.0f;  // (wx * wy) * wz, the stencil's order
                    any = any || w[e] != 0.0f;
                }
                if (!any) continue;
                const float4 r1 = a.coef[3 * (size_t)d + 1], r2 = a.coef[3 * (size_t)d + 2];
                const float v[3] = {r0.w, r1.x, r1.y}, cf[3] = {r1.z, r1.w, r2.x}, cs[3] = {r2.y, r2.z, r2.w};
#pragma unroll
                for (int e = 0; e < 6; e++) {
                    const int ax = e % 3;
                    if (w[e] == 0.0f) continue;  // not a tap (a tap of weight 0 adds nothing either)
                    W[e] += w[e];
                    WV[e] += w[e] * v[ax];
                    if (!wall[e]) {
                        gf[e] += w[e] * cf[ax];
                        gs[e] += w[e] * cs[ax];
                    }
                }
            }
        }
    }
    const double mscale = midpoint && a.flags[1] != 0u ? ldexp(1.0, -mid_exponent(a)) : 0.0;
#pragma unroll
    for (int e = 0; e < 6; e++) {
        if (!has[e]) continue;
        const int ax = e % 3;
        const uint32_t dxa = (uint32_t)nx + (ax == 0), dya = (uint32_t)ny + (ax == 1);
        const size_t f = (size_t)fc[e][0] + dxa * ((size_t)fc[e][1] + (size_t)dya * fc[e][2]);
        float g = gf[e];
        if (mscale != 0.0 && !wall[e]) g += (float)((double)(long long)a.gmid[ax][f] * mscale);
        a.g_fs[ax][f] = make_float2(g, gs[e]);
        a.wsum[ax][f] = make_float2(W[e], WV[e]);
    }
}

// P2G transposed: vel_f = sum_p w v / sum_p w  ->  gather per particle, with
// the normalisation linearised at the unquantised sums k_adj_gather wrote.
__global__ void __launch_bounds__(256) k_adj_p2g(AdjBufs a) {
    const DevParams& P = *a.prm;
    const uint32_t n = P.n;
    const float inv_h = P.inv_h;
    for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d < n; d += gridDim.x * blockDim.x) {
        const float4 pos = a.part[2 * (size_t)d], pvel = a.part[2 * (size_t)d + 1];
        const float q[3] = {(pos.x - P.origin[0]) * inv_h, (pos.y - P.origin[1]) * inv_h, (pos.z - P.origin[2]) * inv_h};
        const float pv[3] = {pvel.x, pvel.y, pvel.z};
        float gX[3] = {0, 0, 0}, gv[3] = {0, 0, 0};
        for (int ax = 0; ax < 3; ax++) {
            const float2* ws = a.wsum[ax];
            const float* gn = a.g_norm[ax];
            stencil(P, ax, q, false, [&](size_t idx, float w, const float* dw) {
                const float2 s = ws[idx];
                const float W = s.x;
                if (!(W > 0.0f)) return;
                const float g = gn[idx] / W;
                gv[ax] += w * g;
                const float diff = (pv[ax] - s.y / W) * g * inv_h;
                for (int b = 0; b < 3; b++) gX[b] += dw[b] * diff;
            });
        }
        float4 s0 = a.g_sorted[2 * (size_t)d], s1 = a.g_sorted[2 * (size_t)d + 1];
        s0.x += gX[0]; s0.y += gX[1]; s0.z += gX[2];
        s1.x += gv[0]; s1.y += gv[1]; s1.z += gv[2];
        a.g_sorted[2 * (size_t)d] = s0;
        a.g_sorted[2 * (size_t)d + 1] = s1;
    }
}

__global__ void __launch_bounds__(256) k_adj_unsort(AdjBufs a) {
    const uint32_t n = a.prm->n;
    for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d < n; d += gridDim.x * blockDim.x) {
        const uint32_t src = a.perm[d];
        a.g_in[2 * (size_t)src] = a.g_sorted[2 * (size_t)d];
        a.g_in[2 * (size_t)src + 1] = a.g_sorted[2 * (size_t)d + 1];
    }
}

cudaError_t launch_adj_g2p(const AdjBufs& a, const LaunchCfg& L, cudaStream_t s) {
    k_adj_g2p<<<L.particle_blocks, 256, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_adj_prhs(const AdjBufs& a, uint32_t C, cudaStream_t s) {
    k_adj_prhs<<<(C + 255) / 256, 256, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_adj_thr(const AdjBufs& a, uint32_t nchunks, double tol_sq, DevParams* cg_prm, cudaStream_t s) {
    k_adj_thr<<<1, 1024, 0, s>>>(a.rhs_part, nchunks, tol_sq, cg_prm);
    return cudaGetLastError();
}
cudaError_t launch_adj_faces(const AdjBufs& a, const uint32_t F3[3], cudaStream_t s) {
    for (int ax = 0; ax < 3; ax++) k_adj_faces<<<(F3[ax] + 255) / 256, 256, 0, s>>>(a, ax);
    k_adj_grav<<<3, 1024, 0, s>>>(a, (F3[0] + 255) / 256, (F3[1] + 255) / 256, (F3[2] + 255) / 256);
    return cudaGetLastError();
}
cudaError_t launch_adj_mid(const AdjBufs& a, const LaunchCfg& L, cudaStream_t s) {
    k_adj_mid<<<L.particle_blocks, 256, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_adj_gather(const AdjBufs& a, uint32_t C, bool midpoint, cudaStream_t s) {
    k_adj_gather<<<(C + 255) / 256, 256, 0, s>>>(a, midpoint ? 1 : 0);
    return cudaGetLastError();
}
cudaError_t launch_adj_p2g(const AdjBufs& a, const LaunchCfg& L, cudaStream_t s) {
    k_adj_p2g<<<L.particle_blocks, 256, 0, s>>>(a);
    return cudaGetLastError();
}
cudaError_t launch_adj_unsort(const AdjBufs& a, const LaunchCfg& L, cudaStream_t s) {
    k_adj_unsort<<<L.particle_blocks, 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace fl
