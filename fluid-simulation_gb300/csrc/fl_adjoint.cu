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
//                   w.r.t. position and velocity, and face gradients of the
//                   final and saved velocities (scatter = transpose of the
//                   trilinear gather; one float2 vector atomic per tap into
//                   the interleaved {final, saved} gradients)
//   k_adj_prhs      gradient.wgsl transposed: dL/dp per liquid cell, the RHS
//                   of the adjoint pressure solve A lambda = dL/dp
//   k_adj_thr       (warm start only) the solve's absolute stopping threshold
//   (k_solve_init + k_cg with the RHS: the adjoint solve)
//   k_adj_faces     divergence.wgsl and gradient.wgsl transposed, then
//                   boundaries.wgsl / forces.wgsl / save_vel.wgsl: gradient of
//                   the normalised P2G face velocity, and dL/dgravity
//   k_adj_p2g_sums  scatter.wgsl without the fixed-point rounding: {sum w,
//                   sum w v} per face (one float2 vector atomic per tap)
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

// Face gradients of a wall-aware gather at q: d(sum w f / W)/d f = w/W.
__device__ __forceinline__ void scatter_faces(const AdjBufs& a, const DevParams& P, const float q[3], const float W[3],
                                              const float gfin[3], const float gsav[3]) {
    #pragma unroll
    for (int ax = 0; ax < 3; ax++) {
        if (!(W[ax] > 0.0f)) continue;
        const float cf = gfin[ax] / W[ax], cs = gsav ? gsav[ax] / W[ax] : 0.0f;
        if (cf == 0.0f && cs == 0.0f) continue;
        float2* gfs = a.g_fs[ax];
        stencil(P, ax, q, true, [&](size_t idx, float w, const float*) {
            atomicAdd(gfs + idx, make_float2(w * cf, w * cs));
        });
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
            scatter_faces(a, P, qm, W2, gpic2, nullptr);
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
        scatter_faces(a, P, q, W, gpic, gsv);
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
    // dL/dg_axis (fixed order within the block, atomics across blocks)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) gg += __shfl_down_sync(0xffffffffu, gg, o);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = gg;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < 8; w++) s += s_red[w];
        if (s != 0.0) atomicAdd(&a.g_grav[axis], s);
    }
}

// P2G transposed: vel_f = sum_p w v / sum_p w  ->  gather per particle.
// scatter.wgsl's sums without the fixed-point rounding: the point at which
// k_adj_p2g linearises the normalisation.  Bin order keeps the atomics of a
// warp on neighbouring faces.
__global__ void __launch_bounds__(256) k_adj_p2g_sums(AdjBufs a) {
    const DevParams& P = *a.prm;
    const uint32_t n = P.n;
    const float inv_h = P.inv_h;
    for (uint32_t d = blockIdx.x * blockDim.x + threadIdx.x; d < n; d += gridDim.x * blockDim.x) {
        const float4 pos = a.part[2 * (size_t)d], pvel = a.part[2 * (size_t)d + 1];
        const float q[3] = {(pos.x - P.origin[0]) * inv_h, (pos.y - P.origin[1]) * inv_h, (pos.z - P.origin[2]) * inv_h};
        const float pv[3] = {pvel.x, pvel.y, pvel.z};
        for (int ax = 0; ax < 3; ax++) {
            float2* ws = a.wsum[ax];
            stencil(P, ax, q, false, [&](size_t idx, float w, const float*) {
                atomicAdd(ws + idx, make_float2(w, w * pv[ax]));
            });
        }
    }
}

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
    return cudaGetLastError();
}
cudaError_t launch_adj_p2g_sums(const AdjBufs& a, const LaunchCfg& L, cudaStream_t s) {
    k_adj_p2g_sums<<<L.particle_blocks, 256, 0, s>>>(a);
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
