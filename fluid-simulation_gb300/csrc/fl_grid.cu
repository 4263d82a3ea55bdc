// fl_grid.cu — cell classification, P2G, grid preparation and projection.
//
//   k_classify   classify.wgsl:25-61 (Solid/Liquid/Air, dilation, liquid count)
//   k_p2g_own    scatter.wgsl:44-117 over the sorted bins: one block per tile
//                of cells accumulates the fixed-point terms of the particles
//                binned in the tile in shared memory, over the faces they
//                reach, then adds the sums to the cleared face arrays with
//                integer reductions (exact and order-free); no float atomics
//   k_p2g_strays the same terms for particles flagged as strays (their
//                multiply-form cell differs from their bin), by global atomics
//   k_grid_prep  normalize.wgsl + save_vel.wgsl + forces.wgsl + boundaries.wgsl
//                per face, then divergence.wgsl + cg_init.wgsl + the first
//                cg_reduce.wgsl tree per 256-cell chunk
//   k_project    gradient.wgsl (the following boundaries pass is a no-op: faces
//                touching a solid are already zero and gradient skips them)
#include "fl_device.cuh"

namespace fl {

__global__ void __launch_bounds__(256) k_classify(DevBufs b, uint32_t C) {
    const DevParams& P = *b.prm;
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    bool liquid = false;
    if (c < C) {
        const uint32_t nx = P.nx, ny = P.ny, nz = P.nz;
        const uint32_t i = c % nx, j = (c / nx) % ny, k = c / (nx * ny);
        const bool boundary = i == 0 || j == 0 || k == 0 || i == nx - 1 || j == ny - 1 || k == nz - 1;
        uint8_t t = CELL_SOLID;
        if (!boundary) {
            const uint32_t th = P.thresh;
            const uint32_t* occ = b.counts;
            liquid = occ[c] >= th;
            if (!liquid && P.dilation) {
                liquid = occ[c - 1] >= th || occ[c + 1] >= th || occ[c - nx] >= th || occ[c + nx] >= th ||
                         occ[c - nx * ny] >= th || occ[c + nx * ny] >= th;
            }
            t = liquid ? CELL_LIQUID : CELL_AIR;
        }
        b.ct[c] = t;
    }
    const uint32_t m = __ballot_sync(0xffffffffu, liquid);
    if ((threadIdx.x & 31u) == 0 && m) atomicAdd(&b.st->liquid, (uint32_t)__popc(m));
}

// ---------------------------------------------------------------------------
// P2G

constexpr int P2G_BATCH = 4;  // particles in flight per thread

// k_p2g_own: one 256-thread block per 8^3 tile of cells, visiting only the
// particles binned in the tile (each particle once; a tile that also read its
// one-cell halo, to own its faces outright, visited about 1.95 per particle
// at 128^3).  A particle of cell c
// reaches faces c..c+1 along the face axis and c-1..c+1 along the other two
// (scatter.wgsl:55-67), so the block accumulates its fixed-point terms over a
// box of (TILE+1) x (TILE+2) x (TILE+2) faces per axis -- the tile's faces
// and a one-face rim -- in shared memory, then adds every nonzero sum to the
// face arrays (cleared before the launch) with integer reductions.  Integer
// sums are order-free, so num/den equal the reference's atomic scatter
// exactly, whatever order the blocks add in.
constexpr int PB_A = TILE + 1;                  // box faces along the face axis
constexpr int PB_O = TILE + 2;                  // box faces along the other axes
constexpr int PB_N = PB_A * PB_O * PB_O;        // box faces per axis
constexpr int P2G_OWN_ROWS = TILE * TILE;       // (y, z) rows of a tile

__device__ __forceinline__ void p2g_box(const DevParams& P, DevStats* st, const int o[3], int axis, const float q[3],
                                        float vcomp, int32_t* s_num, int32_t* s_den) {
    float t[3];
    int base[3];
#pragma unroll
    for (int bb = 0; bb < 3; bb++) {
        const float g = __fadd_rn(q[bb], bb == axis ? 0.0f : -0.5f);
        base[bb] = floor_to_i32(g) - (o[bb] - (bb == axis ? 0 : 1));  // box coordinate of the first tap
        t[bb] = __fsub_rn(g, floorf(g));
    }
    // A particle that is not a stray has floor(q) == its bin cell, so the taps
    // lie in the box (first tap 0..TILE-1 along the face axis, 0..TILE along
    // the others); anything else is recorded and skipped, never written.
    const uint32_t lim[3] = {axis == 0 ? (uint32_t)TILE - 1u : (uint32_t)TILE, axis == 1 ? (uint32_t)TILE - 1u : (uint32_t)TILE,
                             axis == 2 ? (uint32_t)TILE - 1u : (uint32_t)TILE};
    if ((uint32_t)base[0] > lim[0] || (uint32_t)base[1] > lim[1] || (uint32_t)base[2] > lim[2]) {
        atomicCAS(&st->status, 0u, 7u /* FL_INTERNAL */);
        return;
    }
    const int sx = axis == 0 ? PB_A : PB_O, sy = axis == 1 ? PB_A : PB_O;
    const float scale = P.fixed_scale;
#pragma unroll
    for (int dk = 0; dk < 2; dk++) {
        const float wz = tent(t[2], dk);
#pragma unroll
        for (int dj = 0; dj < 2; dj++) {
            const float wy = tent(t[1], dj);
#pragma unroll
            for (int di = 0; di < 2; di++) {
                const float wx = tent(t[0], di);
                const float w = __fmul_rn(__fmul_rn(wx, wy), wz);
                if (w <= 0.0f) continue;
                const int li = (base[0] + di) + sx * ((base[1] + dj) + sy * (base[2] + dk));
                atomicAdd(&s_num[li], fixed_round(__fmul_rn(__fmul_rn(w, vcomp), scale)));
                atomicAdd(&s_den[li], fixed_round(__fmul_rn(w, scale)));
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_p2g_own(DevBufs b, int tiles_x, int tiles_y) {
    __shared__ int32_t s_num[3][PB_N];
    __shared__ int32_t s_den[3][PB_N];
    __shared__ uint32_t s_row_beg[P2G_OWN_ROWS];      // first sorted particle of each row of the tile
    __shared__ uint32_t s_row_off[P2G_OWN_ROWS + 1];  // prefix of the row lengths
    __shared__ uint32_t s_wsum[2];
    const DevParams& P = *b.prm;
    const int nx = (int)P.nx, ny = (int)P.ny, nz = (int)P.nz;
    const int tile = blockIdx.x;
    const int x0 = (tile % tiles_x) * TILE, y0 = ((tile / tiles_x) % tiles_y) * TILE, z0 = (tile / (tiles_x * tiles_y)) * TILE;
    const int xe = min(x0 + TILE, nx), ye = min(y0 + TILE, ny), ze = min(z0 + TILE, nz);
    const int rows_y = ye - y0, rows = rows_y * (ze - z0);
    uint32_t len = 0;
    if ((int)threadIdx.x < rows) {
        const uint32_t cy = (uint32_t)(y0 + (int)threadIdx.x % rows_y), cz = (uint32_t)(z0 + (int)threadIdx.x / rows_y);
        const uint32_t c0 = (uint32_t)x0 + P.nx * (cy + P.ny * cz), c1 = c0 + (uint32_t)(xe - x0 - 1);
        const uint32_t pbeg = b.offsets[c0];
        len = b.offsets[c1] + b.counts[c1] - pbeg;
        s_row_beg[threadIdx.x] = pbeg;
    }
    // exclusive prefix of the row lengths (rows <= 64: warps 0..1)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    {
        uint32_t x = len;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (warp < 2 && lane == 31) s_wsum[warp] = x;
        __syncthreads();
        if ((int)threadIdx.x < rows) s_row_off[threadIdx.x] = (warp == 1 ? s_wsum[0] : 0u) + x - len;
        if (threadIdx.x == 0) s_row_off[rows] = s_wsum[0] + s_wsum[1];
    }
    const uint32_t total = s_wsum[0] + s_wsum[1];
    if (total == 0) return;  // no particle binned in the tile: nothing to add (the face arrays are cleared)
    for (int i = threadIdx.x; i < 3 * PB_N; i += blockDim.x) {
        (&s_num[0][0])[i] = 0;
        (&s_den[0][0])[i] = 0;
    }
    __syncthreads();
    const float inv_h = P.inv_h;
    const float o0 = P.origin[0], o1 = P.origin[1], o2 = P.origin[2];
    const int orig[3] = {x0, y0, z0};
    // Within each group of 256 particle indices thread t takes (t % 32) * 8
    // + t / 32, so the lanes of a warp hold particles of different cells (8
    // per cell when dense) and their shared-memory atomics rarely meet.
    const uint32_t swz = (threadIdx.x & 31u) * 8u + (threadIdx.x >> 5);
    for (uint32_t g0 = 0; g0 < total; g0 += 256u * P2G_BATCH) {
        float4 pos[P2G_BATCH], vel[P2G_BATCH];
        bool use[P2G_BATCH];
#pragma unroll
        for (int k = 0; k < P2G_BATCH; k++) {
            const uint32_t f = g0 + 256u * k + swz;
            use[k] = f < total;
            uint32_t pp = 0;
            if (use[k]) {
                int lo = 0, hi = rows - 1;  // last row with s_row_off[row] <= f
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (s_row_off[mid] <= f) lo = mid;
                    else hi = mid - 1;
                }
                pp = s_row_beg[lo] + (f - s_row_off[lo]);
            }
            pos[k] = use[k] ? b.part_sorted[2 * (size_t)pp] : make_float4(0.f, 0.f, 0.f, 1.f);
            vel[k] = use[k] ? b.part_sorted[2 * (size_t)pp + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
        }
#pragma unroll
        for (int k = 0; k < P2G_BATCH; k++) {
            if (!use[k] || pos[k].w != 0.0f) continue;  // stray: handled by k_p2g_strays
            const float q[3] = {__fmul_rn(__fsub_rn(pos[k].x, o0), inv_h), __fmul_rn(__fsub_rn(pos[k].y, o1), inv_h),
                                __fmul_rn(__fsub_rn(pos[k].z, o2), inv_h)};
            p2g_box(P, b.st, orig, 0, q, vel[k].x, s_num[0], s_den[0]);
            p2g_box(P, b.st, orig, 1, q, vel[k].y, s_num[1], s_den[1]);
            p2g_box(P, b.st, orig, 2, q, vel[k].z, s_num[2], s_den[2]);
        }
    }
    __syncthreads();

    // Add the box to the face arrays: every nonzero sum of a face inside the grid.
    for (int axis = 0; axis < 3; axis++) {
        const int sx = axis == 0 ? PB_A : PB_O, sy = axis == 1 ? PB_A : PB_O;
        const int fx0 = x0 - (axis != 0), fy0 = y0 - (axis != 1), fz0 = z0 - (axis != 2);
        const int dx = (int)face_dim(P, axis, 0), dy = (int)face_dim(P, axis, 1), dz = (int)face_dim(P, axis, 2);
        for (int li = threadIdx.x; li < PB_N; li += blockDim.x) {
            const int32_t vn = s_num[axis][li], vd = s_den[axis][li];
            if ((vn | vd) == 0) continue;
            const int fi = fx0 + li % sx, fj = fy0 + (li / sx) % sy, fk = fz0 + li / (sx * sy);
            if (fi < 0 || fj < 0 || fk < 0 || fi >= dx || fj >= dy || fk >= dz) continue;
            const size_t gidx = (size_t)fi + (size_t)dx * ((size_t)fj + (size_t)dy * fk);
            if (vn) atomicAdd(&b.num[axis][gidx], vn);
            if (vd) atomicAdd(&b.den[axis][gidx], vd);
        }
    }
}

__global__ void __launch_bounds__(256) k_p2g_strays(DevBufs b) {
    const DevParams& P = *b.prm;
    const uint32_t ns = b.st->strays;
    const int n3[3] = {(int)P.nx, (int)P.ny, (int)P.nz};
    for (uint32_t s = blockIdx.x * blockDim.x + threadIdx.x; s < ns; s += gridDim.x * blockDim.x) {
        const uint32_t d = b.stray_list[s];
        const float4 pos = b.part_sorted[2 * (size_t)d];
        const float4 vel = b.part_sorted[2 * (size_t)d + 1];
        const float q[3] = {__fmul_rn(__fsub_rn(pos.x, P.origin[0]), P.inv_h),
                            __fmul_rn(__fsub_rn(pos.y, P.origin[1]), P.inv_h),
                            __fmul_rn(__fsub_rn(pos.z, P.origin[2]), P.inv_h)};
        const float vc[3] = {vel.x, vel.y, vel.z};
        for (int axis = 0; axis < 3; axis++) {
            int dim[3];
            float t[3];
            int base[3];
            for (int bb = 0; bb < 3; bb++) {
                dim[bb] = n3[bb] + (axis == bb ? 1 : 0);
                const float g = __fadd_rn(q[bb], bb == axis ? 0.0f : -0.5f);
                base[bb] = floor_to_i32(g);
                t[bb] = __fsub_rn(g, (float)base[bb]);
            }
            for (int dk = 0; dk < 2; dk++) {
                const int kk = base[2] + dk;
                if (kk < 0 || kk >= dim[2]) continue;
                const float wz = tent(t[2], dk);
                for (int dj = 0; dj < 2; dj++) {
                    const int jj = base[1] + dj;
                    if (jj < 0 || jj >= dim[1]) continue;
                    const float wy = tent(t[1], dj);
                    for (int di = 0; di < 2; di++) {
                        const int ii = base[0] + di;
                        if (ii < 0 || ii >= dim[0]) continue;
                        const float wx = tent(t[0], di);
                        const float w = __fmul_rn(__fmul_rn(wx, wy), wz);
                        if (w <= 0.0f) continue;
                        const size_t idx = (size_t)ii + (size_t)dim[0] * ((size_t)jj + (size_t)dim[1] * kk);
                        atomicAdd(&b.num[axis][idx], fixed_round(__fmul_rn(__fmul_rn(w, vc[axis]), P.fixed_scale)));
                        atomicAdd(&b.den[axis][idx], fixed_round(__fmul_rn(w, P.fixed_scale)));
                    }
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// grid prep

// One face after normalize -> save_vel -> forces -> boundaries.
// Returns the pre-force (saved) value in *saved.
// One face after normalize -> save_vel -> forces -> boundaries, from
// preloaded values: the face's fixed-point sums (dn, nm), its coordinate
// along the axis (comp, of nax cells) and the types of the cells below (tl)
// and above (th) it, CELL_SOLID outside the grid.  Returns the face value;
// *saved gets the pre-force (saved) value.
__device__ __forceinline__ float face_value(const DevParams& P, int axis, int32_t dn, int32_t nm, uint32_t comp,
                                            uint32_t nax, uint8_t tl, uint8_t th, float* saved) {
    float v = 0.0f;
    if (dn > 0) v = __fdiv_rn(__int2float_rn(nm), __int2float_rn(dn));  // normalize.wgsl:21-26
    *saved = v;                                                          // save_vel.wgsl:18
    const bool wet = (comp > 0 && tl == CELL_LIQUID) || (comp < nax && th == CELL_LIQUID);
    if (wet) v = __fadd_rn(v, __fmul_rn(P.grav[axis], P.dt));  // forces.wgsl:75-83
    if (comp == 0 || comp == nax || tl == CELL_SOLID || th == CELL_SOLID) v = 0.0f;  // boundaries.wgsl:43-60
    return v;
}

// cg_reduce.wgsl:38-49 tree over a 256-thread block (s has 256 floats).
// Steps 128/64/32 go through shared memory, 16..1 through shuffles of warp 0;
// the pairing (i with i+off) is the same at every level.
__device__ __forceinline__ float block_tree256(float prod, float* s) {
    const int t = threadIdx.x;
    s[t] = prod;
    __syncthreads();
    if (t < 128) s[t] = __fadd_rn(s[t], s[t + 128]);
    __syncthreads();
    if (t < 64) s[t] = __fadd_rn(s[t], s[t + 64]);
    __syncthreads();
    float v = 0.0f;
    if (t < 32) {
        v = __fadd_rn(s[t], s[t + 32]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = __fadd_rn(v, __shfl_down_sync(0xffffffffu, v, o));
    }
    return v;
}

// (A x)_c of cg_spmv.wgsl:46-68 / cg_init.wgsl:24-48, neighbour order -x,+x,-y,+y,-z,+z.
__device__ __forceinline__ float apply_A(const uint8_t* ct, const float* x, size_t c, size_t nx, size_t nxy, float xc) {
    float cnt = 0.0f, sum = 0.0f;
    const size_t nb[6] = {c - 1, c + 1, c - nx, c + nx, c - nxy, c + nxy};
#pragma unroll
    for (int s = 0; s < 6; s++) {
        const uint8_t t = ct[nb[s]];
        if (t != CELL_SOLID) {
            cnt = __fadd_rn(cnt, 1.0f);
            if (t == CELL_LIQUID) sum = __fadd_rn(sum, x[nb[s]]);
        }
    }
    return __fsub_rn(__fmul_rn(cnt, xc), sum);
}

// Stencil mask of a liquid (hence interior) cell, for the CG.
__device__ __forceinline__ uint16_t stencil_info(const uint8_t* ct, size_t c, size_t nx, size_t nxy) {
    const size_t nb[6] = {c - 1, c + 1, c - nx, c + nx, c - nxy, c + nxy};
    uint32_t info = 1u, cnt = 0u;
#pragma unroll
    for (int s = 0; s < 6; s++) {
        const uint8_t t = ct[nb[s]];
        if (t != CELL_SOLID) cnt++;
        if (t == CELL_LIQUID) info |= 2u << s;
    }
    return (uint16_t)(info | (cnt << 7));
}

__global__ void __launch_bounds__(256) k_grid_prep(DevBufs b, uint32_t C) {
    __shared__ float s_tree[256];
    __shared__ float2 s_red[8];
    const DevParams& P = *b.prm;
    const uint32_t chunk = blockIdx.x;
    const uint32_t c = chunk * 256 + threadIdx.x;
    bool liquid = false;
    float prod = 0.0f;
    Df pdf = {0.0f, 0.0f};
    if (c < C) {
        // Every load a cell needs is issued before its results are used: the
        // lower faces' sums and cell types first, then (liquid cells) the
        // upper faces', the neighbours' types and pressures; all stores come
        // after.  The arithmetic is face_value's and apply_A's, in their order.
        const uint32_t nx = P.nx, ny = P.ny, nz = P.nz;
        const uint32_t i = c % nx, j = (c / nx) % ny, k = c / (nx * ny);
        const size_t nxy = (size_t)nx * ny;
        const size_t i0 = (size_t)i + (size_t)(nx + 1) * ((size_t)j + (size_t)ny * k);  // u face (i, j, k)
        const size_t i1 = (size_t)i + (size_t)nx * ((size_t)j + (size_t)(ny + 1) * k);  // v face (i, j, k)
        const size_t i2 = c;                                                            // w face (i, j, k)
        const int32_t d0 = b.den[0][i0], n0 = b.num[0][i0], d1 = b.den[1][i1], n1 = b.num[1][i1];
        const int32_t d2 = b.den[2][i2], n2 = b.num[2][i2];
        const uint8_t tc = b.ct[c];
        const uint8_t tmx = i > 0 ? b.ct[c - 1] : CELL_SOLID, tmy = j > 0 ? b.ct[c - nx] : CELL_SOLID,
                      tmz = k > 0 ? b.ct[c - nxy] : CELL_SOLID;
        // the grid's far faces, written by the last cell of each line
        const bool eu = i == nx - 1, ev = j == ny - 1, ew = k == nz - 1;
        const int32_t ed0 = eu ? b.den[0][i0 + 1] : 0, en0 = eu ? b.num[0][i0 + 1] : 0;
        const int32_t ed1 = ev ? b.den[1][i1 + nx] : 0, en1 = ev ? b.num[1][i1 + nx] : 0;
        const int32_t ed2 = ew ? b.den[2][i2 + nxy] : 0, en2 = ew ? b.num[2][i2 + nxy] : 0;
        float su, sv, sw;
        const float ul = face_value(P, 0, d0, n0, i, nx, tmx, tc, &su);
        const float vl = face_value(P, 1, d1, n1, j, ny, tmy, tc, &sv);
        const float wl = face_value(P, 2, d2, n2, k, nz, tmz, tc, &sw);
        liquid = tc == CELL_LIQUID;
        if (liquid) {
            // divergence.wgsl:36-58 (liquid cells are interior, so i+1 <= nx-1)
            const int32_t du = b.den[0][i0 + 1], nu = b.num[0][i0 + 1], dv = b.den[1][i1 + nx], nv = b.num[1][i1 + nx];
            const int32_t dw = b.den[2][i2 + nxy], nw = b.num[2][i2 + nxy];
            const uint8_t tpx = b.ct[c + 1], tpy = b.ct[c + nx], tpz = b.ct[c + nxy];
            const bool drift_on = P.stiff > 0.0f && P.rest > 0.0f;
            const uint32_t occ = drift_on ? b.counts[c] : 0u;
            const bool warm = P.warm != 0u;
            const size_t nb6[6] = {c - 1, c + 1, c - nx, c + nx, c - nxy, c + nxy};
            float pn[6];
#pragma unroll
            for (int s2 = 0; s2 < 6; s2++) pn[s2] = warm ? b.p[nb6[s2]] : 0.0f;
            const float p_initial = warm ? b.p[c] : 0.0f;
            float unused;
            const float uh = face_value(P, 0, du, nu, i + 1, nx, tc, tpx, &unused);
            const float vh = face_value(P, 1, dv, nv, j + 1, ny, tc, tpy, &unused);
            const float wh = face_value(P, 2, dw, nw, k + 1, nz, tc, tpz, &unused);
            float dvg = __fmul_rn(__fadd_rn(__fadd_rn(__fsub_rn(uh, ul), __fsub_rn(vh, vl)), __fsub_rn(wh, wl)), P.inv_h);
            if (drift_on) {
                const float over = __fdiv_rn(fmaxf(0.0f, __fsub_rn(__uint2float_rn(occ), P.rest)), P.rest);
                const float drift = fminf(__fmul_rn(P.stiff, over), P.drift_clamp);
                dvg = __fsub_rn(dvg, drift);
            }
            // cg_init.wgsl:66-81; (A p)_c of cg_init.wgsl:24-48, order -x,+x,-y,+y,-z,+z
            const float rhs = __fmul_rn(-P.scale_rhs, dvg);
            const uint8_t t6[6] = {tmx, tpx, tmy, tpy, tmz, tpz};
            float ap = 0.0f;
            uint32_t info = 1u, ncnt = 0u;
            {
                float cnt = 0.0f, sum = 0.0f;
#pragma unroll
                for (int s2 = 0; s2 < 6; s2++) {
                    const uint8_t t = t6[s2];
                    if (t != CELL_SOLID) {
                        cnt = __fadd_rn(cnt, 1.0f);
                        ncnt++;
                        if (t == CELL_LIQUID) sum = __fadd_rn(sum, pn[s2]);
                    }
                    if (t == CELL_LIQUID) info |= 2u << s2;
                }
                if (warm) ap = __fsub_rn(__fmul_rn(cnt, p_initial), sum);
            }
            const float rc = __fsub_rn(rhs, ap);
            if (b.div) b.div[c] = dvg;
            if (!warm) b.p[c] = 0.0f;
            b.r[c] = rc;
            b.dA[c] = rc;
            b.cinfo[c] = (uint16_t)(info | (ncnt << 7));
            prod = __fmul_rn(rc, rc);
            pdf = df_prod(rc, rc);
        } else {
            b.p[c] = 0.0f;
            b.r[c] = 0.0f;
            b.dA[c] = 0.0f;
            b.cinfo[c] = 0;
            if (b.div) b.div[c] = 0.0f;
        }
        b.vel[0][i0] = ul;
        b.sav[0][i0] = su;
        b.vel[1][i1] = vl;
        b.sav[1][i1] = sv;
        b.vel[2][i2] = wl;
        b.sav[2][i2] = sw;
        float se;
        if (eu) {
            b.vel[0][i0 + 1] = face_value(P, 0, ed0, en0, nx, nx, tc, CELL_SOLID, &se);
            b.sav[0][i0 + 1] = se;
        }
        if (ev) {
            b.vel[1][i1 + nx] = face_value(P, 1, ed1, en1, ny, ny, tc, CELL_SOLID, &se);
            b.sav[1][i1 + nx] = se;
        }
        if (ew) {
            b.vel[2][i2 + nxy] = face_value(P, 2, ed2, en2, nz, nz, tc, CELL_SOLID, &se);
            b.sav[2][i2 + nxy] = se;
        }
    }
    const int nliq = __syncthreads_count(liquid);
    const float v = block_tree256(prod, s_tree);
    // float-float partial of this chunk (fixed order: warp shuffles, then warps in order)
    pdf = warp_sum_df(pdf);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = make_float2(pdf.hi, pdf.lo);
    __syncthreads();
    if (threadIdx.x == 0) {
        Df a = {0.0f, 0.0f};
        for (int w = 0; w < 8; w++) a = df_add(a, Df{s_red[w].x, s_red[w].y});
        b.part_rr[chunk] = v;
        b.chunk_rr_df[chunk] = make_float2(a.hi, a.lo);
        b.chunk_flag[chunk] = (uint8_t)(nliq < 255 ? nliq : 255);
    }
}

// gradient.wgsl:23-67 on the cell's three lower faces: an interior face
// with no solid side and a liquid side gets vel -= coeff * (p_hi - p_lo).
// The cell types, pressures and face values are loaded before any face is
// written (the kernel is latency-bound, and a face's store would otherwise
// hold back the next face's loads).
__global__ void __launch_bounds__(256) k_project(DevBufs b, uint32_t C) {
    const DevParams& P = *b.prm;
    const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= C) return;
    const uint32_t nx = P.nx, ny = P.ny;
    const uint32_t i = c % nx, j = (c / nx) % ny, k = c / (nx * ny);
    const size_t nxy = (size_t)nx * ny;
    const size_t lo[3] = {c - 1, c - nx, c - nxy};
    const size_t idx[3] = {(size_t)i + (size_t)(nx + 1) * ((size_t)j + (size_t)ny * k),
                           (size_t)i + (size_t)nx * ((size_t)j + (size_t)(ny + 1) * k), (size_t)c};
    const bool inner[3] = {i > 0, j > 0, k > 0};  // comp == nax never holds for a lower face (comp < n)
    const uint8_t ht = b.ct[c];
    uint8_t lt[3];
#pragma unroll
    for (int a = 0; a < 3; a++) lt[a] = inner[a] ? b.ct[lo[a]] : CELL_SOLID;
    bool on[3];
#pragma unroll
    for (int a = 0; a < 3; a++)  // gradient.wgsl:45-60
        on[a] = inner[a] && lt[a] != CELL_SOLID && ht != CELL_SOLID && (lt[a] == CELL_LIQUID || ht == CELL_LIQUID);
    if (!(on[0] || on[1] || on[2])) return;
    const float ph = b.p[c];
    float pl[3], v[3];
#pragma unroll
    for (int a = 0; a < 3; a++) {
        pl[a] = on[a] ? b.p[lo[a]] : 0.0f;
        v[a] = on[a] ? b.vel[a][idx[a]] : 0.0f;
    }
#pragma unroll
    for (int a = 0; a < 3; a++)
        if (on[a]) b.vel[a][idx[a]] = __fsub_rn(v[a], __fmul_rn(P.coeff_grad, __fsub_rn(ph, pl[a])));
}

// Stand-alone solve: cg_init.wgsl:50-87 from a given divergence field (the
// tail of k_grid_prep without the face passes).
__global__ void __launch_bounds__(256) k_solve_init(DevBufs b, uint32_t C, const float* __restrict__ div) {
    __shared__ float s_tree[256];
    __shared__ float2 s_red[8];
    const DevParams& P = *b.prm;
    const uint32_t chunk = blockIdx.x;
    const uint32_t c = chunk * 256 + threadIdx.x;
    bool liquid = false;
    float prod = 0.0f;
    Df pdf = {0.0f, 0.0f};
    if (c < C) {
        liquid = b.ct[c] == CELL_LIQUID;
        if (liquid) {
            const float rhs = __fmul_rn(-P.scale_rhs, div[c]);
            float ap = 0.0f;
            if (P.warm) {
                const float p_initial = b.p[c];
                ap = apply_A(b.ct, b.p, c, P.nx, (size_t)P.nx * P.ny, p_initial);
            } else {
                b.p[c] = 0.0f;
            }
            const float rc = __fsub_rn(rhs, ap);
            b.r[c] = rc;
            b.dA[c] = rc;
            b.cinfo[c] = stencil_info(b.ct, c, P.nx, (size_t)P.nx * P.ny);
            prod = __fmul_rn(rc, rc);
            pdf = df_prod(rc, rc);
        } else {
            b.p[c] = 0.0f;
            b.r[c] = 0.0f;
            b.dA[c] = 0.0f;
            b.cinfo[c] = 0;
        }
    }
    const int nliq = __syncthreads_count(liquid);
    const float v = block_tree256(prod, s_tree);
    // float-float partial of this chunk (fixed order: warp shuffles, then warps in order)
    pdf = warp_sum_df(pdf);
    if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = make_float2(pdf.hi, pdf.lo);
    __syncthreads();
    if (threadIdx.x == 0) {
        Df a = {0.0f, 0.0f};
        for (int w = 0; w < 8; w++) a = df_add(a, Df{s_red[w].x, s_red[w].y});
        b.part_rr[chunk] = v;
        b.chunk_rr_df[chunk] = make_float2(a.hi, a.lo);
        b.chunk_flag[chunk] = (uint8_t)(nliq < 255 ? nliq : 255);
    }
}

cudaError_t launch_solve_init(const DevBufs& b, uint32_t C, const float* div, cudaStream_t s) {
    k_solve_init<<<(C + 255) / 256, 256, 0, s>>>(b, C, div);
    return cudaGetLastError();
}

cudaError_t launch_classify(const DevBufs& b, uint32_t C, cudaStream_t s) {
    k_classify<<<(C + 255) / 256, 256, 0, s>>>(b, C);
    return cudaGetLastError();
}

cudaError_t launch_p2g(const DevBufs& b, const LaunchCfg& L, uint32_t nx, uint32_t ny, uint32_t nz, cudaStream_t s,
                       bool clear) {
    const int tx = (int)((nx + TILE - 1) / TILE), ty = (int)((ny + TILE - 1) / TILE), tz = (int)((nz + TILE - 1) / TILE);
    // scatter.wgsl's accumulators start at zero (the reference's clear pass)
    for (int a = 0; clear && a < 3; a++) {
        const size_t faces = (size_t)(nx + (a == 0)) * (ny + (a == 1)) * (nz + (a == 2));
        cudaError_t e = cudaMemsetAsync(b.num[a], 0, 4 * faces, s);
        if (e == cudaSuccess) e = cudaMemsetAsync(b.den[a], 0, 4 * faces, s);
        if (e != cudaSuccess) return e;
    }
    k_p2g_own<<<tx * ty * tz, 256, 0, s>>>(b, tx, ty);
    k_p2g_strays<<<L.num_sms, 256, 0, s>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_grid_prep(const DevBufs& b, uint32_t C, cudaStream_t s) {
    k_grid_prep<<<(C + 255) / 256, 256, 0, s>>>(b, C);
    return cudaGetLastError();
}

cudaError_t launch_project(const DevBufs& b, uint32_t C, cudaStream_t s) {
    k_project<<<(C + 255) / 256, 256, 0, s>>>(b, C);
    return cudaGetLastError();
}

}  // namespace fl
