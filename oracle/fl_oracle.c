/*
 * fl_oracle.c — CPU oracle of fluid-lab's FLIP/PIC substep.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path (see fl_oracle.h).
 * Build: oracle/build_oracle.py (gcc -O2 -ffp-contract=off -fopenmp); the
 * no-contraction flag matters on aarch64, where GCC fuses a*b+c by default.
 *
 * Citations: S/ = app/crates/fluid-lab/src/, SH/ = S/gpu/shaders/ of the
 * reference project.
 */
#include "fl_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#define OMP_FOR _Pragma("omp parallel for schedule(static)")
#define OMP_FOR_REDUCE_SUM(v) _Pragma("omp parallel for schedule(static) reduction(+ : liquid)")
#else
#define OMP_FOR
#define OMP_FOR_REDUCE_SUM(v)
#endif

#define ATOMIC_INC_U32(ptr) __atomic_fetch_add((ptr), 1u, __ATOMIC_RELAXED)

/* f32 -> i32 with round-half-to-even (WGSL round(), SH/scatter.wgsl:71-72)
 * and saturation (NaN -> 0), the semantics of PTX cvt.rni.s32.f32. */
static inline int32_t f2i_rn_sat(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x <= -2147483648.0f) return INT32_MIN;
    return (int32_t)rintf(x);
}
static inline int64_t d2l_rn_sat(double x) {
    if (x != x) return 0;
    if (x >= 9223372036854775808.0) return INT64_MAX;
    if (x <= -9223372036854775808.0) return INT64_MIN;
    return (int64_t)rint(x);
}
/* u32(f32) of WGSL: truncate, saturate, NaN -> 0. */
static inline uint32_t f2u_sat(float x) {
    if (!(x > 0.0f)) return 0u;
    if (x >= 4294967296.0f) return UINT32_MAX;
    return (uint32_t)x;
}
/* i32 of an integral floating value (vec3<i32>(floor(g))), saturating. */
static inline int32_t r2i_floor_f(float x) {
    if (x != x) return 0;
    if (x >= 2147483648.0f) return INT32_MAX;
    if (x <= -2147483648.0f) return INT32_MIN;
    return (int32_t)x;
}
static inline int32_t r2i_floor_d(double x) {
    if (x != x) return 0;
    if (x >= 2147483648.0) return INT32_MAX;
    if (x <= -2147483648.0) return INT32_MIN;
    return (int32_t)x;
}

static int g_threads = 0;
void orc_set_threads(int n) {
    g_threads = n;
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#endif
}
int orc_get_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---------------- f32 instantiation: the reference's arithmetic ---------------- */
#define R float
#define SFX _f32
#define IS_F32 1
#define ACC uint32_t /* i32 atomics wrap; unsigned arithmetic wraps the same way */
#define TO_ACC(x) ((uint32_t)f2i_rn_sat(x))
#define ACC_TO_R(a) ((float)(int32_t)(a))
#define ACC_POSITIVE(a) ((int32_t)(a) > 0)
#define ATOMIC_ADD_ACC(ptr, v) __atomic_fetch_add((ptr), (v), __ATOMIC_RELAXED)
#define FLOOR floorf
#define FMIN fminf
#define FMAX fmaxf
#define SQRT sqrtf
#define r2i_floor r2i_floor_f
#include "fl_oracle_step.inc"
#undef R
#undef SFX
#undef IS_F32
#undef ACC
#undef TO_ACC
#undef ACC_TO_R
#undef ACC_POSITIVE
#undef FLOOR
#undef FMIN
#undef FMAX
#undef SQRT
#undef r2i_floor

/* ---------------- f64 instantiation: the same step in double ---------------- */
/* P2G accumulates in double: integral values (the fixed-point rounding of
 * scatter.wgsl, exact sums below 2^53) by default, or the unrounded terms when
 * exact P2G is on — the smooth forward used for finite differences. */
static int g_exact_p2g = 0;
void orc_set_exact_p2g(int on) { g_exact_p2g = on != 0; }
static inline double f64_acc_term(double x) { return g_exact_p2g ? x : (double)d2l_rn_sat(x); }
static inline void atomic_add_f64(double* p, double v) {
#ifdef _OPENMP
#pragma omp atomic
#endif
    *p += v;
}
#undef ATOMIC_ADD_ACC
#define ATOMIC_ADD_ACC(ptr, v) atomic_add_f64((ptr), (v))
#define R double
#define SFX _f64
#define IS_F32 0
#define ACC double
#define TO_ACC(x) f64_acc_term(x)
#define ACC_TO_R(a) (a)
#define ACC_POSITIVE(a) ((a) > 0.0)
#define FLOOR floor
#define FMIN fmin
#define FMAX fmax
#define SQRT sqrt
#define r2i_floor r2i_floor_d
#include "fl_oracle_step.inc"
#undef R
#undef SFX
#undef IS_F32
#undef ACC
#undef TO_ACC
#undef ACC_TO_R
#undef ACC_POSITIVE
#undef FLOOR
#undef FMIN
#undef FMAX
#undef SQRT
#undef r2i_floor

/* ========================================================================= */
/* Restatements of the reference's Rust CPU functions (for its own KATs).     */
/* Grid: GridDims with per-axis counts, uniform h, origin (S/sim/mod.rs:40-48) */

/* S/lib.rs:1163-1173 */
uint32_t orc_ref_cell_key(const float pos[3], const float origin[3], float h, const uint32_t dims[3]) {
    float g[3] = {(pos[0] - origin[0]) / h, (pos[1] - origin[1]) / h, (pos[2] - origin[2]) / h};
    uint32_t c[3];
    for (int a = 0; a < 3; a++) c[a] = (uint32_t)fminf(fmaxf(floorf(g[a]), 0.0f), (float)(dims[a] - 1));
    return c[0] + dims[0] * (c[1] + dims[1] * c[2]);
}

/* S/lib.rs:1176-1184 */
void orc_ref_exclusive_scan(const uint32_t* hist, uint32_t n, uint32_t* out) {
    uint32_t acc = 0;
    for (uint32_t c = 0; c < n; c++) {
        out[c] = acc;
        acc += hist[c];
    }
}

/* S/lib.rs:1188-1211 */
void orc_ref_counting_sort(const float* pos3, uint32_t n, const float origin[3], float h,
                           const uint32_t dims[3], uint32_t* perm_out, uint32_t* keys_out) {
    uint32_t cells = dims[0] * dims[1] * dims[2];
    uint32_t* hist = (uint32_t*)calloc(cells, 4);
    uint32_t* cursor = (uint32_t*)calloc(cells, 4);
    for (uint32_t p = 0; p < n; p++) {
        keys_out[p] = orc_ref_cell_key(pos3 + 3 * (size_t)p, origin, h, dims);
        hist[keys_out[p]]++;
    }
    orc_ref_exclusive_scan(hist, cells, cursor);
    for (uint32_t p = 0; p < n; p++) {
        uint32_t k = keys_out[p];
        uint32_t dst = cursor[k]++;
        perm_out[dst] = p;
    }
    free(hist);
    free(cursor);
}

/* S/sim/mod.rs:124-146 world_to_cell / clamp_idx */
static uint32_t clamp_idx(float f, uint32_t n) {
    if (f < 0.0f) return 0;
    uint32_t i = f2u_sat(f);
    return i >= n ? n - 1 : i;
}
uint32_t orc_ref_world_to_cell(uint32_t nx, uint32_t ny, uint32_t nz, float h, const float origin[3],
                               const float p[3], uint32_t ijk[3]) {
    float fi = floorf((p[0] - origin[0]) / h);
    float fj = floorf((p[1] - origin[1]) / h);
    float fk = floorf((p[2] - origin[2]) / h);
    ijk[0] = clamp_idx(fi, nx);
    ijk[1] = clamp_idx(fj, ny);
    ijk[2] = clamp_idx(fk, nz);
    return ijk[0] + nx * (ijk[1] + ny * ijk[2]);
}

/* S/sim/mod.rs:151-169 */
void orc_ref_classify_cells(uint32_t nx, uint32_t ny, uint32_t nz, const uint8_t* occupied,
                            uint8_t* out) {
    for (uint32_t k = 0; k < nz; k++)
        for (uint32_t j = 0; j < ny; j++)
            for (uint32_t i = 0; i < nx; i++) {
                uint32_t c = i + nx * (j + ny * k);
                int boundary = i == 0 || j == 0 || k == 0 || i == nx - 1 || j == ny - 1 || k == nz - 1;
                out[c] = boundary ? FL_CELL_SOLID : (occupied[c] ? FL_CELL_LIQUID : FL_CELL_AIR);
            }
}

static void face_dims(uint32_t nx, uint32_t ny, uint32_t nz, int axis, uint32_t d[3]) {
    d[0] = nx + (axis == 0);
    d[1] = ny + (axis == 1);
    d[2] = nz + (axis == 2);
}

/* S/sim/mod.rs:404-416 face_touches_static_solid */
static int ref_touches_static(uint32_t nx, uint32_t ny, uint32_t nz, int axis, uint32_t i, uint32_t j,
                              uint32_t k) {
    if (axis == 0) return i <= 1 || i >= nx - 1 || j == 0 || j >= ny - 1 || k == 0 || k >= nz - 1;
    if (axis == 1) return i == 0 || i >= nx - 1 || j <= 1 || j >= ny - 1 || k == 0 || k >= nz - 1;
    return i == 0 || i >= nx - 1 || j == 0 || j >= ny - 1 || k <= 1 || k >= nz - 1;
}

/* S/sim/mod.rs:418-433 */
void orc_ref_fill_wall_zeroed_faces(uint32_t nx, uint32_t ny, uint32_t nz, int axis, float value,
                                    float* out) {
    uint32_t d[3];
    face_dims(nx, ny, nz, axis, d);
    for (uint32_t k = 0; k < d[2]; k++)
        for (uint32_t j = 0; j < d[1]; j++)
            for (uint32_t i = 0; i < d[0]; i++) {
                uint32_t idx = i + d[0] * (j + d[1] * k);
                out[idx] = ref_touches_static(nx, ny, nz, axis, i, j, k) ? 0.0f : value;
            }
}

/* S/sim/mod.rs:435-500 sample_mac_pair (division form of the cell coordinate). */
void orc_ref_sample_mac_pair(uint32_t nx, uint32_t ny, uint32_t nz, float h, const float origin[3],
                             int axis, const float p[3], const float* final_vel,
                             const float* saved_vel, int wall_aware, float out[2]) {
    uint32_t d[3];
    face_dims(nx, ny, nz, axis, d);
    float off[3] = {-0.5f, -0.5f, -0.5f};
    off[axis] = 0.0f;
    float g[3];
    long base[3];
    float t[3];
    for (int a = 0; a < 3; a++) {
        g[a] = (p[a] - origin[a]) / h + off[a];
        base[a] = (long)floorf(g[a]);
        t[a] = g[a] - (float)base[a];
    }
    float fin = 0.0f, sav = 0.0f, wsum = 0.0f;
    for (int dk = 0; dk < 2; dk++) {
        long k = base[2] + dk;
        if (k < 0 || k >= (long)d[2]) continue;
        float wz = dk == 1 ? t[2] : 1.0f - t[2];
        for (int dj = 0; dj < 2; dj++) {
            long j = base[1] + dj;
            if (j < 0 || j >= (long)d[1]) continue;
            float wy = dj == 1 ? t[1] : 1.0f - t[1];
            for (int di = 0; di < 2; di++) {
                long i = base[0] + di;
                if (i < 0 || i >= (long)d[0]) continue;
                if (wall_aware && ref_touches_static(nx, ny, nz, axis, (uint32_t)i, (uint32_t)j, (uint32_t)k))
                    continue;
                float wx = di == 1 ? t[0] : 1.0f - t[0];
                float weight = wx * wy * wz;
                size_t idx = (size_t)i + d[0] * ((size_t)j + d[1] * (size_t)k);
                fin += weight * final_vel[idx];
                sav += weight * saved_vel[idx];
                wsum += weight;
            }
        }
    }
    if (wsum > 0.0f) {
        out[0] = fin / wsum;
        out[1] = sav / wsum;
    } else {
        out[0] = 0.0f;
        out[1] = 0.0f;
    }
}

/* S/sim/pressure.rs:43-66 */
void orc_ref_compute_divergence(uint32_t nx, uint32_t ny, uint32_t nz, float h, const float* u,
                                const float* v, const float* w, const uint8_t* ct, float* div) {
    for (uint32_t c = 0; c < nx * ny * nz; c++) div[c] = 0.0f;
    for (uint32_t k = 0; k < nz; k++)
        for (uint32_t j = 0; j < ny; j++)
            for (uint32_t i = 0; i < nx; i++) {
                uint32_t c = i + nx * (j + ny * k);
                if (ct[c] != FL_CELL_LIQUID) continue;
                float du = u[(i + 1) + (nx + 1) * (j + ny * k)] - u[i + (nx + 1) * (j + ny * k)];
                float dv = v[i + nx * ((j + 1) + (ny + 1) * k)] - v[i + nx * (j + (ny + 1) * k)];
                float dw = w[i + nx * (j + ny * (k + 1))] - w[i + nx * (j + ny * k)];
                div[c] = (du + dv + dw) / h;
            }
}

/* S/sim/pressure.rs:72-117 jacobi_iteration */
static void ref_jacobi_iteration(uint32_t nx, uint32_t ny, uint32_t nz, const uint8_t* ct,
                                 const float* div, float scale, const float* p_in, float* p_out) {
    for (uint32_t k = 0; k < nz; k++)
        for (uint32_t j = 0; j < ny; j++)
            for (uint32_t i = 0; i < nx; i++) {
                uint32_t c = i + nx * (j + ny * k);
                if (ct[c] != FL_CELL_LIQUID) { p_out[c] = 0.0f; continue; }
                uint32_t nb[6] = {c - 1, c + 1, c - nx, c + nx, c - nx * ny, c + nx * ny};
                float sum = 0.0f, n = 0.0f;
                for (int s = 0; s < 6; s++) {
                    if (ct[nb[s]] == FL_CELL_SOLID) continue;
                    if (ct[nb[s]] == FL_CELL_AIR) n += 1.0f;
                    else { sum += p_in[nb[s]]; n += 1.0f; }
                }
                p_out[c] = n > 0.0f ? (sum - scale * div[c]) / n : 0.0f;
            }
}

/* SH/pressure.wgsl:26-61: red-black Gauss-Seidel, in place, from zero;
 * `iters` times the red phase ((i+j+k)&1 == 0) then the black phase.  The
 * per-cell update is jacobi_iteration's formula with the neighbours read from
 * the same buffer; non-liquid cells stay 0. */
void orc_ref_rbgs_solve(uint32_t nx, uint32_t ny, uint32_t nz, float h, float rho, float dt,
                        const uint8_t* ct, const float* div, uint32_t iters, float* p_out) {
    uint32_t C = nx * ny * nz;
    float scale = rho * h * h / dt;
    memset(p_out, 0, 4 * (size_t)C);
    for (uint32_t it = 0; it < iters; it++)
        for (uint32_t phase = 0; phase < 2; phase++)
            for (uint32_t k = 0; k < nz; k++)
                for (uint32_t j = 0; j < ny; j++)
                    for (uint32_t i = 0; i < nx; i++) {
                        uint32_t c = i + nx * (j + ny * k);
                        if (ct[c] != FL_CELL_LIQUID || ((i + j + k) & 1u) != phase) continue;
                        uint32_t nb[6] = {c - 1, c + 1, c - nx, c + nx, c - nx * ny, c + nx * ny};
                        float sum = 0.0f, cnt = 0.0f;
                        for (int s = 0; s < 6; s++) {
                            if (ct[nb[s]] == FL_CELL_SOLID) continue;
                            cnt += 1.0f;
                            if (ct[nb[s]] == FL_CELL_LIQUID) sum += p_out[nb[s]];
                        }
                        p_out[c] = cnt > 0.0f ? (sum - scale * div[c]) / cnt : 0.0f;
                    }
}

/* S/sim/pressure.rs:120-136 jacobi_solve; ProjectionParams::rhs_scale :31-33 */
void orc_ref_jacobi_solve(uint32_t nx, uint32_t ny, uint32_t nz, float h, float rho, float dt,
                          const uint8_t* ct, const float* div, uint32_t iters, float* p_out) {
    uint32_t C = nx * ny * nz;
    float scale = rho * h * h / dt;
    float* a = (float*)calloc(C, 4);
    float* b = (float*)calloc(C, 4);
    for (uint32_t it = 0; it < iters; it++) {
        ref_jacobi_iteration(nx, ny, nz, ct, div, scale, a, b);
        float* t = a; a = b; b = t;
    }
    memcpy(p_out, a, 4 * (size_t)C);
    free(a);
    free(b);
}

/* S/sim/pressure.rs:145-179 */
void orc_ref_apply_poisson(uint32_t nx, uint32_t ny, uint32_t nz, const uint8_t* ct, const float* x,
                           float* out) {
    for (uint32_t k = 0; k < nz; k++)
        for (uint32_t j = 0; j < ny; j++)
            for (uint32_t i = 0; i < nx; i++) {
                uint32_t c = i + nx * (j + ny * k);
                out[c] = 0.0f;
                if (ct[c] != FL_CELL_LIQUID) continue;
                uint32_t nb[6] = {c - 1, c + 1, c - nx, c + nx, c - nx * ny, c + nx * ny};
                float n = 0.0f, sum = 0.0f;
                for (int s = 0; s < 6; s++) {
                    if (ct[nb[s]] == FL_CELL_SOLID) continue;
                    if (ct[nb[s]] == FL_CELL_AIR) n += 1.0f;
                    else { n += 1.0f; sum += x[nb[s]]; }
                }
                out[c] = n * x[c] - sum;
            }
}

/* S/sim/pressure.rs:182-188 */
static double ref_dot(const float* a, const float* b, uint32_t n) {
    double acc = 0.0;
    for (uint32_t c = 0; c < n; c++) acc += (double)a[c] * (double)b[c];
    return acc;
}

/* S/sim/pressure.rs:235-309 cg_solve_with_options (pressure_rhs :202-218,
 * residual_from_pressure :220-233). */
uint32_t orc_ref_cg_solve(uint32_t nx, uint32_t ny, uint32_t nz, float h, float rho, float dt,
                          const uint8_t* ct, const float* div, uint32_t iters, const float* p_init,
                          float tol, float* p_out, double* rs_initial_out, double* rs_final_out) {
    uint32_t n = nx * ny * nz;
    float scale = rho * h * h / dt;
    float* b = (float*)calloc(n, 4);
    float* p = (float*)calloc(n, 4);
    float* r = (float*)calloc(n, 4);
    float* d = (float*)calloc(n, 4);
    float* q = (float*)calloc(n, 4);
    for (uint32_t c = 0; c < n; c++)
        if (ct[c] == FL_CELL_LIQUID) b[c] = -scale * div[c];
    if (p_init)
        for (uint32_t c = 0; c < n; c++)
            if (ct[c] == FL_CELL_LIQUID) p[c] = p_init[c];
    if (p_init) {
        orc_ref_apply_poisson(nx, ny, nz, ct, p, q);
        for (uint32_t c = 0; c < n; c++) r[c] = b[c] - q[c];
    } else {
        memcpy(r, b, 4 * (size_t)n);
    }
    memcpy(d, r, 4 * (size_t)n);
    double rs_old = ref_dot(r, r, n);
    double rs_initial = rs_old;
    int has_target = tol >= 0.0f && isfinite(tol);
    double target = has_target ? (double)tol * (double)tol * rs_initial : 0.0;
    uint32_t iterations = 0;
    for (uint32_t it = 0; it < iters; it++) {
        if (rs_old <= 0.0) break;
        orc_ref_apply_poisson(nx, ny, nz, ct, d, q);
        double dq = ref_dot(d, q, n);
        if (fabs(dq) < 1e-30) break;
        float alpha = (float)(rs_old / dq);
        for (uint32_t c = 0; c < n; c++) {
            p[c] += alpha * d[c];
            r[c] -= alpha * q[c];
        }
        double rs_new = ref_dot(r, r, n);
        iterations++;
        if (has_target && rs_new <= target) {
            rs_old = rs_new;
            break;
        }
        float beta = (float)(rs_new / rs_old);
        for (uint32_t c = 0; c < n; c++) d[c] = r[c] + beta * d[c];
        rs_old = rs_new;
    }
    memcpy(p_out, p, 4 * (size_t)n);
    if (rs_initial_out) *rs_initial_out = rs_initial;
    if (rs_final_out) *rs_final_out = rs_old;
    free(b); free(p); free(r); free(d); free(q);
    return iterations;
}

/* S/sim/pressure.rs:337-426 subtract_gradient / apply_face; grad_coeff :36-38 */
static void ref_apply_face(float coeff, const float* p, const uint8_t* ct, long lo, long hi, float* vel) {
    int lo_solid = lo < 0 ? 1 : ct[lo] == FL_CELL_SOLID;
    int hi_solid = hi < 0 ? 1 : ct[hi] == FL_CELL_SOLID;
    if (lo_solid || hi_solid) { *vel = 0.0f; return; }
    float p_hi = p[hi], p_lo = p[lo];
    *vel -= coeff * (p_hi - p_lo);
}
void orc_ref_subtract_gradient(uint32_t nx, uint32_t ny, uint32_t nz, float h, float rho, float dt,
                               const float* p, const uint8_t* ct, float* u, float* v, float* w) {
    float coeff = (dt / rho) / h;
    for (uint32_t k = 0; k < nz; k++)
        for (uint32_t j = 0; j < ny; j++)
            for (uint32_t i = 0; i <= nx; i++) {
                long lo = i == 0 ? -1 : (long)((i - 1) + nx * (j + ny * k));
                long hi = i == nx ? -1 : (long)(i + nx * (j + ny * k));
                ref_apply_face(coeff, p, ct, lo, hi, &u[i + (nx + 1) * (j + ny * k)]);
            }
    for (uint32_t k = 0; k < nz; k++)
        for (uint32_t j = 0; j <= ny; j++)
            for (uint32_t i = 0; i < nx; i++) {
                long lo = j == 0 ? -1 : (long)(i + nx * ((j - 1) + ny * k));
                long hi = j == ny ? -1 : (long)(i + nx * (j + ny * k));
                ref_apply_face(coeff, p, ct, lo, hi, &v[i + nx * (j + (ny + 1) * k)]);
            }
    for (uint32_t k = 0; k <= nz; k++)
        for (uint32_t j = 0; j < ny; j++)
            for (uint32_t i = 0; i < nx; i++) {
                long lo = k == 0 ? -1 : (long)(i + nx * (j + ny * (k - 1)));
                long hi = k == nz ? -1 : (long)(i + nx * (j + ny * k));
                ref_apply_face(coeff, p, ct, lo, hi, &w[i + nx * (j + ny * k)]);
            }
}

/* S/sim/pressure.rs:431-450 */
float orc_ref_l2_divergence(uint32_t n_cells, const float* div, const uint8_t* ct) {
    double acc = 0.0;
    for (uint32_t c = 0; c < n_cells; c++)
        if (ct[c] == FL_CELL_LIQUID) acc += (double)div[c] * (double)div[c];
    return (float)sqrt(acc);
}
float orc_ref_max_abs_divergence(uint32_t n_cells, const float* div, const uint8_t* ct) {
    float m = 0.0f;
    for (uint32_t c = 0; c < n_cells; c++)
        if (ct[c] == FL_CELL_LIQUID) m = fmaxf(m, fabsf(div[c]));
    return m;
}

/* ---- slice.wgsl:41-141: WGSL mix(e1, e2, e3) = e1*(1-e3) + e2*e3, clamp =
 * min(max(e, lo), hi), length = sqrt(x*x + y*y + z*z); all in f32. */
static float slice_mix(float a, float b, float s) { return a * (1.0f - s) + b * s; }
static float slice_clamp01(float t) { return fminf(fmaxf(t, 0.0f), 1.0f); }
static void slice_mix3(const float a[3], const float b[3], float s, float out[3]) {
    for (int c = 0; c < 3; c++) out[c] = slice_mix(a[c], b[c], s);
}
static void slice_diverging(float t, float out[3]) {
    static const float blue[3] = {0.0f, 0.2f, 0.9f}, white[3] = {1.0f, 1.0f, 1.0f}, red[3] = {0.9f, 0.05f, 0.05f};
    const float tc = slice_clamp01(t);
    if (tc < 0.5f) slice_mix3(blue, white, tc * 2.0f, out);
    else slice_mix3(white, red, (tc - 0.5f) * 2.0f, out);
}
static void slice_speed(float t, float out[3]) {
    static const float c0[3] = {0.0f, 0.0f, 0.8f}, c1[3] = {0.0f, 0.9f, 0.9f}, c2[3] = {1.0f, 1.0f, 0.0f},
                       c3[3] = {0.9f, 0.0f, 0.0f};
    const float tc = slice_clamp01(t);
    if (tc < 0.333f) slice_mix3(c0, c1, tc / 0.333f, out);
    else if (tc < 0.667f) slice_mix3(c1, c2, (tc - 0.333f) / 0.333f, out);
    else slice_mix3(c2, c3, (tc - 0.667f) / 0.333f, out);
}

void orc_grid_slice(uint32_t nx, uint32_t ny, uint32_t nz, const uint8_t* ct, const float* p, const float* u,
                    const float* v, const float* w, uint32_t mode, uint32_t k, float* rgba_out) {
    (void)nz;
    for (uint32_t j = 0; j < ny; j++)
        for (uint32_t i = 0; i < nx; i++) {
            const size_t idx = (size_t)i + nx * ((size_t)j + (size_t)ny * k);
            const uint8_t t = ct[idx];
            float c[3] = {0.0f, 0.0f, 0.0f};
            int visible;
            if (mode == 0u) {
                visible = t != FL_CELL_AIR;
                if (t == FL_CELL_SOLID) { c[0] = 0.40f; c[1] = 0.40f; c[2] = 0.46f; }
                else { c[0] = 0.20f; c[1] = 0.55f; c[2] = 1.00f; }
            } else if (mode == 1u) {
                visible = t == FL_CELL_LIQUID;
                if (visible) slice_diverging(slice_clamp01(p[idx] / 2000.0f * 0.5f + 0.5f), c);
            } else {
                visible = t == FL_CELL_LIQUID;
                if (visible) {
                    const float u0 = u[i + (size_t)(nx + 1) * (j + (size_t)ny * k)];
                    const float u1 = u[(i + 1) + (size_t)(nx + 1) * (j + (size_t)ny * k)];
                    const float v0 = v[i + (size_t)nx * (j + (size_t)(ny + 1) * k)];
                    const float v1 = v[i + (size_t)nx * ((j + 1) + (size_t)(ny + 1) * k)];
                    const float w0 = w[i + (size_t)nx * (j + (size_t)ny * k)];
                    const float w1 = w[i + (size_t)nx * (j + (size_t)ny * (k + 1))];
                    const float au = (u0 + u1) * 0.5f, av = (v0 + v1) * 0.5f, aw = (w0 + w1) * 0.5f;
                    const float spd = sqrtf(au * au + av * av + aw * aw);
                    slice_speed(slice_clamp01(spd / 4.0f), c);
                }
            }
            float* o = rgba_out + 4 * ((size_t)i + (size_t)nx * j);
            o[0] = c[0]; o[1] = c[1]; o[2] = c[2]; o[3] = visible ? 1.0f : 0.0f;
        }
}

/* ---- gpu/fluid.rs:1838-1913 generate_particles, sequential (f32) ---- */
static float rust_clampf(float x, float lo, float hi) {
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}
static int32_t rust_f32_to_i32(float q) {
    if (q != q) return 0;
    if (q >= 2147483647.0f) return 2147483647;
    if (q <= -2147483648.0f) return INT32_MIN;
    return (int32_t)q;
}

uint32_t orc_ref_generate_particles(const float origin[3], float h, const uint32_t gdim[3], const float* blocks,
                                    uint32_t nblocks, uint32_t particle_count, float* out, uint32_t capacity) {
    float extent[3], lo[3], hi[3];
    for (int a = 0; a < 3; a++) {
        extent[a] = (float)gdim[a] * h;
        lo[a] = origin[a] + h * 1.05f;
        hi[a] = origin[a] + extent[a] - h * 1.05f;
    }
    float total_vol = 0.0f;
    for (uint32_t b = 0; b < nblocks; b++) {
        float e[3];
        for (int a = 0; a < 3; a++) {
            const float wmin = origin[a] + blocks[6 * b + a] * extent[a];
            const float wmax = origin[a] + blocks[6 * b + 3 + a] * extent[a];
            e[a] = wmax - wmin;
        }
        total_vol += fmaxf(e[0] * e[1] * e[2], 1e-6f);
    }
    total_vol = fmaxf(total_vol, 1e-6f);
    const float total_target = (float)(particle_count > 1u ? particle_count : 1u);
    uint32_t st = 0x12345678u;
    uint32_t n = 0;
    for (uint32_t b = 0; b < nblocks; b++) {
        float wmin[3], e[3];
        for (int a = 0; a < 3; a++) {
            wmin[a] = origin[a] + blocks[6 * b + a] * extent[a];
            const float wmax = origin[a] + blocks[6 * b + 3 + a] * extent[a];
            e[a] = wmax - wmin[a];
        }
        const float vol = fmaxf(e[0] * e[1] * e[2], 1e-6f);
        const float target = fmaxf(total_target * (vol / total_vol), 1.0f);
        const float spacing = fmaxf(cbrtf(vol / target), 1e-4f);
        int32_t cnt[3];
        for (int a = 0; a < 3; a++) {
            const int32_t c = rust_f32_to_i32(floorf(e[a] / spacing));
            cnt[a] = c > 1 ? c : 1;
        }
        for (int32_t ix = 0; ix < cnt[0]; ix++)
            for (int32_t iy = 0; iy < cnt[1]; iy++)
                for (int32_t iz = 0; iz < cnt[2]; iz++) {
                    const int32_t idx[3] = {ix, iy, iz};
                    float pos[3];
                    for (int a = 0; a < 3; a++) {
                        st = st * 1664525u + 1013904223u;
                        const float r = (float)(st >> 8) / 16777216.0f;
                        const float j = (r - 0.5f) * spacing * 0.5f;
                        pos[a] = rust_clampf(wmin[a] + ((float)idx[a] + 0.5f) * spacing + j, lo[a], hi[a]);
                    }
                    if (n < capacity) {
                        float* o = out + 8 * (size_t)n;
                        o[0] = pos[0]; o[1] = pos[1]; o[2] = pos[2];
                        o[3] = o[4] = o[5] = o[6] = o[7] = 0.0f;
                    }
                    n++;
                }
    }
    return n;
}

