/*
 * fl_oracle.h — CPU oracle of fluid-lab's per-substep FLIP/PIC step.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the checker the CUDA path is compared
 * against: it may be linked or called only by tests/, __graft_entry__.smoke()
 * and bench.py's CPU baseline.  The product library (libfluidgb) never uses it.
 *
 * Two builds of one source: `_f32` restates the reference's WGSL arithmetic
 * (f32, non-contracted, source order; fixed-point i32 P2G; f32 CG dots in the
 * 256-wide two-level tree of cg_reduce.wgsl / cg_reduce_final.wgsl), and `_f64`
 * is the same step carried out in double precision (the FP64 oracle).
 * The `orc_ref_*` functions restate the reference's Rust CPU "spec-as-code"
 * (app/crates/fluid-lab/src/sim/mod.rs, sim/pressure.rs, lib.rs sort mirror) so
 * that the oracle can be pinned to the reference's own known-answer tests.
 */
#ifndef FL_ORACLE_H
#define FL_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#include "../include/fluidgb.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_handle_f32 orc_handle_f32;
typedef struct orc_handle_f64 orc_handle_f64;

/* ---- step oracle (mirrors the fl_* ABI) ---- */
#define ORC_DECL(SFX)                                                                            \
    orc_handle##SFX* orc_create##SFX(const fl_params* p, uint32_t capacity);                     \
    void orc_destroy##SFX(orc_handle##SFX* h);                                                   \
    int orc_set_params##SFX(orc_handle##SFX* h, const fl_params* p);                             \
    int orc_set_particles##SFX(orc_handle##SFX* h, const float* aos32, uint32_t n);              \
    int orc_get_particles##SFX(orc_handle##SFX* h, float* out, uint32_t* ids);                   \
    int orc_step##SFX(orc_handle##SFX* h, uint32_t substeps);                                    \
    int orc_apply_impulse##SFX(orc_handle##SFX* h, const float dv[3]);                           \
    int orc_reset##SFX(orc_handle##SFX* h);                                                      \
    int orc_get_grid##SFX(orc_handle##SFX* h, const fl_grid_view* v);                            \
    int orc_get_bins##SFX(orc_handle##SFX* h, uint32_t* counts, uint32_t* offsets,               \
                          uint32_t* perm);                                                       \
    int orc_get_stats##SFX(orc_handle##SFX* h, fl_stats* s);                                     \
    int orc_get_divergence##SFX(orc_handle##SFX* h, float* out);                                 \
    int orc_set_gravity_d##SFX(orc_handle##SFX* h, const double g[3]);                           \
    int orc_add_velocity_d##SFX(orc_handle##SFX* h, const double* dv, double eps);               \
    int orc_mean_position_d##SFX(orc_handle##SFX* h, double out[3]);                             \
    int orc_add_position_d##SFX(orc_handle##SFX* h, const double* dx, double eps);               \
    int orc_set_pressure##SFX(orc_handle##SFX* h, const float* p);                               \
    int orc_solve_pressure##SFX(uint32_t nx, uint32_t ny, uint32_t nz, const uint8_t* ct,        \
                                const float* div, const float* p_in, float* p_out, float h,      \
                                float rho, float dt, uint32_t max_iters, uint32_t warm,          \
                                float tol, uint32_t precision, fl_stats* st);

ORC_DECL(_f32)
ORC_DECL(_f64)

/* _f64 only: 1 = accumulate P2G terms unrounded (a smooth forward for finite
 * differences), 0 = the reference's 2^16 fixed-point rounding (default). */
void orc_set_exact_p2g(int on);

/* Number of OpenMP threads the oracle uses (0 = library default). */
void orc_set_threads(int n);
int orc_get_threads(void);

/* ---- restatements of the reference's Rust CPU functions (for its KATs) ---- */

/* lib.rs:1163-1173 cell_key (also mark.wgsl:39-43). */
uint32_t orc_ref_cell_key(const float pos[3], const float origin[3], float h, const uint32_t dims[3]);
/* lib.rs:1176-1184 exclusive_scan. */
void orc_ref_exclusive_scan(const uint32_t* hist, uint32_t n, uint32_t* out);
/* lib.rs:1188-1211 counting_sort (stable).  pos: 3 floats each. */
void orc_ref_counting_sort(const float* pos3, uint32_t n, const float origin[3], float h,
                           const uint32_t dims[3], uint32_t* perm_out, uint32_t* keys_out);
/* sim/mod.rs:124-132 world_to_cell; returns cell index, writes ijk. */
uint32_t orc_ref_world_to_cell(uint32_t nx, uint32_t ny, uint32_t nz, float h, const float origin[3],
                               const float p[3], uint32_t ijk[3]);
/* sim/mod.rs:151-169 classify_cells (occupied: one byte per cell, 0/1). */
void orc_ref_classify_cells(uint32_t nx, uint32_t ny, uint32_t nz, const uint8_t* occupied,
                            uint8_t* out);
/* sim/mod.rs:462-525 sample_mac_pair (test helper, wall-aware gather). axis 0..2. */
void orc_ref_sample_mac_pair(uint32_t nx, uint32_t ny, uint32_t nz, float h, const float origin[3],
                             int axis, const float p[3], const float* final_vel,
                             const float* saved_vel, int wall_aware, float out[2]);
/* sim/mod.rs:426-441 fill_wall_zeroed_faces. */
void orc_ref_fill_wall_zeroed_faces(uint32_t nx, uint32_t ny, uint32_t nz, int axis, float value,
                                    float* out);
/* sim/pressure.rs:43-66 compute_divergence (no drift term). */
void orc_ref_compute_divergence(uint32_t nx, uint32_t ny, uint32_t nz, float h, const float* u,
                                const float* v, const float* w, const uint8_t* ct, float* div);
/* pressure.wgsl:26-61 red-black Gauss-Seidel from zero, `iters` red+black phases. */
void orc_ref_rbgs_solve(uint32_t nx, uint32_t ny, uint32_t nz, float h, float rho, float dt,
                        const uint8_t* ct, const float* div, uint32_t iters, float* p_out);
/* sim/pressure.rs:72-136 jacobi_solve. */
void orc_ref_jacobi_solve(uint32_t nx, uint32_t ny, uint32_t nz, float h, float rho, float dt,
                          const uint8_t* ct, const float* div, uint32_t iters, float* p_out);
/* sim/pressure.rs:145-179 apply_poisson. */
void orc_ref_apply_poisson(uint32_t nx, uint32_t ny, uint32_t nz, const uint8_t* ct, const float* x,
                           float* out);
/* sim/pressure.rs:235-309 cg_solve_with_options.  p_init may be NULL (cold);
 * tol < 0 = no tolerance.  Returns iterations; writes residuals if non-NULL. */
uint32_t orc_ref_cg_solve(uint32_t nx, uint32_t ny, uint32_t nz, float h, float rho, float dt,
                          const uint8_t* ct, const float* div, uint32_t iters, const float* p_init,
                          float tol, float* p_out, double* rs_initial, double* rs_final);
/* sim/pressure.rs:337-426 subtract_gradient. */
void orc_ref_subtract_gradient(uint32_t nx, uint32_t ny, uint32_t nz, float h, float rho, float dt,
                               const float* p, const uint8_t* ct, float* u, float* v, float* w);
/* sim/pressure.rs:431-450 diagnostics. */
float orc_ref_l2_divergence(uint32_t n_cells, const float* div, const uint8_t* ct);
float orc_ref_max_abs_divergence(uint32_t n_cells, const float* div, const uint8_t* ct);

/* generate_particles (gpu/fluid.rs:1838-1913) as the reference runs it: one
 * sequential loop over blocks and lattice points drawing from a single seeded
 * LCG.  blocks: 6 floats each (min xyz, max xyz, normalized).  Writes up to
 * `capacity` particles (8 floats each, zero velocity); returns the layout's
 * particle count. */
uint32_t orc_ref_generate_particles(const float origin[3], float h, const uint32_t gdim[3], const float* blocks,
                                    uint32_t nblocks, uint32_t particle_count, float* out, uint32_t capacity);

/* The per-cell arithmetic of the slice debug renderer (shaders/slice.wgsl:69-141)
 * for the XY slice at k: rgba_out[4*(i + nx*j) + c] = {r, g, b, visible}. */
void orc_grid_slice(uint32_t nx, uint32_t ny, uint32_t nz, const uint8_t* ct, const float* p, const float* u,
                    const float* v, const float* w, uint32_t mode, uint32_t k, float* rgba_out);

#ifdef __cplusplus
}
#endif
#endif
