/*
 * fluidgb.h — C ABI of the GB300-native (sm_103a) FLIP/PIC substep.
 *
 * The library replaces the per-substep compute passes of fluid-lab's
 * `GpuFluid` (app/crates/fluid-lab/src/gpu/fluid.rs) behind plain C types:
 * particle buffers in, particle buffers out, and the same 128-byte `Params`
 * settings block.  All functions return an `fl_status`; none aborts and no
 * kernel traps.  A handle is not thread-safe; different handles may be used
 * from different threads.  Work is enqueued on the handle's CUDA stream and is
 * asynchronous until `fl_sync` or a call that copies to host memory.
 *
 * Reference interfaces replaced (file:line within the reference project):
 *   GpuFluid::new / GpuContext::recreate_fluid  app/crates/fluid-lab/src/gpu/fluid.rs:247-318,
 *                                               app/crates/fluid-lab/src/gpu/mod.rs:500-625
 *   GpuContext::step(substeps)                  app/crates/fluid-lab/src/gpu/mod.rs:950-989
 *   record_prep_pre_sort / record_sort /
 *   record_prep_post_sort / record_pressure /
 *   record_finish                               app/crates/fluid-lab/src/gpu/fluid.rs:1436-1715
 *   live setters (set_flip_blend ...)           app/crates/fluid-lab/src/gpu/fluid.rs:1294-1371
 *   apply_impulse                               app/crates/fluid-lab/src/gpu/fluid.rs:1374-1395
 *   reset                                       app/crates/fluid-lab/src/gpu/fluid.rs:1408-1418
 *   particle_buffer()                           app/crates/fluid-lab/src/gpu/fluid.rs:1208-1214
 */
#ifndef FLUIDGB_H
#define FLUIDGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FL_ABI_VERSION 1u

typedef enum fl_status {
    FL_OK = 0,
    FL_INVALID_ARG = 1,   /* bad pointer, size, or parameter; nothing was enqueued */
    FL_OOM = 2,           /* device or host allocation failed */
    FL_CUDA_ERROR = 3,    /* a CUDA runtime call failed; see fl_last_error */
    FL_NOT_CONVERGED = 4, /* reserved: CG stopped at the iteration cap (informational) */
    FL_TIMEOUT = 5,       /* a bounded device-side wait expired; the context stays usable */
    FL_NO_DEVICE = 6,     /* no CUDA device, or it is not an sm_103 part */
    FL_INTERNAL = 7
} fl_status;

/* Cell classification, same numbering as the reference's `CellType`
 * (app/crates/fluid-lab/src/sim/mod.rs:30-36). */
enum { FL_CELL_SOLID = 0, FL_CELL_LIQUID = 1, FL_CELL_AIR = 2 };

/* CG inner-product precision (extension field `cg_precision`).  The FP32
 * vector arithmetic (directions, SpMV, updates) is the same in all three. */
enum {
    FL_CG_F32 = 0,      /* reference arithmetic: f32 two-level 256-wide tree dots (cg_reduce.wgsl) */
    FL_CG_F64 = 1,      /* extended-precision inner products, residual norm and convergence
                           test in float-float (~48-bit significand) on the FP32 pipe */
    FL_CG_F64_IEEE = 2  /* inner products, residual norm, alpha/beta quotients and convergence
                           test in IEEE double: exact f32 x f32 products, double sums, trees and
                           combines (the CPU reference CG's f64 dot, sim/pressure.rs:182-188);
                           the initial residual's per-chunk partials are float-float */
};

/*
 * fl_params — the reference's 128-byte `Params` uniform
 * (app/crates/fluid-lab/src/gpu/fluid.rs:25-39, filled at :289-318), field for
 * field, followed by a 32-byte extension block.  A caller holding the
 * reference's `Params` bytes can copy them into the first 128 bytes.
 */
typedef struct fl_params {
    uint32_t dims[4];   /* nx (legacy, ignored), particle_count (ignored: set by
                           fl_set_particles), pressure_iters (0 -> 1), warm_start */
    float geom[4];      /* h, inv_h, dt, fixed_scale (2^16) */
    float phys[4];      /* gravity_y (legacy, ignored), rho, flip_blend, wall_friction */
    float origin[4];    /* world position of cell (0,0,0)'s min corner; w ignored */
    float grav[4];      /* gx, gy, gz, _ */
    float spc[4];       /* rest_per_cell, volume_stiffness, drift_clamp, _ */
    float cls[4];       /* liquid_threshold, surface_dilation, cfl, _ */
    uint32_t gdim[4];   /* nx, ny, nz, 0 */
    /* ---- extension block (not part of the reference's Params) ---- */
    float pressure_tolerance; /* relative residual tolerance; 0 = off; clamped to
                                 [0, 0.1] like set_pressure_residual_tolerance
                                 (fluid.rs:47-50, :1362-1369) */
    uint32_t cg_precision;    /* FL_CG_F32, FL_CG_F64 or FL_CG_F64_IEEE */
    uint32_t advect_order;    /* 1 = forward Euler (reference g2p.wgsl:186); 2 = midpoint */
    uint32_t sort_period;     /* accepted for drop-in compatibility; the layout is
                                 re-sorted every substep (the gather-form P2G reads bins) */
    uint32_t pressure_solver; /* FL_SOLVER_CG (the reference's CG) or FL_SOLVER_MGPCG */
    uint32_t reserved[3];     /* must be zero */
} fl_params;

/* Pressure solvers.  FL_SOLVER_CG is the reference's CG (cg_*.wgsl).
 * FL_SOLVER_MGPCG preconditions the same CG with a multigrid V-cycle whose
 * smoother is the reference's red-black Gauss-Seidel sweep (pressure.wgsl):
 * same operator, warm start, iteration cap and stopping test, far fewer
 * iterations; the pressure agrees with the CG's to the tolerance, not bit for
 * bit.  Reductions are float-float in both precisions. */
#define FL_SOLVER_CG 0u
#define FL_SOLVER_MGPCG 1u

typedef struct fl_handle fl_handle;

/* Statistics of the most recent substep. */
typedef struct fl_stats {
    uint32_t liquid_cells;    /* stats[0] of classify.wgsl */
    uint32_t cg_iterations;   /* iterations that ran with `active` set */
    uint32_t stray_particles; /* particles whose P2G base differs from their bin (ulp ties) */
    uint32_t device_status;   /* 0, or the fl_status a kernel recorded */
    uint64_t substeps;        /* substeps run since fl_create / fl_reset */
    double rs_initial;        /* r.r after CG init */
    double rs_final;          /* r.r at exit */
} fl_stats;

/* Host destinations for fl_get_grid; any NULL member is skipped. */
typedef struct fl_grid_view {
    float* u;        /* (nx+1)*ny*nz, final (post-projection) face velocity */
    float* v;        /* nx*(ny+1)*nz */
    float* w;        /* nx*ny*(nz+1) */
    float* u_saved;  /* post-P2G, pre-force snapshot used by the FLIP delta */
    float* v_saved;
    float* w_saved;
    float* pressure; /* nx*ny*nz */
    uint8_t* cell_type; /* nx*ny*nz, FL_CELL_* */
    uint32_t* counts;   /* nx*ny*nz particle histogram (occupancy) */
    uint32_t* offsets;  /* nx*ny*nz exclusive prefix sum of counts */
} fl_grid_view;

/* Version of this ABI (FL_ABI_VERSION of the library that was loaded). */
uint32_t fl_abi_version(void);
const char* fl_status_string(fl_status s);

/* Fill `out` with the reference registry defaults (settings/mod.rs:498-724) for a
 * tank of nx*ny*nz cells of size h whose min corner is `origin` (NULL = centred
 * like fluid.rs:262-269).  Replaces the Params construction at fluid.rs:289-318. */
fl_status fl_params_default(fl_params* out, uint32_t nx, uint32_t ny, uint32_t nz, float h,
                            const float* origin);

/* Allocate device state for a grid and at most `capacity` particles.
 * Replaces GpuFluid::new (fluid.rs:247-1197). */
fl_status fl_create(const fl_params* params, uint32_t capacity, fl_handle** out);
fl_status fl_destroy(fl_handle* h);

/* Live parameter update (fluid.rs:1294-1371).  Grid dimensions cannot change:
 * INVALID_ARG (create a new handle instead, like GpuContext::recreate_fluid). */
fl_status fl_set_params(fl_handle* h, const fl_params* params);
fl_status fl_get_params(const fl_handle* h, fl_params* out);

/* Upload n particles as 8 floats each {pos.xyz, _, vel.xyz, _} (fluid.rs:116-123);
 * they also become the state fl_reset restores.  Particle ids are 0..n-1. */
fl_status fl_set_particles(fl_handle* h, const float* pos_vel_aos32, uint32_t n);
/* Download the current particles (8 floats each) and, if ids_out != NULL, the
 * id of the particle in each slot. */
fl_status fl_get_particles(fl_handle* h, float* pos_vel_aos32_out, uint32_t* ids_out);
fl_status fl_particle_count(const fl_handle* h, uint32_t* n_out);

/* Run `substeps` fixed-dt substeps on the handle's particles (GpuContext::step). */
fl_status fl_step(fl_handle* h, uint32_t substeps);
/* One substep on a caller-owned device buffer of n particles (8 floats each,
 * 16-byte aligned).  The buffer is read, and on return holds the advanced
 * particles in this substep's bin order.  n <= capacity. */
fl_status fl_step_device(fl_handle* h, void* particles_dev, uint32_t n);

/* Host-memory variant: copy n particles from `in` (pinned memory overlaps best)
 * into the handle, run `substeps`, copy the result to `out` (may equal `in`),
 * and wait.  The handle keeps the advanced particles and its warm-start
 * pressure; particle ids are not maintained by this call.  n <= capacity. */
fl_status fl_step_host(fl_handle* h, const float* in, float* out, uint32_t n, uint32_t substeps);

/* Wait for the handle's stream; returns FL_TIMEOUT (and clears it) when a
 * device-side wait of an earlier substep expired.  Replaces the device-lost
 * status word the reference polls (gpu/mod.rs:245-250). */
fl_status fl_sync(fl_handle* h);
/* Limit of every device-side wait of this handle's kernels (the CG exchange
 * polls and the multigrid barrier), in nanoseconds; 0 = the default of 2 s.
 * When a wait runs out, the solve records FL_TIMEOUT and every block returns;
 * the substep finishes with the pressure the solve had reached, the next
 * fl_sync / fl_step_host / read-back reports FL_TIMEOUT, and the handle stays
 * usable.  Applies from the next enqueued substep.  No counterpart in the
 * reference (a WebGPU device has no such watchdog). */
fl_status fl_set_wait_timeout(fl_handle* h, uint64_t ns);
/* Use a caller stream (cudaStream_t passed as void*; NULL = the handle's own). */
fl_status fl_set_stream(fl_handle* h, void* cuda_stream);

/* Add dv to every particle velocity (impulse.wgsl; fluid.rs:1374-1395). */
fl_status fl_apply_impulse(fl_handle* h, const float dv[3]);
/* Restore the particles of the last fl_set_particles and zero the pressure
 * (fluid.rs:1408-1418). */
fl_status fl_reset(fl_handle* h);

/* Copy grid state of the last substep to host memory. */
fl_status fl_get_grid(fl_handle* h, const fl_grid_view* view);
/* Divergence of the last substep's pre-projection velocity, drift term
 * included (divergence.wgsl:22-59): nx*ny*nz floats, 0 off liquid cells. */
fl_status fl_get_divergence(fl_handle* h, float* out);
/* Bins of the last substep's counting sort: per-cell counts and exclusive
 * offsets, and perm[d] = pre-sort slot of the particle placed in slot d.  The
 * permutation is stable (lib.rs:1188-1211).  Any pointer may be NULL. */
fl_status fl_get_bins(fl_handle* h, uint32_t* counts, uint32_t* offsets, uint32_t* perm);
fl_status fl_get_stats(fl_handle* h, fl_stats* out);

/* Checkpoint: particles, ids, warm-start pressure and step counter.  Call with
 * buf == NULL to learn the size.  Resume is bit-exact. */
fl_status fl_save_state(fl_handle* h, void* buf, size_t* size_inout);
fl_status fl_load_state(fl_handle* h, const void* buf, size_t size);

/* Device-buffer particle copies (8 floats per particle, 16-byte aligned):
 * out of the handle (n = fl_particle_count particles and, if ids_dev is not
 * NULL, their ids as fl_get_particles gives them), and into it (n <= capacity;
 * ids become the input slots 0..n-1; the warm-start pressure and the reset
 * copy are kept).  No reference counterpart: the reference's particles live
 * in its own GPU buffers (fluid.rs), which these stand in for. */
fl_status fl_get_particles_device(fl_handle* h, void* dst_dev, uint32_t* ids_dev);
fl_status fl_set_particles_device(fl_handle* h, const void* src_dev, uint32_t n);

/* fl_save_state / fl_load_state with the blob in device memory (same layout
 * and size; 256-byte aligned buffer): checkpoints of a rollout stay in HBM. */
fl_status fl_save_state_device(fl_handle* h, void* dst_dev, size_t* size_inout);
fl_status fl_load_state_device(fl_handle* h, const void* src_dev, size_t size);

/* ---- adjoint (differentiable rollout) ----
 * A tape records the forward intermediates of up to `max_steps` substeps:
 * bin-ordered particles, the bin permutation, cell types, the saved and the
 * final face velocities (36 B per particle, 1 B per cell and 8 B per face,
 * per step).  fl_step_record runs one substep like
 * fl_step(h, 1) and appends it.  fl_step_adjoint pops the last recorded step:
 * given dL/d(particles after the step) — 8 floats per particle, in the order
 * fl_get_particles returns after that step — it writes dL/d(particles before
 * the step) in the order they had before it, and adds dL/d(gravity vector) to
 * dL_dgrav[3].  Discrete choices (bins, cell types, clamps) are held fixed;
 * the fixed-point P2G normalisation is linearised at its unquantised sums;
 * the pressure solve is differentiated as an exact solve, so the adjoint runs
 * a second CG with the same operator, the handle's cg_precision and the
 * tape's adjoint solver (fl_tape_set_adjoint_solver), to `adj_cg_tol`
 * relative residual or `adj_cg_iters` iterations.  Both advection orders and
 * the wall-friction band are differentiated (the friction band's min/max
 * selections and the speed and wall clamps held at the recorded step's
 * choices).  Gradient buffers are device pointers.
 * fl_tape_last_stats: cg_iterations, rs_initial/rs_final and device_status of
 * the last adjoint pressure solve. */
typedef struct fl_tape fl_tape;
fl_status fl_tape_create(fl_handle* h, uint32_t max_steps, fl_tape** out);
fl_status fl_tape_free(fl_tape* t);
fl_status fl_tape_clear(fl_tape* t);
/* Warm start of the adjoint pressure solve (off after fl_tape_create).  When
 * on, each fl_step_adjoint starts its CG from the adjoint pressure of the
 * previous call instead of zero, and stops once |r| <= adj_cg_tol * |dL/dp|
 * (the bound the cold start's relative test gives) or at adj_cg_iters.  Every
 * call, on or off, resets the carried adjoint pressure to zero: a backward
 * pass that begins with it does not depend on earlier ones. */
fl_status fl_tape_set_adjoint_warm_start(fl_tape* t, int enable);
/* Solver of the adjoint pressure systems: FL_SOLVER_CG, FL_SOLVER_MGPCG, or
 * FL_SOLVER_FOLLOW (after fl_tape_create) for the handle's pressure_solver.
 * The adjoint has no reference arithmetic to match, so the multigrid
 * preconditioner may serve a handle whose forward runs the reference's CG. */
#define FL_SOLVER_FOLLOW 0xffffffffu
fl_status fl_tape_set_adjoint_solver(fl_tape* t, uint32_t solver);
fl_status fl_tape_count(const fl_tape* t, uint32_t* n_out);
fl_status fl_tape_last_stats(const fl_tape* t, fl_stats* out);
fl_status fl_step_record(fl_handle* h, fl_tape* t);
fl_status fl_step_adjoint(fl_handle* h, fl_tape* t, const void* dL_dout_dev, void* dL_din_dev, float* dL_dgrav,
                          uint32_t adj_cg_iters, float adj_cg_tol);

/* ---- pressure log (rollouts that recompute without the pressure solve) ----
 * fl_copy_pressure_device copies the pressure field of the last substep
 * (C = nx*ny*nz floats, x fastest) to device memory.  fl_step_replay runs one
 * substep like fl_step(h, 1) with the pressure solve replaced by
 * `pressure_dev`: given the field that the same substep's solve produced, the
 * substep is reproduced bit for bit without its CG.  With a tape (not NULL)
 * the substep is also recorded, as by fl_step_record. */
fl_status fl_copy_pressure_device(fl_handle* h, void* dst_dev);
fl_status fl_step_replay(fl_handle* h, const void* pressure_dev, fl_tape* t);

/* Per-stage device time, measured with CUDA events on the handle's stream
 * (the sections of the reference's GpuTimers, gpu/timing.rs:32-59, grouped by
 * kernel).  While profiling is on, fl_step launches stage by stage and waits at
 * the end of every substep; totals accumulate until fl_reset_stage_times. */
enum {
    FL_STAGE_SORT = 0,      /* clear (histogram, P2G accumulators) + mark + counting sort */
    FL_STAGE_CLASSIFY = 1,  /* classify */
    FL_STAGE_SCATTER = 2,   /* P2G */
    FL_STAGE_PREP = 3,      /* normalize, save_vel, forces, bound_pre, divergence, cg_init */
    FL_STAGE_CG = 4,        /* the CG iterations */
    FL_STAGE_GRADIENT = 5,  /* gradient (+ bound_post) */
    FL_STAGE_G2P = 6,       /* g2p */
    FL_STAGE_COUNT = 7
};
fl_status fl_set_profiling(fl_handle* h, int enable);
/* ms_out[FL_STAGE_COUNT]: summed milliseconds; substeps_out: substeps timed. */
fl_status fl_get_stage_times(fl_handle* h, double* ms_out, uint64_t* substeps_out);
fl_status fl_reset_stage_times(fl_handle* h);

/* The reference's section names, for per-section comparisons: its detailed
 * sections (FINE_SECTIONS, gpu/timing.rs:32-59: "clear" .. "g2p", indices
 * 0-25) followed by its CG categories (CG_CATS, timing.rs:93: "cg_spmv",
 * "cg_reduce", "cg_update", "cg_scalars", indices 26-29).  Fused kernels time
 * several sections at once here, so each section reports the FL_STAGE_* whose
 * time contains it (e.g. "clear", "mark" and "sort" -> FL_STAGE_SORT: one
 * memset clears the histogram and the P2G accumulators at the start of the
 * substep; the four CG categories -> FL_STAGE_CG, one persistent kernel).  fl_section_name returns
 * NULL and fl_section_stage -1 past the end. */
#define FL_SECTION_COUNT 30u
const char* fl_section_name(uint32_t i);
int fl_section_stage(uint32_t i);
/* The reference's coarse rollup (timing.rs PREP_END / FINISH_START): ms_out[0]
 * prep (clear .. bound_pre_w), ms_out[1] pressure (divergence, cg_init and the
 * CG), ms_out[2] finish (gradient .. g2p), from the stage totals.  The grid
 * prep kernel fuses bound_pre with divergence and cg_init, so its whole time
 * counts as prep here. */
fl_status fl_get_coarse_times(fl_handle* h, double* ms_out, uint64_t* substeps_out);

/* ---- scene presets and particle seeding ----
 * The reference's scene presets (app/crates/fluid-lab/src/scene/mod.rs) and
 * its initial particle layout (generate_particles, app/crates/fluid-lab/src/
 * gpu/fluid.rs:1838-1913).  A block is an axis-aligned liquid region in
 * normalized tank space [0,1]^3 (y up). */
typedef struct fl_block {
    float min[3];
    float max[3];
} fl_block;
enum { FL_PRESET_FALLING_BLOB = 0, FL_PRESET_DAM_BREAK = 1, FL_PRESET_DOUBLE_SPLASH = 2 };
#define FL_SCENE_MAX_BLOCKS 16u
/* preset_blocks (scene/mod.rs:204-236): the preset's blocks for a drop height
 * and a fill level in [0,1] (the registry's percentage / 100); `out` holds at
 * least 2 blocks.  Unknown presets are the falling blob (ScenePreset::from_u32). */
fl_status fl_scene_blocks(uint32_t preset, float drop_height, float fill_level, fl_block* out, uint32_t* n_out);
/* seeded_volume_fraction (scene/mod.rs:155-165). */
fl_status fl_scene_seeded_fraction(const fl_block* blocks, uint32_t nblocks, float* out);
/* resolved_particle_count (scene/mod.rs:178-192): override_count when nonzero,
 * else round(seeded cells * density), at least 1024 (0 for an empty scene). */
fl_status fl_scene_particle_count(uint32_t nx, uint32_t ny, uint32_t nz, const fl_block* blocks, uint32_t nblocks,
                                  float density, uint32_t override_count, uint32_t* out);
/* Number of particles generate_particles lays out for these blocks and budget
 * in the settings' tank (origin, cell size h = geom[0], extent = gdim * h). */
fl_status fl_seed_count(const fl_params* params, const fl_block* blocks, uint32_t nblocks, uint32_t particle_count,
                        uint32_t* n_out);
/* generate_particles on the device, into the handle (like fl_set_particles:
 * ids 0..n-1, zero velocity, the state fl_reset restores, pressure zeroed):
 * the jittered lattice per block with the reference's seeded LCG, bit for bit.
 * *n_out = particles written; INVALID_ARG if more than the capacity. */
fl_status fl_seed_particles(fl_handle* h, const fl_block* blocks, uint32_t nblocks, uint32_t particle_count,
                            uint32_t* n_out);

/* ---- headless grid slice ----
 * The per-cell arithmetic of the reference's slice debug renderer
 * (app/crates/fluid-lab/src/gpu/slice.rs, shaders/slice.wgsl:69-141) for the
 * XY cross-section at k (FL_SLICE_MIDDLE = nz/2, the reference's slice): one
 * float4 {r, g, b, visible} per cell, row-major over (i, j), of the last
 * substep's grid.  visible = 0 where the renderer draws nothing (air in
 * FL_SLICE_CELL_TYPE; non-liquid cells in the other modes).  No window,
 * swapchain or graphics API: the image is a buffer.  fl_grid_slice copies
 * nx*ny*4 floats to host memory and waits; fl_grid_slice_device writes a
 * 16-byte aligned device buffer on the handle's stream. */
#define FL_SLICE_MIDDLE 0xffffffffu
enum { FL_SLICE_CELL_TYPE = 0, FL_SLICE_PRESSURE = 1, FL_SLICE_SPEED = 2 };
fl_status fl_grid_slice(fl_handle* h, uint32_t mode, uint32_t slice_k, float* rgba_out);
fl_status fl_grid_slice_device(fl_handle* h, uint32_t mode, uint32_t slice_k, void* rgba_dev);

/* ---- fixed-timestep frame driver ----
 * fl_timestep restates the reference's TimestepController
 * (app/crates/fluid-lab/src/timestep.rs:64-233): a render delta is sanitised,
 * scaled by the simulation speed and clamped to 1/30 s before it enters the
 * accumulator; at most max_substeps substeps of fixed_dt run per frame, and
 * when more were due the rest of the accumulator is dropped.  Host only; no
 * device is needed. */
enum { FL_POLICY_FIXED_DROP_CAP = 0, FL_POLICY_EXPLICIT_EXPORT = 1 };
typedef struct fl_timestep_stats {  /* TimestepFrameStats (timestep.rs:21-50) */
    uint32_t substeps;          /* substeps executed this frame */
    uint32_t natural_substeps;  /* substeps the accumulator wanted before the cap */
    uint32_t max_substeps;
    uint32_t substep_cap_hit;   /* 1 when natural_substeps > max_substeps */
    float fixed_dt;
    float accumulated_before;   /* accumulator after adding the clamped delta */
    float accumulated_after;    /* after draining (and dropping) */
    float dropped_this_frame;   /* seconds dropped by the cap this frame */
    float sim_advanced;         /* seconds of simulation advanced */
    float wall_dt;              /* sanitised render delta, before the clamp */
    float sim_time_scale;
    float real_time_factor;     /* sim_advanced / wall_dt (0 when wall_dt is 0) */
    uint32_t policy;            /* FL_POLICY_* (label: fl_timestep_policy_label) */
} fl_timestep_stats;
typedef struct fl_timestep fl_timestep;
fl_status fl_timestep_create(float fixed_dt, uint32_t max_substeps, fl_timestep** out);
fl_status fl_timestep_free(fl_timestep* t);
/* steps_for_frame_scaled (timestep.rs:98-150); sim_time_scale 1 = steps_for_frame. */
fl_status fl_timestep_steps_for_frame(fl_timestep* t, float render_dt_s, float sim_time_scale, uint32_t* n_out);
fl_status fl_timestep_record_manual_steps(fl_timestep* t, float render_dt_s, uint32_t substeps,
                                          float sim_time_scale);
fl_status fl_timestep_record_export_steps(fl_timestep* t, float sim_dt_s, uint32_t substeps);
fl_status fl_timestep_record_idle_frame(fl_timestep* t, float render_dt_s, float sim_time_scale);
fl_status fl_timestep_reset(fl_timestep* t);
fl_status fl_timestep_last_stats(const fl_timestep* t, fl_timestep_stats* out);
fl_status fl_timestep_total_dropped(const fl_timestep* t, float* out);
fl_status fl_timestep_accumulator(const fl_timestep* t, float* out);
const char* fl_timestep_policy_label(uint32_t policy);
/* The simulation half of FluidApp::frame (app/crates/fluid-lab/src/lib.rs:352-394):
 * running, accumulate render_dt_ms (sanitised, converted to seconds in f32)
 * scaled by sim_speed and run the due substeps on h; paused, reset the
 * accumulator and run one substep if *pending_steps > 0 (decrementing it).
 * *substeps_out (may be NULL) receives the substeps run. */
fl_status fl_frame(fl_handle* h, fl_timestep* t, double render_dt_ms, float sim_speed, int paused,
                   uint32_t* pending_steps, uint32_t* substeps_out);
/* The simulation half of FluidApp::export_frame (lib.rs:570-590): run
 * `substeps` substeps and record them as explicit export steps. */
fl_status fl_export_frame(fl_handle* h, fl_timestep* t, uint32_t substeps, double sim_dt_s);

/* Stand-alone pressure solve on host arrays: the MAC-Poisson CG of
 * cg_init/cg_spmv/.../cg_dir.wgsl with the step's semantics, for cell types
 * (FL_CELL_*), a divergence field and an initial pressure (used only when
 * warm_start != 0).  Replaces sim/pressure.rs cg_solve_with_options
 * (app/crates/fluid-lab/src/sim/pressure.rs:235-309) on the GPU.
 * rhs = -(rho*h*h/dt)*div.  Writes pressure_out and, if non-NULL, stats. */
fl_status fl_solve_pressure(uint32_t nx, uint32_t ny, uint32_t nz, const uint8_t* cell_type,
                            const float* divergence, const float* pressure_in, float* pressure_out,
                            float h, float rho, float dt, uint32_t max_iters, uint32_t warm_start,
                            float tolerance, uint32_t cg_precision, fl_stats* stats_out);

/* The reference's relaxation solvers for the same system, from p = 0:
 * FL_RELAX_JACOBI is jacobi_solve (sim/pressure.rs:68-136), `iters` Jacobi
 * sweeps; FL_RELAX_RBGS is the red-black Gauss-Seidel sweep of pressure.wgsl,
 * `iters` times a red phase then a black phase, in place.  scale = rho*h*h/dt
 * as in ProjectionParams::rhs_scale.  Host arrays of nx*ny*nz cells; the
 * result is bit-identical to the reference arithmetic (f32). */
#define FL_RELAX_JACOBI 0u
#define FL_RELAX_RBGS 1u
fl_status fl_relax_pressure(uint32_t nx, uint32_t ny, uint32_t nz, const uint8_t* cell_type,
                            const float* divergence, float h, float rho, float dt, uint32_t method, uint32_t iters,
                            float* pressure_out);

/* Pressure solve that allocates nothing.  No counterpart in the reference:
 * for callers that cannot call cudaMalloc around the solve (a frame loop with
 * a no-allocation rule, a plugin whose host application owns every device
 * allocation, a process that must not grow its device footprint after
 * start-up).  Same solve and settings as fl_solve_pressure, but inputs and
 * output are DEVICE pointers: cell types (u8), divergence, and pressure
 * (read as the initial guess when warm_start != 0, overwritten with the
 * result); pressure must not overlap the other two (FL_INVALID_ARG).  The CG
 * scratch is one static device array sized for FL_NOALLOC_MAX_CELLS cells
 * (about 4.6 MB, held by every GPU that loads the library until exit); larger
 * grids return FL_INVALID_ARG.  The first call on a device looks up the
 * array's device address (cudaGetSymbolAddress).  All calls share the array:
 * calls that overlap on the GPU race.  Enqueues on `cuda_stream` (NULL =
 * default stream), copies the statistics back and synchronizes that stream,
 * so it cannot be called while the stream is being captured into a graph;
 * fills stats_out if non-NULL.  A failure leaves its message in
 * fl_last_error(NULL). */
#define FL_NOALLOC_MAX_CELLS 262144u
fl_status fl_solve_pressure_noalloc(uint32_t nx, uint32_t ny, uint32_t nz, const uint8_t* cell_type_dev,
                                    const float* divergence_dev, float* pressure_dev, float h, float rho,
                                    float dt, uint32_t max_iters, uint32_t warm_start, float tolerance,
                                    uint32_t cg_precision, void* cuda_stream, fl_stats* stats_out);

/* Message of the last failing call on `h` (or of the last failing fl_create /
 * fl_solve_pressure when h == NULL).  Never NULL. */
const char* fl_last_error(const fl_handle* h);

#ifdef __cplusplus
}
#endif
#endif /* FLUIDGB_H */
