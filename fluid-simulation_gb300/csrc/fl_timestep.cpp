// fl_timestep.cpp — the fixed-timestep frame driver (host code, no device work
// of its own).
//
// fl_timestep restates the reference's TimestepController
// (app/crates/fluid-lab/src/timestep.rs:64-233): render deltas are sanitised,
// scaled by the simulation speed and clamped to 1/30 s before they enter the
// accumulator; at most max_substeps fixed-dt substeps run per frame and, when
// more were due, the rest of the accumulator is dropped (policy
// "fixed-drop-cap").  Arithmetic is f32 in the reference's order (this file is
// compiled with -ffp-contract=off).
//
// fl_frame / fl_export_frame are the simulation half of FluidApp::frame and
// FluidApp::export_frame (app/crates/fluid-lab/src/lib.rs:352-394, :570-590):
// they decide the substep count and run it on a handle through fl_step.
#include <cmath>
#include <new>

#include "../../include/fluidgb.h"

struct fl_timestep {
    float accumulator = 0.0f;
    float fixed_dt = 0.0f;
    uint32_t max_substeps = 0;
    float dropped_time = 0.0f;  // cumulative seconds dropped by the cap
    fl_timestep_stats last{};
};

namespace {

// 1/30 s in f32 (timestep.rs:15)
const float kMaxRenderDt = 1.0f / 30.0f;

// timestep.rs:235-241
float finite_nonnegative(float v) { return std::isfinite(v) ? (v > 0.0f ? v : 0.0f) : 0.0f; }

// timestep.rs:243-249
float real_time_factor(float sim_advanced, float wall_dt) { return wall_dt > 0.0f ? sim_advanced / wall_dt : 0.0f; }

// Rust's `f32 as u32`: saturating, NaN -> 0.
uint32_t f32_to_u32(float x) {
    if (!(x > 0.0f)) return 0u;
    if (x >= 4294967296.0f) return 0xffffffffu;
    return (uint32_t)x;
}

fl_timestep_stats idle_stats(float fixed_dt, uint32_t max_substeps, float wall_dt, float scale) {
    fl_timestep_stats s{};
    s.fixed_dt = fixed_dt;
    s.max_substeps = max_substeps;
    s.wall_dt = wall_dt;
    s.sim_time_scale = scale;
    s.policy = FL_POLICY_FIXED_DROP_CAP;
    return s;
}

}  // namespace

extern "C" {

const char* fl_timestep_policy_label(uint32_t policy) {
    // timestep.rs:18 and :182
    return policy == FL_POLICY_EXPLICIT_EXPORT ? "fixed-explicit-export" : "fixed-drop-cap";
}

fl_status fl_timestep_create(float fixed_dt, uint32_t max_substeps, fl_timestep** out) {
    if (!out) return FL_INVALID_ARG;
    *out = nullptr;
    fl_timestep* t = new (std::nothrow) fl_timestep();
    if (!t) return FL_OOM;
    t->fixed_dt = fixed_dt;
    t->max_substeps = max_substeps;
    *out = t;
    return FL_OK;
}

fl_status fl_timestep_free(fl_timestep* t) {
    delete t;
    return FL_OK;
}

// timestep.rs:98-150 (steps_for_frame_scaled; steps_for_frame is scale 1)
fl_status fl_timestep_steps_for_frame(fl_timestep* t, float render_dt_s, float sim_time_scale, uint32_t* n_out) {
    if (!t || !n_out) return FL_INVALID_ARG;
    const float wall = finite_nonnegative(render_dt_s);
    const float scale = finite_nonnegative(sim_time_scale);
    const float scaled = wall * scale;
    const float clamped = scaled < kMaxRenderDt ? scaled : kMaxRenderDt;
    t->accumulator += clamped;
    const float before = t->accumulator;
    const uint32_t natural = t->fixed_dt > 0.0f ? f32_to_u32(std::floor(t->accumulator / t->fixed_dt)) : 0u;
    const uint32_t n = natural < t->max_substeps ? natural : t->max_substeps;
    t->accumulator -= (float)n * t->fixed_dt;
    float dropped = 0.0f;
    if (natural > t->max_substeps) {
        dropped = t->accumulator;
        t->dropped_time += dropped;
        t->accumulator = 0.0f;
    }
    const float advanced = (float)n * t->fixed_dt;
    fl_timestep_stats s{};
    s.substeps = n;
    s.fixed_dt = t->fixed_dt;
    s.max_substeps = t->max_substeps;
    s.natural_substeps = natural;
    s.substep_cap_hit = natural > t->max_substeps ? 1u : 0u;
    s.accumulated_before = before;
    s.accumulated_after = t->accumulator;
    s.dropped_this_frame = dropped;
    s.sim_advanced = advanced;
    s.wall_dt = wall;
    s.sim_time_scale = scale;
    s.real_time_factor = real_time_factor(advanced, wall);
    s.policy = FL_POLICY_FIXED_DROP_CAP;
    t->last = s;
    *n_out = n;
    return FL_OK;
}

// timestep.rs:154-172
fl_status fl_timestep_record_manual_steps(fl_timestep* t, float render_dt_s, uint32_t substeps,
                                          float sim_time_scale) {
    if (!t) return FL_INVALID_ARG;
    const float wall = finite_nonnegative(render_dt_s);
    const float scale = finite_nonnegative(sim_time_scale);
    const float advanced = (float)substeps * t->fixed_dt;
    fl_timestep_stats s = idle_stats(t->fixed_dt, t->max_substeps, wall, scale);
    s.substeps = substeps;
    s.sim_advanced = advanced;
    s.real_time_factor = real_time_factor(advanced, wall);
    t->last = s;
    return FL_OK;
}

// timestep.rs:176-193
fl_status fl_timestep_record_export_steps(fl_timestep* t, float sim_dt_s, uint32_t substeps) {
    if (!t) return FL_INVALID_ARG;
    const float wall = finite_nonnegative(sim_dt_s);
    const float advanced = (float)substeps * t->fixed_dt;
    fl_timestep_stats s{};
    s.substeps = substeps;
    s.fixed_dt = t->fixed_dt;
    s.max_substeps = substeps;
    s.natural_substeps = substeps;
    s.sim_advanced = advanced;
    s.wall_dt = wall;
    s.sim_time_scale = 1.0f;
    s.real_time_factor = real_time_factor(advanced, wall);
    s.policy = FL_POLICY_EXPLICIT_EXPORT;
    t->last = s;
    return FL_OK;
}

// timestep.rs:197-206
fl_status fl_timestep_record_idle_frame(fl_timestep* t, float render_dt_s, float sim_time_scale) {
    if (!t) return FL_INVALID_ARG;
    t->last = idle_stats(t->fixed_dt, t->max_substeps, finite_nonnegative(render_dt_s),
                         finite_nonnegative(sim_time_scale));
    return FL_OK;
}

// timestep.rs:226-233: zero the accumulator and the per-frame stats; the
// cumulative dropped time is kept.
fl_status fl_timestep_reset(fl_timestep* t) {
    if (!t) return FL_INVALID_ARG;
    t->accumulator = 0.0f;
    t->last = idle_stats(t->fixed_dt, t->max_substeps, 0.0f, 1.0f);
    return FL_OK;
}

fl_status fl_timestep_last_stats(const fl_timestep* t, fl_timestep_stats* out) {
    if (!t || !out) return FL_INVALID_ARG;
    *out = t->last;
    return FL_OK;
}

fl_status fl_timestep_total_dropped(const fl_timestep* t, float* out) {
    if (!t || !out) return FL_INVALID_ARG;
    *out = t->dropped_time;
    return FL_OK;
}

fl_status fl_timestep_accumulator(const fl_timestep* t, float* out) {
    if (!t || !out) return FL_INVALID_ARG;
    *out = t->accumulator;
    return FL_OK;
}

// FluidApp::frame (lib.rs:352-394), simulation half.
fl_status fl_frame(fl_handle* h, fl_timestep* t, double render_dt_ms, float sim_speed, int paused,
                   uint32_t* pending_steps, uint32_t* substeps_out) {
    if (!h || !t) return FL_INVALID_ARG;
    double ms = std::isfinite(render_dt_ms) ? render_dt_ms : 0.0;  // finite_or_zero_f64(..).max(0)
    if (ms < 0.0) ms = 0.0;
    const float dt_s = (float)ms / 1000.0f;
    uint32_t n = 0;
    fl_status s = FL_OK;
    if (!paused) {
        s = fl_timestep_steps_for_frame(t, dt_s, sim_speed, &n);
        if (s == FL_OK && n > 0) s = fl_step(h, n);
    } else {
        fl_timestep_reset(t);
        if (pending_steps && *pending_steps > 0) {
            *pending_steps -= 1;
            n = 1;
            s = fl_step(h, 1);
            fl_timestep_record_manual_steps(t, dt_s, 1, sim_speed);
        } else {
            fl_timestep_record_idle_frame(t, dt_s, sim_speed);
        }
    }
    if (substeps_out) *substeps_out = n;
    return s;
}

// FluidApp::export_frame (lib.rs:570-590), simulation half.
fl_status fl_export_frame(fl_handle* h, fl_timestep* t, uint32_t substeps, double sim_dt_s) {
    if (!h || !t) return FL_INVALID_ARG;
    double dt = std::isfinite(sim_dt_s) ? sim_dt_s : 0.0;
    if (dt < 0.0) dt = 0.0;
    fl_status s = FL_OK;
    if (substeps > 0) s = fl_step(h, substeps);
    fl_timestep_record_export_steps(t, (float)dt, substeps);
    return s;
}

}  // extern "C"
