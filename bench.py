#!/usr/bin/env python
"""FLIP/PIC substep benchmark: steps/s of the 128^3, ~2M-particle dam break.

Workload (default `dam128_2m`): 128^3 unit box, fluid in x<0.5, y<0.5, z<0.5 at
8 jittered particles per interior cell (2,000,376 particles, seed 0x5EED),
dt = 1/120, FLIP 0.95, CG <= 200 iterations at relative tolerance 1e-5.
A step is one full substep (bin -> P2G -> classify -> grid prep -> CG ->
projection -> G2P) through the C ABI.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours:      `value` = steps/s over K device-timed steps (CUDA events on the
           handle's stream, inputs resident in HBM); `e2e` = steps/s through
           fl_step_host with particles in and out of pinned host memory every
           step; `roofline` for the dominant stage; `cpu_baseline` = the CPU
           oracle (a C port of the reference step) on the host cores.
reference: the reference step's CPU restatement (the oracle; the reference is
           Rust + WebGPU and cannot run on this machine) on all host cores.
Multi-GPU: replicas only (independent scenes, seed + rank); value = all
ranks' steps / max-over-ranks time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [os.path.join(REPO, "fluid-simulation_gb300")]

# bin 8 (count, scan x3, scatter, fix, fix_big, gather), classify, p2g 2, prep, cg plan, cg, project, g2p
KERNELS_PER_STEP = 16


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="dam128_2m")
    ap.add_argument("--precision", choices=["f32", "f64", "f64ieee"], default="f32")
    ap.add_argument("--profile-steps", type=int, default=20)
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--cpu-budget", type=float, default=20.0, help="seconds of CPU-baseline sampling")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-mgpcg", action="store_true", help="skip the multigrid-preconditioned solver leg")
    ap.add_argument("--adj-steps", type=int, default=20, help="rollout length of the forward+adjoint leg (0 = off)")
    ap.add_argument("--adj-every", type=int, default=10, help="checkpoint interval of that rollout")
    ap.add_argument("--adj-no-plog", action="store_true",
                    help="recompute segments with their pressure solves (default: replay the logged pressure fields)")
    ap.add_argument("--adj-mgpcg", action="store_true",
                    help="run the forward+adjoint leg on FL_SOLVER_MGPCG (forward and adjoint solves)")
    ap.add_argument("--adj-solver", choices=["follow", "cg", "mgpcg"], default="mgpcg",
                    help="solver of the adjoint pressure systems (default: the multigrid-preconditioned CG; "
                         "the forward keeps the reference CG unless --adj-mgpcg)")
    ap.add_argument("--extra-legs", default="block256,dam128",
                    help="other configurations measured after the headline (comma list; '' = none): "
                         "forward steps/s, stage rooflines, device memory; block256 also forward+adjoint")
    ap.add_argument("--adj-cold", action="store_true",
                    help="start every adjoint pressure solve from zero (default: from the next step's solution)")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def replica_value(world, steps, ms_max):
    """Whole-job steps/s of `world` independent replicas: all ranks' steps over
    the slowest rank's time."""
    return world * steps / (ms_max / 1000.0)


def measured_peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def working_set_bytes(n, nx, ny, nz):
    C = nx * ny * nz
    F = (nx + 1) * ny * nz + nx * (ny + 1) * nz + nx * ny * (nz + 1)
    return 2 * 32 * n + 6 * 4 * n + (4 * 4 + 2 + 5 * 4) * C + 4 * 4 * F


def algorithmic_bytes(stage, n, nx, ny, nz, liquid, iters):
    """Per-launch algorithmic bytes of a stage (the byte model: a particle is
    32 B, a cell array entry 4 B, a cell type 1 B; CG 33 B per liquid cell per
    iteration: p, r, d, q each read and written once, plus the cell type)."""
    C = nx * ny * nz
    F = (nx + 1) * ny * nz + nx * (ny + 1) * nz + nx * ny * (nz + 1)
    return {
        "sort": 80 * n + 16 * C,
        "classify": 4 * C + 1 * C,
        "scatter": 32 * n + 8 * F,
        "prep": 16 * F + 4 * C + 1 * C + 16 * liquid,
        "cg": 33 * liquid * iters,
        "gradient": 8 * F + 5 * C,
        "g2p": 64 * n + 8 * F,
    }[stage]


def cpu_baseline(name, budget_s, seed):
    """The CPU oracle on all host threads from the workload's initial state."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle
    from fluidgb import scenes
    oracle.load()
    threads = os.cpu_count() or 1
    oracle.set_threads(threads)
    p, parts, spec = scenes.workload(name, seed=seed)
    o = oracle.OracleFluid(p, parts.shape[0])
    o.set_particles(parts)
    o.step(1)  # untimed warm-up step
    t0 = time.perf_counter()
    k = 0
    while True:
        o.step(1)
        k += 1
        el = time.perf_counter() - t0
        if el >= budget_s:
            break
    o.close()
    return {"value": k / el, "unit": "steps/s", "cores": threads, "kind": "port",
            "sample": "%d substeps of %s (N=%d, %d^3) after 1 warm-up step, f32 reference arithmetic, %d threads" % (
                k, name, parts.shape[0], spec["n"], threads)}


# The headline metric (steps/s, forward+adjoint ratio, CG bandwidth), shared by both arms.
METRIC = "FLIP steps/s @128^3 ~2M particles; fwd+adjoint/fwd ratio; CG HBM GB/s"


def base_config(workload, spec, n, world):
    """The workload part of the JSON line's config, identical in both arms."""
    return {"workload": workload, "grid": [spec["n"]] * 3, "particles": int(n), "cg_max_iters": spec["iters"],
            "cg_tol": spec["tol"], "flip": 0.95, "dt": "1/120", "parallelism": "replicas" if world > 1 else "single"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from fluidgb import scenes
    budget = max(10.0, min(150.0, 1.5 * args.steps))
    cb = cpu_baseline(args.workload, budget, scenes.DEFAULT_SEED)
    p, parts, spec = scenes.workload(args.workload)
    line = {
        "metric": METRIC,
        "value": cb["value"], "unit": "steps/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 / cb["value"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": base_config(args.workload, spec, parts.shape[0], world),
        "cpu_baseline": cb,
        "e2e": {"value": cb["value"], "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference is Rust+WebGPU (no toolchain or graphics stack here); its step is timed as the C "
                "restatement of its arithmetic (oracle/fl_oracle.c) on the host cores",
    }
    print(json.dumps(line))


def timed_steps(torch, g, k):
    s = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s)
    g.step(k)
    e1.record(s)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1)


def adjoint_leg(torch, p, parts, steps, every, cg_iters, cg_tol, warm=True, plog=True, adj_solver=None):
    """Forward+adjoint of a checkpointed rollout against its forward alone.

    forward: `steps` substeps from `parts` with a device checkpoint every
    `every`, the last segment recorded on the tape, and (with `plog`) every
    substep's pressure field; backward: per earlier segment, restore +
    recompute while recording (with `plog`, each substep replayed with its
    logged pressure instead of its CG: the same bits); every step popped through
    the adjoint (a second solve with the forward's iteration cap, tolerance
    and precision, by `adj_solver` — None: the handle's — started from the
    next step's adjoint pressure unless `warm` is False).  Loss: |centre of mass - (0.7, 0.2, 0.5)|^2.  Timed with CUDA
    events on the rollout's stream."""
    from fluidgb.autograd import Rollout
    n = parts.shape[0]
    free0 = torch.cuda.mem_get_info()[0]
    from fluidgb import FL_SOLVER_FOLLOW
    roll = Rollout(p, n, steps, checkpoint_every=every, adj_cg_iters=cg_iters, adj_cg_tol=cg_tol,
                   adj_warm_start=warm, pressure_log=plog,
                   adj_solver=FL_SOLVER_FOLLOW if adj_solver is None else adj_solver)
    parts_d = torch.from_numpy(parts).cuda()
    target = torch.tensor([0.7, 0.2, 0.5], dtype=torch.float64, device="cuda")
    grav = (p.grav[0], p.grav[1], p.grav[2])

    def loss_grad(final):
        c = final[:, 0:3].double().mean(dim=0)
        g = torch.zeros((n, 8), dtype=torch.float32, device="cuda")
        g[:, 0:3] = (2.0 * (c - target) / n).float()
        return g

    def once():
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        torch.cuda.synchronize()
        e[0].record(roll.stream)
        final, _ = roll.forward(parts_d, grav)
        e[1].record(roll.stream)
        g = loss_grad(final)
        roll.stream.wait_stream(torch.cuda.current_stream())
        roll.backward(g)
        e[2].record(roll.stream)
        torch.cuda.synchronize()
        return e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])

    once()  # warm: graph capture, tape pool
    fwd_ms, bwd_ms = once()
    iters = roll.adj_cg_iterations
    used = free0 - torch.cuda.mem_get_info()[0]
    roll.close()
    return {"workload_steps": steps, "checkpoint_every": every,
            "fwd_ms_per_step": fwd_ms / steps, "fwd_adj_ms_per_step": (fwd_ms + bwd_ms) / steps,
            "ratio": (fwd_ms + bwd_ms) / fwd_ms,
            "backward": "last segment taped during the forward; earlier segments restore + recompute-with-tape" +
                        (" (substeps replayed with their logged pressure fields, no CG)" if plog else " (CG re-solved)") +
                        "; adjoint per step",
            "pressure_log_bytes": steps * int(p.gdim[0]) * int(p.gdim[1]) * int(p.gdim[2]) * 4 if plog else 0,
            "adj_cg_iters_mean": float(sum(iters)) / max(len(iters), 1), "adj_cg_iters_max": max(iters or [0]),
            "adj_cg_max_iters": cg_iters, "adj_cg_tol": cg_tol,
            "adj_cg_start": "warm: previous step's lambda, stop at |r| <= tol |dL/dp|" if warm else "cold: zero",
            "device_bytes": used, "device_bytes_note": "handle + tape + checkpoints + torch buffers of the rollout"}


def stage_profile(g, n, nx, ny, nz, steps, peak):
    """Per-stage CUDA-event times over `steps` substeps, and every stage's
    algorithmic GB/s and fraction of the HBM peak (the byte model above)."""
    g.set_profiling(True)
    g.reset_stage_times()
    liquid_sum = iters_sum = cg_bytes = 0
    for _ in range(steps):
        g.step(1)
        s = g.stats()
        liquid_sum += s["liquid_cells"]
        iters_sum += s["cg_iterations"]
        cg_bytes += algorithmic_bytes("cg", n, nx, ny, nz, s["liquid_cells"], s["cg_iterations"])
    stage_ms, nprof = g.stage_times()
    g.set_profiling(False)
    liquid_avg, iters_avg = liquid_sum / max(nprof, 1), iters_sum / max(nprof, 1)
    roof = {}
    for k, ms in stage_ms.items():
        if ms <= 0.0:
            continue
        b = cg_bytes if k == "cg" else algorithmic_bytes(k, n, nx, ny, nz, liquid_avg, iters_avg) * nprof
        gbs = b / (ms / 1000.0) / 1e9
        roof[k] = {"algorithmic_gbs": gbs, "frac": gbs / peak}
    return ({k: v / max(nprof, 1) for k, v in stage_ms.items()}, roof, liquid_avg, iters_avg, cg_bytes, stage_ms,
            nprof)


def extra_leg(torch, name, stream, steps, warmup, profile_steps, adj_steps, adj_every, peak):
    """Another configuration on the same GPU, after the headline: forward
    steps/s (CUDA events over `steps` substeps after `warmup`), the stages'
    rooflines, the handle's device memory, and (adj_steps > 0) the
    forward+adjoint ratio of a checkpointed rollout."""
    import fluidgb
    from fluidgb import scenes
    p, parts, spec = scenes.workload(name)
    n = parts.shape[0]
    nx = spec["n"]
    free0 = torch.cuda.mem_get_info()[0]
    g = fluidgb.Fluid(p, n)
    handle_bytes = free0 - torch.cuda.mem_get_info()[0]
    g.set_stream(stream.cuda_stream)
    g.set_particles(parts)
    g.step(warmup)
    g.sync()
    ms = timed_steps(torch, g, steps)
    st = g.stats()
    if st["device_status"] != 0:
        raise RuntimeError("device status %d (%s)" % (st["device_status"], name))
    stage_ms, roof, liquid_avg, iters_avg, _, _, _ = stage_profile(g, n, nx, nx, nx, profile_steps, peak)
    g.close()
    tpath = os.path.join(REPO, "profiles", "traffic.json")  # ncu DRAM bytes per launch, where captured
    if os.path.exists(tpath):
        with open(tpath) as f:
            captured = json.load(f).get(name, {})
        for k in roof:
            roof[k]["traffic"] = captured.get(k)
    out = {"workload": name, "grid": [nx] * 3, "particles": int(n), "cg_max_iters": spec["iters"],
           "cg_tol": spec["tol"], "value": steps / (ms / 1000.0), "unit": "steps/s", "ms_per_step": ms / steps,
           "steps": steps, "warmup": warmup, "window": "substeps %d-%d of the scene" % (warmup + 1, warmup + steps),
           "stage_ms_per_step": stage_ms, "stage_roofline": roof, "avg_liquid_cells": liquid_avg,
           "avg_cg_iterations": iters_avg, "handle_device_bytes": handle_bytes}
    if adj_steps > 0:
        out["fwd_adjoint"] = adjoint_leg(torch, p, parts, adj_steps, adj_every, spec["iters"], spec["tol"],
                                         adj_solver=fluidgb.FL_SOLVER_MGPCG)
        out["fwd_adjoint"]["adjoint_solver"] = "mgpcg"
    return out


def run_ours(args):
    import numpy as np
    import torch

    import fluidgb
    from fluidgb import build, scenes

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    build.build()
    fluidgb.load_library()
    prec = {"f32": fluidgb.FL_CG_F32, "f64": fluidgb.FL_CG_F64, "f64ieee": fluidgb.FL_CG_F64_IEEE}[args.precision]
    seed = scenes.DEFAULT_SEED + rank
    p, parts, spec = scenes.workload(args.workload, seed=seed, precision=prec)
    n = parts.shape[0]
    nx = ny = nz = spec["n"]
    # A dedicated stream: the handle enqueues on it and the timing events are
    # recorded on it (torch's default stream has handle 0, which the ABI reads
    # as "the handle's own stream").
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    g = fluidgb.Fluid(p, n)
    g.set_stream(stream.cuda_stream)
    g.set_particles(parts)
    g.step(args.warmup)
    g.sync()

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    ms = timed_steps(torch, g, args.steps)
    barrier()
    clock_rec = clocks.stop()
    st = g.stats()
    if st["device_status"] != 0:
        raise RuntimeError("device status %d" % st["device_status"])
    t = torch.tensor([ms], dtype=torch.float64, device="cuda")
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    ms_max = float(t.item())
    value = replica_value(world, args.steps, ms_max)

    # The extended-precision CG forms on the same scene and schedule:
    # float-float (FL_CG_F64) and IEEE double (FL_CG_F64_IEEE) reductions.
    def precision_leg(form, what):
        q = p.copy()
        q.cg_precision = form
        g64 = fluidgb.Fluid(q, n)
        g64.set_stream(stream.cuda_stream)
        g64.set_particles(parts)
        g64.step(args.warmup)
        g64.sync()
        ms64 = timed_steps(torch, g64, args.steps)
        s64 = g64.stats()
        g64.close()
        return {"value": args.steps / (ms64 / 1000.0), "ms_per_step": ms64 / args.steps,
                "overhead_pct": 100.0 * (ms64 - ms) / ms, "last_cg_iterations": s64["cg_iterations"],
                "reductions": what}

    fp64 = fp64_ieee = None
    if not args.no_fp64 and prec == fluidgb.FL_CG_F32:
        fp64 = precision_leg(fluidgb.FL_CG_F64, "float-float (about 48-bit significand) on the FP32 pipe")
        fp64_ieee = precision_leg(fluidgb.FL_CG_F64_IEEE, "IEEE double: exact products, double sums, trees, "
                                                          "combines, alpha/beta and stopping test")

    # Multigrid-preconditioned CG (opt-in solver) on the same scene and schedule.
    mg = None
    if not args.no_mgpcg:
        q = p.copy()
        q.pressure_solver = fluidgb.FL_SOLVER_MGPCG
        gmg = fluidgb.Fluid(q, n)
        gmg.set_stream(stream.cuda_stream)
        gmg.set_particles(parts)
        gmg.step(args.warmup)
        gmg.sync()
        msmg = timed_steps(torch, gmg, args.steps)
        smg = gmg.stats()
        if smg["device_status"] != 0:
            raise RuntimeError("device status %d (MGPCG)" % smg["device_status"])
        mg = {"value": args.steps / (msmg / 1000.0), "ms_per_step": msmg / args.steps,
              "speedup_vs_cg": ms / msmg, "last_cg_iterations": smg["cg_iterations"],
              "cg_last_cg_iterations": st["cg_iterations"],
              "note": "FL_SOLVER_MGPCG: same operator, warm start, cap and stopping test; results agree with "
                      "the CG's to the tolerance, not bit for bit"}
        gmg.close()

    adj = None
    if args.adj_steps > 0:
        pa = p.copy()
        if args.adj_mgpcg:
            pa.pressure_solver = fluidgb.FL_SOLVER_MGPCG
        adj_solver = {"follow": None, "cg": fluidgb.FL_SOLVER_CG, "mgpcg": fluidgb.FL_SOLVER_MGPCG}[args.adj_solver]
        adj = adjoint_leg(torch, pa, parts, args.adj_steps, args.adj_every, spec["iters"], spec["tol"],
                          warm=not args.adj_cold, plog=not args.adj_no_plog, adj_solver=adj_solver)
        adj["pressure_solver"] = "mgpcg" if args.adj_mgpcg else "cg"
        adj["adjoint_solver"] = adj["pressure_solver"] if adj_solver is None else args.adj_solver
        torch.cuda.set_stream(stream)

    # Per-stage device times (CUDA events between stages on the same stream).
    g.set_profiling(True)
    g.reset_stage_times()
    liquid_sum = iters_sum = 0
    cg_bytes = 0
    for _ in range(args.profile_steps):
        g.step(1)
        s = g.stats()
        liquid_sum += s["liquid_cells"]
        iters_sum += s["cg_iterations"]
        cg_bytes += algorithmic_bytes("cg", n, nx, ny, nz, s["liquid_cells"], s["cg_iterations"])
    stage_ms, nprof = g.stage_times()
    g.set_profiling(False)
    dom = max(stage_ms, key=stage_ms.get)
    liquid_avg = liquid_sum / max(nprof, 1)
    iters_avg = iters_sum / max(nprof, 1)
    if dom == "cg":
        bytes_total = cg_bytes
    else:
        bytes_total = algorithmic_bytes(dom, n, nx, ny, nz, liquid_avg, iters_avg) * nprof
    achieved = bytes_total / (stage_ms[dom] / 1000.0) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = None
    traffic_all = {}
    tpath = os.path.join(REPO, "profiles", "traffic.json")
    if os.path.exists(tpath):
        with open(tpath) as f:
            traffic_all = json.load(f).get(args.workload, {})
        traffic = traffic_all.get(dom)
    # Every stage against the same byte model and peak (transfer GB/s:
    # scatter = P2G, g2p = G2P), with ncu's DRAM bytes per launch where captured.
    stage_roofline = {}
    for k, ms in stage_ms.items():
        if ms <= 0.0:
            continue
        b = cg_bytes if k == "cg" else algorithmic_bytes(k, n, nx, ny, nz, liquid_avg, iters_avg) * nprof
        gbs = b / (ms / 1000.0) / 1e9
        stage_roofline[k] = {"algorithmic_gbs": gbs, "frac": gbs / peak, "traffic": traffic_all.get(k)}

    # End to end through the public C ABI with host buffers.
    pin_in = torch.empty((n, 8), dtype=torch.float32, pin_memory=True)
    pin_out = torch.empty((n, 8), dtype=torch.float32, pin_memory=True)
    a_in, a_out = pin_in.numpy(), pin_out.numpy()
    a_in[:] = g.get_particles(with_ids=False)
    g.step_host(a_in, a_out, 1)  # warm
    a_in, a_out = a_out, a_in
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        g.step_host(a_in, a_out, 1)
        a_in, a_out = a_out, a_in
    e2e_s = time.perf_counter() - t0
    tt = torch.tensor([e2e_s], dtype=torch.float64, device="cuda")
    if world > 1:
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
    e2e_value = world * args.e2e_steps / float(tt.item())
    g.close()

    # The other configurations, one after another (rank 0 of a 1-GPU run):
    # the 256^3 block (forward and forward+adjoint) and the full-depth 128^3
    # dam break (4.19M particles).
    legs = {}
    if rank == 0 and world == 1:
        for name in [x for x in args.extra_legs.split(",") if x and x != args.workload]:
            legs[name] = extra_leg(torch, name, stream, 10, 3, 3, 20 if name == "block256" else 0, 10, peak)
            torch.cuda.set_stream(stream)

    cb = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cb = cpu_baseline(args.workload, args.cpu_budget, seed)

    if rank == 0:
        line = {
            "metric": METRIC,
            "value": value, "unit": "steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32" if prec == fluidgb.FL_CG_F32 else "f32+f64-reductions",
            "data": "synthetic (seeded dam break, seed 0x5EED + rank)",
            "config": dict(base_config(args.workload, spec, n, world),
                           l2="no flush: per-step working set %.0f MB > 129 MB L2" % (
                               working_set_bytes(n, nx, ny, nz) / 1e6),
                           last_cg_iterations=st["cg_iterations"], liquid_cells=st["liquid_cells"]),
            "e2e": {"value": e2e_value, "unit": "steps/s", "h2d_bytes_per_step": 32 * n,
                    "d2h_bytes_per_step": 32 * n,
                    "path": "fl_step_host: pinned host particles in, 1 substep, particles out, synchronous"},
            "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "peak_kind": peak_kind, "traffic": traffic,
                         "bytes_model": "cg: 33 B per liquid cell per iteration" if dom == "cg" else dom,
                         "avg_liquid_cells": liquid_avg, "avg_cg_iterations": iters_avg},
            "stage_ms_per_step": {k: v / max(nprof, 1) for k, v in stage_ms.items()},
            "stage_roofline": stage_roofline,
            "fp64_reductions": fp64,
            "fp64_ieee_reductions": fp64_ieee,
            "mgpcg": mg,
            "fwd_adjoint": adj,
            "configurations": legs or None,
            "cpu_baseline": cb,
            "clocks": clock_rec,
            "gpu_launches": KERNELS_PER_STEP * args.steps,
        }
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
