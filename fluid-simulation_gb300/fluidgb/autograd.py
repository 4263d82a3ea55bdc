"""Differentiable rollouts through the C ABI's adjoint (fl_step_record /
fl_step_adjoint), wrapped in a torch.autograd.Function.

The forward pass runs `steps` substeps and keeps a checkpoint (particles, ids,
warm-start pressure: fl_save_state_device) every `checkpoint_every`
substeps, in device memory; it records the last segment on the tape as it
goes.  The backward pass walks the segments in reverse: the last one is popped
straight from the tape; every earlier one is restored from its checkpoint and
recomputed while recording (the recomputation is bit-identical to the
forward), then popped step by step through the adjoint kernels.  Memory: one
tape of `checkpoint_every` substeps plus the checkpoints; nothing leaves the
GPU.  With checkpoint_every >= steps nothing is recomputed.

With pressure_log (the default) the forward also keeps every substep's
pressure field (4 bytes per cell per substep), and the recomputation replays
each substep with that field in place of its CG (fl_step_replay): the same
bits, without the solve that dominates the substep.

Each adjoint pressure solve starts, by default, from the adjoint pressure of
the step after it (the one solved just before in the backward walk) and stops
at the cold start's bound |r| <= tol |dL/dp| (fl_tape_set_adjoint_warm_start);
adj_warm_start=False starts every solve from zero.  adj_solver chooses the
adjoint solves' solver (FL_SOLVER_CG, FL_SOLVER_MGPCG; by default the
handle's).

Gradients are taken with respect to the initial per-particle state and the
gravity (body-force) vector, as in the differentiable-rollout workload:
`loss = |mean(final positions) - target|^2`, d loss / d(initial velocity, gravity).
"""
import numpy as np
import torch

from ._abi import FL_SOLVER_FOLLOW, Fluid


def _as_device_particles(particles, dev):
    if isinstance(particles, torch.Tensor):
        t = particles.detach().to(device=dev, dtype=torch.float32)
    else:
        t = torch.from_numpy(np.ascontiguousarray(particles, np.float32)).to(dev)
    if t.dim() != 2 or t.shape[1] != 8:
        raise ValueError("particles must be (N, 8) float32: pos.xyz, pad, vel.xyz, pad")
    return t.contiguous()


class Rollout:
    """A checkpointed rollout of one handle.  All buffers live on the current
    CUDA device; the handle runs on a stream of its own, ordered against the
    caller's stream at entry and exit."""

    def __init__(self, params, capacity, steps, checkpoint_every=10, adj_cg_iters=1000, adj_cg_tol=1e-6,
                 adj_warm_start=True, pressure_log=True, adj_solver=FL_SOLVER_FOLLOW):
        self.dev = torch.device("cuda", torch.cuda.current_device())
        self.stream = torch.cuda.Stream(self.dev)
        self.fluid = Fluid(params, capacity)
        self.fluid.set_stream(self.stream.cuda_stream)
        self.params = params.copy()
        self.steps = int(steps)
        self.k = max(1, int(checkpoint_every))
        self.adj_cg_iters = adj_cg_iters
        self.adj_cg_tol = adj_cg_tol
        self.adj_warm_start = bool(adj_warm_start)
        self.cells = int(params.gdim[0]) * int(params.gdim[1]) * int(params.gdim[2])
        self.plog = torch.empty((self.steps, self.cells), dtype=torch.float32, device=self.dev) if pressure_log else None
        self.tape = self.fluid.tape(self.k)
        self.tape.set_adjoint_solver(adj_solver)
        self.checkpoints = {}
        self.taped = None
        self.n = 0
        self.adj_cg_iterations = []

    def close(self):
        self.tape.close()
        self.fluid.close()

    def _enter(self):
        self.stream.wait_stream(torch.cuda.current_stream(self.dev))
        return torch.cuda.stream(self.stream)

    def _leave(self):
        torch.cuda.current_stream(self.dev).wait_stream(self.stream)

    def set_gravity(self, gravity):
        p = self.params.copy()
        p.grav[0], p.grav[1], p.grav[2] = (float(g) for g in gravity)
        p.phys[0] = p.grav[1]
        self.fluid.set_params(p)

    def forward(self, particles0, gravity):
        """particles0: (N, 8) float32 (torch tensor or numpy), input order.
        Returns the final particles (N, 8) and their ids (input slots, int64),
        both CUDA tensors."""
        with self._enter():
            parts = _as_device_particles(particles0, self.dev)
            self.n = parts.shape[0]
            self.set_gravity(gravity)
            self.fluid.set_particles_device(parts.data_ptr(), self.n)
            size = self.fluid.state_size()
            last = ((self.steps - 1) // self.k) * self.k if self.steps else 0
            self.tape.clear()
            for s in range(self.steps):
                if s % self.k == 0:
                    buf = self.checkpoints.get(s)
                    if buf is None or buf.numel() != size:
                        buf = torch.empty(size, dtype=torch.uint8, device=self.dev)
                        self.checkpoints[s] = buf
                    self.fluid.save_state_device(buf.data_ptr(), size)
                if s >= last:
                    self.tape.record()
                else:
                    self.fluid.step(1)
                if self.plog is not None:
                    self.fluid.copy_pressure_device(self.plog[s].data_ptr())
            self.taped = last
            for s in [s for s in self.checkpoints if s >= self.steps or s % self.k]:
                del self.checkpoints[s]
            final = torch.empty((self.n, 8), dtype=torch.float32, device=self.dev)
            ids = torch.empty(self.n, dtype=torch.int32, device=self.dev)
            self.fluid.get_particles_device(final.data_ptr(), ids.data_ptr())
        self._leave()
        return final, ids.long()

    def backward(self, g_final):
        """g_final: dL/d(final particles) (N, 8) in the order forward returned
        them.  Returns dL/d(particles0) (N, 8, CUDA tensor, input order) and
        dL/dgravity (3 doubles)."""
        g_grav = np.zeros(3, np.float64)
        self.adj_cg_iterations = []
        with self._enter():
            g_out = _as_device_particles(g_final, self.dev).clone()
            g_in = torch.empty_like(g_out)
            self.tape.set_adjoint_warm_start(self.adj_warm_start)
            for s0 in sorted(self.checkpoints, reverse=True):
                s1 = min(s0 + self.k, self.steps)
                if s0 != self.taped or len(self.tape) != s1 - s0:
                    buf = self.checkpoints[s0]
                    self.fluid.load_state_device(buf.data_ptr(), buf.numel())
                    self.tape.clear()
                    for s in range(s0, s1):
                        if self.plog is not None:
                            self.fluid.step_replay(self.plog[s].data_ptr(), self.tape)
                        else:
                            self.tape.record()
                self.taped = None
                for _ in range(s0, s1):
                    gg = self.tape.adjoint(g_out.data_ptr(), g_in.data_ptr(), self.adj_cg_iters, self.adj_cg_tol)
                    self.adj_cg_iterations.append(self.tape.last_stats()["cg_iterations"])
                    g_grav += np.asarray(gg, np.float64)
                    g_out, g_in = g_in, g_out
        self._leave()
        return g_out, g_grav


class RolloutFunction(torch.autograd.Function):
    """(initial velocity (N,3), gravity (3,)) -> final positions (N,3), rows by
    particle id.  Initial positions are fixed (ctx input).  Device-resident."""

    @staticmethod
    def forward(ctx, vel0, gravity, pos0, rollout):
        n = pos0.shape[0]
        parts = torch.zeros((n, 8), dtype=torch.float32, device=vel0.device)
        parts[:, 0:3] = pos0.detach()
        parts[:, 4:7] = vel0.detach()
        final, ids = rollout.forward(parts, gravity.detach().cpu().numpy())
        ctx.rollout = rollout
        ctx.save_for_backward(ids)
        out = torch.empty((n, 3), dtype=torch.float32, device=vel0.device)
        out[ids] = final[:, 0:3]
        return out

    @staticmethod
    def backward(ctx, g_pos):
        (ids,) = ctx.saved_tensors
        gf = torch.zeros((ids.numel(), 8), dtype=torch.float32, device=g_pos.device)
        gf[:, 0:3] = g_pos[ids]
        g0, g_grav = ctx.rollout.backward(gf)
        dvel = g0[:, 4:7].contiguous()
        dgrav = torch.tensor(g_grav, dtype=g_pos.dtype, device=g_pos.device)
        return dvel, dgrav, None, None


def com_loss(final_pos, target):
    """Squared distance of the particle centre of mass to `target`."""
    return ((final_pos.mean(dim=0) - target) ** 2).sum()
