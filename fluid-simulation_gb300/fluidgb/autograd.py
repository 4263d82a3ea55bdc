"""Differentiable rollouts through the C ABI's adjoint (fl_step_record /
fl_step_adjoint), wrapped in a torch.autograd.Function.

The forward pass runs `steps` substeps and keeps a checkpoint (particles, ids,
warm-start pressure: fl_save_state) every `checkpoint_every` substeps.  The
backward pass walks the segments in reverse: it restores a segment's
checkpoint, recomputes the segment while recording a tape (the recomputation
is bit-identical to the forward), then pops the tape step by step through the
adjoint kernels.  Memory: one tape of `checkpoint_every` substeps plus the
checkpoints.

Gradients are taken with respect to the initial per-particle state and the
gravity (body-force) vector, as in the differentiable-rollout workload:
`loss = |mean(final positions) - target|^2`, d loss / d(initial velocity, gravity).
"""
import numpy as np
import torch

from ._abi import Fluid


class Rollout:
    def __init__(self, params, capacity, steps, checkpoint_every=10, adj_cg_iters=1000, adj_cg_tol=1e-6):
        self.fluid = Fluid(params, capacity)
        self.params = params.copy()
        self.steps = int(steps)
        self.k = max(1, int(checkpoint_every))
        self.adj_cg_iters = adj_cg_iters
        self.adj_cg_tol = adj_cg_tol
        self.tape = self.fluid.tape(self.k)
        self.checkpoints = {}

    def close(self):
        self.tape.close()
        self.fluid.close()

    def forward(self, particles0, gravity):
        """particles0: (N, 8) float32 array (input order).  Returns the final
        particles (N, 8) and their ids (input slots)."""
        p = self.params.copy()
        p.grav[0], p.grav[1], p.grav[2] = (float(g) for g in gravity)
        p.phys[0] = p.grav[1]
        self.fluid.set_params(p)
        self.fluid.set_particles(np.ascontiguousarray(particles0, np.float32))
        self.checkpoints = {}
        for s in range(self.steps):
            if s % self.k == 0:
                self.checkpoints[s] = self.fluid.save_state()
            self.fluid.step(1)
        return self.fluid.get_particles()

    def backward(self, g_final, final_ids):
        """g_final: dL/d(final particles) (N, 8) in the order returned by
        forward.  Returns dL/d(particles0) (N, 8) in input order and dL/dgravity."""
        dev = torch.device("cuda")
        g_out = torch.from_numpy(np.ascontiguousarray(g_final, np.float32)).to(dev)
        g_in = torch.empty_like(g_out)
        g_grav = np.zeros(3, np.float64)
        starts = sorted(self.checkpoints)
        for s0 in reversed(starts):
            s1 = min(s0 + self.k, self.steps)
            self.fluid.load_state(self.checkpoints[s0])
            self.tape.clear()
            for _ in range(s0, s1):
                self.tape.record()
            torch.cuda.synchronize()
            for _ in range(s0, s1):
                gg = self.tape.adjoint(g_out.data_ptr(), g_in.data_ptr(), self.adj_cg_iters, self.adj_cg_tol)
                g_grav += np.asarray(gg, np.float64)
                g_out, g_in = g_in, g_out
        return g_out.cpu().numpy(), g_grav


class RolloutFunction(torch.autograd.Function):
    """(initial velocity (N,3), gravity (3,)) -> final positions (N,3), rows by
    particle id.  Initial positions are fixed (ctx input)."""

    @staticmethod
    def forward(ctx, vel0, gravity, pos0, rollout):
        n = pos0.shape[0]
        parts = np.zeros((n, 8), np.float32)
        parts[:, 0:3] = pos0.detach().cpu().numpy()
        parts[:, 4:7] = vel0.detach().cpu().numpy()
        final, ids = rollout.forward(parts, gravity.detach().cpu().numpy())
        ctx.rollout = rollout
        ctx.ids = ids
        out = np.empty((n, 3), np.float32)
        out[ids] = final[:, 0:3]
        return torch.from_numpy(out).to(vel0.device)

    @staticmethod
    def backward(ctx, g_pos):
        ids = ctx.ids
        g = g_pos.detach().cpu().numpy()
        gf = np.zeros((ids.size, 8), np.float32)
        gf[:, 0:3] = g[ids]
        g0, g_grav = ctx.rollout.backward(gf, ids)
        dvel = torch.from_numpy(np.ascontiguousarray(g0[:, 4:7])).to(g_pos.device)
        dgrav = torch.tensor(g_grav, dtype=g_pos.dtype, device=g_pos.device)
        return dvel, dgrav, None, None


def com_loss(final_pos, target):
    """Squared distance of the particle centre of mass to `target`."""
    return ((final_pos.mean(dim=0) - target) ** 2).sum()
