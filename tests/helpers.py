"""Shared helpers of the test suite (oracle runs, digests, id ordering)."""
import hashlib

import numpy as np

from fluidgb import scenes


def run(oracle, name="dam32", steps=5, variant="f32", threads=0, **kw):
    """Run the CPU oracle on a named workload; returns (particles, ids), grid, bins, stats."""
    p, parts, spec = scenes.workload(name, **kw)
    oracle.set_threads(threads)
    o = oracle.OracleFluid(p, parts.shape[0], variant)
    o.set_particles(parts)
    o.step(steps)
    out = o.get_particles(), o.get_grid(), o.get_bins(), o.stats()
    o.close()
    oracle.set_threads(0)
    return out


def by_id(parts, ids):
    """Rows reordered so that row i is the particle with id i."""
    out = np.empty_like(parts)
    out[ids] = parts
    return out


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()
