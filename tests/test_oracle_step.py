"""Step-level properties of the CPU oracle (CPU only).

The oracle restates the reference step (binning -> P2G -> classify -> forces /
boundaries -> divergence -> CG -> projection -> G2P).  These tests check the
properties the GPU parity tests rely on: determinism for any thread count,
agreement of the f32 and f64 variants, conservation and containment, and the
committed golden digests (so the oracle gives the same bits on every host).
"""
import json
import os

import numpy as np
import pytest

from fluidgb import scenes
from helpers import by_id, digest, run

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def test_thread_count_does_not_change_bits(oracle):
    (a, ia), ga, _, sa = run(oracle, steps=4, threads=1)
    (b, ib), gb, _, sb = run(oracle, steps=4, threads=4)
    assert np.array_equal(a, b) and np.array_equal(ia, ib)
    for k in ga:
        assert np.array_equal(ga[k], gb[k]), k
    assert sa["cg_iterations"] == sb["cg_iterations"]


def test_f32_and_f64_variants_agree(oracle):
    (a, ia), ga, _, _ = run(oracle, steps=5, variant="f32")
    (b, ib), gb, _, _ = run(oracle, steps=5, variant="f64")
    pa, pb = by_id(a, ia), by_id(b, ib)
    # 5 steps of 1/120 s: positions agree to well under a cell (h = 1/32)
    assert np.abs(pa[:, :3] - pb[:, :3]).max() < 1e-3
    assert np.abs(pa[:, 4:7] - pb[:, 4:7]).max() < 5e-2


def test_particles_conserved_and_inside_walls(oracle):
    (x, ids), g, (counts, offsets, perm), st = run(oracle, steps=6)
    n = x.shape[0]
    assert np.array_equal(np.sort(ids), np.arange(n, dtype=np.uint32))
    h = 1.0 / 32
    lo, hi = np.float32(0 + h * 1.05), np.float32(1 - h * 1.05)
    assert x[:, :3].min() >= lo - 1e-7 and x[:, :3].max() <= hi + 1e-7
    assert counts.sum() == n
    assert np.array_equal(offsets, np.concatenate([[0], np.cumsum(counts)[:-1]]).astype(np.uint32))
    assert np.array_equal(np.sort(perm), np.arange(n, dtype=np.uint32))
    assert st["liquid_cells"] > 0 and st["cg_iterations"] == 40


def test_projection_reduces_divergence(oracle):
    p, parts, _ = scenes.workload("dam32", tol=0.0)
    o = oracle.OracleFluid(p, parts.shape[0])
    o.set_particles(parts)
    o.step(3)
    st = o.stats()
    assert st["rs_final"] < 1e-3 * st["rs_initial"]


def test_impulse_and_reset(oracle):
    p, parts, _ = scenes.workload("dam32")
    o = oracle.OracleFluid(p, parts.shape[0])
    o.set_particles(parts)
    o.apply_impulse([0.5, 0.0, -0.25])
    x, _ = o.get_particles()
    assert np.allclose(x[:, 4], parts[:, 4] + 0.5) and np.allclose(x[:, 6], parts[:, 6] - 0.25)
    o.step(2)
    o.reset()
    y, ids = o.get_particles()
    assert np.array_equal(y, parts) and np.array_equal(ids, np.arange(parts.shape[0], dtype=np.uint32))


@pytest.mark.parametrize("case", json.load(open(os.path.join(GOLDEN, "oracle_digests.json")))["cases"]
                         if os.path.exists(os.path.join(GOLDEN, "oracle_digests.json")) else [],
                         ids=lambda c: c["name"])
def test_oracle_matches_committed_golden_digest(oracle, case):
    """tests/golden/make_golden.py wrote these on the development host; the
    same bits must come out on any host (x86-64 or aarch64)."""
    (x, ids), g, (counts, offsets, perm), st = run(oracle, name=case["workload"], steps=case["steps"],
                                                   variant=case["variant"], **case.get("overrides", {}))
    assert digest(x, ids) == case["particles"]
    assert digest(g["u"], g["v"], g["w"], g["pressure"]) == case["grid"]
    assert digest(counts, offsets, perm) == case["bins"]
    assert st["cg_iterations"] == case["cg_iterations"]
