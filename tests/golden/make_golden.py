"""Write tests/golden/oracle_digests.json: SHA-256 digests of the CPU oracle's
outputs for small seeded workloads.  The tests recompute them on whatever host
they run on (the oracle is built -ffp-contract=off, so x86-64 and aarch64 must
agree bit for bit) and the GPU tests compare the CUDA path to the same oracle.

Run from the repository root:  python tests/golden/make_golden.py
"""
import json
import os
import sys

REPO = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [os.path.join(REPO, "fluid-simulation_gb300"), os.path.join(REPO, "oracle"), os.path.join(REPO, "tests")]

import oracle  # noqa: E402
from helpers import digest, run  # noqa: E402

CASES = [
    dict(name="dam32_f32_3", workload="dam32", steps=3, variant="f32"),
    dict(name="dam32_f32_cg64_3", workload="dam32", steps=3, variant="f32", overrides=dict(precision=1)),
    dict(name="dam32_f64_2", workload="dam32", steps=2, variant="f64"),
    dict(name="block64_f32_1", workload="block64", steps=1, variant="f32"),
]


def main():
    oracle.load()
    out = []
    for c in CASES:
        (x, ids), g, (counts, offsets, perm), st = run(oracle, name=c["workload"], steps=c["steps"],
                                                       variant=c["variant"], **c.get("overrides", {}))
        d = dict(c)
        d.update(particles=digest(x, ids), grid=digest(g["u"], g["v"], g["w"], g["pressure"]),
                 bins=digest(counts, offsets, perm), cg_iterations=int(st["cg_iterations"]))
        out.append(d)
        print(c["name"], d["particles"][:16], st["cg_iterations"])
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_digests.json")
    with open(path, "w") as f:
        json.dump({"generator": "tests/golden/make_golden.py", "cases": out}, f, indent=1)


if __name__ == "__main__":
    main()
