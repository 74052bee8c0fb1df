"""Generates tests/golden/op_counts.json: the algorithmic FP32 work of each benchmark workload.

For the three single-mesh workloads (sphere16k, torus262k, star1310k) it records, per test class
(sat1, ray1, sat2, ray2), the number of tests the work counts define and the FP32 operations the
reference's predicates execute on them, early exits included (oracle.Run.count_ops).  The
benchmark reads the per-test averages to state the algorithmic operations of a launch.

Run: `python tests/golden/make_op_counts.py` (a few seconds to a minute on a multicore host).
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))


def counts(cfg, threads=0):
    from oracle import oracle as orc

    import workloads as W

    tris, spec = W.make(cfg)
    run = orc.Run(tris, spec, fill=orc.FILL_CAND, threads=threads)
    _, s2, r2 = run.level2_state(0, run.B, threads)
    tests = {"sat1": run.sat1_tests(), "ray1": run.ray1_candidates(), "sat2": s2, "ray2": r2}
    ops = run.count_ops(0, run.B, threads)
    return {k: {"tests": int(tests[k]), "ops": int(ops[k])} for k in tests}


def main():
    import workloads as W

    out = {"what": "FP32 add/sub/mul/div executed by the reference predicates over the algorithmic "
                   "tests (early exits included); per-exit counts in oracle/gpv_oracle.c"}
    for cfg in (W.C1, W.C2, W.C3):
        out[cfg["name"]] = counts(cfg)
        print(cfg["name"], out[cfg["name"]], flush=True)
    with open(os.path.join(HERE, "op_counts.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
