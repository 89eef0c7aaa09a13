"""Per-launch device time and algorithmic bytes of the FIM patch kernel.

    python sci-solver_level-set_gb300/launch_profile.py [--n 96] [--steps 1] [--launches 4]

Builds the curvature-flow workload of the benchmark at n^3 cells (seeded
jittered cube, three spheres, 3x3x3-vertex patches), turns per-kernel
profiling on before the first step and runs `steps` time steps kernel by
kernel.  It prints one line per FIM launch (the first `launches` of them,
all when 0): kind (sweep / check), device time from CUDA events on the
library's stream, and the algorithmic slab bytes of the patch visits and
checks that launch ran, then their sums.

No FIM kernel runs before the first profiled step and a step's FIM work is
deterministic, so the FIM launches that `ncu -k regex:k_fim -c <launches>`
captures on this same command are the ones printed here: their DRAM bytes
(dram__bytes_read.sum + dram__bytes_write.sum) compare directly with the
printed algorithmic bytes.
"""
import argparse
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import lsgb300  # noqa: E402
import synth  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=96, help="cells per side")
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--launches", type=int, default=4, help="FIM launches to print (0: all)")
    args = ap.parse_args()
    w = synth.workload("c3", seed=0, n=args.n)
    ls = lsgb300.from_workload(w)
    ls.set_profile(True)
    ls.reset_stats()
    ls.step(args.steps)
    kinds, ms, nbytes = ls.launch_log()
    k = len(kinds) if args.launches <= 0 else min(args.launches, len(kinds))
    for i in range(k):
        print(json.dumps({"launch": i, "kind": "sweep" if kinds[i] == 0 else "check",
                          "ms": round(float(ms[i]), 5), "algorithmic_bytes": int(nbytes[i]),
                          "gb_per_s": round(float(nbytes[i]) / (float(ms[i]) * 1e6), 1) if ms[i] > 0 else None}))
    print(json.dumps({"workload": "c3 curvature flow %d^3 cells" % w["n"], "fim_launches_total": int(len(kinds)),
                      "printed": k, "sum_ms": round(float(ms[:k].sum()), 5),
                      "sum_algorithmic_bytes": int(nbytes[:k].sum())}))
    ls.close()


if __name__ == "__main__":
    main()
