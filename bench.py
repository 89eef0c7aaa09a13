#!/usr/bin/env python
"""Benchmark of the narrowband level-set time step on GB300.

Workload (default): 128^3-cell jittered Freudenthal cube (2,146,689 vertices,
12,582,912 tetrahedra), union of 3 seeded spheres, mean-curvature flow with
dt = 0.5 h^2, narrowband 6h, 3x3x3-vertex patches (79,507 patches).  A step is
one time step: seed search, fast-iterative-method redistance of the
narrowband, narrowband selection, curvature update.

Metric: narrowband vertex-updates per second, one update = one vertex with
|phi| <= w after the step's redistance.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With --gpus N > 1 (launched by torch.distributed.run) every rank runs an
independent replica of the workload (the time step does not shard: the
wavefront couples neighbouring patches in every FIM iteration); the timed region is bracketed by a barrier and the maximum time
over ranks is reported.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "sci-solver_level-set_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import numpy as np  # noqa: E402

METRIC = "narrowband vertex-updates/s (curvature flow, 128^3 jittered cube, 3 spheres)"
UNIT = "vertex-updates/s"
# max |phi - phi_FP64| / h of the fast build over 3 steps of this workload,
# measured by the GPU test named in ACCURACY
C3_FAST_MAX_ERR_H = 9.44e-5


# the two kernel builds and what the GPU tests establish about their accuracy
BUILDS = {
    "fast": "fast: FMA contraction, approximate division and square root, planar-wave tet solver",
    "bit-exact": "bit-exact: no FMA contraction, the reference's tet solver in its operand order",
}
ACCURACY = {
    # printed per step by the test (3 curvature steps of this workload,
    # against the CPU oracle run entirely in FP64)
    "fast": {"max_err_vs_fp64_h": C3_FAST_MAX_ERR_H,
             "source": "tests/test_gpu_configs.py::test_c3_curvature_128_cells_full_size (3 steps at 128^3, "
                       "max |phi - phi_FP64| over the band per step, asserted <= 1e-3 h)"},
    "bit-exact": {"equals_oracle_bitwise": True,
                  "source": "tests/test_gpu_configs.py::test_c3_curvature_128_cells_full_size (phi, narrowband "
                            "sets and work counters equal to the CPU oracle bit for bit over 2 steps at 128^3)"},
}


def job_totals(ms, updates, dist=None):
    """Whole-job timing over independent replicas: the slowest rank's time
    and the sum of all ranks' narrowband vertex-updates."""
    if dist is None:
        return ms, float(updates)
    import torch

    t = torch.tensor([ms, float(updates)], dtype=torch.float64)
    tmax = t.clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    tsum = t.clone()
    dist.all_reduce(tsum, op=dist.ReduceOp.SUM)
    return float(tmax[0]), float(tsum[1])


def env_rank():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread is not None:
            self.thread.join(timeout=2)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_value(key):
    """A figure of the committed ncu summary of the FIM kernel
    (profiles/k_fim_sweep_c3.md, lines "key: value"), or None."""
    path = os.path.join(ROOT, "profiles", "k_fim_sweep_c3.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.strip().startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


def profile_traffic(algorithmic_bytes_per_launch):
    """DRAM bytes per launch of the FIM kernel: the DRAM / algorithmic byte
    ratio of the committed ncu capture (the same launches' DRAM bytes and
    algorithmic bytes, launch_profile.py) times this run's algorithmic bytes
    per launch (the kernel reads a fixed slab per patch visit, so traffic
    grows with the visits), or None."""
    ratio = profile_value("traffic_ratio")
    if ratio is None:
        return None
    return ratio * algorithmic_bytes_per_launch


class OracleRun:
    """CPU oracle (the FP32 port of the reference's algorithm) on the same
    workload: warm-up steps once, then timed samples from the warm state
    with any thread count (each sample's first step seeds over all
    patches, as a fresh reference GenerateData call does)."""

    def __init__(self, w, warm, threads, precision=32):
        import lsoracle

        self.w = w
        self.ol = lsoracle.OracleLayout(w["dim"], w["xyz"], w["elems"], w["npart"], w["nparts"])
        self.kind = lsoracle.UPDATE[w["update"]]
        self.precision = precision
        self.phi = w["phi0"]
        if warm > 0:
            hist, _, _, _ = self.ol.solve(self._params(threads), w["phi0"], w["vel"], warm, nb_sets=False)
            self.phi = hist[-1]

    def _params(self, threads):
        w = self.w
        return self.ol.params(update_kind=self.kind, dt=w["dt"], bandwidth=w["bandwidth"], curv_coeff=1.0,
                              nthreads=threads, precision=self.precision)

    def rate(self, nsteps, threads):
        """(vertex-updates/s, seconds, stats) of nsteps timed steps."""
        t0 = time.perf_counter()
        _, _, _, st = self.ol.solve(self._params(threads), self.phi, self.w["vel"], nsteps, nb_sets=False)
        sec = time.perf_counter() - t0
        return st["nb_vertex_updates"] / sec, sec, st


def oracle_rate(w, nsteps, warm, threads, precision=32):
    """`warm` untimed steps then `nsteps` timed steps of the CPU oracle."""
    return OracleRun(w, warm, threads, precision).rate(nsteps, threads)


# wall-clock budget of the reference arm's timed steps (the oracle port takes
# about 1.2 s per 128^3 step on 16 Grace cores): the requested step count
# runs whole unless it would exceed this
REFERENCE_BUDGET_S = 180.0


def one_core_sample(run, per_step_s_multi, threads):
    """One step of the same oracle on one host core (the reference's own CPU
    code is single-threaded), from the same warm state."""
    rate1, sec1, _ = run.rate(1, 1)
    return {"value": rate1, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": "1 timed step of the full workload from the warm state, FP32 oracle port, 1 thread "
                      "(%.1f s; %d threads: %.2f s per step)" % (sec1, threads, per_step_s_multi)}


def run_reference_arm(args, w, rank):
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    warm = max(args.warmup, 0)
    t0 = time.perf_counter()
    run = OracleRun(w, warm, threads)
    warm_s = time.perf_counter() - t0
    # the requested steps, unless the measured warm-up rate says they would
    # exceed the budget
    per_step = warm_s / warm if warm > 0 else 0.0
    k = args.steps
    note = None
    if per_step > 0 and per_step * k > REFERENCE_BUDGET_S:
        k = max(1, int(REFERENCE_BUDGET_S / per_step))
        note = "%d of the %d requested steps: %.1f s per step would exceed the %.0f s budget" % (
            k, args.steps, per_step, REFERENCE_BUDGET_S)
    rate, sec, st = run.rate(k, threads)
    sample = "%d timed steps after %d warm-up step(s) of the full workload, FP32 oracle port, %d threads" % (
        k, warm, threads)
    cfg = {"workload": w["label"], "steps_requested": args.steps, "steps_run": k}
    if note:
        cfg["note"] = note
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus, "steps": k,
        "warmup": warm, "ms_per_step": 1000.0 * sec / k, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded jittered cube, sphere-union SDF)",
        "config": cfg,
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "cpu_baseline_1core": one_core_sample(run, sec / k, threads),
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_batched(args, rank, world, local):
    """64 independent jittered cubes (16..64 cells per side, log-uniform),
    advection by random rigid rotations, stepped as one batch (one patch set,
    one launch sequence per step) and, for comparison, one handle per mesh
    stepped in turn on the same GPU.  With --learned the batch runs with the
    learned warm start (network trained first, train_network), next to the
    plain batch."""
    import lsgb300
    import synth
    import torch

    if world > 1 and rank != 0:
        return 0
    torch.cuda.set_device(local)
    ws = synth.workload_batch(0)
    nv = sum(len(w["xyz"]) for w in ws)
    ne = sum(len(w["elems"]) for w in ws)
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")
    net, training = (train_network(args.n) if args.learned else (None, None))

    # patch side and FIM setting tuned over the whole batch (2 timed steps per
    # candidate); the timed batches use the pick
    tb = lsgb300.LevelSetBatch()
    for w in ws:
        tb.add(lsgb300.from_workload(w, setup=False, structured_block=3))
    trials, best = tb.autotune(2)
    tb.close()
    pick = trials[best]
    tune = {"patch_side_vertices": pick["patch_size"], "fim_ctas_per_sm": pick["fim_ctas_per_sm"],
            "trials": [[t["patch_size"], t["fim_ctas_per_sm"], round(t["ms_per_step"], 3)] for t in trials]}

    def run_batch(learned):
        b = lsgb300.LevelSetBatch()
        for w in ws:
            b.add(lsgb300.from_workload(w, setup=False, structured_block=pick["patch_size"],
                                        fim_ctas_per_sm=pick["fim_ctas_per_sm"]))
        b.setup()
        if learned:
            b.set_learned(net, margin=0.3, reset_mode=0)
        for _ in range(args.warmup):
            b.solve(1)
        b.reset_stats()
        clocks = ClockSampler(local)
        clocks.start()
        ms = 0.0
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            before = b.stats()["ms_total"]
            b.solve(1)
            ms += b.stats()["ms_total"] - before
        clocks.stop()
        st = b.stats()
        phis = [b.phi(i) for i in range(len(ws))]
        b.close()
        return ms, st, clocks.summary(), phis

    learned_part = None
    if args.learned:
        ms_l, st_l, clk_l, ph_l = run_batch(True)
    ms, st, clk, ph = run_batch(False)
    value = st["nb_vertex_updates"] / (ms / 1000.0)
    if args.learned:
        value_l = st_l["nb_vertex_updates"] / (ms_l / 1000.0)
        diff = 0.0
        for w, a, c in zip(ws, ph_l, ph):
            band = np.abs(c) <= w["bandwidth"]
            if band.any():
                diff = max(diff, float(np.max(np.abs(a[band] - c[band])) / w["h"]))
        learned_part = {"value": value_l, "unit": UNIT, "ms_per_step": ms_l / args.steps, "clocks": clk_l,
                        "training": training, "warm_vertices": st_l["warm_vertices"],
                        "moved_beyond_1e-3h": st_l["moved_vertices"], "unsupported_resets": st_l["unsupported_resets"],
                        "support_rounds": st_l["support_rounds"], "fallbacks_to_plain": st_l["learned_fallbacks"],
                        "patch_visits_per_step": st_l["patch_visits"] / args.steps,
                        "learned_batched_over_plain_batched": value_l / value,
                        "max_abs_diff_vs_plain_h": diff}
    # the same meshes one handle at a time (the reference's one-mesh-per-solver use)
    seq_ms, seq_updates = 0.0, 0
    for w in ws:
        ls = lsgb300.from_workload(w, structured_block=pick["patch_size"], fim_ctas_per_sm=pick["fim_ctas_per_sm"])
        for _ in range(args.warmup):
            ls.step(1)
        ls.reset_stats()
        for _ in range(args.steps):
            ls.step(1)
        s = ls.stats()
        seq_ms += s["ms_total"]
        seq_updates += s["nb_vertex_updates"]
        ls.close()
    seq_value = seq_updates / (seq_ms / 1000.0)
    line = {
        "metric": "narrowband vertex-updates/s (batched advection, 64 jittered cubes 16..64 cells per side)",
        "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (seeded jittered cubes, 1-3 sphere unions, random rigid rotations)",
        "config": {"workload": "c5 batch of %d meshes (%d verts, %d tets), w=5h, CFL 0.5" % (len(ws), nv, ne),
                   "autotune": tune,
                   "l2": "flushed between timed steps (256 MB write)", "parallelism": "single GPU",
                   "fim_iters_per_step": st["fim_iters"] / args.steps,
                   "patch_visits_per_step": st["patch_visits"] / args.steps,
                   "nb_patches_per_step": st["nb_patches"] / args.steps},
        "sequential": {"value": seq_value, "unit": UNIT, "ms_per_step": seq_ms / args.steps,
                       "how": "one handle per mesh, meshes stepped in turn, same steps"},
        "batched_over_sequential": value / seq_value,
        "learned": learned_part,
        "clocks": clk,
        "e2e": None,
        "gpu_launches": int(st["kernel_launches"]),
    }
    print(json.dumps(line), flush=True)
    return 0


# training pairs (features of a vertex before the redistance, its signed
# distance / h after it) from this project's own FIM: seeded runs of the
# 3D-advection and curvature-flow families, other seeds than the benchmark's
PAIR_SOURCES = (  # (family, cells per side, seed, pairs to collect)
    ("c3", 128, 1, 9_000_000), ("c3", 128, 2, 9_000_000), ("c2", 32, 3, 1_500_000), ("c2", 32, 4, 1_500_000))
PAIR_CAPACITY = 24 * 1024 * 1024
TRAIN_EPOCHS, TRAIN_BATCH, TRAIN_LR = 20, 65536, 1e-3


def train_network(n_eval):
    """Collects about 21 M training pairs (PAIR_SOURCES), trains the network
    on the GPU (Adam, batch 65,536), and measures its error on pairs of the
    benchmark workload (seed 0, n_eval^3 cells) that it was not trained on."""
    import lsgb300
    import synth

    m = lsgb300.MLP(11)
    m.reserve_pairs(PAIR_CAPACITY)
    t0 = time.perf_counter()
    sources = []
    for name, n, seed, quota in PAIR_SOURCES:
        ls = lsgb300.from_workload(synth.workload(name, n=n, seed=seed))
        start = m.num_pairs()
        steps = 0
        while m.num_pairs() - start < quota and steps < 100:
            ls.learn_collect(m, 4)
            steps += 4
        sources.append({"workload": "%s %d^3 seed %d" % (name, n, seed), "steps": steps,
                        "pairs": m.num_pairs() - start})
        ls.close()
    collect_s = time.perf_counter() - t0
    npairs = m.num_pairs()
    t0 = time.perf_counter()
    loss = m.train_pairs(epochs=TRAIN_EPOCHS, batch=TRAIN_BATCH, lr=TRAIN_LR, seed=1)
    train_s = time.perf_counter() - t0
    # held-out error: pairs of the benchmark workload, appended after training
    first = m.num_pairs()
    ls = lsgb300.from_workload(synth.workload("c3", n=n_eval, seed=0))
    ls.learn_collect(m, 4)
    ls.close()
    err = m.eval_pairs(first, m.num_pairs() - first)
    q = lambda x: float(np.quantile(err, x)) if err.size else None  # noqa: E731
    info = {"pairs": npairs, "sources": sources, "collect_s": collect_s, "train_s": train_s,
            "epochs": TRAIN_EPOCHS, "batch": TRAIN_BATCH, "lr": TRAIN_LR, "last_epoch_loss": loss,
            "batches": TRAIN_EPOCHS * ((npairs + TRAIN_BATCH - 1) // TRAIN_BATCH),
            "ms_per_batch": 1000.0 * train_s / max(1, TRAIN_EPOCHS * ((npairs + TRAIN_BATCH - 1) // TRAIN_BATCH)),
            "held_out": {"workload": "c3 %d^3 seed 0, 4 steps" % n_eval, "pairs": int(err.size),
                         "abs_err_h": {"p50": q(0.5), "p90": q(0.9), "p99": q(0.99),
                                       "max": float(err.max()) if err.size else None},
                         "frac_within_h": {"1e-3": float((err <= 1e-3).mean()) if err.size else None,
                                           "1e-2": float((err <= 1e-2).mean()) if err.size else None,
                                           "1e-1": float((err <= 1e-1).mean()) if err.size else None}}}
    return m, info


def run_learned(args, rank, world, local):
    """The curvature-flow workload with the learned warm start: the network
    trained on the GPU (train_network), then timed steps at --n cells per
    side with the warm start (margin 0.3 h, whole-patch resets) next to the
    same steps of the plain path."""
    import lsgb300
    import synth
    import torch

    if world > 1 and rank != 0:
        return 0
    torch.cuda.set_device(local)
    m, training = train_network(args.n)
    w = synth.workload("c3", seed=0, n=args.n)
    nv = len(w["xyz"])
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    def timed(learned):
        ls = lsgb300.from_workload(w)
        if learned:
            ls.set_learned(m, margin=0.3, reset_mode=0)
        for _ in range(args.warmup):
            ls.step(1)
        ls.reset_stats()
        ms = 0.0
        phis = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            before = ls.stats()["ms_total"]
            ls.step(1)
            ms += ls.stats()["ms_total"] - before
            phis.append(ls.phi())
        st = ls.stats()
        ls.close()
        return ms, st, np.array(phis)

    ms_l, st_l, ph_l = timed(True)
    ms_p, st_p, ph_p = timed(False)
    band = np.abs(ph_p) <= w["bandwidth"]
    err = np.abs(ph_l - ph_p)[band] / w["h"]
    value = st_l["nb_vertex_updates"] / (ms_l / 1000.0)
    plain = st_p["nb_vertex_updates"] / (ms_p / 1000.0)
    line = {
        "metric": "narrowband vertex-updates/s (curvature flow with the learned warm start, %d^3 jittered cube)"
                  % w["n"],
        "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_l / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 (network bf16, fp32 accumulate)", "data": "synthetic (seeded jittered cube, sphere-union SDF)",
        "config": {"workload": "c4 learned warm start on c3 %d^3 (%d verts)" % (w["n"], nv),
                   "l2": "flushed between timed steps (256 MB write)",
                   "training": training,
                   "warm_vertices": st_l["warm_vertices"], "moved_beyond_1e-3h": st_l["moved_vertices"],
                   "unsupported_resets": st_l["unsupported_resets"], "support_rounds": st_l["support_rounds"],
                   "fallbacks_to_plain": st_l["learned_fallbacks"],
                   "patch_visits": st_l["patch_visits"], "check_visits": st_l["check_visits"]},
        "plain": {"value": plain, "ms_per_step": ms_p / args.steps, "patch_visits": st_p["patch_visits"],
                  "check_visits": st_p["check_visits"]},
        "learned_over_plain": value / plain,
        "max_abs_diff_vs_plain_h": float(err.max()) if err.size else 0.0,
        "e2e": None,
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=128, help="cells per side (128 = the benchmark workload)")
    ap.add_argument("--fp64-flagged", action="store_true", help="precision form")
    ap.add_argument("--bit-exact", action="store_true",
                    help="the bit-exact kernel build (no FMA contraction, the reference's tet solver), which "
                         "equals the CPU oracle bit for bit")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ctas", type=int, default=0, help="FIM CTAs per SM (2, 3, 4; 5 = two element copies per thread; 0 = library default)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep 3x3x3-vertex patches and the default FIM CTAs per SM instead of the autotuner's pick")
    ap.add_argument("--learned", action="store_true",
                    help="c5: also run the batch with the learned warm start (the network is trained first)")
    ap.add_argument("--workload", default="c3", choices=["c3", "c4", "c5"],
                    help="c3: the 128^3 curvature-flow benchmark; c4: the same with the learned warm start; "
                         "c5: 64 independent meshes as one batch")
    args = ap.parse_args()
    rank, world, local = env_rank()
    if args.workload == "c5":
        return run_batched(args, rank, world, local)
    if args.workload == "c4":
        return run_learned(args, rank, world, local)

    import synth

    w = synth.workload("c3", seed=0, n=args.n)
    w["label"] = "c3 curvature flow %d^3 cells x 6 tets (%d verts, %d tets), w=6h, dt=0.5h^2" % (
        w["n"], len(w["xyz"]), len(w["elems"]))
    if args.impl == "reference":
        return run_reference_arm(args, w, rank)

    import lsgb300
    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist_mod

        dist_mod.init_process_group("gloo")
        dist = dist_mod
    torch.cuda.set_device(local)
    extra = {"fim_ctas_per_sm": args.ctas} if args.ctas else {}
    tune = None
    if args.no_autotune:
        ls = lsgb300.from_workload(w, fp64_flagged=args.fp64_flagged, bit_exact=args.bit_exact, **extra)
    else:
        # structured blocks of a tuned side (the autotuner times 2 steps per
        # candidate patch size and CTAs-per-SM setting, from phi0)
        flags = (lsgb300.FP64_FLAGGED if args.fp64_flagged else 0) | (lsgb300.BITEXACT if args.bit_exact else 0)
        p = lsgb300.default_params(time_step=w["dt"], bandwidth=w["bandwidth"], update_kind=lsgb300.UPDATE_CURVATURE,
                                   curv_coeff=1.0, partition_type=1, side_lengths=w["n"] + 1, block_size=3,
                                   flags=flags, **extra)
        ls = lsgb300.LevelSet(False, p)
        ls.set_mesh(w["xyz"], w["elems"])
        ls.set_phi(w["phi0"])
        ls.set_velocity(w["vel"])
        trials, best = ls.autotune(2)
        tp = ls.get_params()
        tune = {"patch_side_vertices": tp.block_size, "fim_ctas_per_sm": tp.fim_ctas_per_sm,
                "trials": [[t["patch_size"], t["fim_ctas_per_sm"], round(t["ms_per_step"], 3)] for t in trials]}
    nv = len(w["xyz"])
    # L2 flush buffer (larger than the 129 MB L2), written between timed steps
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    for _ in range(args.warmup):
        ls.step(1)
    ls.reset_stats()
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    ms = 0.0
    launched = 0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        before = ls.stats()["ms_total"]
        launched += ls.step(1)
        ms += ls.stats()["ms_total"] - before
    barrier()
    clocks.stop()
    st = ls.stats()
    updates = st["nb_vertex_updates"]
    ms_job, updates_job = job_totals(ms, updates, dist)
    value = updates_job / (ms_job / 1000.0)
    # our kernels launched inside the timed region (graph kernels included)
    gpu_launches = int(st["kernel_launches"])

    # end to end through the C ABI with host buffers: phi in (host) -> step -> phi out (host)
    phi_h = ls.phi()
    out_h = np.empty_like(phi_h)
    # one untimed step through the same host buffers first: the output
    # array's pages are then populated, as in a caller that reuses its buffers
    ls.step_host(phi_h, out_h)
    phi_h, out_h = out_h, phi_h
    e2e_steps = max(1, min(args.steps, 10))
    before = ls.stats()["nb_vertex_updates"]
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ls.step_host(phi_h, out_h)
        phi_h, out_h = out_h, phi_h
    barrier()
    e2e_sec = time.perf_counter() - t0
    e2e_updates = ls.stats()["nb_vertex_updates"] - before
    e2e_value = e2e_updates / e2e_sec

    # roofline of the dominant kernel (FIM patch sweep): per-launch
    # algorithmic slab bytes / per-launch device time, CUDA events on the
    # library's stream around each sweep launch
    ls.set_profile(True)
    ls.reset_stats()
    prof_steps = 2
    ls.step(prof_steps)
    ps = ls.stats()
    ls.set_profile(False)
    peak, peak_kind = load_peaks()
    # the FIM patch kernel: sweep launches and neighbour-check launches (a
    # check that activates its patch runs the patch's visit in the same launch)
    fim_launches = max(ps["n_sweep"] + ps["n_check"], 1)
    sweep_ms = (ps["ms_sweep"] + ps["ms_check"]) / fim_launches
    bytes_per_launch = ps["sweep_slab_bytes"] / fim_launches
    achieved = bytes_per_launch / (sweep_ms / 1000.0) / 1e9 if sweep_ms > 0 else 0.0
    step_ms_prof = (ps["ms_sweep"] + ps["ms_check"] + ps["ms_schedule"] + ps["ms_seed"] + ps["ms_narrowband"]
                    + ps["ms_update"])
    kernel_ms = {k: ps["ms_" + k] / prof_steps for k in ("sweep", "check", "schedule", "seed", "narrowband", "update")}
    # the sweep kernel the run used: two element copies per thread at the
    # setting 5 (patches of up to 384 copies), one per thread otherwise
    sweep_kernel = "k_fim_pair" if ls.get_params().fim_ctas_per_sm == 5 else "k_fim_compact"
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": profile_traffic(bytes_per_launch),
                "kernel": sweep_kernel + " (FIM patch sweep and check launches)",
                "traffic_source": "this run's algorithmic bytes per launch x the DRAM/algorithmic ratio of an ncu "
                                  "capture (dram__bytes_read.sum + dram__bytes_write.sum) of this kernel build's "
                                  "first FIM launches at 96^3, profiles/k_fim_sweep_c3.md",
                "traffic_ratio": profile_value("traffic_ratio"),
                "peak_source": peak_kind,
                "share_of_step": ((ps["ms_sweep"] + ps["ms_check"]) / step_ms_prof) if step_ms_prof > 0 else None,
                "algorithmic_bytes_per_launch": bytes_per_launch, "avg_launch_ms": sweep_ms,
                # the FIM kernel is bound by instruction issue of the local
                # solvers, not by HBM: issue slots active from the committed
                # ncu capture of its sweep and check launches
                "limiter": "SM instruction issue (FP32/ALU/MUFU of the local solvers); DRAM at 4-13 % of peak",
                "issue_slots_active": profile_value("issue_slots_active")}

    cpu = None
    cpu1 = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        run = OracleRun(w, 1, threads)
        rate, sec, _ = run.rate(2, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "2 timed steps after 1 warm-up step of the full workload, FP32 oracle port (%.1f s)" % sec}
        cpu1 = one_core_sample(run, sec / 2, threads)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_job / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" + ("+f64flagged" if args.fp64_flagged else ""),
            "data": "synthetic (seeded jittered cube, sphere-union SDF)",
            "config": {"workload": w["label"], "l2": "flushed between timed steps (256 MB write)",
                       "parallelism": "replicas" if world > 1 else "single GPU",
                       "fim_iters_per_step": st["fim_iters"] / args.steps,
                       "patch_visits_per_step": st["patch_visits"] / args.steps,
                       "check_visits_per_step": st["check_visits"] / args.steps,
                       "nb_patches_per_step": st["nb_patches"] / args.steps,
                       "flagged_fp64_solves": st["flagged_copies"],
                       "kernel_ms_per_step_profiled": kernel_ms,
                       "patch_side_vertices": ls.get_params().block_size,
                       "build": BUILDS["bit-exact" if args.bit_exact else "fast"],
                       "accuracy": ACCURACY["bit-exact" if args.bit_exact else "fast"],
                       "autotune": tune},
            "clocks": clocks.summary(),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": 4 * nv, "d2h_bytes_per_step": 4 * nv,
                    "steps": e2e_steps},
            "gpu_launches": gpu_launches,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "cpu_baseline_1core": cpu1,
        }
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
