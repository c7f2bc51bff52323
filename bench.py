"""Benchmark of the Barnes-Hut gravity step: particle-steps/s at N = 1,048,576, theta = 0.5.

Workload: a major merger of two disk + bulge + NFW-halo galaxies of 524,288 particles each
(seeded synthetic stand-in, gravitas_gb300.ics.merger), theta 0.5 with quadrupoles, softening
0.02, global KDK steps of dt = 1e-3 (kick, drift, tree build, walk, kick). One step advances all
N particles. The leaf size (and the mixed walk's group size) of each walk is chosen first by the
library's autotuner (gbh_autotune) at theta 0.5 for the shortest force evaluation with RMS force
error <= 2e-3; --leaf fixes it instead.

  value       mixed walk (warp-cooperative FP32 + compensated sums, FP64 state), state resident
              in HBM, device time of K steps from CUDA events on the library's stream, L2
              flushed (256 MiB write) between steps
  e2e         the same step through gbh_step_kdk with pinned host buffers: state copied in and
              out inside every timed step (wall clock)
  plain       the same step with the plain all-FP32 walk (the CUDA twin of the Metal kernel)
  roofline    the walk kernel: algorithmic FLOP (50 per accepted quadrupole node, 18 per leaf
              pair, 8 per opened node, counted by the reference per-star walk of the CPU oracle)
              per launch / its CUDA-event duration, against this GPU's FP32 FMA peak measured
              in the same run
  errors      RMS and p99 relative force error of both walks against the FP64 direct sum on
              4,096 seeded targets
  cpu_baseline  the CPU restatement of the reference step at the mixed walk's leaf size, best of
              5 single steps on every host thread (and one step on one thread)
  configs     the batched forest (5 steps after the autotuner's sweep) and the galaxy (50
              six-level block steps), run short (--no-configs leaves them out)

--impl reference times the CPU restatement of the reference's Barnes-Hut step (oracle/, FP64,
all host threads) on the same workload at the reference solver's default leaf size, 24, and at
leaf 32 (the leaf sizes the autotuner picks between here), and reports the faster.

--workload adjoint and --workload forest print the lines of the differentiable and the batched
workloads instead (see run_adjoint and run_forest); --workload sweep runs the merger at theta
0.3, 0.5 and 0.8 for 200 steps each (run_sweep), --workload galaxy the 131,072-body galaxy in
500 six-level block steps (run_galaxy), --workload scaling the Plummer sphere from 1M to 64M
bodies (run_scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s @N=1M θ=0.5: mixed vs plain GPU walk at RMS force err ≤2e-3"
N_DEFAULT = 1 << 20
THETA, EPS, DT = 0.5, 0.02, 1e-3
# DRAM bytes (read + write) of one walk launch on this workload (a force evaluation of
# `bench.py --profile mixed --leaf L`), by kernel and leaf size, from ncu captures of
# dram__bytes_read.sum + dram__bytes_write.sum. Stored figures,
# not measured in the bench's own run (a counter capture cannot run inside a timed region).
WALK_TRAFFIC_BYTES = {(32, 24): 55_931_904, (32, 32): 61_613_568,  # (stars per group, leaf size)
                      (64, 24): 58_973_952, (64, 32): 67_039_232}
TUNE_LEAVES = [8, 12, 16, 24, 32]
RMS_BOUND = 2e-3
REFERENCE_LEAF = 24  # bh.go:17-19, the reference solver's default leaf size
# leaf sizes the reference arm times: its own default and the leaves the autotuner picks between
# for the mixed walk on this workload; the arm reports the fastest
REFERENCE_LEAVES = (24, 32)
CPU_BEST_OF = 5
FIELDS = ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az")


def workload_name(n):
    return (f"merger N={n} (2 x {n // 2} disk+bulge+NFW-halo galaxies, pericentre 5, separation 40), "
            f"theta={THETA}, eps={EPS}, dt={DT}, global KDK steps")


def max_over_ranks(x: float, world: int, device: str) -> float:
    """The largest x over the ranks of the default process group (x itself on one rank)."""
    if world == 1:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_value(n: int, steps: int, ms_max: float, world: int) -> float:
    """Whole-job particle-steps/s of `world` independent replicas, each advancing n particles by
    `steps` steps, timed by the slowest rank (ms_max milliseconds)."""
    return world * n * steps / (ms_max * 1e-3)


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("LOCAL_RANK", "0"))


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device, self.rows, self.proc, self.first = device, [], None, 0

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            # the timed region starts once the sampler is live (its first line), at most 3 s later
            t0 = time.perf_counter()
            while not self.rows and self.proc.poll() is None and time.perf_counter() - t0 < 3.0:
                time.sleep(0.01)
            self.first = len(self.rows)  # samples taken before the timed region are not counted
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows[self.first:] if len(self.rows) > self.first else self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except (ValueError, IndexError):
                continue
            for name, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(n, seed=0):
    from gravitas_gb300 import ics
    return ics.merger(n, seed=seed)


def cpu_reference_steps(s, steps, leaf, workers=0, count=False, initial=None, group=64):
    """Times full KDK steps of the CPU oracle (the reference's algorithm, FP64) on a copy of s;
    optionally also returns, at the initial state, the reference walk's interaction counts and
    the counts of the group walk the mixed walk executes (groups of `group` sorted stars). The
    initial forces are computed untimed, or taken from `initial` (a state whose accelerations
    are s's forces: the oracle's forces do not depend on its thread count)."""
    from oracle import oracle as O
    counts = None
    if count:
        t = O.Tree(s["px"], s["py"], s["pz"], s["mass"], theta=THETA, leaf=leaf, workers=workers)
        counts = (t.counts(EPS, workers=workers), t.group_counts(group, workers=workers))
        del t
    src = s if initial is None else initial
    st = {k: np.array(src[k], copy=True) for k in (*FIELDS, "mass")}
    if initial is None:
        O.kdk(st, dt=DT, eps=EPS, theta=THETA, leaf=leaf, nsteps=0, workers=workers)  # initial forces
    first = {k: v.copy() for k, v in st.items()}
    t0 = time.perf_counter()
    O.kdk(st, dt=DT, eps=EPS, theta=THETA, leaf=leaf, nsteps=steps, acc_valid=True, workers=workers)
    return time.perf_counter() - t0, counts, first


def run_reference(args):
    """The reference arm: the CPU restatement of the reference's Barnes-Hut step (oracle/, FP64,
    every host thread) on the headline workload, at each leaf size of REFERENCE_LEAVES (one
    warm-up step, then up to --steps timed steps, at most about 30 s per leaf); the line reports
    the fastest leaf."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    n = args.n
    s = make_workload(n)
    cores = os.cpu_count() or 1
    leaves = (args.leaf,) if args.leaf else REFERENCE_LEAVES
    per_leaf = {}
    first = None
    for leaf in leaves:
        warm, _, first_l = cpu_reference_steps(s, 1, leaf, workers=0)
        k = max(1, min(args.steps, int(30.0 / max(warm, 1e-3))))
        el, _, _ = cpu_reference_steps(s, k, leaf, workers=0, initial=first_l)
        per_leaf[leaf] = {"value": n * k / el, "steps": k, "ms_per_step": el / k * 1e3}
    leaf = max(per_leaf, key=lambda L: per_leaf[L]["value"])
    value, k = per_leaf[leaf]["value"], per_leaf[leaf]["steps"]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": args.gpus,
        "steps": k, "warmup": 1, "ms_per_step": per_leaf[leaf]["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(n), "requested_steps": args.steps, "leaf_size": leaf,
                   "tuning": f"fastest of leaf sizes {list(leaves)} (the reference solver's default, bh.go:17-19, "
                             f"and the leaf sizes the GPU autotuner picks between on this workload)"},
        "per_leaf": {str(L): v for L, v in per_leaf.items()},
        "cpu_baseline": {"value": value, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                         "sample": f"{k} full KDK steps of the {n}-particle workload at leaf {leaf} after one warm-up "
                                   f"step (C++ restatement of the reference CPU Barnes-Hut, FP64, {cores} threads; "
                                   f"Go is not available)"},
        "e2e": {"value": value, "unit": "particle-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def rel_err_stats(got, want):
    e = np.linalg.norm(got - want, axis=1) / np.linalg.norm(want, axis=1)
    return {"rms": float(np.sqrt(np.mean(e ** 2))), "p99": float(np.percentile(e, 99)),
            "median": float(np.median(e)), "max": float(e.max())}


def run(args):
    import torch

    from gravitas_gb300 import abi

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    P = abi.ptr
    n = args.n
    s = make_workload(n, seed=0)
    ctx = abi.Context(local)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def upload(state):
        ctx.call("gbh_state_upload", n, *[P(state[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")],
                 None, None, None, P(state["mass"]), None, None)

    # leaf (and group) size of each walk: the autotuner at theta 0.5 under the RMS bound
    upload(s)
    tuned = {}
    for walk in ("mixed", "plain"):
        base = abi.make_params(THETA, EPS, args.leaf or 8, False, False, walk)
        if args.leaf:
            tuned[walk] = (base, None)
            continue
        best, table = ctx.autotune(base, thetas=[THETA], leaves=TUNE_LEAVES,
                                   groups=[64, 32] if walk == "mixed" else [64], rms_bound=RMS_BOUND,
                                   sample=4096, reps=3)
        tuned[walk] = (best, [{k: (round(v, 6) if isinstance(v, float) else v) for k, v in e.items()
                               if k in ("leaf_size", "group_size", "ms", "rms_err")} for e in table])
    leaf = tuned["mixed"][0].leaf_size

    def timed_steps(walk, steps, warmup, diag=None):
        par = tuned[walk][0]
        upload(s)
        if diag is not None:
            diag.append(ctx.diagnostics(par))
        for _ in range(warmup):
            ctx.call("gbh_state_step", par, DT, 1)
        barrier()
        tot = walk_ms = build_ms = 0.0
        launches = 0
        for _ in range(steps):
            flush.fill_(1)  # L2 flush (256 MiB) outside the step's events
            torch.cuda.synchronize()
            ctx.call("gbh_state_step", par, DT, 1)
            t = ctx.timings()
            tot += t["total_ms"]
            walk_ms += t["walk_ms"]
            build_ms += t["build_ms"]
            launches += t["launches"]
        barrier()
        if diag is not None:
            diag.append(ctx.diagnostics(par))
        return tot, walk_ms, build_ms, launches, t["nnodes"]

    peak = ctx.probe_fp32_peak(100.0)

    # headline: mixed walk, resident state
    diag = []
    with Clocks(local) as clk:
        t_mixed, w_mixed, b_mixed, launches, nnodes = timed_steps("mixed", args.steps, args.warmup, diag)
    clocks = clk.summary()
    e0, e1 = diag[0]["total"], diag[1]["total"]
    l0, l1 = np.array(diag[0]["angular_momentum"]), np.array(diag[1]["angular_momentum"])
    drift = {"steps": args.warmup + args.steps, "dt": DT, "energy_rel": abs((e1 - e0) / e0),
             "angular_momentum_rel": float(np.linalg.norm(l1 - l0) / np.linalg.norm(l0)),
             "energy_method": "tree potential at theta 0.5 from the list walk with a potential sink (FP32 "
                              "interactions, compensated per-star sums, FP64 total) + FP64 kinetic "
                              "(gbh_state_diagnostics with the step's parameters)"}
    t_plain, w_plain, b_plain, _, _ = timed_steps("plain", args.steps, args.warmup)

    def maxr(x):
        return max_over_ranks(x, world, f"cuda:{local}")

    t_mixed, t_plain = maxr(t_mixed), maxr(t_plain)
    value = replica_value(n, args.steps, t_mixed, world)
    plain_value = replica_value(n, args.steps, t_plain, world)

    # end to end: host state in pinned memory, one gbh_step_kdk per step (copies inside)
    host = {k: torch.from_numpy(np.array(s[k], copy=True)).pin_memory() for k in (*FIELDS, "mass")}
    par = tuned["mixed"][0]
    hp = [host[k].data_ptr() for k in FIELDS]

    def e2e_step(acc_valid):
        ctx.call("gbh_step_kdk", par, DT, 1, acc_valid, n, *[P(x) for x in hp], P(host["mass"].data_ptr()),
                 None, None)

    e2e_step(0)
    for _ in range(max(args.warmup - 1, 0)):
        e2e_step(1)
    barrier()
    e2e_wall = 0.0
    h2d = d2h = 0
    for _ in range(args.steps):
        flush.fill_(1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step(1)
        e2e_wall += time.perf_counter() - t0
        tm = ctx.timings()
        h2d, d2h = tm["h2d_bytes"], tm["d2h_bytes"]
    e2e_wall = maxr(e2e_wall)
    e2e_value = replica_value(n, args.steps, e2e_wall * 1e3, world)

    # force errors of both walks against the FP64 direct sum on 4096 seeded targets
    rng = np.random.default_rng(1234)
    targets = np.sort(rng.choice(n, 4096, replace=False)).astype(np.int64)
    want = np.zeros((3, 4096))
    ctx.call("gbh_direct_accelerations", abi.make_params(0, EPS, 0, False, False, "fp64"), n, P(s["px"]),
             P(s["py"]), P(s["pz"]), P(s["mass"]), None, P(targets), 4096, P(want[0]), P(want[1]), P(want[2]))
    want = want.T
    errs = {}
    for walk in ("mixed", "plain"):
        a = [np.zeros(n) for _ in range(3)]
        ctx.call("gbh_accelerations", tuned[walk][0], n, P(s["px"]),
                 P(s["py"]), P(s["pz"]), P(s["mass"]), None, None, P(a[0]), P(a[1]), P(a[2]))
        errs[walk] = rel_err_stats(np.stack(a, axis=1)[targets], want)

    # the batched and the galaxy configurations, run short beside the headline (their own
    # workloads print full lines: --workload forest, --workload galaxy)
    configs = None
    if rank == 0 and not args.no_configs:
        configs = {"forest": forest_summary(local, 5, 2, table=False),
                   "galaxy": galaxy_summary(local, 50, compare=False)}

    line = None
    if rank == 0:
        # CPU baseline leg: the oracle (reference algorithm) on the host cores at the GPU arm's leaf
        # size, best of CPU_BEST_OF single steps after one warm-up step (a bounded sample), plus the
        # reference walk's interaction counts behind the algorithmic FLOP figure
        group = tuned["mixed"][0].group_size or 64
        kernel = f"k_walk_lists ({group}-star groups, {group // 32} star(s) a lane)"
        _, (counts, gcounts), first = cpu_reference_steps(s, 1, leaf, workers=0, count=True, group=group)
        cpu_times = [cpu_reference_steps(s, 1, leaf, workers=0, initial=first)[0] for _ in range(CPU_BEST_OF)]
        el = min(cpu_times)
        cores = os.cpu_count() or 1
        # the same step on one thread (initial forces reused from the run above)
        el1, _, _ = cpu_reference_steps(s, 1, leaf, workers=1, initial=first)
        n_pn, n_pp, n_open = counts
        flop = 50 * n_pn + 18 * n_pp + 8 * n_open
        flop_exec = 50 * gcounts[0] + 18 * gcounts[1] + 8 * gcounts[2]
        walk_s = w_mixed / args.steps * 1e-3
        achieved = flop / walk_s / 1e12
        line = {
            "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_mixed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 walk, f64 state", "data": "synthetic",
            "config": {"workload": workload_name(n), "parallelism": "replicas" if world > 1 else "1 gpu",
                       "l2": "flushed (256 MiB write) between timed steps; events cover each step only",
                       "leaf_size": leaf, "group_size": group, "list_depth": tuned["mixed"][0].list_depth,
                       "plain_leaf_size": tuned["plain"][0].leaf_size,
                       "tuning": "gbh_autotune at theta 0.5, RMS force error <= 2e-3 on 4096 stars" if not args.leaf
                       else "fixed by --leaf"},
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": WALK_TRAFFIC_BYTES.get((group, leaf)),
                         "traffic_source": "stored, not measured in this run: ncu dram__bytes_read.sum + "
                                           "dram__bytes_write.sum of one launch of this kernel at this leaf size "
                                           "on this workload (null: not captured for this kernel and leaf size)",
                         "kernel": kernel, "flop_per_launch": flop,
                         "peak_source": "FP32 FMA microbenchmark in this run (gbh_probe_fp32_peak); "
                                        "MEASURED_PEAKS.json has no FP32 figure",
                         "walk_ms": w_mixed / args.steps, "build_ms": b_mixed / args.steps,
                         "executed": {"flop_per_launch": flop_exec, "over_credited": flop_exec / flop,
                                      "achieved": flop_exec / walk_s / 1e12,
                                      "frac": flop_exec / walk_s / 1e12 / peak,
                                      "source": f"oracle group-walk counts (orc_tree_group_counts) for "
                                                f"{group}-star groups at the same theta and leaf: every star "
                                                f"of a group takes part in each of its group's visits, as in "
                                                f"{kernel}; same FLOP weights"}},
            "cpu_baseline": {"value": n / el, "unit": "particle-steps/s", "cores": cores, "kind": "port",
                             "sample": f"best of {CPU_BEST_OF} full KDK steps of the {n}-particle workload at leaf "
                                       f"{leaf} after one warm-up step, C++ restatement of the reference CPU "
                                       f"Barnes-Hut (FP64), {cores} threads",
                             "step_seconds": cpu_times,
                             "single_core": {"value": n / el1, "unit": "particle-steps/s", "cores": 1,
                                             "sample": "the same full KDK step on one thread"}},
            "e2e": {"value": e2e_value, "unit": "particle-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "api": "gbh_step_kdk on pinned host buffers, 1 step per call"},
            "gpu_launches": launches,
            "clocks": clocks,
            "plain": {"value": plain_value, "ms_per_step": t_plain / args.steps, "walk_ms": w_plain / args.steps,
                      "force_error": errs["plain"], "speedup_mixed_over_plain": value / plain_value},
            "autotune": {"mixed": tuned["mixed"][1], "plain": tuned["plain"][1]},
            "force_error": errs["mixed"],
            "drift": drift,
            "interactions": {"accepted_nodes": n_pn, "leaf_pairs": n_pp, "opened_nodes": n_open,
                             "per_star": (n_pn + n_pp) / n, "nodes": nnodes,
                             "per_s": (n_pn + n_pp) / walk_s,
                             "per_s_of_step": (n_pn + n_pp) * args.steps / (t_mixed * 1e-3),
                             "source": "the reference per-star walk's node and leaf-pair interactions "
                                       "(oracle counts at the initial state) per second of walk time and "
                                       "of full-step time"},
        }
        if configs:
            line["configs"] = configs
        print(json.dumps(line), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def run_profile(args):
    """A short launch sequence for ncu captures: upload the workload, then two force
    evaluations with the chosen walk (tree build + walk each). --profile adjoint runs one
    forward + backward of the 32,768-body adjoint workload over 4 steps (checkpoints every 2);
    --profile forest two force evaluations of the 64-system forest at the autotuner's choice
    (theta 0.7, leaf 16, group 64); --profile build two force evaluations of a Plummer sphere of
    --n bodies (leaf 32), for captures of the build kernels."""
    from gravitas_gb300 import abi
    P = abi.ptr
    if args.profile == "adjoint":
        from gravitas_gb300 import ics, sim
        s, targets = ics.adjoint_problem(ADJ_N, seed=0)
        ctx = abi.Context(0)
        loss, _, _, _ = sim.trajectory_loss_gradient(s, targets, ADJ_DT, ADJ_EPS, 4, 2, abi.ADJ_FP32, ctx)
        t = ctx.timings()
        print(json.dumps({"profile": "adjoint", "n": ADJ_N, "steps": 4, "loss": loss, "bwd_ms": t["total_ms"],
                          "pair_ms": t["walk_ms"], "launches": t["launches"]}))
        ctx.close()
        return 0
    if args.profile == "build":
        from gravitas_gb300 import ics
        n = args.n
        s = ics.plummer(n, seed=0)
        ctx = abi.Context(0)
        ctx.call("gbh_state_upload", n, *[P(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None, None,
                 P(s["mass"]), None, None)
        par = abi.make_params(THETA, 0.01, args.leaf or 32, False, False, "mixed", group_size=64)
        for _ in range(2):
            ctx.call("gbh_state_accelerations", par)
        t = ctx.timings()
        print(json.dumps({"profile": "build", "n": n, "build_ms": t["build_ms"], "walk_ms": t["walk_ms"],
                          "nnodes": t["nnodes"], "launches": t["launches"]}))
        ctx.close()
        return 0
    if args.profile == "forest":
        from gravitas_gb300 import ics
        s, off = ics.forest(nsys=64, seed=0)
        ctx = abi.Context(0, abi.CFG_PAIRED if args.paired else 0)
        ctx.forest_upload(off, s["px"], s["py"], s["pz"], s["vx"], s["vy"], s["vz"], s["mass"], s["kind"],
                          s["alive"])
        # the autotuner's pick for this forest (theta 0.7, leaf 32, 64-star groups); --leaf overrides
        par = abi.make_params(0.7, EPS, args.leaf or 32, False, False, "mixed", group_size=64)
        for _ in range(2):
            ctx.call("gbh_state_accelerations", par)
        t = ctx.timings()
        print(json.dumps({"profile": "forest", "leaf": par.leaf_size, "n": int(off[-1]), "build_ms": t["build_ms"], "walk_ms": t["walk_ms"],
                          "nnodes": t["nnodes"], "launches": t["launches"]}))
        ctx.close()
        return 0
    n = args.n
    s = make_workload(n, seed=0)
    ctx = abi.Context(0, abi.CFG_PAIRED if args.paired else 0)
    ctx.call("gbh_state_upload", n, *[P(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None, None,
             P(s["mass"]), None, None)
    leaf = args.leaf or REFERENCE_LEAF
    par = abi.make_params(THETA, EPS, leaf, False, False, args.profile, group_size=args.group)
    for _ in range(2):
        ctx.call("gbh_state_accelerations", par)
    t = ctx.timings()
    print(json.dumps({"profile": args.profile, "n": n, "leaf": leaf, "group": args.group, "build_ms": t["build_ms"],
                      "walk_ms": t["walk_ms"], "nnodes": t["nnodes"], "launches": t["launches"]}))
    ctx.close()
    return 0


ADJ_N, ADJ_STEPS, ADJ_EVERY, ADJ_EPS, ADJ_DT = 32768, 1000, 50, 0.01, 1e-3
ADJ_TREE_LEAF = 16
ADJ_FLOP_FORCE, ADJ_FLOP_VJP = 18, 51  # algorithmic FLOP per ordered pair (force; kick adjoint)


def run_adjoint(args):
    """The differentiable workload: gradient of L = mean |x_T - target|^2 with respect to the
    initial positions, velocities and masses through gbh_fwd_save / gbh_bwd, on a Plummer
    sphere of 32,768 lognormal-mass bodies, 1,000 KDK steps of 1e-3, softening 0.01, checkpoints
    every 50 steps, FP32 pair kernels. Checked against central differences (h = 1e-4) of the
    same forward on --fd-coords coordinates. Beside it (tree_force) the gradient through the
    Barnes-Hut force at theta 0.5 (the tree adjoint, lists frozen per step), timed and checked on
    --tree-coords coordinates against differences of the same tree forward. One line of JSON; not
    the headline workload."""
    from gravitas_gb300 import abi, ics, sim
    from oracle import oracle as O
    rank, world, local = dist_env()
    n, T, K = args.n if args.n != N_DEFAULT else ADJ_N, ADJ_STEPS, ADJ_EVERY
    s, targets = ics.adjoint_problem(n, seed=0)
    ctx = abi.Context(local)
    x0 = np.stack([s["px"], s["py"], s["pz"]], 1)
    v0 = np.stack([s["vx"], s["vy"], s["vz"]], 1)
    peak = ctx.probe_fp32_peak(50.0)
    for _ in range(args.warmup):
        sim.trajectory_loss_gradient(s, targets, ADJ_DT, ADJ_EPS, T, K, abi.ADJ_FP32, ctx)
    walls, dev, pair = [], [], []
    with Clocks(local) as clk:
        for _ in range(args.steps):
            t0 = time.perf_counter()
            loss, dx, dv, dm = sim.trajectory_loss_gradient(s, targets, ADJ_DT, ADJ_EPS, T, K, abi.ADJ_FP32, ctx)
            walls.append(time.perf_counter() - t0)
            tf = ctx.timings()  # of gbh_bwd; the forward's were read below
            dev.append(tf["total_ms"])
            pair.append(tf["walk_ms"])
    # device and pair-kernel time of one forward, read separately
    ctx.fwd_save(x0, v0, s["mass"], ADJ_DT, ADJ_EPS, T, K, abi.ADJ_FP32)
    tfw = ctx.timings()
    ms_grad = statistics.median(walls) * 1e3
    dev_ms = tfw["total_ms"] + statistics.median(dev)
    pair_ms = tfw["walk_ms"] + statistics.median(pair)
    nck = (T + K - 1) // K
    pairs = n * (n - 1)
    flop = pairs * (ADJ_FLOP_FORCE * (2 * T + 1 - nck) + ADJ_FLOP_VJP * (T + 1))
    achieved = flop / (pair_ms * 1e-3) / 1e12
    # central differences of the same forward on random velocity and mass coordinates
    rng = np.random.default_rng(5)
    h, errs, scale = 1e-4, [], float(np.abs(np.concatenate([dv.ravel(), dm])).max())
    pure, small = [], 0  # |g - fd| / |fd| without the floor; coordinates whose |fd| is below the floor
    flagged = []
    for q in range(args.fd_coords):
        i, c = int(rng.integers(n)), int(rng.integers(3))
        vals = []
        for sign in (1.0, -1.0):
            v, m = v0.copy(), s["mass"].copy()
            if q % 2 == 0:
                v[i, c] += sign * h
            else:
                m[i] += sign * h
            xT, _ = ctx.fwd_save(x0, v, m, ADJ_DT, ADJ_EPS, T, T, abi.ADJ_FP32)
            vals.append(float(np.sum((xT - targets) ** 2) / n))
        fd = (vals[0] - vals[1]) / (2 * h)
        g = dv[i, c] if q % 2 == 0 else dm[i]
        errs.append(abs(g - fd) / max(abs(fd), 1e-3 * scale))
        pure.append(abs(g - fd) / abs(fd) if fd != 0 else float("inf"))
        if errs[-1] > 1e-3:
            flagged.append((i, c, q, float(g), fd, errs[-1]))
        small += abs(fd) < 1e-3 * scale
    # For each coordinate off by more than 1e-3 the quotient is taken again at 2h and h/2. Two
    # error sources show: the O(h^2) truncation of the central difference (a mass is about 3e-5
    # here, so h = 1e-4 is no small step for a mass coordinate: the quotients then converge as h^2,
    # and the Richardson value (4 fd(h/2) - fd(h)) / 3 removes that term), and the rounding of the
    # FP32 pair forces of the forward (an FP64 forward of 1,000 steps at this size takes hours at
    # GB300's FP64 rate), which the spread of the three quotients bounds.
    noise = []
    for (i, c, q, g, fd, e) in flagged:
        alt = []
        for hh in (2 * h, h / 2):
            vals = []
            for sign in (1.0, -1.0):
                v, m = v0.copy(), s["mass"].copy()
                if q % 2 == 0:
                    v[i, c] += sign * hh
                else:
                    m[i] += sign * hh
                xT, _ = ctx.fwd_save(x0, v, m, ADJ_DT, ADJ_EPS, T, T, abi.ADJ_FP32)
                vals.append(float(np.sum((xT - targets) ** 2) / n))
            alt.append((vals[0] - vals[1]) / (2 * hh))
        fds = [fd] + alt
        rich = (4 * alt[1] - fd) / 3
        noise.append({"coord": ("v" if q % 2 == 0 else "m") + f"[{i}]" + (f"[{c}]" if q % 2 == 0 else ""),
                      "g": g, "fd_h_2h_half": fds, "rel_err": e,
                      "fd_spread_rel": (max(fds) - min(fds)) / max(abs(fd), 1e-30),
                      "richardson": rich, "rel_err_richardson": abs(g - rich) / max(abs(rich), 1e-3 * scale)})
    worst_x = max([x for x in errs if x <= 1e-3] + [r["rel_err_richardson"] for r in noise], default=None)
    # the same gradient against central differences of the tree dynamics (theta 0.5, mixed walk,
    # leaf 8): the opening-test discontinuities are far below the difference quotient at h = 1e-4
    tree_errs = []
    par = abi.make_params(THETA, ADJ_EPS, 8, False, False, "mixed")
    F = ("px", "py", "pz", "vx", "vy", "vz", "ax", "ay", "az")
    for q in range(args.fd_coords // 2):
        i, c = int(rng.integers(n)), int(rng.integers(3))
        vals = []
        for sign in (1.0, -1.0):
            st = {k: (s[k].copy() if k in s else np.zeros(n)) for k in F}
            st[("vx", "vy", "vz")[c]][i] += sign * h
            ctx.call("gbh_step_kdk", par, ADJ_DT, T, 0, n, *[abi.ptr(st[k]) for k in F], abi.ptr(s["mass"]), None,
                     None)
            x = np.stack([st["px"], st["py"], st["pz"]], 1)
            vals.append(float(np.sum((x - targets) ** 2) / n))
        fd = (vals[0] - vals[1]) / (2 * h)
        tree_errs.append(abs(dv[i, c] - fd) / max(abs(fd), 1e-3 * scale))
    # The tree force (theta 0.5): the adjoint of the list walk with each step's lists
    # frozen, timed like the direct-sum gradient and checked against central differences of the
    # same tree forward (velocities at h, masses at 1e-2 of their value)
    tree = None
    if args.tree_coords > 0:
        tl = lambda: sim.trajectory_loss_gradient(s, targets, ADJ_DT, ADJ_EPS, T, K, abi.ADJ_FP32, ctx,
                                                  abi.ADJ_TREE, THETA, ADJ_TREE_LEAF)
        tl()
        twalls = []
        for _ in range(max(1, args.steps)):
            t0 = time.perf_counter()
            _, tdx, tdv, tdm = tl()
            twalls.append(time.perf_counter() - t0)
        tscale_v, tscale_m = float(np.abs(tdv).max()), float(np.abs(tdm).max())
        terrs = []
        for q in range(args.tree_coords):
            i, c = int(rng.integers(n)), int(rng.integers(3))
            hh = h if q % 2 == 0 else 1e-2 * float(s["mass"][i])
            vals = []
            for sign in (1.0, -1.0):
                v, m = v0.copy(), s["mass"].copy()
                if q % 2 == 0:
                    v[i, c] += sign * hh
                else:
                    m[i] += sign * hh
                xT, _ = ctx.fwd_save(x0, v, m, ADJ_DT, ADJ_EPS, T, T, abi.ADJ_FP32, abi.ADJ_TREE, THETA, ADJ_TREE_LEAF)
                vals.append(float(np.sum((xT - targets) ** 2) / n))
            fd = (vals[0] - vals[1]) / (2 * hh)
            g = tdv[i, c] if q % 2 == 0 else tdm[i]
            terrs.append(abs(g - fd) / max(abs(fd), 1e-3 * (tscale_v if q % 2 == 0 else tscale_m)))
        tree = {"theta": THETA, "leaf": ADJ_TREE_LEAF, "walk": "list walk, 32-star groups split among warps, quadrupoles",
                "ms_per_gradient": statistics.median(twalls) * 1e3,
                "value": n * T / statistics.median(twalls), "unit": "particle-steps/s",
                "fd_check": {"coords": len(terrs), "h_v": h, "h_m": "1e-2 m_i",
                             "max_rel": float(max(terrs)) if terrs else None,
                             "median_rel": float(np.median(terrs)) if terrs else None,
                             "p90_rel": float(np.percentile(terrs, 90)) if terrs else None,
                             "error": "|g - fd| / max(|fd|, 1e-3 max|g|), fd of the same tree forward"}}
    # CPU baseline: the oracle's FP64 adjoint on a bounded sample (all bodies, 4 steps)
    cpu = None
    if rank == 0:
        xT4 = {k: s[k].copy() for k in ("px", "py", "pz", "vx", "vy", "vz", "mass")}
        t0 = time.perf_counter()
        O.kdk_direct(xT4, ADJ_DT, ADJ_EPS, 4)
        gx4 = 2 * (np.stack([xT4["px"], xT4["py"], xT4["pz"]], 1) - targets) / n
        O.adjoint_direct(s, ADJ_DT, ADJ_EPS, 4, 2, gx4, np.zeros_like(gx4))
        el = time.perf_counter() - t0
        cpu = {"value": n * 4 / el, "unit": "particle-steps/s", "cores": os.cpu_count() or 1, "kind": "port",
               "sample": f"FP64 direct-sum adjoint of the oracle, all {n} bodies, 4 steps, checkpoints every 2 "
                         f"(forward + backward), {os.cpu_count()} threads"}
    line = {
        "metric": f"adjoint particle-steps/s @N={n}: gradient of a final-position loss, {T} KDK steps",
        "value": n * T / (ms_grad * 1e-3), "unit": "particle-steps/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_grad, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 pairs, f64 state", "data": "synthetic",
        "config": {"workload": f"Plummer N={n}, lognormal(0.3) masses, eps={ADJ_EPS}, dt={ADJ_DT}, {T} steps, "
                               f"checkpoints every {K}, targets = x0 rotated 30 deg about z + N(0, 0.01^2)",
                   "loss": loss},
        "device_ms_per_gradient": dev_ms, "pair_kernel_ms": pair_ms,
        "roofline": {"bound": "fp32", "kernels": "k_force32 + k_vjp32", "achieved": achieved, "peak": peak,
                     "unit": "TFLOP/s", "frac": achieved / peak, "flop_per_pair": [ADJ_FLOP_FORCE, ADJ_FLOP_VJP],
                     "peak_source": "FP32 FMA probe of this run"},
        "fd_check": {"coords": len(errs), "h": h, "max_rel": float(max(errs)) if errs else None,
                     "median_rel": float(np.median(errs)) if errs else None,
                     "error": "|g - fd| / max(|fd|, 1e-3 max|g|)",
                     "pure": {"error": "|g - fd| / |fd|", "max_rel": float(max(pure)) if pure else None,
                              "median_rel": float(np.median(pure)) if pure else None,
                              "p90_rel": float(np.percentile(pure, 90)) if pure else None,
                              "coords_below_floor": int(small)},
                     "above_1e-3": noise,
                     "max_rel_extrapolated": worst_x,
                     "extrapolated": "every coordinate at h, except those above 1e-3 there, which take the "
                                     "Richardson value of h and h/2"},
        "fd_check_tree_dynamics": {"coords": len(tree_errs), "h": h, "theta": THETA, "walk": "mixed, leaf 8",
                                   "max_rel": float(max(tree_errs)) if tree_errs else None,
                                   "median_rel": float(np.median(tree_errs)) if tree_errs else None},
        "cpu_baseline": cpu, "clocks": clk.summary(),
    }
    if tree:
        line["tree_force"] = tree
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()
    return 0


def forest_summary(local, steps, warmup, table=True):
    """The batched workload: 64 independent Plummer or disk+bulge+halo systems of log-uniform
    N in [2048, 65536] and scale radius in [0.5, 2], one state (gbh_forest_upload). The autotuner
    (gbh_autotune) sweeps theta {0.4, 0.5, 0.7} x leaf {4, 8, 16, 32} x group {32, 64} for the
    fastest force evaluation with RMS error <= 2e-3; then `steps` KDK steps run with the chosen
    parameters (one build and one walk launch per step for all systems; device time from CUDA
    events, L2 flushed between steps), and every system is checked against its own FP64 direct
    sum on sampled stars. Returns a dict (the forest line's fields)."""
    import torch

    from gravitas_gb300 import abi, ics
    P = abi.ptr
    s, off = ics.forest(nsys=64, seed=0)
    n, nsys = int(off[-1]), len(off) - 1
    ctx = abi.Context(local)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")

    def upload():
        ctx.forest_upload(off, s["px"], s["py"], s["pz"], s["vx"], s["vy"], s["vz"], s["mass"], s["kind"],
                          s["alive"])

    upload()
    base = abi.make_params(0.5, EPS, 8, False, False, "mixed")
    t0 = time.perf_counter()
    best, tab = ctx.autotune(base, rms_bound=2e-3, sample=2048, reps=3)
    tune_s = time.perf_counter() - t0
    default = [e for e in tab if (e["theta"], e["leaf_size"], e["group_size"]) == (0.5, 8, 64)][0]
    upload()
    for _ in range(warmup):
        ctx.call("gbh_state_step", best, DT, 1)
    torch.cuda.synchronize()
    tot = walk_ms = build_ms = 0.0
    launches = 0
    with Clocks(local) as clk:
        for _ in range(steps):
            flush.fill_(1)
            torch.cuda.synchronize()
            ctx.call("gbh_state_step", best, DT, 1)
            t = ctx.timings()
            tot += t["total_ms"]
            walk_ms += t["walk_ms"]
            build_ms += t["build_ms"]
            launches += t["launches"]
    # per-system check of the stepped state's forces against each system's own FP64 direct sum
    ctx.call("gbh_state_accelerations", best)
    st = {k: np.zeros(n) for k in FIELDS}
    ctx.call("gbh_state_download", *[P(st[k]) for k in FIELDS])
    a = np.stack([st["ax"], st["ay"], st["az"]], 1)
    rms, p99 = [], []
    fp64 = abi.make_params(0, EPS, 0, False, False, "fp64")
    for q in range(nsys):
        lo, hi = int(off[q]), int(off[q + 1])
        tg = np.arange(0, hi - lo, max(1, (hi - lo) // 256), dtype=np.int64)
        want = np.zeros((3, len(tg)))
        sub = {k: np.ascontiguousarray(st[k][lo:hi]) for k in ("px", "py", "pz")}
        m = np.ascontiguousarray(s["mass"][lo:hi])
        kd = np.ascontiguousarray(s["kind"][lo:hi])
        ctx.call("gbh_direct_accelerations", fp64, hi - lo, P(sub["px"]), P(sub["py"]), P(sub["pz"]), P(m), P(kd),
                 P(tg), len(tg), P(want[0]), P(want[1]), P(want[2]))
        e = np.linalg.norm(a[lo:hi][tg] - want.T, axis=1) / np.linalg.norm(want.T, axis=1)
        rms.append(float(np.sqrt(np.mean(e ** 2))))
        p99.append(float(np.percentile(e, 99)))
    ctx.close()
    out = {
        "value": n * steps / (tot * 1e-3), "unit": "particle-steps/s", "steps": steps, "warmup": warmup,
        "ms_per_step": tot / steps, "n": n, "systems": nsys,
        "workload": f"forest of {nsys} Plummer or disk+bulge+halo systems, N_i log-uniform in [2048, 65536], "
                    f"scale U[0.5, 2], eps={EPS}, dt={DT}, global KDK steps",
        "chosen": {"theta": best.theta, "leaf_size": best.leaf_size, "group_size": best.group_size,
                   "list_depth": best.list_depth},
        "autotune": {"seconds": tune_s, "candidates": len(tab),
                     "chosen_force_ms": min(e["ms"] for e in tab if e["meets"]) if any(e["meets"] for e in tab)
                     else None, "default_force_ms": default["ms"], "default_rms_err": default["rms_err"]},
        "walk_ms": walk_ms / steps, "build_ms": build_ms / steps, "gpu_launches": launches,
        "launches_per_step": launches / steps,
        "force_error_per_system": {"max_rms": max(rms), "median_rms": float(np.median(rms)), "max_p99": max(p99)},
        "clocks": clk.summary(),
    }
    if table:
        out["autotune"]["table"] = [{k: (round(v, 6) if isinstance(v, float) else v) for k, v in e.items()}
                                    for e in tab]
    return out


def run_forest(args):
    """The batched workload's own line (forest_summary with --steps and --warmup)."""
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    f = forest_summary(local, args.steps, args.warmup)
    line = {
        "metric": f"forest particle-steps/s: {f['systems']} systems, N={f['n']}, autotuned at RMS force err <= 2e-3",
        "value": f["value"], "unit": f["unit"], "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": f["ms_per_step"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 walk, f64 state", "data": "synthetic",
        "config": {"workload": f["workload"], "l2": "flushed (256 MiB write) between timed steps"},
        **{k: f[k] for k in ("chosen", "autotune", "walk_ms", "build_ms", "gpu_launches", "launches_per_step",
                             "force_error_per_system", "clocks")},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def run_scaling(args):
    """Throughput against N on one GPU: equal-mass Plummer spheres of 1M, 4M, 16M and 64M bodies
    (eps 0.01, theta 0.5, leaf 32, 64-star groups, dt 1e-3), global KDK steps of the mixed walk
    with the state resident in HBM. For each N: device ms per step split into build and walk,
    particle-steps/s, and the device memory the library holds. One line of JSON."""
    import torch

    from gravitas_gb300 import abi, ics
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    P = abi.ptr
    rows = []
    for n in args.sizes:
        s = ics.plummer(n, seed=0)
        ctx = abi.Context(local)
        free0, total = torch.cuda.mem_get_info(local)
        ctx.call("gbh_state_upload", n, *[P(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None, None,
                 P(s["mass"]), None, None)
        par = abi.make_params(THETA, 0.01, 32, False, False, "mixed", group_size=64)
        for _ in range(max(args.warmup, 1)):
            ctx.call("gbh_state_step", par, DT, 1)
        tot = walk = build = 0.0
        for _ in range(args.steps):
            ctx.call("gbh_state_step", par, DT, 1)
            t = ctx.timings()
            tot += t["total_ms"]
            walk += t["walk_ms"]
            build += t["build_ms"]
        free1, _ = torch.cuda.mem_get_info(local)
        rows.append({"n": n, "ms_per_step": tot / args.steps, "walk_ms": walk / args.steps,
                     "build_ms": build / args.steps, "particle_steps_per_s": n * args.steps / (tot * 1e-3),
                     "device_gb": (free0 - free1) / 1e9, "nodes": t["nnodes"]})
        ctx.close()
        del s
        if rank == 0:
            print(json.dumps({"scaling_row": rows[-1]}), flush=True)
    if rank == 0:
        print(json.dumps({"metric": "particle-steps/s vs N, Plummer, theta 0.5, mixed walk", "unit": "particle-steps/s",
                          "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "data": "synthetic",
                          "rows": rows, "hbm_total_gb": total / 1e9}), flush=True)
    return 0


def run_sweep(args):
    """The large-merger configuration's theta sweep: the 1M merger at theta 0.3, 0.5 and 0.8
    (mixed walk, leaf 32, 64-star groups, eps 0.02), 200 global KDK steps of dt = 1e-3 each
    (the default --steps of this workload), graph-replayed in one call. Per theta: particle-steps/s from CUDA events,
    walk and build time, RMS / p99 force error of the initial forces against the FP64 direct sum
    on 4,096 seeded stars, and the drift of energy and angular momentum over the run, all
    measured with one estimator (the mixed-walk tree potential at theta 0.5). One line of JSON."""
    import torch

    from gravitas_gb300 import abi
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if rank != 0:
        return 0
    P = abi.ptr
    n = args.n
    s = make_workload(n)
    steps = args.steps
    ctx = abi.Context(local)
    rng = np.random.default_rng(1234)
    targets = np.sort(rng.choice(n, 4096, replace=False)).astype(np.int64)
    want = np.zeros((3, 4096))
    ctx.call("gbh_direct_accelerations", abi.make_params(0, EPS, 0, False, False, "fp64"), n, P(s["px"]),
             P(s["py"]), P(s["pz"]), P(s["mass"]), None, P(targets), 4096, P(want[0]), P(want[1]), P(want[2]))
    want = want.T
    est = abi.make_params(0.5, EPS, 32, False, False, "mixed", group_size=64)  # the drift estimator
    rows = []
    with Clocks(local) as clk:
        for theta in (0.3, 0.5, 0.8):
            par = abi.make_params(theta, EPS, args.leaf or 32, False, False, "mixed", group_size=64)
            ctx.call("gbh_state_upload", n, *[P(s[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None,
                     None, P(s["mass"]), None, None)
            ctx.call("gbh_state_accelerations", par)
            a = [np.zeros(n) for _ in range(3)]
            ctx.call("gbh_state_download", None, None, None, None, None, None, P(a[0]), P(a[1]), P(a[2]))
            err = rel_err_stats(np.stack(a, axis=1)[targets], want)
            d0 = ctx.diagnostics(est)
            ctx.call("gbh_state_step", par, DT, steps)
            t = ctx.timings()
            d1 = ctx.diagnostics(est)
            l0, l1 = np.array(d0["angular_momentum"]), np.array(d1["angular_momentum"])
            rows.append({"theta": theta, "ms_per_step": t["total_ms"] / steps, "walk_ms": t["walk_ms"] / steps,
                         "build_ms": t["build_ms"] / steps,
                         "particle_steps_per_s": n * steps / (t["total_ms"] * 1e-3), "force_error": err,
                         "energy_drift": abs((d1["total"] - d0["total"]) / d0["total"]),
                         "angular_momentum_drift": float(np.linalg.norm(l1 - l0) / np.linalg.norm(l0)),
                         "nodes": t["nnodes"], "launches_per_step": t["launches"] / steps})
            print(json.dumps({"sweep_row": rows[-1]}), flush=True)
    ctx.close()
    print(json.dumps({"metric": "merger theta sweep: particle-steps/s, force error and drift per theta",
                      "unit": "particle-steps/s", "n_gpus": 1, "steps": steps, "data": "synthetic",
                      "config": {"workload": workload_name(n), "leaf_size": args.leaf or 32, "dt": DT, "group_size": 64,
                                 "estimator": "energy and angular momentum from gbh_state_diagnostics with the "
                                              "mixed walk at theta 0.5 for every row",
                                 "l2": "not flushed: the steps run back to back in one graph-replayed call"},
                      "rows": rows, "clocks": clk.summary()}), flush=True)
    return 0


def galaxy_summary(local, steps, leaf=0, compare=True):
    """The galaxy configuration: the 131,072-body disk + bulge + NFW-halo galaxy (halo particles at
    4x the disk particle mass), eps 0.02, theta 0.5, power-of-two block steps with 6 levels driven
    by eta sqrt(eps / |a|), eta 0.025, `steps` block steps of T = 1.6e-2, mixed walk at the leaf
    the autotuner picks (or `leaf`). Returns block steps per second, particle-steps/s (each block
    step advances every particle by T), the events and walked stars, and the energy and
    angular-momentum drift; with `compare`, also the first 50 block steps' simulated time in
    global steps at the finest rung (T / 32), timed and with its drift, for the scheme's saving."""
    import torch

    from gravitas_gb300 import abi, ics
    P = abi.ptr
    g = ics.galaxy(131072, seed=0)
    n = len(g["px"])
    T, levels, eta, eps = 1.6e-2, 6, 0.025, 0.02
    ctx = abi.Context(local)

    def upload():
        ctx.call("gbh_state_upload", n, *[P(g[k]) for k in ("px", "py", "pz", "vx", "vy", "vz")], None, None, None,
                 P(g["mass"]), P(g["kind"]), P(g["alive"]))

    upload()
    base = abi.make_params(THETA, eps, leaf or 16, False, False, "mixed")
    if leaf:
        par = base
    else:
        par, _ = ctx.autotune(base, thetas=[THETA], leaves=TUNE_LEAVES, groups=[64, 32], rms_bound=RMS_BOUND,
                              sample=4096, reps=3)

    def run_block(nsteps):
        upload()
        ctx.step_block(par, T, eta, levels, 1)  # warm-up: buffers and captured graphs
        upload()
        d0 = ctx.diagnostics(par)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        st = ctx.step_block(par, T, eta, levels, nsteps)
        torch.cuda.synchronize()
        el = time.perf_counter() - t0
        d1 = ctx.diagnostics(par)
        return el, st, d0, d1

    def drifts(d0, d1):
        l0, l1 = np.array(d0["angular_momentum"]), np.array(d1["angular_momentum"])
        return abs((d1["total"] - d0["total"]) / d0["total"]), float(np.linalg.norm(l1 - l0) / np.linalg.norm(l0))

    with Clocks(local) as clk:
        el, st, d0, d1 = run_block(steps)
        de, dl = drifts(d0, d1)
        cmp = None
        if compare:
            short = min(steps, 50)
            el_s, st_s, s0, s1 = run_block(short)
            de_s, _ = drifts(s0, s1)
            upload()
            f0 = ctx.diagnostics(par)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ctx.call("gbh_state_step", par, T / 32, 32 * short)
            torch.cuda.synchronize()
            el_g = time.perf_counter() - t0
            de_g, _ = drifts(f0, ctx.diagnostics(par))
            cmp = {"block_steps": short, "block_seconds": el_s, "block_energy_drift": de_s,
                   "global_steps": 32 * short, "global_seconds": el_g, "global_energy_drift": de_g,
                   "speedup": el_g / el_s}
    ctx.close()
    out = {
        "value": n * steps / el, "unit": "particle-steps/s", "steps": steps,
        "workload": f"galaxy N={n} (40 % exponential disk, 10 % Hernquist bulge, 50 % NFW halo at 4x the disk "
                    f"particle mass), eps={eps}, theta={THETA}, {levels} levels, eta={eta}, T={T}",
        "leaf_size": par.leaf_size, "group_size": par.group_size or 64, "list_depth": par.list_depth,
        "timing": "wall clock around one gbh_state_step_block call (host reads one event tick per event)",
        "block_steps_per_s": steps / el, "events": st["substeps"], "walked_stars": st["evaluations"],
        "walked_fraction": st["evaluations"] / (n * st["substeps"]) if st["substeps"] else None,
        "energy_drift": de, "angular_momentum_drift": dl, "clocks": clk.summary()}
    if cmp:
        out["vs_finest_rung_global_steps"] = cmp
    return out


def run_galaxy(args):
    """The galaxy configuration's own line (galaxy_summary with --steps, default 500)."""
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if rank != 0:
        return 0
    gsum = galaxy_summary(local, args.steps, args.leaf)
    line = {"metric": "galaxy block steps: particle-steps/s (each block step advances all particles by T)",
            "value": gsum["value"], "unit": gsum["unit"], "n_gpus": 1, "steps": args.steps, "data": "synthetic",
            "config": {k: gsum[k] for k in ("workload", "leaf_size", "group_size", "list_depth", "timing")}}
    line.update({k: v for k, v in gsum.items() if k not in line["config"] and k not in ("value", "unit", "steps")})
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (default 10; 200 for --workload sweep)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=N_DEFAULT)
    ap.add_argument("--leaf", type=int, default=0,
                    help="leaf size; 0 (default) lets the autotuner choose for each walk")
    ap.add_argument("--profile", choices=["mixed", "plain", "fp64", "adjoint", "forest", "build"], default=None,
                    help="run only two force evaluations with this walk (for ncu captures)")
    ap.add_argument("--workload", choices=["merger", "adjoint", "forest", "scaling", "sweep", "galaxy"],
                    default="merger",
                    help="adjoint: the differentiable workload (gbh_fwd_save / gbh_bwd); forest: 64 systems in "
                         "one state with the autotuner; sweep: the merger at theta 0.3 / 0.5 / 0.8; galaxy: the "
                         "131,072-body galaxy in block steps; scaling: 1M to 64M bodies; each prints its own "
                         "JSON line")
    ap.add_argument("--group", type=int, default=0, choices=[0, 32, 64],
                    help="--profile mixed: the mixed walk's group size (0: the library's default)")
    ap.add_argument("--paired", action="store_true",
                    help="--profile mixed / forest: 64-star groups take the paired walk (GBH_CFG_PAIRED), for "
                         "captures of k_walk_mixed2")
    ap.add_argument("--no-configs", action="store_true",
                    help="headline: leave out the short forest and galaxy runs reported beside it")
    ap.add_argument("--fd-coords", type=int, default=16, help="adjoint: coordinates checked by central differences")
    ap.add_argument("--tree-coords", type=int, default=8,
                    help="adjoint: coordinates of the tree-force gradient checked by central differences (0: no "
                         "tree-force gradient)")
    ap.add_argument("--sizes", type=int, nargs="+", default=[1 << 20, 1 << 22, 1 << 24, 1 << 26],
                    help="scaling: body counts")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = {"sweep": 200, "galaxy": 500}.get(args.workload, 10)
    if args.workload == "adjoint":
        return run_adjoint(args)
    if args.workload == "forest":
        return run_forest(args)
    if args.workload == "scaling":
        return run_scaling(args)
    if args.workload == "sweep":
        return run_sweep(args)
    if args.workload == "galaxy":
        return run_galaxy(args)
    if args.profile:
        return run_profile(args)
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run(args)


if __name__ == "__main__":
    sys.exit(main())
