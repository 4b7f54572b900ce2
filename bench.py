#!/usr/bin/env python
"""Benchmark of the vortex-particle FMM hot path on GB300.

One step = one full RK stage of the reference's FMMCalculator::advance
(fmmCalculator.hpp:919-1005) on device-resident bodies: tree build, interaction
lists, P2M/M2M, M2L, L2L, L2P + P2P, stretching and the stage update.  The
workload is the uniform cloud: N = 1,048,576 positions uniform in [-1, 1]^3,
strengths N(0, 1e-3), sigma = 1.3 * 2 * N^(-1/3), theta = 0.5, leaf 64, RK2;
synthetic inputs from a seed.  Metric: particle evaluations (velocity + J +
dalpha/dt at one body for one RHS evaluation) per second, whole job.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With torchrun, each rank runs an independent replica on its own GPU (the
single-system FMM does not shard without a halo exchange the reference does
not have); value = sum of all ranks' particle evaluations / max rank time.
--impl reference times the CPU implementation of the same path (the oracle
restatement of the reference's own FMM, OpenMP, all host cores) on the same
workload, one stage per step.
"""
from __future__ import annotations

import argparse
import ctypes
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

METRIC = "particle-evals/sec at N=1M, mixed vs FP64 GPU FMM at <=1e-6 rel L2 err"
UNIT = "particle-evals/s"


def parse(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=40)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--fp64-steps", type=int, default=2, help="timed FP64 steps for the mixed-vs-FP64 comparison (0: skip)")
    ap.add_argument("--n", type=int, default=1 << 20)
    ap.add_argument("--p", type=int, default=10)
    ap.add_argument("--ncrit", type=int, default=64)
    ap.add_argument("--theta", type=float, default=0.5)
    ap.add_argument("--dt", type=float, default=0.01)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="bodies in the CPU baseline's cloud (0: the full workload, the same state the GPU times)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true")
    ap.add_argument("--out", default=None, help="also write the JSON line to this file")
    ap.add_argument("--autotune", action="store_true",
                    help="also report the opt-in autotuner's choice (leaf size, M2L batch) and its stage time")
    ap.add_argument("--workload", default="cloud", choices=["cloud", "rings64", "adjoint", "wing", "ring"],
                    help="cloud: the headline N = 2^20 cloud; rings64: 64 independent rings, batched; "
                         "adjoint: reverse-mode gradient of the leapfrogging rings; wing: wing + wake, 400 RK2 steps "
                         "of shedding; ring: the 32,512-body ring, 10 RK2 steps with relaxation (FP64)")
    ap.add_argument("--wing-steps", type=int, default=400, help="wing workload: steps")
    ap.add_argument("--wing-check", type=int, default=50, help="wing workload: accuracy check every this many steps")
    ap.add_argument("--m2l-kernel", default="auto", choices=["auto", "tensor", "cuda"],
                    help="mixed-mode M2L at p = 8..10: by size (auto), tensor cores, or CUDA cores")
    ap.add_argument("--orders", default="6,14",
                    help="other expansion orders of the cloud reported beside the headline (stage times, errors); '' = none")
    ap.add_argument("--adj-steps", type=int, default=50, help="adjoint workload: RK3 steps")
    ap.add_argument("--cs-dirs", type=int, default=2, help="adjoint workload: complex-step check directions (0 = none)")
    return ap.parse_args(argv)


# ----------------------------------------------------------------- distributed
class Dist:
    """Replica bookkeeping: rank/world from torchrun's environment; barriers and
    max-reductions over gloo (no data-path collective exists)."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def sum(self, v: float) -> float:
        if not self.pg:
            return v
        import torch
        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.SUM)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples (SM clock, throttle reasons) during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.rows: list[list[str]] = []
        self.proc = None
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self) -> dict:
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows if len(r) >= 9 for k in range(4) if "Active" in r[5 + k]
                          and "Not" not in r[5 + k]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ----------------------------------------------------------------- helpers
def m2l_flops_per_pair(p: int) -> int:
    """Useful complex multiply-adds of one M2L (j + n <= p - 1, all k <= j,
    all m), 8 flops each, 3 components: 24 * sum_j (j+1)(p-j)^2."""
    return 24 * sum((j + 1) * (p - j) ** 2 for j in range(p))


P2P_FLOPS = 84  # per body-body interaction, counted from multipoleKernels.hpp:239-283

# DRAM bytes (read + write) per unit of the mixed-precision evaluation kernels
# at p = 10, from ncu captures of 2^19-body clouds: per M2L pair for the
# CUDA-core M2L (3,881,744 pairs) and the tensor-core M2L (3,847,952 pairs), per
# body for the fused leaf kernel and for the split one's near + far passes
# (profiles/k_m2l32v2_k_l2p_p2p32_cloud512K_p10.md, profiles/k_m2l_tc_cloud512K_p10.md,
# profiles/k_l2p_p2p32_cloud512K_p10.md, profiles/k_l2p_p2p32_split_cloud512K_p10.md).
NCU_TRAFFIC_MIXED_P10 = {"m2l": 359.0e6 / 3881744, "m2l_tc": (961.3e6 + 93.5e6) / 3847952,
                         "l2p_p2p": (125.1e6 + 40.5e6) / 524288, "l2p_p2p_split": (24.2e6 + 201.5e6) / 524288}
# tensor-pipe share of the tensor M2L's cycles in the same capture
NCU_TC_PIPE_ACTIVE = 0.233
# dense TF32 tensor rate relative to dense BF16 (nominal GB300 figures, 1.1 and
# 2.25 PFLOP/s), applied to the measured BF16 rate
TF32_PER_BF16 = 1.1 / 2.25


def measured_peaks() -> dict:
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return json.load(f)
    except OSError:
        return {}


def cpu_baseline(args, threads: int | None = None) -> dict:
    """The oracle restatement of the reference's FMM (OpenMP, host cores): one
    full stage (tree, lists, evaluation, Euler update) of the timed cloud (or
    of a smaller cloud of the same recipe with --cpu-sample)."""
    from oracle import oracle as O
    from uvlm_gb300 import workloads
    lib = O.oracle()
    cores = lib.vo_set_threads(threads or os.cpu_count() or 1)
    n = args.cpu_sample or args.n
    b = workloads.cloud(n, seed=1000 if n == args.n else 11)
    t0 = time.perf_counter()
    O.advance(b, args.p, args.ncrit, args.theta, args.dt, 1, 0)
    t = time.perf_counter() - t0
    what = "the timed cloud" if n == args.n else f"a {n}-body cloud of the same recipe"
    return {"value": n / t, "unit": UNIT, "cores": cores, "kind": "port", "seconds": t, "same_config": n == args.n,
            "sample": f"one stage (tree, lists, FMM evaluation, update) of {what} (p={args.p}, theta={args.theta}, "
                      f"leaf {args.ncrit}); the reference's own headers, compiled with OpenMP, ran 2.1x slower than "
                      f"this port on a 131,072-body cloud (8 cores), so the port is the faster CPU baseline"}


def config_of(args, l2: str) -> dict:
    return {"workload": "uniform cloud, one RK2 stage of the same initial state every step", "n_bodies": args.n, "p": args.p, "theta": args.theta,
            "ncrit": args.ncrit, "integrator": "RK2", "precision": args.precision, "l2": l2}


# ----------------------------------------------------------------- arms
def run_reference(args, dist: Dist) -> dict | None:
    if dist.rank != 0:
        return None
    from oracle import oracle as O
    O.build_oracle()
    for _ in range(args.warmup):
        cpu_baseline(args)
    vals, secs = [], []
    for _ in range(args.steps):
        r = cpu_baseline(args)
        vals.append(r["value"])
        secs.append(r["seconds"])
    value = (args.cpu_sample or args.n) * len(secs) / sum(secs)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(secs) / len(secs), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded uniform cloud)",
            "config": dict(config_of(args, "n/a (CPU)"), precision="fp64"), "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": r["cores"], "kind": "port", "sample": r["sample"]},
            "same_config": r["same_config"],
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    return line


def run_ours(args, dist: Dist) -> dict | None:
    from uvlm_gb300 import FMMCalculator, direct, lib, workloads
    from uvlm_gb300._lib import BODY_DTYPE
    n = args.n
    calc = FMMCalculator(p=args.p, ncrit=args.ncrit, theta=args.theta, integration="RK2", precision=args.precision,
                         device=dist.local_rank, m2l_kernel=args.m2l_kernel)
    h = calc.handle
    L = lib()
    bodies = workloads.cloud(n, seed=1000 + dist.rank)
    # every step is the same stage of the same cloud: the initial bodies are
    # loaded again before each step (outside the timed region), so each timed
    # step builds the same tree and lists and does the same work
    for w in range(args.warmup):
        calc.load(bodies)
        calc.stage(0, args.dt)
    L.vfmm_synchronize(h)
    dist.barrier()
    clocks = ClockSampler(dist.local_rank)
    clocks.start()
    launches = 0
    times = []
    ms = ctypes.c_float()
    for k in range(args.steps):
        calc.load(bodies)   # restore the initial state (untimed)
        L.vfmm_flush_l2(h)  # evict L2 between timed steps (untimed)
        L.vfmm_event_record(h, 0)
        launches0 = L.vfmm_launch_count(h)
        calc.stage(0, args.dt)
        launches += L.vfmm_launch_count(h) - launches0
        L.vfmm_event_record(h, 1)
        L.vfmm_event_elapsed(h, 0, 1, ctypes.byref(ms))
        times.append(ms.value * 1e-3)
    L.vfmm_synchronize(h)
    clk = clocks.stop()
    dist.barrier()
    total = sum(times)
    tmax = dist.max(total)
    value = dist.world * n * args.steps / tmax
    phases = calc.phase_times()
    stats = calc.stats()

    # roofline of the dominant kernel (phase timings of the last step, CUDA events on the handle's stream)
    peak_fp = ctypes.c_double()
    L.vfmm_measure_fma_peak(h, 0 if args.precision == "fp64" else 1, ctypes.byref(peak_fp))
    m2l_flops = m2l_flops_per_pair(args.p) * stats["m2l_pairs"]
    p2p_flops = P2P_FLOPS * stats["p2p_interactions"]
    tensor = args.precision == "mixed" and stats.get("m2l_tensor", 0) == 1
    split = phases.get("p2p_near", 0.0) > 0
    # with the split leaf kernel the near pass runs on a second stream beside
    # M2L: its own events time it (near pass + far pass), and M2L stays the
    # phase on the critical path
    cand = {"m2l": (phases["m2l"], m2l_flops),
            "l2p_p2p": (phases["p2p_near"] + phases["l2p_far"] if split else phases["l2p_p2p"], p2p_flops)}

    def roof_of(kern):
        t_k, f_k = cand[kern]
        achieved = f_k / (t_k * 1e-3) / 1e12
        traffic = None
        if args.precision == "mixed" and args.p == 10:
            key = "m2l_tc" if kern == "m2l" and tensor else ("l2p_p2p_split" if kern == "l2p_p2p" and split else kern)
            traffic = NCU_TRAFFIC_MIXED_P10[key] * (stats["m2l_pairs"] if kern == "m2l" else n)
        r = {"kernel": kern, "achieved": achieved, "unit": "TFLOP/s", "traffic": traffic,
             "traffic_source": "DRAM bytes per unit from an ncu capture of a 2^19-body cloud at p = 10, scaled by "
                               "this launch's units (M2L pairs or bodies); null for other orders",
             "algorithmic_flops_per_launch": f_k, "kernel_ms": t_k}
        if kern == "m2l" and tensor:
            bf16 = measured_peaks().get("bf16_tflops")
            peak = bf16 * TF32_PER_BF16 if bf16 else 1900.0 * TF32_PER_BF16
            r.update({"bound": "tensor", "peak": peak, "frac": achieved / peak,
                      "kernel": "m2l: k_m2l_tc (tcgen05.mma kind::tf32, three TF32 products per FP32 product) "
                                "with its tile/class pre-pass",
                      "peak_source": ("of measured: MEASURED_PEAKS.json bf16_tflops (burst) x 1.1/2.25, the dense "
                                      "TF32:BF16 ratio" if bf16 else "of fallback: 1.9 PFLOP/s bf16 x 1.1/2.25"),
                      "tensor_pipe_active_ncu": NCU_TC_PIPE_ACTIVE,
                      "note": "achieved counts the algorithmic M2L flops (24 T(p) per pair); the tensor core "
                              "executes about 3x that for the TF32 splits and the dense 128-row operator, and "
                              "the kernel is staging-bound (tensor pipe 23% busy in ncu), not pipe-bound"})
        else:
            if kern == "l2p_p2p" and split:
                r.update({"kernel": "l2p_p2p: k_l2p_p2p32 split, near pass (MODE 1) + far pass (MODE 2)",
                          "near_ms": phases["p2p_near"], "far_ms": phases["l2p_far"],
                          "note": "the near pass shares every SM with the tensor M2L for the M2L's duration (one "
                                  "leaf block beside the M2L block), then runs alone; achieved is over the two "
                                  "passes' own event times, so it includes the shared stretch"})
            r.update({"bound": "fp64" if args.precision == "fp64" else "fp32", "peak": peak_fp.value,
                      "frac": achieved / peak_fp.value if peak_fp.value else None,
                      "peak_source": "measured on this GPU in this run: FMA-chain probe kernel "
                                     "(vfmm_measure_fma_peak); MEASURED_PEAKS.json has no CUDA-core figure"})
        return r

    dom = "m2l" if split else max(cand, key=lambda k: cand[k][0])
    roof = roof_of(dom)
    roof["other"] = roof_of("l2p_p2p" if dom == "m2l" else "m2l")

    # end to end through the public API: vfmm_advance on pinned host AoS bodies
    host = bodies.copy()
    L.vfmm_host_register(host.ctypes.data, host.nbytes)
    calc.advance(host, args.dt)  # warm-up
    dist.barrier()
    e2e_t = []
    for _ in range(args.e2e_steps):
        host[:] = bodies  # the same initial cloud every step (untimed)
        t0 = time.perf_counter()
        calc.advance(host, args.dt)
        e2e_t.append(time.perf_counter() - t0)
    L.vfmm_host_unregister(host.ctypes.data)
    e2e_total = dist.max(sum(e2e_t))
    stages = calc.num_stages
    e2e_value = dist.world * n * stages * len(e2e_t) / e2e_total

    accuracy = None
    if not args.no_accuracy and dist.rank == 0 and args.precision == "mixed":
        accuracy = accuracy_at(args.p, bodies, args, mixed_calc=calc)
    calc.close()

    fp64 = None
    if args.precision == "mixed" and args.fp64_steps > 0:
        fp64 = time_fp64(args, dist, bodies)
    orders = []
    if args.precision == "mixed" and args.orders:
        for p in [int(x) for x in args.orders.split(",") if x.strip()]:
            o = time_order(p, bodies, args, dist, steps=3, fp64_steps=1)
            if dist.rank == 0 and not args.no_accuracy:
                o["accuracy"] = accuracy_at(p, bodies, args)
            orders.append(o)
    if dist.rank != 0:
        return None
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * tmax / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32",
            "data": "synthetic (seeded uniform cloud; no dataset)",
            "config": config_of(args, "flushed between steps (256 MB write)"),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": n * BODY_DTYPE.itemsize,
                    "d2h_bytes_per_step": n * BODY_DTYPE.itemsize,
                    "note": f"vfmm_advance (RK2 = {stages} stages) on pinned host exafmm::Body arrays, wall clock; "
                            "h2d counts the whole records, of which the step reads X, alpha and the radius "
                            "(the host-link lines those fields touch)"},
            "gpu_launches": int(launches),
            "roofline": roof, "clocks": clk, "phases_ms": phases, "tree": stats}
    if accuracy:
        line["accuracy"] = accuracy
    if fp64:
        line["fp64"] = fp64
        line["fp64"]["speedup_mixed_vs_fp64"] = fp64["ms_per_step"] / line["ms_per_step"]
    if orders:
        line["other_orders"] = orders
    if args.autotune:
        with FMMCalculator(p=args.p, ncrit=args.ncrit, theta=args.theta, integration="RK2", precision=args.precision,
                           device=dist.local_rank) as ct:
            line["autotuned"] = ct.autotune(bodies, args.dt)
            line["autotuned"]["note"] = ("opt-in: another leaf size builds another tree than the reference's ncrit; "
                                         "stage times from the tuner's own CUDA-event timing, L2 not flushed")
    if not args.no_cpu_baseline and dist.world == 1:
        line["cpu_baseline"] = {k: v for k, v in cpu_baseline(args).items() if k != "seconds"}
    return line


def time_fp64(args, dist: Dist, bodies) -> dict:
    """The plain FP64 GPU FMM on the same fixed workload (the drop-in mode),
    timed the same way for the mixed-vs-FP64 comparison."""
    from uvlm_gb300 import FMMCalculator
    with FMMCalculator(p=args.p, ncrit=args.ncrit, theta=args.theta, integration="RK2", precision="fp64",
                       device=dist.local_rank) as c:
        t = time_fixed_stage(c, bodies, args.dt, args.fp64_steps, warmup=1)
        ph = c.phase_times()
    tot = dist.max(sum(t))
    return {"ms_per_step": tot / len(t), "value": dist.world * args.n * len(t) / (tot * 1e-3), "steps": len(t),
            "phases_ms": ph}


def evaluate_state(c, bodies):
    """init + calculate of `bodies` on calculator c; returns the bodies in
    tree order, with a column of their original indices."""
    bb = bodies.copy()
    bb["drdt_old"] = np.arange(bb.size)  # survives init/calculate: recovers the tree permutation
    c.init(bb)
    c.calculate()
    c.copyBodies2Host(bb)
    return bb


def rl2(a, r) -> float:
    return float(np.linalg.norm(a - r) / np.linalg.norm(r))


def accuracy_at(p: int, bodies, args, mixed_calc=None, targets: int = 4096) -> dict:
    """Errors of the timed state (the initial cloud, one evaluation) at order p:
    mixed against the FP64 FMM on every body, and both against the
    model-consistent FP64 direct sum (regularised kernel on P2P-list leaf
    pairs, singular elsewhere: the sum the FMM approximates) on `targets`
    bodies; FP64 FMM against the plain regularised direct sum beside it."""
    from uvlm_gb300 import FMMCalculator, direct
    own = mixed_calc is None
    cm = mixed_calc or FMMCalculator(p=p, ncrit=args.ncrit, theta=args.theta, precision="mixed")
    mix = evaluate_state(cm, bodies)
    if own:
        cm.close()
    with FMMCalculator(p=p, ncrit=args.ncrit, theta=args.theta, precision="fp64") as c64:
        f64 = evaluate_state(c64, bodies)
        tgt = np.sort(np.random.default_rng(4096).choice(bodies.size, size=min(targets, bodies.size), replace=False))
        um, Jm = c64.direct_model(tgt)
    assert (mix["X"] == f64["X"]).all(), "mixed and FP64 trees differ"
    Jm = Jm.reshape(-1, 9)
    acc = {"p": p,
           "velocity_rel_l2_vs_fp64_fmm": rl2(mix["velocity"], f64["velocity"]),
           "J_rel_l2_vs_fp64_fmm": rl2(mix["J"], f64["J"]),
           "dadt_rel_l2_vs_fp64_fmm": rl2(mix["dadt"], f64["dadt"]),
           "bodies_compared": int(bodies.size),
           "model_direct_targets": int(tgt.size),
           "mixed_velocity_rel_l2_vs_model_direct": rl2(mix["velocity"][tgt], um),
           "mixed_J_rel_l2_vs_model_direct": rl2(mix["J"][tgt].reshape(-1, 9), Jm),
           "fp64_velocity_rel_l2_vs_model_direct": rl2(f64["velocity"][tgt], um),
           "fp64_J_rel_l2_vs_model_direct": rl2(f64["J"][tgt].reshape(-1, 9), Jm)}
    if p == args.p:
        ref = direct(f64[tgt].copy(), f64)  # all pairs regularised (order of the sources is immaterial)
        acc["fp64_velocity_rel_l2_vs_regularised_direct"] = rl2(f64["velocity"][tgt], ref["velocity"])
        acc["mixed_velocity_rel_l2_vs_regularised_direct"] = rl2(mix["velocity"][tgt], ref["velocity"])
    acc["note"] = ("timed state (initial cloud, one evaluation).  *_vs_fp64_fmm: precision error of the mixed path "
                   "(the <=1e-6 bar); *_vs_model_direct: FP64 direct sum with the FMM's own kernel split, so "
                   "the FMM's truncation error at this order and theta (the reference's MAC on cell half-widths), the "
                   "same for FP64 and mixed; *_vs_regularised_direct: all pairs regularised, which the reference's "
                   "singular far field does not approximate")
    return acc


def time_order(p: int, bodies, args, dist: Dist, steps: int, fp64_steps: int) -> dict:
    """Mixed and FP64 stage times of the same fixed workload at order p."""
    from uvlm_gb300 import FMMCalculator
    out = {"p": p}
    for prec, k in (("mixed", steps), ("fp64", fp64_steps)):
        if k <= 0:
            continue
        with FMMCalculator(p=p, ncrit=args.ncrit, theta=args.theta, integration="RK2", precision=prec,
                           device=dist.local_rank) as c:
            t = time_fixed_stage(c, bodies, args.dt, k, warmup=1)
            out[f"{prec}_ms_per_stage"] = dist.max(sum(t)) / len(t)
            if prec == "mixed":
                out["phases_ms"] = c.phase_times()
    if "fp64_ms_per_stage" in out and "mixed_ms_per_stage" in out:
        out["speedup_mixed_vs_fp64"] = out["fp64_ms_per_stage"] / out["mixed_ms_per_stage"]
    return out


def time_fixed_stage(c, bodies, dt: float, steps: int, warmup: int = 1) -> list:
    """ms of `steps` timed stages, each from the same loaded state, L2 flushed."""
    from uvlm_gb300 import lib
    L = lib()
    h = c.handle
    ms = ctypes.c_float()
    for _ in range(warmup):
        c.load(bodies)
        c.stage(0, dt)
    t = []
    for _ in range(steps):
        c.load(bodies)
        L.vfmm_flush_l2(h)
        L.vfmm_event_record(h, 0)
        c.stage(0, dt)
        L.vfmm_event_record(h, 1)
        L.vfmm_event_elapsed(h, 0, 1, ctypes.byref(ms))
        t.append(ms.value)
    return t


def run_rings64(args, dist: Dist) -> dict | None:
    """64 independent vortex rings (N log-uniform in [2k, 60k], random radius,
    core, circulation and orientation), p = 8, theta = 0.5, leaf 32, RK2, one
    step = one advance of every ring, through vfmm_advance_batch on host
    arrays (copies included); the same systems advanced one after another on
    the same handles are timed beside it."""
    from uvlm_gb300 import FMMCalculator, advance_batch, workloads
    systems = workloads.ring_batch(64, seed=7 + dist.rank)
    ntot = sum(b.size for b in systems)
    kw = dict(p=8, ncrit=32, theta=0.5, integration="RK2", precision=args.precision, device=dist.local_rank)
    tuned = None
    if args.autotune:
        # leaf size, P2P tile and M2L batch tuned per size bucket (N within a
        # factor of 2) on the bucket's median system, then used by every handle
        # of the bucket
        buckets = {}
        for i, b in enumerate(systems):
            buckets.setdefault(int(np.log2(b.size)), []).append(i)
        tuned = {}
        for key, idx in sorted(buckets.items()):
            med = sorted(idx, key=lambda i: systems[i].size)[len(idx) // 2]
            with FMMCalculator(**kw) as c:
                t = c.autotune(systems[med], args.dt)
            tuned[key] = {"systems": len(idx), "ncrit": t["ncrit"], "m2l_batch": t["m2l_batch"], "p2p_chunk": t["p2p_chunk"],
                          "ms_per_stage": t["ms_per_stage"], "default_ms_per_stage": t["default_ms_per_stage"]}
        mixed = args.precision == "mixed"
        calcs = [FMMCalculator(**dict(kw, ncrit=tuned[int(np.log2(b.size))]["ncrit"],
                                      m2l_batch=tuned[int(np.log2(b.size))]["m2l_batch"] if mixed else 0,
                                      p2p_chunk=tuned[int(np.log2(b.size))]["p2p_chunk"] if mixed else 0))
                 for b in systems]
    else:
        calcs = [FMMCalculator(**kw) for _ in systems]
    work = [b.copy() for b in systems]
    for _ in range(args.warmup):
        advance_batch(calcs, work, args.dt)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        advance_batch(calcs, work, args.dt)
    tb = dist.max(time.perf_counter() - t0)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for c, b in zip(calcs, work):
            c.advance(b, args.dt)
    ts = dist.max(time.perf_counter() - t0)
    for c in calcs:
        c.close()
    if dist.rank != 0:
        return None
    evals = dist.world * ntot * 2 * args.steps  # RK2: two evaluations per step
    return {"metric": "particle-evals/sec, 64 independent rings, batched advance", "value": evals / tb, "unit": UNIT,
            "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tb / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32", "data": "synthetic (seeded rings; no dataset)",
            "config": {"workload": "64 rings, N log-uniform [2k, 60k], RK2 step per ring", "bodies_total": ntot, "p": 8,
                       "theta": 0.5, "ncrit": 32, "precision": args.precision, "timing": "host wall clock, copies included"},
            "sequential": {"value": evals / ts, "ms_per_step": 1e3 * ts / args.steps,
                           "note": "the same systems advanced one vfmm_advance after another"},
            "autotuned_buckets": tuned}


def run_adjoint(args, dist: Dist) -> dict | None:
    """Reverse-mode gradient of the leapfrogging-ring objective: two coaxial
    rings of 512 stations x 127 points (130,048 bodies) at z = 0 and 0.5,
    p = 8, theta = 0.5, leaf 32, 50 RK3 steps of dt = 0.01 with a checkpoint
    every 10 steps; objective = kinetic energy sum u.(x cross alpha) + z-impulse
    at the final state; gradient with respect to all initial positions and
    strengths.  Timed on the host around vfmm_adjoint (copies included), beside
    the forward sweep alone.  The check leg compares the FP64 gradient of the
    8,128-body sub-case (32 stations) with the oracle's whole-step complex step
    along random directions (theta = 0.47: CPU and GPU trajectories agree in
    every tree and list decision only without exact MAC ties)."""
    import ctypes
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.leapfrog(512, seed=dist.rank)
    kw = dict(p=8, ncrit=32, theta=0.5, integration="RK3", precision=args.precision, device=dist.local_rank)
    steps, every = args.adj_steps, 10
    with FMMCalculator(**kw) as c:
        c.adjoint(b, args.dt, 1, 1)  # warm-up: buffers and kernels
        dist.barrier()
        t0 = time.perf_counter()
        c.adjoint(b, args.dt, steps, every, gradient=False)
        tf = dist.max(time.perf_counter() - t0)
        t0 = time.perf_counter()
        v, gx, ga = c.adjoint(b, args.dt, steps, every)
        tg = dist.max(time.perf_counter() - t0)
    check = None
    if dist.rank == 0 and args.cs_dirs > 0:
        from oracle.oracle import oracle
        b8 = workloads.leapfrog(32, seed=0)
        n8 = b8.size
        with FMMCalculator(p=8, ncrit=32, theta=0.47, integration="RK3", precision="fp64", device=dist.local_rank) as c:
            v8, gx8, ga8 = c.adjoint(b8, args.dt, steps, every)
        rng = np.random.default_rng(2024)
        nd = args.cs_dirs
        dx = rng.normal(size=(nd, n8, 3))
        da = rng.normal(size=(nd, n8, 3)) * np.abs(b8["alpha"]).max()
        wI = np.array([0.0, 0.0, 1.0])
        val, der = ctypes.c_double(), np.zeros(nd)
        t0 = time.perf_counter()
        oracle().vo_cs_objective(b8.ctypes.data, n8, 8, 32, 0.47, 2, 0, args.dt, steps, 1.0, wI.ctypes.data, dx.ctypes.data,
                                 da.ctypes.data, nd, ctypes.byref(val), der.ctypes.data, 0.0, 0, 0, 0.0)
        tcs = time.perf_counter() - t0
        an = np.einsum("kij,ij->k", dx, gx8) + np.einsum("kij,ij->k", da, ga8)
        check = {"case": "2 rings x 32 stations x 127 (8,128 bodies), FP64, theta 0.47, 50 RK3 steps", "directions": nd,
                 "max_rel_err_vs_complex_step": float(np.max(np.abs(an - der) / np.abs(der))),
                 "value_rel_diff": abs(v8 - val.value) / abs(val.value), "complex_step_seconds": tcs}
    if dist.rank != 0:
        return None
    return {"metric": f"reverse-mode gradient wall time, 2 leapfrogging rings (130,048 bodies), {steps} RK3 steps", "value": tg, "unit": "s",
            "n_gpus": dist.world, "steps": steps, "warmup": 1, "ms_per_step": 1e3 * tg / steps, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32",
            "data": "synthetic (seeded rings; no dataset)",
            "config": {"workload": "leapfrogging rings 2 x 512 x 127, KE + z-impulse objective", "bodies": int(b.size), "p": 8,
                       "theta": 0.5, "ncrit": 32, "checkpoint_every": every, "precision": args.precision,
                       "timing": "host wall clock around vfmm_adjoint, copies included"},
            "forward_seconds": tf, "gradient_over_forward": tg / tf, "objective": v, "complex_step_check": check}


def run_wing(args, dist: Dist) -> dict | None:
    """Wing + wake (workloads.WingWake): AR 8, chord 1, 40 x 10 panels, 5
    degrees, U = (1, 0, 0), 400 particles shed per step (10 per TE panel), 400
    RK2 steps of dt = 0.02, mixed precision, p = 10, theta = 0.5, leaf 64.
    Each step appends the shed particles and advances all of them through
    vfmm_advance on host arrays (copies included), as the reference's driver
    calls FMMCalculator::advance (src/main.cpp:291-293).  Every --wing-check
    steps the current state is evaluated in mixed precision and in FP64 and
    compared, both against the model-consistent FP64 direct sum on 2048
    bodies, and one FP64 stage of that state is timed."""
    from uvlm_gb300 import FMMCalculator, workloads
    from uvlm_gb300._lib import BODY_DTYPE
    w = workloads.WingWake(dt=0.02)
    kw = dict(p=10, ncrit=64, theta=0.5, integration="RK2", device=dist.local_rank)
    # relaxation (factor 0.3) after each step: without it the stretching of
    # the rolled-up sheet grew without bound after ~70 steps (|alpha| x 1e8 by
    # step 90, in FP64 as in mixed precision); the reference's driver has no
    # working relaxation (relaxation.hpp does not compile)
    calc = FMMCalculator(precision=args.precision, relax=0.3, **kw)
    bodies = np.zeros(0, BODY_DTYPE)
    evals, wall, checks = 0.0, 0.0, []
    for k in range(args.wing_steps):
        bodies = np.concatenate([bodies, w.shed()])
        t0 = time.perf_counter()
        calc.advance(bodies, w.dt)
        wall += time.perf_counter() - t0
        evals += 2.0 * bodies.size
        if dist.rank == 0 and ((k + 1) % args.wing_check == 0 or k + 1 == args.wing_steps):
            st = bodies.copy()
            with FMMCalculator(precision="mixed", **kw) as cm, FMMCalculator(precision="fp64", **kw) as c64:
                mix = evaluate_state(cm, st)
                f64 = evaluate_state(c64, st)
                tgt = np.sort(np.random.default_rng(k).choice(st.size, size=min(2048, st.size), replace=False))
                um, Jm = c64.direct_model(tgt)
                c64.load(st)
                t64 = time_fixed_stage(c64, st, w.dt, 1, warmup=0)[0]
                cm.load(st)
                tmx = time_fixed_stage(cm, st, w.dt, 1, warmup=1)[0]
            Jm = Jm.reshape(-1, 9)
            checks.append({"step": k + 1, "bodies": int(st.size),
                           "velocity_rel_l2_vs_fp64_fmm": rl2(mix["velocity"], f64["velocity"]),
                           "J_rel_l2_vs_fp64_fmm": rl2(mix["J"], f64["J"]),
                           "mixed_velocity_rel_l2_vs_model_direct": rl2(mix["velocity"][tgt], um),
                           "fp64_velocity_rel_l2_vs_model_direct": rl2(f64["velocity"][tgt], um),
                           "mixed_J_rel_l2_vs_model_direct": rl2(mix["J"][tgt].reshape(-1, 9), Jm),
                           "mixed_ms_per_stage": tmx, "fp64_ms_per_stage": t64})
    calc.close()
    evals_all = dist.sum(evals)
    wall_max = dist.max(wall)
    if dist.rank != 0:
        return None
    return {"metric": "particle-evals/sec, wing + wake, 400 RK2 steps of shedding (to 160,000 particles)",
            "value": evals_all / wall_max, "unit": UNIT, "n_gpus": dist.world, "steps": args.wing_steps, "warmup": 0,
            "ms_per_step": 1e3 * wall_max / args.wing_steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f32",
            "data": "synthetic (prescribed elliptic bound circulation; no dataset)",
            "config": {"workload": "wing AR 8, 40 x 10 panels, 5 deg, U = (1, 0, 0), 10 particles shed per TE panel and step, "
                                   "RK2 dt = 0.02, relaxation 0.3", "final_bodies": int(bodies.size), "p": 10, "theta": 0.5, "ncrit": 64,
                       "precision": args.precision,
                       "timing": "host wall clock around vfmm_advance on host arrays (copies included), every step"},
            "checks": checks}


def run_ring(args, dist: Dist) -> dict | None:
    """The plain FP64 ring (32,512 bodies: 256 stations x 127), p = 8, theta
    = 0.5, leaf 32, 10 RK2 steps of dt = 0.01 with relaxation (factor 0.3)
    after each step, through vfmm_advance on host arrays; the oracle
    restatement of the reference's advance on the host cores beside it."""
    from oracle import oracle as O
    from uvlm_gb300 import FMMCalculator, workloads
    b = workloads.ring(256, seed=0)
    steps = 10
    with FMMCalculator(p=8, ncrit=32, theta=0.5, integration="RK2", relax=0.3, precision=args.precision,
                       device=dist.local_rank) as c:
        c.advance(b.copy(), 0.01)  # warm-up
        bb = b.copy()
        t0 = time.perf_counter()
        for _ in range(steps):
            c.advance(bb, 0.01)
        tg = dist.max(time.perf_counter() - t0)
    tc = None
    cores = None
    if dist.rank == 0 and not args.no_cpu_baseline:
        cores = O.oracle().vo_set_threads(os.cpu_count() or 1)
        t0 = time.perf_counter()
        O.advance(b, 8, 32, 0.5, 0.01, steps, 1, relax=0.3)
        tc = time.perf_counter() - t0
    if dist.rank != 0:
        return None
    evals = dist.world * b.size * 2 * steps
    line = {"metric": "particle-evals/sec, vortex ring 32,512 bodies, 10 RK2 steps with relaxation", "value": evals / tg,
            "unit": UNIT, "n_gpus": dist.world, "steps": steps, "warmup": 1, "ms_per_step": 1e3 * tg / steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if args.precision == "fp64" else "f32", "data": "synthetic (seeded ring; no dataset)",
            "config": {"workload": "ring 256 x 127, RK2 dt 0.01, relaxation 0.3", "bodies": int(b.size), "p": 8, "theta": 0.5,
                       "ncrit": 32, "precision": args.precision, "timing": "host wall clock around vfmm_advance, copies included"}}
    if tc is not None:
        line["cpu_baseline"] = {"value": b.size * 2 * steps / tc, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": "the same 10 steps on the host cores", "seconds": tc}
    return line


def main(argv=None):
    args = parse(argv)
    dist = Dist()
    if args.impl == "reference":
        line = run_reference(args, dist)
    elif args.workload == "rings64":
        line = run_rings64(args, dist)
    elif args.workload == "adjoint":
        line = run_adjoint(args, dist)
    elif args.workload == "wing":
        line = run_wing(args, dist)
    elif args.workload == "ring":
        line = run_ring(args, dist)
    else:
        from uvlm_gb300 import _build, _lib
        if not os.path.exists(_lib.LIB_PATH):
            _build.build()
        line = run_ours(args, dist)
    if line is not None:
        s = json.dumps(line)
        print(s, flush=True)
        if args.out:
            with open(args.out, "w") as f:
                f.write(s + "\n")
    dist.close()


if __name__ == "__main__":
    main()
