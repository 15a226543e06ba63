"""Benchmark: batched rigid-body step, instance-steps/s on one GB300.

Workload (default): 65,536 serial revolute chains, n ~ U{2..48}, random
principal axes, l ~ U(0.2, 1) m, m ~ U(0.5, 2) kg, rod inertias,
q0 ~ U(−π, π), v0 ~ N(0, 1), open-loop τ ~ N(0, 1) resampled every 10 steps,
semi-implicit Euler at dt = 5e-4.  One bench "step" is one integrator step of
every instance; the timed region runs `--steps` of them in one persistent
launch.  Four forms are timed: FP64 through the reference's route (CRBA +
solve), FP64 articulated-body algorithm, mixed precision (articulated-body
algorithm with FP32 kinematics and double-float articulated inertias) and
CRBA with FP64 iterative refinement.  `value` is the fastest form whose per-step q̈ stays within 1e-5
of FP64 CRBA on ≥ 99 % of instances, at the initial and the final states.

`--impl reference` times the CPU restatement of the reference's `simulate`
(the Rust crate cannot be built here) on all host cores over a bounded sample
of the same workload.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "gorilla-physics_gb300"))
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

METRIC = "instance-steps/sec mixed vs FP64 GPU at stated qdd error"
UNIT = "instance-steps/s"
DT = {0: 1e-3, 1: 5e-4, 2: 1e-4, 3: 2e-4}
CONFIG_NAME = {0: "acrobot", 1: "serial-chain", 2: "floating-cube", 3: "quadruped"}
CONTROL = {0: "host", 1: "open_loop", 2: "host", 3: "pd"}
# each configuration's own batch and length (1,024 acrobots × 10,000 steps;
# 65,536 chains × 2,000; 32,768 cubes × 20,000; 16,384 quadrupeds × 10,000)
CONFIG_INSTANCES = {0: 1024, 1: 65536, 2: 32768, 3: 16384}
CONFIG_STEPS = {0: 10000, 1: 2000, 2: 20000, 3: 10000}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default: the configuration's own length; 2000 for --cuboids / --vstep)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gpb", choices=["gpb", "reference"])
    ap.add_argument("--config", type=int, default=1)
    ap.add_argument("--instances", type=int, default=None,
                    help="instances per GPU (default: the configuration's own batch; 65536 for --cuboids / --vstep)")
    ap.add_argument("--seed", type=int, default=2026)
    ap.add_argument("--mix-chains", type=int, default=0,
                    help="also step this many serial chains in the same batch (one control law for all)")
    ap.add_argument("--skip-cpu", action="store_true", help="omit the cpu_baseline leg")
    ap.add_argument("--warps-per-sm", type=int, default=0,
                    help="resident warps per SM of the step kernel (0: the autotuner chooses)")
    ap.add_argument("--precision", default="all", choices=["all", "fp64", "mixed", "refined"])
    ap.add_argument("--serve", action="store_true",
                    help="serving mix instead: Poisson arrivals, latency percentiles per rate")
    ap.add_argument("--serve-rates", default="1000,5000,20000", help="arrival rates, requests/s")
    ap.add_argument("--serve-seconds", type=float, default=10.0, help="arrival window per rate")
    ap.add_argument("--serve-drain", type=float, default=150.0, help="max seconds to drain after it")
    ap.add_argument("--serve-precisions", default="mixed,fp64")
    ap.add_argument("--serve-budget-gb", type=float, default=150.0, help="HBM budget of the slot pool")
    ap.add_argument("--serve-algorithm", default="aba", choices=["aba", "crba"])
    ap.add_argument("--serve-slo", action="store_true",
                    help="serving target: isolated time per request, peak sustainable load, "
                         "latency / isolated time at 50 %% of the peak")
    ap.add_argument("--serve-load", type=float, default=0.5, help="fraction of the peak for --serve-slo")
    ap.add_argument("--serve-peak-rate", type=float, default=20000.0,
                    help="arrival rate (requests/s) of the saturating run of --serve-slo")
    ap.add_argument("--cuboids", action="store_true",
                    help="cuboid-collider workload: build_gripper batches (GJK/EPA jaw-cube "
                         "contacts) and independent collision queries")
    ap.add_argument("--pairs", type=int, default=1 << 22, help="collision queries per timed launch")
    ap.add_argument("--vstep", action="store_true",
                    help="velocity stepping (friction-cone impulses) on cubes resting on the ground")
    args = ap.parse_args()
    other = args.cuboids or args.vstep
    if args.steps is None:
        args.steps = 2000 if other else CONFIG_STEPS[args.config]
    if args.instances is None:
        args.instances = 65536 if other else CONFIG_INSTANCES[args.config]
    return args


def kernel_source_hash() -> str:
    """First 16 hex digits of the SHA-256 of the CUDA/C++ sources (names and
    contents): ncu-derived figures in profiles/ are used only for the build
    they were captured on."""
    import hashlib

    h = hashlib.sha256()
    for f in sorted((ROOT / "gorilla-physics_gb300" / "csrc").iterdir()):
        if f.is_file():
            h.update(f.name.encode())
            h.update(f.read_bytes())
    return h.hexdigest()[:16]


_FLUSH = {}
L2_NOTE = ("L2 flushed (a 256 MB device write, twice the 129 MB L2) before each timed launch; "
           "the K steps inside one persistent launch reuse the batch's tables and state on chip by design")


def flush_l2(local: int) -> None:
    """Writes 256 MB on the device so that the next timed launch starts with a cold L2."""
    import torch

    buf = _FLUSH.get(local)
    if buf is None:
        buf = _FLUSH[local] = torch.empty(32 << 20, dtype=torch.float64, device=f"cuda:{local}")
    buf.zero_()
    torch.cuda.synchronize(local)


def shard_seed(seed: int, rank: int) -> int:
    """Each rank steps its own instances (weak scaling: no data-path collective)."""
    return seed + 1000 * rank


def all_reduce(x: float, op: str, world: int, device: str) -> float:
    """Max or sum of a per-rank scalar (timings: max over ranks; work: sum)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi samples during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=10)

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                for n, val in zip(names, f[5:9]):
                    if val.lower().startswith("active"):
                        reasons.add(n)
        finally:
            os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        load = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(load), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_reference(model, q0, v0, aux, config, steps, seconds_target=12.0, threads=None):
    """The oracle (CPU restatement of the reference path) on a bounded sample."""
    import oracle

    threads = threads or os.cpu_count() or 1
    qo, vo, _ = model.offsets()
    sample = min(model.n, 4096)
    K = max(1, steps)
    # calibrate on a tiny run, then size the sample to ≈ seconds_target
    cal_n = min(sample, 8 * threads)
    q, v = q0.copy(), v0.copy()
    kw = dict(control=CONTROL[config], ctl_all=aux if config == 3 else None, seed=7,
              resample_every=10, sigma=1.0, kp=50.0, kd=2.0, threads=threads)
    t = time.perf_counter()
    oracle.simulate_batch(model, q, v, DT[config], 2, end=cal_n, **kw)
    per = (time.perf_counter() - t) / (cal_n * 2)
    K = max(1, min(K, int(seconds_target / max(per * sample, 1e-9))))
    if K < 5:
        sample = max(threads, int(seconds_target / max(per * 5, 1e-9)))
        sample = min(sample, model.n)
        K = 5
    q, v = q0.copy(), v0.copy()
    t = time.perf_counter()
    oracle.simulate_batch(model, q, v, DT[config], K, end=sample, **kw)
    dt = time.perf_counter() - t
    return {"value": sample * K / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {sample} of {model.n} instances x {K} steps "
                      f"(oracle restatement, {threads} host threads)"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    import oracle

    oracle.build()
    # inputs from the CPU build of the workload generator: this arm loads no CUDA library
    M, q0, v0, aux = oracle.from_config(args.config, args.instances, seed=args.seed)
    threads = os.cpu_count() or 1
    qo, vo, _ = M.offsets()
    sample = min(M.n, 4096)
    kw = dict(control=CONTROL[args.config], ctl_all=aux if args.config == 3 else None, seed=7,
              resample_every=10, sigma=1.0, kp=50.0, kd=2.0, threads=threads)
    q, v = q0.copy(), v0.copy()
    # per step: one integrator step of the sampled instances; sized so that the
    # whole --steps run stays within a few minutes
    t = time.perf_counter()
    oracle.simulate_batch(M, q, v, DT[args.config], 1, end=min(sample, 64 * threads), **kw)
    per_inst_step = (time.perf_counter() - t) / min(sample, 64 * threads)
    budget = 120.0
    sample = int(min(sample, max(threads, budget / max(args.steps * per_inst_step, 1e-9))))
    for _ in range(args.warmup):
        oracle.simulate_batch(M, q, v, DT[args.config], 1, end=sample, **kw)
    t = time.perf_counter()
    oracle.simulate_batch(M, q, v, DT[args.config], args.steps, end=sample, **kw)
    el = time.perf_counter() - t
    value = sample * args.steps / el
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded Philox)",
        "impl": "reference",
        "config": {"workload": f"{CONFIG_NAME[args.config]} x {args.instances}",
                   "instances_timed": sample, "dt": DT[args.config], "integrator": "semi-implicit Euler"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"first {sample} instances x {args.steps} steps, oracle "
                                   f"restatement of the reference path (Rust crate unbuildable here)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_reference_cuboids(args):
    """--cuboids --impl reference: the oracle on the gripper workload, rank 0 only."""
    rank, _, _ = dist_env()
    if rank != 0:
        return 0
    import oracle

    oracle.build()
    M, q0, v0 = gripper_batch(args.instances, args.seed)
    base = cpu_cuboids(M, q0, v0, args.steps)
    line = {"metric": "instance-steps/s of build_gripper batches (GJK/EPA cuboid contacts)",
            "value": base["value"], "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded numpy draws)", "impl": "reference",
            "config": {"workload": f"gripper x {args.instances}", "dt": CUBOID_DT,
                       "integrator": "semi-implicit Euler"},
            "cpu_baseline": base,
            "e2e": {"value": base["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


VMAX_BOUNDED = 1e4


def qdd_error(B, gpb, precision, algorithm, where, lanes=1):
    """Per-instance q̈ error of (precision, algorithm) against the FP64 form of
    the reference's route (CRBA + solve), at the batch's current state.  That
    FP64 form agrees with the oracle to ≤ max(1e-10, 5e-15 cond(M)).  With
    several lanes per instance the form's q̈ is read from one step of the
    body-parallel mapping itself: semi-implicit Euler evaluates q̈ at the
    current state, and (v1 − v0) / dt recovers it to |v|·ε/dt."""
    ok = B.status() == 0
    B.set_algorithm(gpb.ALGO_CRBA)
    a = B.dynamics_continuous(None, precision=gpb.FP64)
    B.set_algorithm(algorithm)
    if lanes > 1:
        B.set_mapping(lanes)
        qs, vs = B.state()
        dt = 1e-3
        B.step(dt, None, gpb.SEMI_IMPLICIT_EULER, precision)
        b = (B.state()[1] - vs) / dt
        B.update(qs, vs)
    else:
        b = B.dynamics_continuous(None, precision=precision)
    vo = B.v_offset
    _, vel = B.state()
    err, rel, vmax = [], [], []
    for i in np.nonzero(ok)[0]:
        vmax.append(np.max(np.abs(vel[vo[i]:vo[i + 1]])) if vo[i + 1] > vo[i] else 0.0)
        x, y = b[vo[i]:vo[i + 1]], a[vo[i]:vo[i + 1]]
        d = np.max(np.abs(x - y)) if y.size else 0.0
        m = np.max(np.abs(y)) if y.size else 0.0
        e = d / max(m, 1.0)
        r = d / m if m > 0 else (0.0 if d == 0 else np.inf)
        err.append(e if np.isfinite(e) else np.inf)
        rel.append(r if np.isfinite(r) else np.inf)
    err, rel, vmax = np.asarray(err), np.asarray(rel), np.asarray(vmax)
    fin = err[np.isfinite(err)]
    rfin = rel[np.isfinite(rel)]
    # a trajectory that semi-implicit Euler has blown up (velocities growing
    # without bound, 1e29 and beyond, before they turn into NaN) has no
    # meaningful q̈ to compare: the gate uses the instances still bounded
    bnd = np.isfinite(vmax) & (vmax <= VMAX_BOUNDED)
    eb = err[bnd]
    return {"max": float(fin.max()) if fin.size else None,
            "p99": float(np.quantile(err, 0.99)), "median": float(np.median(err)),
            "frac_le_1e-5": float(np.mean(err <= 1e-5)), "nonfinite": int(np.sum(~np.isfinite(err))),
            "instances": int(err.size), "state": where,
            "norm": "max|Δq̈| / max(max|q̈_fp64,crba|, 1) per instance",
            "bounded": {"max": float(eb[np.isfinite(eb)].max()) if np.isfinite(eb).any() else None,
                        "frac_le_1e-5": float(np.mean(eb <= 1e-5)) if eb.size else 1.0,
                        "instances": int(eb.size), "excluded": int(err.size - eb.size),
                        "criterion": f"max|v| <= {VMAX_BOUNDED:g} (rad/s or m/s): trajectories not blown up"},
            "relative": {"max": float(rfin.max()) if rfin.size else None,
                         "p99": float(np.quantile(rel, 0.99)), "frac_le_1e-5": float(np.mean(rel <= 1e-5)),
                         "norm": "max|Δq̈| / max|q̈_fp64,crba| per instance (no floor)"}}


def run_gpu(args):
    rank, world, local = dist_env()
    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    import gpb
    from gpb import Batch, Model
    from gpb.flops import aba_model_flops, model_flops

    L = gpb.lib()
    ctx = gpb.Context(local)
    # weak scaling: every rank owns its own instances (seed offset by rank)
    M, q0, v0, aux = Model.from_config(args.config, args.instances, seed=shard_seed(args.seed, rank))
    if args.mix_chains > 0:  # e.g. quadrupeds and chains in the same persistent launch
        M2, q2, v2, _ = Model.from_config(1, args.mix_chains, seed=shard_seed(args.seed, rank) + 7)
        M = Model.concat([M, M2])
        q0, v0 = np.concatenate([q0, q2]), np.concatenate([v0, v2])
        aux = np.concatenate([aux, np.zeros_like(v2)])  # PD targets 0 for the chains
    B = Batch(M, ctx)
    kw = dict(control=CONTROL[args.config], tau=aux if args.config == 3 else None, seed=7,
              resample_every=10, sigma=1.0, kp=50.0, kd=2.0)
    dt = DT[args.config]

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def reduce_max(x):
        return all_reduce(x, "max", world, f"cuda:{local}")

    def reduce_sum(x):
        return all_reduce(x, "sum", world, f"cuda:{local}")

    # the four forms: (precision, algorithm, per-instance FP64 flops of one step)
    MODES = {
        "fp64_crba": (gpb.FP64, gpb.ALGO_CRBA, model_flops(M, 0)),
        "fp64": (gpb.FP64, gpb.ALGO_ABA, aba_model_flops(M, False)),
        "mixed": (gpb.MIXED, gpb.ALGO_ABA, aba_model_flops(M, True)),
        "refined": (gpb.MIXED_REFINED, gpb.ALGO_CRBA, model_flops(M, 0)),
    }
    precs = {"all": list(MODES), "fp64": ["fp64_crba", "fp64"], "mixed": ["mixed"],
             "refined": ["refined"]}[args.precision]
    results = {}
    launch = {}
    errs = {}
    for name in precs:
        prec, algo, inst_flops = MODES[name]
        B.set_algorithm(algo)
        B.update(q0, v0)
        B.clear_status()
        # launch shape for this workload and form (short trials, state restored)
        if args.warps_per_sm:
            B.set_launch(args.warps_per_sm)
            B.set_mapping(1)
            w, c, lanes = args.warps_per_sm, 0, 1
        else:
            w, c, lanes = B.autotune(dt, 0, prec, trial_steps=10, **kw)
        launch[name] = {"warps_per_sm": w, "coop_min_dof": c, "lanes_per_instance": lanes}
        if lanes > 1:  # the body-parallel mapping factors H whatever the algorithm setting
            inst_flops = MODES["fp64_crba"][2]
        if args.warmup:
            B.simulate_steps(args.warmup, dt, 0, prec, step0=0, **kw)
        barrier()
        ctx.synchronize()
        flush_l2(local)
        with Clocks(local) as clk:
            l0 = ctx.launches
            t0 = time.perf_counter()
            B.simulate_steps(args.steps, dt, 0, prec, step0=args.warmup, **kw)
            kernel_ms = L.gpb_last_launch_ms(ctx.h)
            ctx.synchronize()
            wall = time.perf_counter() - t0
            timed_launches = ctx.launches - l0
        barrier()
        kernel_ms = reduce_max(kernel_ms)
        bad = int(np.sum(B.status() != 0))
        done = B.steps_done()
        if name != "fp64_crba":  # q̈ error at the final state of this form's own trajectory
            errs[name] = {"final": qdd_error(B, gpb, prec, algo, f"after this form's {args.steps}-step timed run",
                                             lanes)}
        # only completed instance-steps count (a diverged instance freezes)
        results[name] = {"kernel_ms": kernel_ms, "wall_s": wall, "clocks": clk.summary(),
                         "failed_instances": bad, "launches": timed_launches, "lanes": lanes,
                         "done": reduce_sum(float(done.sum())),
                         "flops": reduce_sum(float(np.dot(done, inst_flops.astype(np.float64))))}
        if lanes > 1 and world == 1:
            # the autotuner chose several lanes per instance: the same run with
            # one lane per instance (4 and 8 warps per SM), for comparison
            B.set_mapping(1)
            best = None
            for w1 in (4, 8):
                B.set_launch(w1)
                B.update(q0, v0)
                B.clear_status()
                ctx.synchronize()
                flush_l2(local)
                B.simulate_steps(args.steps, dt, 0, prec, step0=args.warmup, **kw)
                ms1 = L.gpb_last_launch_ms(ctx.h)
                if best is None or ms1 < best[0]:
                    best = (ms1, w1, float(B.steps_done().sum()))
            launch[name]["one_lane"] = {"value": best[2] / (best[0] * 1e-3), "warps_per_sm": best[1],
                                        "kernel_ms": best[0]}
            B.set_mapping(lanes)
            B.set_launch(w)
    # q̈ error of every form against FP64 CRBA at the configuration's initial
    # states (the final states were measured after each form's run)
    B.update(q0, v0)
    B.clear_status()
    for name in errs:
        prec, algo, _ = MODES[name]
        errs[name]["initial"] = qdd_error(B, gpb, prec, algo, "the configuration's initial states",
                                          launch[name]["lanes_per_instance"])
    # headline: the fastest form that meets the stated bound (every instance
    # whose trajectory is not blown up within 1e-5 at both states); the FP64
    # forms are exact to round-off
    head_name = max([p for p in precs if p.startswith("fp64")] or precs[:1],
                    key=lambda n: results[n]["done"] / results[n]["kernel_ms"])
    for name in ["mixed", "refined"]:
        e = errs.get(name)
        if name in results and e and all(x["bounded"]["frac_le_1e-5"] == 1.0 for x in e.values()):
            if results[name]["kernel_ms"] < results[head_name]["kernel_ms"]:
                head_name = name
    # e2e through the public API: host (pinned) state in, K steps, state out
    q_h = torch.from_numpy(q0).pin_memory()
    v_h = torch.from_numpy(v0).pin_memory()
    qn, vn = q_h.numpy(), v_h.numpy()
    prec, algo, _ = MODES[head_name]
    B.set_algorithm(algo)
    # the headline form's own launch shape (the later forms' autotuning changed it)
    B.set_launch(launch[head_name]["warps_per_sm"])
    B.set_coop(launch[head_name]["coop_min_dof"])
    B.set_mapping(launch[head_name]["lanes_per_instance"])
    barrier()
    ctx.synchronize()
    flush_l2(local)
    t0 = time.perf_counter()
    B.update(qn, vn)
    B.simulate_steps(args.steps, dt, 0, prec, step0=0, **kw)
    qo, vo_ = B.state()
    e2e_s = time.perf_counter() - t0
    e2e_s = reduce_max(e2e_s)
    e2e_done = reduce_sum(float(B.steps_done().sum()))

    head = results[head_name]
    value = head["done"] / (head["kernel_ms"] * 1e-3)

    def peak(precision):
        t = __import__("ctypes").c_double()
        gpb._abi.check(L.gpb_fma_peak(local, precision, 32, __import__("ctypes").byref(t)), "gpb_fma_peak")
        return t.value

    p64, p32 = peak(gpb.FP64), peak(gpb.MIXED)

    WORK = {"fp64_crba": "CRBA + RNEA + Cholesky flops (gpb.flops.model_flops)",
            "fp64": "articulated-body algorithm flops (gpb.flops.aba_model_flops)",
            "mixed": "FP64 share of the mixed articulated-body algorithm (gpb.flops.aba_model_flops(mixed=True))",  # configurations without the instruction count
            "refined": "CRBA-equivalent flops (the FP64 residual is a part of them)"}
    # The mixed form runs its precision-critical recursion in double-float on the
    # FP32 pipes: no single pipe is near its peak, and its roofline is the SM's
    # instruction issue rate (the warp-instruction rate of the measured FP32 FMA
    # microbenchmark) against its executed warp instructions per instance-step.
    warp_inst_peak = p32 * 1e12 / 64 / 1e9  # G warp-instructions/s (64 flops per FFMA warp instruction)

    # DRAM bytes per instance-step from the committed ncu capture (small case of the
    # same workload), scaled to this launch's completed instance-steps
    src_hash = kernel_source_hash()
    stale = []
    try:
        tb = json.loads((ROOT / "profiles" / "dram_traffic_per_instance_step.json").read_text())
        traffic_per = {}
        for k, t in tb.get(CONFIG_NAME[args.config], {}).items():
            if t.get("source_sha16") == src_hash:
                traffic_per[k] = t
            else:  # captured on another build: not this kernel's figures
                stale.append(k)
    except (OSError, ValueError):
        traffic_per = {}
    hbm_peak = None
    try:
        hbm_peak = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        pass

    def roof(name, res):
        ach = res["flops"] / (res["kernel_ms"] * 1e-3) / 1e12
        per = res["flops"] / max(res["done"], 1.0)
        # the ncu table describes the one-lane kernels
        t = traffic_per.get(name) if res["lanes"] == 1 else None
        if name == "mixed" and t and "warp_instructions_per_instance_step" in t and not args.mix_chains:
            wi = t["warp_instructions_per_instance_step"]
            ach_i = wi * res["done"] / (res["kernel_ms"] * 1e-3) / 1e9
            out = {"bound": "issue", "achieved": ach_i, "peak": warp_inst_peak, "unit": "G warp-instructions/s",
                   "frac": ach_i / warp_inst_peak, "traffic": None,
                   "peak_source": "measured FP32 FMA microbenchmark (gpb_fma_peak), this run, in warp instructions",
                   "work": f"{wi:.0f} executed warp instructions per instance-step (ncu, {t['capture']}); "
                           f"{per:.0f} FP64 flops per instance-step remain on the FP64 pipe"}
        else:
            out = {"bound": "fp64", "achieved": ach, "peak": p64, "unit": "TFLOP/s", "frac": ach / p64,
                   "traffic": None, "peak_source": "measured FP64 FMA microbenchmark (gpb_fma_peak), this run",
                   "work": f"{per:.0f} FP64 flops per completed instance-step (mean): "
                           + (WORK[name] if res["lanes"] == 1 else WORK["fp64_crba"])}
        if t and not args.mix_chains:
            bytes_launch = t["dram_bytes_per_instance_step"] * res["done"]
            out["traffic"] = bytes_launch
            out["traffic_source"] = "ncu dram__bytes_read+write, " + t["capture"] + ", scaled to this launch"
            if hbm_peak:
                gbs = bytes_launch / (res["kernel_ms"] * 1e-3) / 1e9
                out["hbm"] = {"achieved": gbs, "peak": hbm_peak, "unit": "GB/s", "frac": gbs / hbm_peak,
                              "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)"}
        return out

    DTYPE = {"fp64_crba": "f64", "fp64": "f64",
             "mixed": "f32 kinematics/bias + double-f32 articulated inertias + f64 state"
             if launch.get("mixed", {}).get("lanes_per_instance", 1) == 1
             else "f64 (the body-parallel mapping computes in FP64 for GPB_MIXED requests)",
             "refined": "f32 solve + f64 residual refinement + f64 state"}
    ALGO0 = {"fp64_crba": "CRBA + Cholesky (the reference's route)", "fp64": "articulated-body algorithm",
             "mixed": "articulated-body algorithm", "refined": "CRBA + Cholesky, iterative refinement"}

    def algo_label(name):
        lanes = (launch.get(name) or {}).get("lanes_per_instance", 1)
        if lanes == 1:
            return ALGO0[name]
        return f"CRBA + Cholesky in FP64, body-parallel: {lanes} lanes per instance"

    ALGO = {k: algo_label(k) for k in ALGO0}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": head["kernel_ms"] / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": DTYPE[head_name],
        "data": "synthetic (seeded Philox4x32-10 draws of the configuration's distributions)",
        "config": {"workload": f"{CONFIG_NAME[args.config]} x {args.instances}"
                               + (f" + serial-chain x {args.mix_chains}" if args.mix_chains else "") + " per GPU",
                   "precision_mode": head_name, "algorithm": ALGO[head_name],
                   "dof": "U{2..48}" if args.config == 1 else None, "dt": dt,
                   "integrator": "semi-implicit Euler", "control": CONTROL[args.config],
                   "l2": L2_NOTE},
        "gpu_launches": head["launches"],
    }
    line["modes"] = {}
    for name, r in results.items():
        line["modes"][name] = {
            "value": r["done"] / (r["kernel_ms"] * 1e-3), "ms_per_step": r["kernel_ms"] / args.steps,
            "algorithm": ALGO[name], "dtype": DTYPE[name], "roofline": roof(name, r),
            "launch": launch.get(name),
            "qdd_rel_err_vs_fp64_crba": errs.get(name)}
    for base in ("fp64", "fp64_crba"):
        if base in results:
            for name in ("mixed", "refined", "fp64"):
                if name in results and name != base:
                    line[f"{name}_over_{base}"] = line["modes"][name]["value"] / line["modes"][base]["value"]
    line["roofline"] = roof(head_name, head)
    line["kernel_source_sha16"] = src_hash
    if stale:
        line["ncu_tables_stale"] = {"forms": stale, "note": "profiles/dram_traffic_per_instance_step.json "
                                    "was captured on other sources; its traffic and instruction counts are not used"}
    line["peaks_measured"] = {"fp64_tflops": p64, "fp32_tflops": p32}
    line["clocks"] = head["clocks"]
    line["failed_instances"] = {k: r["failed_instances"] for k, r in results.items()}
    line["completed_fraction"] = {k: r["done"] / ((args.instances + args.mix_chains) * world * args.steps)
                                  for k, r in results.items()}
    line["e2e"] = {"value": e2e_done / e2e_s, "unit": UNIT,
                   "h2d_bytes_per_step": (qn.nbytes + vn.nbytes) / args.steps,
                   "d2h_bytes_per_step": (qo.nbytes + vo_.nbytes) / args.steps,
                   "note": "gpb_set_state (pinned host) + gpb_simulate + gpb_get_state"}
    if rank == 0 and not args.skip_cpu:
        line["cpu_baseline"] = cpu_reference(M, q0, v0, aux, args.config, args.steps)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# ---------------------------------------------------------------------------
# serving mix: acrobot / chain / cube / quadruped = 40/30/20/10 %, horizons
# log-uniform in [100, 50000] steps, Poisson arrivals, continuous batching

SERVE_MIX = (0.4, 0.3, 0.2, 0.1)
SERVE_HORIZON = (100, 50000)


def serve_classes(budget_bytes, algorithm="aba"):
    """Slot classes of the serving mix (chains split by DOF), budget shares by
    expected occupancy (mix share × mean per-step cost), and per-class chunk
    steps that make one tick cost about the same for every class."""
    from gpb.serve import SlotClass

    def cost(nb, nv, nc):  # FP64 flops per step (leading terms of gpb.flops)
        if algorithm == "aba":
            return 620 * nb + 130 * nc + (60 * nb if nc else 0)
        return 625 * nb + 11 * nv * (nv + 1) / 2 + nv ** 3 / 3 + 2 * nv * nv + 80 * nc

    specs = [((2, 2, 2, 0, 0), SERVE_MIX[0])]
    for hi in (8, 16, 24, 32, 40, 48):
        specs.append(((hi, hi, hi, 0, 0), SERVE_MIX[1] * 8 / 47))
    specs[-1] = (specs[-1][0], SERVE_MIX[1] * 7 / 47)  # n = 2..48: 47 values
    specs[1] = (specs[1][0], SERVE_MIX[1] * 7 / 47)
    specs.append(((1, 7, 6, 8, 1), SERVE_MIX[2]))
    specs.append(((13, 19, 18, 4, 1), SERVE_MIX[3]))
    from gpb.serve import plan

    cmax = max(cost(s[0], s[2], s[3]) for s, _ in specs)
    _, nbytes = plan([SlotClass(*s, packs=1) for s, _ in specs])
    out = []
    for (s, share), nb in zip(specs, nbytes):
        c = cost(s[0], s[2], s[3])
        # concurrent slots ∝ share × residence time (∝ cost); bytes ∝ slots × pack bytes
        # acrobots and chains are planar chains: their classes run the specialised passes
        out.append(SlotClass(*s, weight=share * c * float(nb), chunk_steps=max(1, int(round(16 * cmax / c))),
                             planar_only=s[3] == 0))
    return out


def run_serve(args):
    import torch

    torch.cuda.set_device(0)
    import gpb
    from gpb import Model
    from gpb.serve import Server

    ctx = gpb.Context(0)
    prec_of = {"fp64": gpb.FP64, "mixed": gpb.MIXED, "refined": gpb.MIXED_REFINED}
    runs = []
    for pname in args.serve_precisions.split(","):
        for rate in [float(r) for r in args.serve_rates.split(",")]:
            t_arr, cfg, horizon, per = serve_stream(rate, args.serve_seconds, args.seed)
            n = len(t_arr)
            S = Server(ctx, serve_classes(int(args.serve_budget_gb * 1e9), args.serve_algorithm),
                       precision=prec_of[pname],
                       chunk_steps=16, hbm_budget_bytes=int(args.serve_budget_gb * 1e9),
                       algorithm=gpb.ALGO_ABA if args.serve_algorithm == "aba" else gpb.ALGO_CRBA)
            lat, trace, wall = serve_run(S, gpb, t_arr, cfg, horizon, per, args.serve_seconds, args.serve_drain)
            ok = np.isfinite(lat)
            offered = float(rate * np.mean(horizon)) if n else 0.0
            runs.append({
                "precision": pname, "rate_req_s": rate, "requests": n, "completed": int(ok.sum()),
                "censored": int((~ok).sum()),
                "latency_s": {"p50": float(np.quantile(lat[ok], 0.5)) if ok.any() else None,
                              "p99": float(np.quantile(lat[ok], 0.99)) if ok.any() else None,
                              "max": float(lat[ok].max()) if ok.any() else None},
                "latency_by_config_p50_s": {CONFIG_NAME[c]: float(np.median(lat[ok & (cfg == c)]))
                                            for c in range(4) if (ok & (cfg == c)).any()},
                "offered_instance_steps_per_s": offered,
                "achieved_in_window_instance_steps_per_s": steps_rate(trace, 0.0, args.serve_seconds),
                "wall_s": wall, "ticks": int(trace.shape[0]),
                "pool_bytes": S.stats()["pool_bytes"]})
            S.close()
            print(json.dumps(runs[-1]), file=sys.stderr, flush=True)
    line = {"metric": "serving latency (p50/p99) and throughput, Poisson arrivals",
            "unit": "s", "n_gpus": 1, "higher_is_better": False,
            "config": {"workload": "serving mix acrobot/chain/cube/quadruped = 40/30/20/10 %",
                       "horizon_steps": "log-uniform [100, 50000]",
                       "arrival_window_s": args.serve_seconds, "hbm_budget_gb": args.serve_budget_gb,
                       "admission": "FIFO per slot class; pool sized to the budget"},
            "data": "synthetic (seeded)", "runs": runs}
    print(json.dumps(line))
    ctx.close()
    return 0


def serve_stream(rate, seconds, seed):
    """Poisson arrivals of the serving mix: arrival times, configuration, horizon
    and the instance each request takes from its configuration's seeded model."""
    from gpb import Model

    rng = np.random.default_rng(seed)
    n = int(rng.poisson(rate * seconds))
    t_arr = np.sort(rng.uniform(0.0, seconds, n))
    cfg = rng.choice(4, size=n, p=SERVE_MIX)
    lo, hi = np.log(SERVE_HORIZON[0]), np.log(SERVE_HORIZON[1])
    horizon = np.exp(rng.uniform(lo, hi, n)).astype(np.int64)
    per = []
    for c in range(4):
        idx = np.nonzero(cfg == c)[0]
        M, q0, v0, aux = Model.from_config(c, max(len(idx), 1), seed=seed + 17 * c)
        per.append({"idx": idx, "M": M, "q0": q0, "v0": v0, "aux": aux, "next": 0, "t": t_arr[idx]})
    return t_arr, cfg, horizon, per


def serve_run(S, gpb, t_arr, cfg, horizon, per, window, drain):
    """Feeds the stream to server S in real time for `window` seconds, then
    runs at most `drain` seconds more.  Returns per-request
    latency (NaN if not finished), the (time, instance-steps run) samples of
    every tick and the wall time."""
    n = len(t_arr)
    req_of, lat = {}, np.full(n, np.nan)
    trace = []
    t0 = time.perf_counter()
    while True:
        now = time.perf_counter() - t0
        for c, P in enumerate(per):
            upto = int(np.searchsorted(P["t"], now, side="right"))
            if upto > P["next"]:
                a, b = P["next"], upto
                ids = S.submit(P["M"], a, b - a, P["q0"], P["v0"], dt=DT[c], steps=horizon[P["idx"][a:b]],
                               control=CONTROL[c], tau=P["aux"] if c == 3 else None, seed=7 + c, kp=50.0,
                               kd=2.0, keys=0)
                for rid, r in zip(ids.tolist(), P["idx"][a:b].tolist()):
                    req_of[rid] = r
                P["next"] = b
        st = S.stats()
        if all(P["next"] == len(P["idx"]) for P in per) and st["pending"] == 0 and st["active"] == 0:
            break
        if now > window + drain:
            break
        if st["pending"] == 0 and st["active"] == 0:
            continue
        S.tick()
        tdone = time.perf_counter() - t0
        trace.append((tdone, S.stats()["steps"]))
        done = S.completed()
        if done.size:
            for rid in done.tolist():
                r = req_of.pop(rid)
                lat[r] = tdone - t_arr[r]
            S.forget(done)
    return lat, np.asarray(trace).reshape(-1, 2), time.perf_counter() - t0


def steps_rate(trace, t_from, t_to):
    """Instance-steps per second run between two times of a serve_run trace."""
    if trace.shape[0] < 2:
        return 0.0
    s0, s1 = np.interp([t_from, t_to], trace[:, 0], trace[:, 1])
    return float((s1 - s0) / max(t_to - t_from, 1e-9))


def run_serve_slo(args):
    """The serving target: p99 latency against the isolated-request time at a
    fraction (default 50 %) of the peak sustainable load.

    1. Isolated time: single requests on an empty server — per configuration
       the time of a short and a long horizon (chains at five DOF counts), a
       linear model a + b·H per configuration (chains: b interpolated in DOF).
    2. Peak: arrivals far above what the GPU can run (offered 20× the measured
       throughput), so that the running set only grows; the instance-steps run
       (gpb_server_stats.steps) in the second half of the window over that
       half's length is the saturated throughput.
    3. Load: Poisson arrivals at load × peak ÷ mean horizon for the arrival
       window, then drained; per request the slowdown latency ÷ isolated time.
    Throughput of the load run counts the instance-steps run inside the
    arrival window only."""
    import torch

    torch.cuda.set_device(0)
    import gpb
    from gpb import Model
    from gpb.serve import Server

    ctx = gpb.Context(0)
    prec_of = {"fp64": gpb.FP64, "mixed": gpb.MIXED}
    algo = gpb.ALGO_ABA if args.serve_algorithm == "aba" else gpb.ALGO_CRBA
    budget = int(args.serve_budget_gb * 1e9)
    mean_h = (SERVE_HORIZON[1] - SERVE_HORIZON[0]) / math.log(SERVE_HORIZON[1] / SERVE_HORIZON[0])
    out_runs = []
    for pname in args.serve_precisions.split(","):
        def server():
            return Server(ctx, serve_classes(budget, args.serve_algorithm), precision=prec_of[pname],
                          chunk_steps=16, hbm_budget_bytes=budget, algorithm=algo)

        # 1. isolated times
        S = server()
        iso = {}
        H_lo, H_hi = 200, 4000
        probe = {0: [None], 1: [2, 13, 25, 37, 48], 2: [None], 3: [None]}
        for c in range(4):
            M, q0, v0, aux = Model.from_config(c, 256, seed=args.seed + 5 * c)
            nv = np.diff(M.offsets()[1])
            for dof in probe[c]:
                j = 0 if dof is None else int(np.argmin(np.abs(nv - dof)))
                T = []
                for H in (H_lo, H_hi):
                    t0 = time.perf_counter()
                    S.submit(M, j, 1, q0, v0, dt=DT[c], steps=H, control=CONTROL[c],
                             tau=aux if c == 3 else None, seed=7 + c, kp=50.0, kd=2.0, keys=0)
                    while True:
                        S.tick()
                        d = S.completed()
                        if d.size:
                            S.forget(d)
                            break
                    T.append(time.perf_counter() - t0)
                b = (T[1] - T[0]) / (H_hi - H_lo)
                iso[(c, int(nv[j]) if dof is not None else None)] = (T[0] - b * H_lo, b)
        S.close()
        chain_dofs = sorted(k[1] for k in iso if k[0] == 1)

        def t_iso(c, dof, H):
            if c != 1:
                a, b = iso[(c, None)]
                return a + b * H
            a = np.interp(dof, chain_dofs, [iso[(1, d)][0] for d in chain_dofs])
            b = np.interp(dof, chain_dofs, [iso[(1, d)][1] for d in chain_dofs])
            return a + b * H

        # 2. peak sustainable throughput (closed loop: the queue never empties)
        w = max(args.serve_seconds, 10.0)
        t_arr, cfg, horizon, per = serve_stream(args.serve_peak_rate, w, args.seed + 1)
        S = server()
        _, trace, _ = serve_run(S, gpb, t_arr, cfg, horizon, per, w, 0.0)
        S.close()
        peak = steps_rate(trace, w / 2, min(w, trace[-1, 0]))

        # 3. the load run at args.serve_load of the peak
        rate = args.serve_load * peak / mean_h
        t_arr, cfg, horizon, per = serve_stream(rate, args.serve_seconds, args.seed)
        dof = np.zeros(len(t_arr), np.int64)
        for c, P in enumerate(per):
            nvs = np.diff(P["M"].offsets()[1])
            dof[P["idx"]] = nvs[:len(P["idx"])]
        S = server()
        lat, trace, wall = serve_run(S, gpb, t_arr, cfg, horizon, per, args.serve_seconds, args.serve_drain)
        S.close()
        ok = np.isfinite(lat)
        tiso = np.array([t_iso(int(cfg[r]), int(dof[r]), int(horizon[r])) for r in range(len(t_arr))])
        slow = lat / tiso

        def q(x, p):
            return float(np.quantile(x, p)) if x.size else None

        by_cfg = {}
        for c in range(4):
            m = ok & (cfg == c)
            by_cfg[CONFIG_NAME[c]] = {"requests": int(m.sum()), "latency_p99_s": q(lat[m], 0.99),
                                      "isolated_p99_s": q(tiso[m], 0.99),
                                      "slowdown_p50": q(slow[m], 0.5), "slowdown_p99": q(slow[m], 0.99)}
        run = {"precision": pname, "peak_instance_steps_per_s": peak, "peak_arrival_rate_req_s": args.serve_peak_rate,
               "load_fraction": args.serve_load,
               "rate_req_s": rate, "requests": int(len(t_arr)), "completed": int(ok.sum()),
               "censored": int((~ok).sum()),
               "latency_s": {"p50": q(lat[ok], 0.5), "p99": q(lat[ok], 0.99)},
               "isolated_s": {"p50": q(tiso[ok], 0.5), "p99": q(tiso[ok], 0.99)},
               "p99_over_isolated_p99": (q(lat[ok], 0.99) / q(tiso[ok], 0.99)) if ok.any() else None,
               "slowdown": {"p50": q(slow[ok], 0.5), "p99": q(slow[ok], 0.99), "max": float(slow[ok].max())
                            if ok.any() else None,
                            "definition": "latency ÷ the same request's isolated time (class, DOF, horizon)"},
               "by_config": by_cfg,
               "achieved_in_window_instance_steps_per_s": steps_rate(trace, 0.0, args.serve_seconds),
               "offered_instance_steps_per_s": rate * mean_h,
               "isolated_model": {f"{CONFIG_NAME[k[0]]}{'' if k[1] is None else ' n=' + str(k[1])}":
                                  {"fixed_s": a, "per_step_s": b} for k, (a, b) in iso.items()},
               "wall_s": wall}
        out_runs.append(run)
        print(json.dumps(run), file=sys.stderr, flush=True)
    line = {"metric": "serving p99 latency over the isolated-request time at a fraction of peak load",
            "unit": "ratio", "n_gpus": 1, "higher_is_better": False,
            "config": {"workload": "serving mix acrobot/chain/cube/quadruped = 40/30/20/10 %",
                       "horizon_steps": "log-uniform [100, 50000]", "arrival_window_s": args.serve_seconds,
                       "hbm_budget_gb": args.serve_budget_gb, "algorithm": args.serve_algorithm},
            "data": "synthetic (seeded)", "runs": out_runs}
    print(json.dumps(line))
    ctx.close()
    return 0


# ---------------------------------------------------------------------------
# cuboid colliders: build_gripper batches (both jaws 0.02-0.07 m into the cube,
# every evaluation runs 3 GJK/EPA pair queries per instance) and independent
# collision queries (gpb_collide_cuboids_device)

CUBOID_DT = 1e-5  # the squeezed 0.1 kg cube's regularised friction needs it


def gripper_batch(n, seed):
    from gpb import Model, builders

    M = Model.from_mechanisms([builders.build_gripper()] * n)
    q, v = builders.gripper_states(np.random.default_rng(seed), n)
    return M, q.ravel(), v.ravel()


def run_cuboids(args):
    rank, world, local = dist_env()
    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    import ctypes

    import gpb
    from gpb import Batch, builders
    from gpb.flops import aba_model_flops, model_flops

    L = gpb.lib()
    ctx = gpb.Context(local)
    n = args.instances
    M, q0, v0 = gripper_batch(n, shard_seed(args.seed, rank))
    B = Batch(M, ctx)
    work = json.loads((ROOT / "profiles" / "collision_work.json").read_text())
    pair_flops = work["gripper"]["mean_flops_per_evaluation"]
    MODES = {"fp64": (gpb.FP64, gpb.ALGO_ABA, aba_model_flops(M, False)),
             "fp64_crba": (gpb.FP64, gpb.ALGO_CRBA, model_flops(M, 0)),
             "mixed": (gpb.MIXED, gpb.ALGO_ABA, aba_model_flops(M, True))}

    def peak():
        t = ctypes.c_double()
        gpb._abi.check(L.gpb_fma_peak(local, gpb.FP64, 32, ctypes.byref(t)), "gpb_fma_peak")
        return t.value

    p64 = peak()
    results = {}
    for name, (prec, algo, inst_flops) in MODES.items():
        B.set_algorithm(algo)
        B.update(q0, v0)
        B.clear_status()
        w, _, _ = B.autotune(CUBOID_DT, 0, prec, trial_steps=10)
        if args.warmup:
            B.simulate_steps(args.warmup, CUBOID_DT, 0, prec)
        if world > 1:
            torch.distributed.barrier()
        ctx.synchronize()
        flush_l2(local)
        with Clocks(local) as clk:
            l0 = ctx.launches
            B.simulate_steps(args.steps, CUBOID_DT, 0, prec, step0=args.warmup)
            kernel_ms = L.gpb_last_launch_ms(ctx.h)
            ctx.synchronize()
            launches = ctx.launches - l0
        kernel_ms = all_reduce(kernel_ms, "max", world, f"cuda:{local}")
        done = B.steps_done()
        flops = float(np.dot(done, inst_flops.astype(np.float64))) + float(done.sum()) * pair_flops
        results[name] = {"kernel_ms": kernel_ms, "clocks": clk.summary(), "launches": launches,
                         "warps_per_sm": w, "failed_instances": int(np.sum(B.status() != 0)),
                         "done": all_reduce(float(done.sum()), "sum", world, f"cuda:{local}"),
                         "flops": all_reduce(flops, "sum", world, f"cuda:{local}")}
    head_name = max(("fp64", "fp64_crba"), key=lambda k: results[k]["done"] / results[k]["kernel_ms"])
    head = results[head_name]

    def roof(r, extra):
        ach = r["flops"] / (r["kernel_ms"] * 1e-3) / 1e12
        return {"bound": "fp64", "achieved": ach, "peak": p64, "unit": "TFLOP/s", "frac": ach / p64,
                "traffic": None, "peak_source": "measured FP64 FMA microbenchmark (gpb_fma_peak), this run",
                "work": extra}

    # independent collision queries on device buffers, CUDA events on the stream
    # the kernel runs on
    queries = {}
    stream = torch.cuda.Stream()  # a stream of its own: events and kernel on the same one
    for kind in ("shallow", "deep"):
        rng = np.random.default_rng(shard_seed(args.seed, rank))
        pa, da, pb, db = builders.cuboid_pairs(rng, args.pairs, kind)
        dev = {k: torch.from_numpy(np.ascontiguousarray(x)).cuda() for k, x in
               (("pa", pa), ("da", da), ("pb", pb), ("db", db))}
        res = torch.empty(args.pairs, dtype=torch.int32, device="cuda")
        ca = torch.empty((args.pairs, 3), dtype=torch.float64, device="cuda")
        cb = torch.empty_like(ca)

        def launch():
            gpb.collision.collide_cuboids_device(ctx, args.pairs, dev["pa"].data_ptr(), dev["da"].data_ptr(),
                                                 dev["pb"].data_ptr(), dev["db"].data_ptr(), res.data_ptr(),
                                                 ca.data_ptr(), cb.data_ptr(), stream.cuda_stream)

        torch.cuda.synchronize()
        for _ in range(3):
            launch()
        torch.cuda.synchronize()
        reps = 10
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        l0 = ctx.launches
        with Clocks(local) as clk:
            e0.record(stream)
            for _ in range(reps):
                launch()
            e1.record(stream)
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        assert ctx.launches - l0 == reps
        per = work["pairs_" + kind]["mean_flops"]
        ach = args.pairs * per / (ms * 1e-3) / 1e12
        queries[kind] = {"pairs_per_s": args.pairs / (ms * 1e-3), "ms_per_launch": ms, "launches": reps,
                         "hit_fraction": float((res == 1).float().mean()),
                         "failed": int((res < 0).sum()), "clocks": clk.summary(),
                         "roofline": {"bound": "fp64", "achieved": ach, "peak": p64, "unit": "TFLOP/s",
                                      "frac": ach / p64, "traffic": None,
                                      "work": f"{per:.0f} FP64 operations per query (mean, "
                                              f"profiles/collision_work.json: {work['pairs_' + kind]['sample']})"}}
        del dev, res, ca, cb
    # e2e through the public API: pinned host state in, K steps, state out
    q_h = torch.from_numpy(q0).pin_memory().numpy()
    v_h = torch.from_numpy(v0).pin_memory().numpy()
    prec, algo, _ = MODES[head_name]
    B.set_algorithm(algo)
    ctx.synchronize()
    t0 = time.perf_counter()
    B.update(q_h, v_h)
    B.simulate_steps(args.steps, CUBOID_DT, 0, prec)
    qo, vo = B.state()
    e2e_s = all_reduce(time.perf_counter() - t0, "max", world, f"cuda:{local}")
    e2e_done = all_reduce(float(B.steps_done().sum()), "sum", world, f"cuda:{local}")
    line = {
        "metric": "instance-steps/s of build_gripper batches (GJK/EPA cuboid contacts)",
        "value": head["done"] / (head["kernel_ms"] * 1e-3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": head["kernel_ms"] / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded numpy draws of gripper states and cuboid pairs)",
        "config": {"workload": f"gripper x {n} per GPU (3 cuboid pairs per evaluation)",
                   "algorithm": {"fp64": "articulated-body algorithm",
                                 "fp64_crba": "CRBA + Cholesky (the reference's route)"}[head_name],
                   "dt": CUBOID_DT, "integrator": "semi-implicit Euler", "control": "host (zero torque)",
                   "l2": L2_NOTE},
        "gpu_launches": head["launches"],
        "roofline": roof(head, f"{pair_flops:.0f} FP64 operations of the 3 pair queries per evaluation "
                               f"(profiles/collision_work.json) + the dynamics flops (gpb.flops)"),
        "clocks": head["clocks"],
        "modes": {k: {"value": r["done"] / (r["kernel_ms"] * 1e-3), "ms_per_step": r["kernel_ms"] / args.steps,
                      "warps_per_sm": r["warps_per_sm"], "failed_instances": r["failed_instances"],
                      "roofline": roof(r, "as above")} for k, r in results.items()},
        "collision_queries": {"n_pairs": args.pairs, **queries},
        "e2e": {"value": e2e_done / e2e_s, "unit": UNIT, "h2d_bytes_per_step": (q_h.nbytes + v_h.nbytes) / args.steps,
                "d2h_bytes_per_step": (qo.nbytes + vo.nbytes) / args.steps,
                "note": "gpb_set_state (pinned host) + gpb_simulate + gpb_get_state"},
    }
    line["kernel_source_sha16"] = kernel_source_hash()
    if rank == 0 and not args.skip_cpu:
        line["cpu_baseline"] = cpu_cuboids(M, q0, v0, args.steps)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def cpu_cuboids(M, q0, v0, steps, seconds_target=12.0):
    """The oracle on a bounded sample of the gripper batch, all host threads."""
    import oracle

    threads = os.cpu_count() or 1
    q, v = q0.copy(), v0.copy()
    cal = min(M.n, 8 * threads)
    t = time.perf_counter()
    oracle.simulate_batch(M, q, v, CUBOID_DT, 2, end=cal, threads=threads)
    per = (time.perf_counter() - t) / (cal * 2)
    sample = min(M.n, 4096)
    K = max(5, min(steps, int(seconds_target / max(per * sample, 1e-9))))
    q, v = q0.copy(), v0.copy()
    t = time.perf_counter()
    oracle.simulate_batch(M, q, v, CUBOID_DT, K, end=sample, threads=threads)
    el = time.perf_counter() - t
    return {"value": sample * K / el, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"first {sample} of {M.n} grippers x {K} steps (oracle restatement, {threads} host threads)"}


# ---------------------------------------------------------------------------
# velocity stepping: the floating-cube configuration's cubes placed resting on
# the ground (1-4 corners in contact), one friction-cone program per cube-step

VSTEP_DT = 1e-3


def resting_cubes(n, seed):
    from gpb import Model, builders

    M, _, _, _ = Model.from_config(2, n, seed=seed)
    side = 2.0 * np.abs(M.contact_params.reshape(-1, 6)[::8, 0])  # first corner: (l/2, l/2, -l/2)
    q, v = builders.resting_cube_states(np.random.default_rng(seed), M, lambda i: side[i], tilt=0.005)
    return M, q, v


def run_vstep(args):
    rank, world, local = dist_env()
    import torch

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    import gpb
    from gpb import Batch

    L = gpb.lib()
    ctx = gpb.Context(local)
    n = args.instances
    M, q0, v0 = resting_cubes(n, shard_seed(args.seed, rank))
    B = Batch(M, ctx)
    B.update(q0, v0)
    w, _, _ = B.autotune(VSTEP_DT, gpb.VELOCITY_STEPPING, gpb.FP64, trial_steps=5)
    if args.warmup:
        B.simulate_steps(args.warmup, VSTEP_DT, gpb.VELOCITY_STEPPING)
    ctx.synchronize()
    flush_l2(local)
    with Clocks(local) as clk:
        l0 = ctx.launches
        B.simulate_steps(args.steps, VSTEP_DT, gpb.VELOCITY_STEPPING, step0=args.warmup)
        kernel_ms = L.gpb_last_launch_ms(ctx.h)
        ctx.synchronize()
        launches = ctx.launches - l0
    kernel_ms = all_reduce(kernel_ms, "max", world, f"cuda:{local}")
    done = all_reduce(float(B.steps_done().sum()), "sum", world, f"cuda:{local}")
    failed = int(np.sum(B.status() != 0))
    # e2e: pinned host state in, K steps, state out
    q_h = torch.from_numpy(q0).pin_memory().numpy()
    v_h = torch.from_numpy(v0).pin_memory().numpy()
    ctx.synchronize()
    t0 = time.perf_counter()
    B.update(q_h, v_h)
    B.clear_status()
    B.simulate_steps(args.steps, VSTEP_DT, gpb.VELOCITY_STEPPING)
    qo, vo = B.state()
    e2e_s = all_reduce(time.perf_counter() - t0, "max", world, f"cuda:{local}")
    e2e_done = all_reduce(float(B.steps_done().sum()), "sum", world, f"cuda:{local}")
    # FP64 roofline: executed FP64 operations per instance-step (ncu thread-level
    # counters of predicated-on lanes, 2 per FMA) from the committed capture
    import ctypes

    tpk = ctypes.c_double()
    gpb._abi.check(L.gpb_fma_peak(local, gpb.FP64, 32, ctypes.byref(tpk)), "gpb_fma_peak")
    roof = None
    try:
        wk = json.loads((ROOT / "profiles" / "vstep_work.json").read_text())
        ach = done / (kernel_ms * 1e-3) * wk["fp64_flops_per_instance_step"] / 1e12
        roof = {"bound": "fp64", "achieved": ach, "peak": tpk.value, "unit": "TFLOP/s", "frac": ach / tpk.value,
                "traffic": None, "peak_source": "measured FP64 FMA microbenchmark (gpb_fma_peak), this run",
                "work": f"{wk['fp64_flops_per_instance_step']:.0f} FP64 operations per instance-step "
                        f"({wk['source']})"}
    except (OSError, ValueError, KeyError):
        pass
    line = {
        "metric": "instance-steps/s of velocity stepping (friction-cone impulse program per step)",
        "value": done / (kernel_ms * 1e-3), "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": kernel_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (the floating-cube configuration's cubes, seeded resting states)",
        "config": {"workload": f"resting cube x {n} per GPU (8 corner contacts, ground plane)",
                   "dt": VSTEP_DT, "integrator": "velocity stepping", "warps_per_sm": w,
                   "l2": L2_NOTE},
        "gpu_launches": launches, "clocks": clk.summary(), "failed_instances": failed, "roofline": roof,
        "e2e": {"value": e2e_done / e2e_s, "unit": UNIT, "h2d_bytes_per_step": (q_h.nbytes + v_h.nbytes) / args.steps,
                "d2h_bytes_per_step": (qo.nbytes + vo.nbytes) / args.steps,
                "note": "gpb_set_state (pinned host) + gpb_simulate + gpb_get_state"},
    }
    if rank == 0 and not args.skip_cpu:
        import oracle

        threads = os.cpu_count() or 1
        qc, vc = q0.copy(), v0.copy()
        cal = min(n, 8 * threads)
        t = time.perf_counter()
        oracle.simulate_batch(M, qc, vc, VSTEP_DT, 2, integrator=gpb.VELOCITY_STEPPING, end=cal, threads=threads)
        per = (time.perf_counter() - t) / (cal * 2)
        sample = min(n, 4096)
        K = max(5, min(args.steps, int(12.0 / max(per * sample, 1e-9))))
        qc, vc = q0.copy(), v0.copy()
        t = time.perf_counter()
        oracle.simulate_batch(M, qc, vc, VSTEP_DT, K, integrator=gpb.VELOCITY_STEPPING, end=sample,
                              threads=threads)
        el = time.perf_counter() - t
        line["cpu_baseline"] = {"value": sample * K / el, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"first {sample} of {n} cubes x {K} steps (oracle restatement, "
                                          f"{threads} host threads)"}
    line["kernel_source_sha16"] = kernel_source_hash()
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference_cuboids(args) if args.cuboids else run_reference(args)
    if args.serve_slo:
        return run_serve_slo(args)
    if args.serve:
        return run_serve(args)
    if args.cuboids:
        return run_cuboids(args)
    if args.vstep:
        return run_vstep(args)
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())
