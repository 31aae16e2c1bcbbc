#!/usr/bin/env python
"""Benchmark of the flow right-hand side on GB300.

A step is one right-hand-side evaluation of the pseudo-fermion FRG flow:
compute_dΣ! followed by compute_dΓ_2l! (the reference's src/Flow/flow_self.jl
and src/Flow/compute.jl) on a seeded synthetic state of the pyrochlore
lattice, L = 6, nearest-neighbour Heisenberg J1 = 1, SU(2), 50/15/10 positive
frequencies, Λ = 1, vertex entries N(0, 0.05) plus the bare coupling on the
Ω = 0 slice of the t-channel spin component.  The metric is right-hand-side
evaluations per second of the mixed-precision GPU path; the FP64 GPU path,
the mixed path's error against it and the CPU oracle are reported beside it.

The full-flow leg (``full_flow``) runs the flow of the same lattice and
model, pyrochlore L = 6 two-loop (Λ 50 → 0.01 or the breakdown, χ measured
after every accepted step), in FP64 and in mixed precision, and the mixed
right-hand side once more on the FP64 flow's accepted step sequence; it
reports the wall times and χ(ω = 0) of the mixed flows against the FP64 one
(``--flow`` selects the square L = 3 one-loop or the kagome L = 8 U(1)-DM
three-loop flow instead).  The warm-start leg (``--warm-start TRAIN,TEST``,
honeycomb J1-J2-J3) counts parquet iterations from the bare couplings, the
mean training vertex, the least-squares part alone and the least-squares
part with the network.  ``--sweep N`` runs N square J1-J2 flows sharing the
GPU.  Before the warm-up the team shape of the passes is picked by the
autotuner.

``--impl reference`` times the CPU restatement of the reference's algorithm
(the reference is Julia, which is not installed on these machines) on all
host cores: full right-hand sides of the same workload, as many as fit its
time budget.
"""
from __future__ import annotations

import argparse
import csv
import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import __graft_entry__ as entry  # noqa: E402

METRIC = "full-flow s & dΓ evals/s, mixed vs FP64 GPU on 1 GB300 at ≤1e-6 rel χ err"
UNIT = "dΓ evals/s"
WORKLOAD = "pyrochlore-L6-2l"
GAMMA_TOL = (1e-8, 1e-4)
SIGMA_TOL = (1e-8, 1e-4)


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default=WORKLOAD)
    p.add_argument("--fp64-steps", type=int, default=2)
    p.add_argument("--ref-seconds", type=float, default=150.0,
                   help="CPU time budget of the reference arm's timed steps (full right-hand sides)")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    p.add_argument("--no-e2e", action="store_true", help="skip the host-buffer end-to-end leg (profiling runs)")
    p.add_argument("--no-flow", action="store_true", help="skip the full-flow leg")
    p.add_argument("--team-shape", default="", help="lanes x sites per lane of the passes (empty: autotuned)")
    p.add_argument("--flow-final", type=float, default=0.01, help="final cutoff of the full-flow leg")
    p.add_argument("--flow-precisions", default="fp64,mixed", help="precisions of the full-flow leg")
    p.add_argument("--flow", default="pyrochlore-L6-2l", choices=sorted(FLOWS), help="workload of the full-flow leg")
    p.add_argument("--no-replay", action="store_true", help="skip the mixed replay of the FP64 flow's steps")
    p.add_argument("--sweep", type=int, default=0,
                   help="instances of the coupling-sweep leg (square J1-J2, L in 3,4,5,6,8; 0: skip)")
    p.add_argument("--warm-start", default="64,16",
                   help="train,test counts of the learned parquet warm-start leg (honeycomb J1-J2-J3; empty: skip)")
    p.add_argument("--warm-lambda", type=float, default=2.0, help="cutoff of the warm-start leg's parquet solves")
    p.add_argument("--warm-meshes", default="25/15/10", help="positive σ/Ω/ν frequencies of the warm-start leg")
    p.add_argument("--warm-k", type=int, default=32, help="principal components of the warm start")
    return p.parse_args()


def config(args, w, extra=None):
    c = {"workload": w.name, "lattice": w.lattice, "L": w.size, "model": w.model, "J": w.J, "symmetry": w.symmetry,
         "loops": w.loops, "Lambda": w.Lam, "num_sigma": w.num_sigma, "num_omega": w.num_omega, "num_nu": w.num_nu,
         "eval": w.eval, "gamma_tol": list(GAMMA_TOL), "sigma_tol": list(SIGMA_TOL), "noise": w.noise, "seed": w.seed,
         "l2": "flushed between timed steps (256 MiB write); the vertex is L2-resident within a step",
         "parallelism": f"replicas x{args.gpus}"}
    if extra:
        c.update(extra)
    return c


# ---------------------------------------------------------------------------
# clocks (nvidia-smi sampled during the timed region)
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.file = tempfile.NamedTemporaryFile(prefix="clocks_", suffix=".csv", delete=False)
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.file,
                                         stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        self.file.close()

    def summary(self, busy_frac: float = 0.0):
        rows = []
        try:
            with open(self.file.name) as fh:
                for r in csv.reader(fh):
                    if len(r) >= 9:
                        rows.append([x.strip() for x in r])
        except OSError:
            pass
        os.unlink(self.file.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def ncu_profile_summary():
    """Figures of the committed ncu summary of the dominant kernel (profiles/eval_kernel_traffic.txt): the
    workload and precision it was captured on, DRAM bytes of all wave-kernel launches of one right-hand
    side, and the issue, occupancy and cache figures of one captured eval_kernel launch; or None."""
    p = ROOT / "profiles" / "eval_kernel_traffic.txt"
    if not p.exists():
        return None
    out = {}
    for line in p.read_text().splitlines():
        if line.strip() and not line.startswith("#"):
            k, _, v = line.partition(" ")
            v = v.strip()
            try:
                out[k] = float(v)
            except ValueError:
                out[k] = v
    return out


# ---------------------------------------------------------------------------
# CPU baseline: the oracle (CPU restatement) over every channel task, timed in full
# ---------------------------------------------------------------------------
def sigma_corr_of(w) -> bool:
    """The Σ corrections of compute_dΓ_ml! belong to three or more loops (the launcher's default)."""
    return w.loops >= 3


def cpu_rhs_seconds(O, P, a, w):
    """Wall seconds of one full right-hand side of the oracle (dΣ, then dΓ over all channel tasks)."""
    da = np.zeros_like(a.buf)
    t0 = time.perf_counter()
    O.dsigma(P, w.Lam, a.buf, da, *SIGMA_TOL)
    O.dgamma(P, w.loops, w.Lam, a.buf, da, w.eval, gtol=GAMMA_TOL, sigma_corr=sigma_corr_of(w), stol=SIGMA_TOL)
    return time.perf_counter() - t0


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    entry.load_package()
    import pffrg_gb300.workloads as wl

    O = entry.load_oracle()
    w = wl.WORKLOADS[args.workload]
    lat, r, m, a = wl.build_state(w)
    threads = os.cpu_count() or 1
    P = O.Problem(r, m, symmetry=w.symmetry, S=w.S, num_threads=threads)
    # Every step is one full right-hand side (no task sample).  A step takes seconds on the CPU, so
    # the run does at most one untimed warm-up step and as many of the requested timed steps as fit
    # in the time budget (--ref-seconds); "steps" and "warmup" report what was run.
    warm = min(args.warmup, 1)
    t_first = None
    for _ in range(warm):
        t_first = cpu_rhs_seconds(O, P, a, w)
    n = args.steps
    if t_first is not None:
        n = max(1, min(args.steps, int(args.ref_seconds // t_first)))
    times = [cpu_rhs_seconds(O, P, a, w) for _ in range(n)]
    per = float(np.mean(times))
    value = 1.0 / per
    sample = (f"{n} full right-hand sides (dΣ + dΓ over every channel task) after {warm} untimed; "
              f"{args.steps} steps were requested, the CPU budget is {args.ref_seconds:.0f} s; "
              "CPU restatement of the reference algorithm (Julia is not installed)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": n, "warmup": warm, "requested_steps": args.steps, "requested_warmup": args.warmup,
            "ms_per_step": per * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config(args, w), "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads,
                                                        "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# replicas: every rank runs the whole workload on its own GPU (no data-path collective)
# ---------------------------------------------------------------------------
def max_over_ranks(x: float, dist, device) -> float:
    """The largest of the ranks' values (the slowest replica sets the step time)."""
    if not dist:
        return x
    import torch

    t = torch.tensor([x], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world: int, seconds_per_step: float) -> float:
    """Right-hand sides per second of all replicas together (one per rank and step)."""
    return world / seconds_per_step


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def ours(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)

    pkg = entry.load_package()
    import pffrg_gb300._capi as C
    import pffrg_gb300.workloads as wl
    from pffrg_gb300.flow import FlowContext

    w = wl.WORKLOADS[args.workload]
    lat, r, m, a = wl.build_state(w)
    lay = a.layout
    action_bytes = lay.size * 8
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def barrier():
        torch.cuda.synchronize(dev)
        if dist:
            dist.barrier()

    ctx = FlowContext(r, m, symmetry=w.symmetry, S=w.S, precision="mixed", device=local)
    ctx.upload(C.SLOT_A, a)
    # the team shape of the quadrature passes, picked by timing one right-hand side per candidate
    # (or given, for profiling runs that must launch the same kernels every time)
    if args.team_shape:
        team = tuple(int(x) for x in args.team_shape.split("x"))
        ctx.set_team_shape(*team)
    else:
        team = ctx.autotune_team_shape(w.Lam, w.eval, loops=w.loops, gamma_tol=GAMMA_TOL, sigma_tol=SIGMA_TOL)

    def rhs():
        ctx.rhs(w.Lam, w.eval, loops=w.loops, gamma_tol=GAMMA_TOL, sigma_tol=SIGMA_TOL, sigma_corr=sigma_corr_of(w))

    # warm-up
    for _ in range(args.warmup):
        rhs()
    ctx.set_timing(True)
    ctx.read_stats(reset=True)
    barrier()
    with ClockSampler(local) as clocks:
        t_wall0 = time.perf_counter()
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize(dev)
            rhs()
        barrier()
        t_wall = time.perf_counter() - t_wall0
    st = ctx.read_stats(reset=True)
    ctx.set_timing(False)
    ms_step = st["rhs_ms"] / args.steps
    pass_ms_step = st["pass_ms"] / args.steps
    launches_step = st["launches"] / args.steps
    pass_launches_step = st["pass_launches"] / args.steps
    evals_step = st["integrand_evals"]
    alg_bytes_step = st["algorithmic_values"] * 4  # FP32 vertex values on the mixed path
    t_max = max_over_ranks(ms_step, dist, dev)
    value = replica_throughput(world, t_max * 1e-3)

    # mixed result for the error report
    da_mixed = pkg.action.Action.empty_like(a)
    ctx.download(C.SLOT_DA, da_mixed)

    # FP64 comparator on the same state
    fp64_ms, err_mixed = None, None
    if args.fp64_steps > 0:
        fp64_ms, err_mixed = fp64_leg(args, ctx, pkg, C, a, rhs, flush, dev, da_mixed)

    # end to end through the reference-facing calls with host (pinned) buffers
    e2e = None
    if not args.no_e2e:
        e2e = end_to_end(args, ctx, pkg, C, a, w, flush, dev, dist, world)
    ctx.close()

    clk = clocks.summary()
    peak, peak_kind = measured_peaks()
    achieved = alg_bytes_step / (pass_ms_step * 1e-3) / 1e9 if pass_ms_step > 0 else None
    # DRAM bytes per pass launch: the captured wave launch's DRAM rate times the pass time (the
    # traffic of a pass is taken proportional to its kernel time; the capture is one level)
    # DRAM bytes per pass launch: the wave kernels of one right-hand side captured with ncu, divided by
    # the right-hand side's passes; issue and cache figures from one captured eval_kernel launch
    prof = ncu_profile_summary()
    if not (prof and prof.get("workload") == w.name and prof.get("precision") == "mixed"):
        prof = {}
    traffic = (prof["dram_bytes_per_rhs"] / prof["passes_per_rhs"]) if "dram_bytes_per_rhs" in prof else None

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    flow = None
    if world == 1 and not args.no_flow:
        flow = flow_leg(args, local)
    sweep = sweep_leg(args, local) if world == 1 and args.sweep > 0 else None
    warm = warm_start_leg(args, local) if world == 1 and args.warm_start else None
    # CPU baseline (oracle, all host cores, bounded strided sample), rank 0 at N=1 only
    cpu = None
    if world == 1 and not args.no_cpu:
        O = entry.load_oracle()
        threads = os.cpu_count() or 1
        secs = cpu_rhs_seconds(O, O.Problem(r, m, symmetry=w.symmetry, S=w.S, num_threads=threads), a, w)
        cpu = {"value": 1.0 / secs, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"one full right-hand side (dΣ + dΓ over every channel task), {secs:.1f} s; "
                         "CPU restatement of the reference algorithm"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_max, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 integrand / f64 quadrature bookkeeping", "data": "synthetic",
        "config": config(args, w, {"precision": "mixed", "wall_ms_per_step": t_wall * 1e3 / args.steps,
                                   "team_shape": "%dx%d" % team, "vertex_bytes": action_bytes}),
        "e2e": e2e,
        "gpu_launches": int(round(launches_step * args.steps)),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None, "traffic": traffic,
                     "kernel": "quadrature wave kernels of the dΓ passes", "peak_kind": peak_kind,
                     "algorithmic_bytes_per_step": alg_bytes_step, "kernel_ms_per_step": pass_ms_step,
                     "launches_per_step": pass_launches_step,
                     "algorithmic_bytes_per_launch": (alg_bytes_step / pass_launches_step)
                     if pass_launches_step else None,
                     "traffic_note": "DRAM bytes per pass launch: all wave-kernel launches of one right-hand side "
                                     "under ncu / passes per right-hand side (profiles/eval_kernel_traffic.txt)",
                     "limiter": prof.get("limiter"),
                     "issue_active_frac": prof["issue_active_pct"] / 100 if "issue_active_pct" in prof else None,
                     "warps_active_per_sm": prof.get("warps_active_per_sm"),
                     "l1_hit_frac": prof["l1_hit_pct"] / 100 if "l1_hit_pct" in prof else None,
                     "l1_throughput_frac": prof["l1_throughput_pct"] / 100 if "l1_throughput_pct" in prof else None,
                     "l2_throughput_frac": prof["l2_throughput_pct"] / 100 if "l2_throughput_pct" in prof else None,
                     "profile_team_shape": prof.get("team_shape")},
        "cpu_baseline": cpu,
        "fp64": {"value": 1e3 / fp64_ms, "unit": UNIT, "ms_per_step": fp64_ms,
                 "mixed_speedup": fp64_ms / ms_step,
                 "vs_cpu_baseline": (1e3 / fp64_ms) / cpu["value"] if cpu else None} if fp64_ms else None,
        "mixed_vs_cpu_baseline": value / cpu["value"] if cpu else None,
        "mixed_vs_fp64_rel_err": err_mixed,
        "full_flow": flow,
        "sweep": sweep,
        "warm_start": warm,
        "integrand_evals_per_step": evals_step,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


# the full flow of the square-lattice case: L = 3, nearest-neighbour Heisenberg, 1 loop, 50/15/10
# frequencies, bare couplings at Λ = 50 (no parquet start), Bogacki-Shampine tolerance 1e-3, χ at
# every accepted step; both precisions pass the same checkpoints, where their χ(ω = 0) is compared
FLOWS = {
    "square-L3-1l": dict(name="square", size=3, model="heisenberg", symmetry="su2", J=[[1.0]], num_sigma=50,
                         num_omega=15, num_nu=10, num_chi=10, initial=50.0, ode_tol=(1e-3, 1e-3), parquet=False,
                         loops=1),
    # the flow of the benchmark lattice: pyrochlore L = 6, nearest-neighbour Heisenberg, 2 loops, same meshes
    "pyrochlore-L6-2l": dict(name="pyrochlore", size=6, model="heisenberg", symmetry="su2", J=[[1.0]],
                             num_sigma=50, num_omega=15, num_nu=10, num_chi=10, initial=50.0, ode_tol=(1e-3, 1e-3),
                             parquet=False, loops=2),
    # the largest configuration: kagome L = 8 XXZ + DM (J⊥ = 1, Jz = 0.8, Dz = 0.2), U(1)-DM, 3 loops,
    # 60/20/15 frequencies
    "kagome-L8-3l-u1dm": dict(name="kagome", size=8, model="kagome-xxz-dm", symmetry="u1-dm",
                              J=[[1.0, 0.8, 0.2]], num_sigma=60, num_omega=20, num_nu=15, num_chi=10, initial=50.0,
                              ode_tol=(1e-3, 1e-3), parquet=False, loops=3),
}
FLOW_CPS = [20.0, 10.0, 5.0, 2.0, 1.0, 0.5, 0.2, 0.1, 0.05, 0.02]


def _chi0(res):
    """χ(ω = 0) of every site at every measured cutoff of a run (the χ meshes adapt, ω = 0 stays);
    U(1)-DM runs stack χxx, χzz, χxy."""
    return {round(L, 12): (np.concatenate([x[:, 0] for x in c]) if isinstance(c, list) else c[:, 0])
            for (L, mesh, c) in res.chi}


def _chi_err(cm, cf, keys):
    errs = {}
    for L in keys:
        a, b = cm.get(round(L, 12)), cf.get(round(L, 12))
        if a is not None and b is not None:
            errs[str(L)] = float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
    return errs


def flow_leg(args, dev_index):
    """Full flows (ODE steps, χ after every accepted step, resampling) of one workload, Λ 50 -> final, in
    FP64 and mixed precision: seconds, steps and χ(ω = 0) of the mixed flow against the FP64 flow at the
    shared checkpoints.  The mixed right-hand side also replays the FP64 flow's accepted (Λ, dΛ)
    sequence, so that its χ at every one of those cutoffs differs from the FP64 one by the arithmetic
    alone (the two free-running flows choose their steps from their own error ratios)."""
    from pffrg_gb300.launcher import launch

    kw = dict(FLOWS[args.flow])
    name, size, model, sym, J = (kw.pop(k) for k in ("name", "size", "model", "symmetry", "J"))
    runs = {}
    for prec in [s for s in args.flow_precisions.split(",") if s]:
        t0 = time.perf_counter()
        res = launch("", name, size, model, sym, J, final=args.flow_final, cps=FLOW_CPS, precision=prec,
                     device=dev_index, **kw)
        runs[prec] = (time.perf_counter() - t0, res)
    if "fp64" in runs and "mixed" in runs and not args.no_replay:
        t0 = time.perf_counter()
        res = launch("", name, size, model, sym, J, final=args.flow_final, cps=FLOW_CPS, precision="mixed",
                     device=dev_index, schedule=runs["fp64"][1].steps, **kw)
        runs["mixed_replay"] = (time.perf_counter() - t0, res)
    out = {"workload": "%s L=%d %s %s, %d loop, %d/%d/%d, Λ 50 -> %g, ODE tol 1e-3, bare start"
                       % (name, size, model, sym, kw["loops"], kw["num_sigma"], kw["num_omega"], kw["num_nu"],
                          args.flow_final)}
    for prec, (secs, res) in runs.items():
        out[prec] = {"seconds": secs, "accepted_steps": len(res.Lam), "rejected_steps": res.rejected,
                     "final_lambda": res.Lam[-1] if res.Lam else None, "reason": res.reason or "final cutoff",
                     "timers_s": {k: round(v, 3) for k, v in res.timers.items()},
                     "rhs_evaluations": res.rhs_evals}
    if "mixed" in runs and "fp64" in runs:
        out["speedup_mixed_vs_fp64"] = runs["fp64"][0] / runs["mixed"][0]
        cf = _chi0(runs["fp64"][1])
        out["chi_static_rel_err_mixed_vs_fp64"] = _chi_err(_chi0(runs["mixed"][1]), cf, FLOW_CPS)
        if "mixed_replay" in runs:
            cr = _chi0(runs["mixed_replay"][1])
            every = _chi_err(cr, cf, [L for (L, mesh, c) in runs["fp64"][1].chi])
            out["chi_static_rel_err_replay_vs_fp64"] = {
                "checkpoints": _chi_err(cr, cf, FLOW_CPS),
                "max_over_steps": max(every.values()) if every else None,
                "steps_compared": len(every),
                "steps_above_1e-6": sum(1 for v in every.values() if v > 1e-6)}
    return out


SWEEP = dict(num_sigma=30, num_omega=10, num_nu=8, num_chi=6, initial=50.0, final=0.1, ode_tol=(1e-3, 1e-3),
             parquet=False)


def sweep_leg(args, dev_index):
    """Coupling sweep: n square-lattice J1-J2 Heisenberg flows (J2 ~ U[0, 1], seed 2; L = 3, 4, 5, 6, 8 round
    robin), mixed precision, all on one GPU from concurrent streams; against the same instances run one
    after the other, with the on-site χ(ω=0) of each concurrent run against its single run."""
    from pffrg_gb300.launcher import launch
    from pffrg_gb300.sweep import launch_sweep, square_j1j2_sweep

    inst = square_j1j2_sweep(args.sweep)
    t0 = time.perf_counter()
    res = launch_sweep(inst, workers=16, device=dev_index, precision="mixed", **SWEEP)
    t_sweep = time.perf_counter() - t0
    n_ref = min(len(inst), 8)
    t0 = time.perf_counter()
    ref = [launch("", i.name, i.size, i.model, i.symmetry, i.J, device=dev_index, precision="mixed", **SWEEP)
           for i in inst[:n_ref]]
    t_one = (time.perf_counter() - t0) / n_ref
    errs = [float(np.max(np.abs(a.chi[-1][2][0] - b.chi[-1][2][0])) / np.max(np.abs(b.chi[-1][2][0])))
            for a, b in zip(res, ref)]
    return {"workload": "square J1-J2 (J2 ~ U[0,1], seed 2), L in 3,4,5,6,8, 1 loop, 30/10/8, Λ 50 -> 0.1, "
                        "mixed, %d instances" % len(inst),
            "seconds": t_sweep, "instances_per_s": len(inst) / t_sweep,
            "serial_seconds_per_instance": t_one, "speedup_vs_serial": t_one * len(inst) / t_sweep,
            "max_chi_rel_diff_vs_single_runs": max(errs) if errs else None}


def warm_start_leg(args, dev_index):
    """The learned parquet warm start on honeycomb J1-J2-J3 (L=5, (J2, J3) ~ U[0, 0.5]^2, seed 3):
    fit on `train` converged parquet vertices, then parquet iterations to the residual from the bare
    couplings and from the prediction on `test` held-out couplings (FP64)."""
    from pffrg_gb300.launcher import launch
    from pffrg_gb300.warmstart import ParquetWarmStart, coupling_features, vertex_mask

    n_train, n_test = (int(x) for x in args.warm_start.split(","))
    Lam = args.warm_lambda
    sizes = dict(zip(("num_sigma", "num_omega", "num_nu"), (int(x) for x in args.warm_meshes.split("/"))))
    kw = dict(num_chi=4, initial=Lam, final=Lam, parquet=True, parquet_tol=(1e-8, 1e-8), max_iter=200,
              precision="fp64", correlations=False, device=dev_index, **sizes)
    rng = np.random.default_rng(3)
    J = [[[1.0], [float(a)], [float(b)]] for a, b in rng.uniform(0.0, 0.5, size=(n_train + n_test, 2))]
    t0 = time.perf_counter()
    feats, verts = [], []
    for j in J[:n_train]:
        res = launch("", "honeycomb", 5, "heisenberg", "su2", j, **kw)
        feats.append(coupling_features(j))
        verts.append(res.action.buf[vertex_mask(res.action)].copy())
    t_data = time.perf_counter() - t0
    t0 = time.perf_counter()
    ws = ParquetWarmStart(k=args.warm_k, hidden=(64, 64))
    loss = ws.fit(feats, verts, epochs=8000, lr=3e-3)
    t_fit = time.perf_counter() - t0

    class Part:
        """A start predicted by one part of the fitted model (the ablation)."""

        def __init__(self, part):
            self.part = part

        def predict(self, f):
            return ws.predict(f, self.part)

    starts = {"bare": None, "mean": Part("mean"), "lsq": Part("lsq"), "full": Part("full")}
    its = {k: [] for k in starts}
    start_err = {k: [] for k in starts if k != "bare"}
    diffs, rates = [], []
    for j in J[n_train:]:
        ref = None
        for name, st in starts.items():
            r = launch("", "honeycomb", 5, "heisenberg", "su2", j, warm_start=st, **kw)
            its[name].append(r.parquet_iterations)
            msk = vertex_mask(r.action)
            if ref is None:
                ref = r.action.buf[msk].copy()
                h = r.parquet_residuals
                if len(h) > 2:  # geometric contraction of the bare iteration's residual
                    rates.append(float((h[-1] / h[1]) ** (1.0 / (len(h) - 2))))
                continue
            scale = float(np.max(np.abs(ref)))
            start_err[name].append(float(np.max(np.abs(st.predict(coupling_features(j)) - ref))) / scale)
            diffs.append(float(np.max(np.abs(r.action.buf[msk] - ref))) / scale)
    mean_it = {k: float(np.mean(v)) for k, v in its.items()}
    return {"workload": "honeycomb J1-J2-J3 L=5, (J2,J3) ~ U[0,0.5]^2 seed 3, %s, Λ=%g, residual 1e-8, FP64"
                        % (args.warm_meshes, Lam),
            "train": n_train, "test": n_test, "components": args.warm_k, "data_seconds": t_data,
            "fit_seconds": t_fit, "fit_loss": loss,
            "iterations_mean": mean_it,
            "iteration_ratio": {k: mean_it["bare"] / max(v, 1e-9) for k, v in mean_it.items() if k != "bare"},
            "start_error_median": {k: float(np.median(v)) for k, v in start_err.items()},
            "bare_contraction_per_iteration_median": float(np.median(rates)) if rates else None,
            "max_converged_vertex_rel_diff": max(diffs) if diffs else None}


def fp64_leg(args, ctx, pkg, C, a, rhs, flush, dev, da_mixed):
    """FP64 right-hand sides on the same state: time per step and the mixed path's error."""
    import torch

    ctx.set_precision("fp64")
    rhs()
    ctx.set_timing(True)
    ctx.read_stats(reset=True)
    for _ in range(args.fp64_steps):
        flush.zero_()
        torch.cuda.synchronize(dev)
        rhs()
    st64 = ctx.read_stats(reset=True)
    ctx.set_timing(False)
    fp64_ms = st64["rhs_ms"] / args.fp64_steps
    da64 = pkg.action.Action.empty_like(a)
    ctx.download(C.SLOT_DA, da64)
    err = float(np.max(np.abs(da_mixed.buf - da64.buf)) / np.max(np.abs(da64.buf)))
    ctx.set_precision("mixed")
    return fp64_ms, err


def end_to_end(args, ctx, pkg, C, a, w, flush, dev, dist, world):
    """The same metric through pffrg_dsigma + pffrg_dgamma with host (pinned) buffers."""
    import ctypes

    import torch

    lay = a.layout
    action_bytes = lay.size * 8
    lib = C.load()
    nbytes = action_bytes
    pa = lib.pffrg_host_alloc(nbytes)
    pd = lib.pffrg_host_alloc(nbytes)
    ha = np.frombuffer((ctypes.c_double * lay.size).from_address(pa), dtype=np.float64)
    hd = np.frombuffer((ctypes.c_double * lay.size).from_address(pd), dtype=np.float64)
    A_host = pkg.action.Action(a.symmetry, lay.num_sites, lay.num_sigma, lay.num_omega, lay.num_nu, a.S, ha)
    D_host = pkg.action.Action(a.symmetry, lay.num_sites, lay.num_sigma, lay.num_omega, lay.num_nu, a.S, hd)
    A_host.buf[:] = a.buf
    for _ in range(1):
        D_host.buf[:] = 0.0
        ctx.compute_dsigma(w.Lam, A_host, D_host, SIGMA_TOL)
        ctx.compute_dgamma(w.Lam, A_host, D_host, w.eval, GAMMA_TOL, loops=w.loops, sigma_corr=sigma_corr_of(w),
                           sigma_tol=SIGMA_TOL)
    e2e_times = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize(dev)
        D_host.buf[:] = 0.0
        t0 = time.perf_counter()
        ctx.compute_dsigma(w.Lam, A_host, D_host, SIGMA_TOL)
        ctx.compute_dgamma(w.Lam, A_host, D_host, w.eval, GAMMA_TOL, loops=w.loops, sigma_corr=sigma_corr_of(w),
                           sigma_tol=SIGMA_TOL)
        e2e_times.append(time.perf_counter() - t0)
    e2e_s = max_over_ranks(float(np.mean(e2e_times)), dist, dev)
    e2e_value = replica_throughput(world, e2e_s)
    h2d = 4 * action_bytes  # a and da uploaded by each of the two calls
    d2h = 2 * action_bytes  # da returned by each call
    lib.pffrg_host_free(pa)
    lib.pffrg_host_free(pd)
    return {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h}


def main():
    args = parse()
    if args.impl == "reference":
        return reference_arm(args)
    return ours(args)


if __name__ == "__main__":
    sys.exit(main())
