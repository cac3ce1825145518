#!/usr/bin/env python3
"""Benchmark of the explicit meshless time step on GB300.

Workload (default): two elastic rings (r_in 0.03 m, r_out 0.04 m, centres 0.09 m
apart) on a dx = 0.05 mm lattice, ~1.76M particles, total-Lagrangian SPH with the
Randles-Libersky correction and penalty contact (the rings_tl_contact structure),
E 1e7 Pa, nu 0.4, rho 1200 kg/m^3, +-10 m/s, h = 1.3 dx, dt = 0.3 h / c0, mixed
precision (FP32 pair sums, FP64 position/velocity RK4 state and 2x2 inversions).
Synthetic, seeded data of the workload's shapes (there is no external dataset).

Metric: particle-steps/s = particles x RK4 steps / time, the whole step included
(4 stages, contact, boundary update).  One JSON line on rank 0.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload c2|c1|c3|c4|corot|godunov|potential|ulweak|tlweak|tlfem|ulfem]
                  [--precision mixed|fp64|fp64_strict]

The family workloads (corot, godunov, potential, ulweak, tlweak, tlfem, ulfem) are
ensembles of the reference's own two-ring set-up of that family (ulfem: FP64 forms
only).

With --impl reference it times the reference's CPU implementation of the same path
(single-threaded; the reference's own build where this host has one, else the oracle
restatement) on all host cores.
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
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "particle-steps/s on 1 GB300: plain FP64 vs mixed/batched at <=1e-4 rel err"
UNIT = "particle-steps/s"


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


FAMILIES = ("corot", "godunov", "potential", "ulweak", "tlweak", "tlfem", "ulfem")
FP64_ONLY = ("ulfem",)  # the weak UL form on element maps has no mixed form (no per-stage RKPM)


def workload_desc(name: str, dx: float | None, instances: int = 512) -> dict:
    if name in FAMILIES:
        from mfree_iwf_gb300 import scenarios as S
        return {"workload": f"ensemble of {instances} two-ring impacts, {S.FAMILY_RING_SETUPS[name]}(81) each "
                            "(the reference's set-up), per-instance E~U[8e6,1.2e7] Pa, seeded"}
    if name == "c4":
        return {"workload": f"ensemble of {instances} ring impacts, Gray-Monaghan SPH, per-instance dx~U[0.2,1] mm, "
                            "E~U[5e6,5e7] Pa, nu~U[0.3,0.45], speed~U[5,40] m/s, seeded"}
    if name == "c3":
        return {"workload": f"plate tension 0.1 x 0.02 m, weak-form TL + RKPM, dx={(dx or 2e-5)*1e3:g} mm, "
                            "+-1 m/s pull, 1% seeded jitter"}
    if name == "c2":
        return {"workload": f"ring impact, total-Lagrangian SPH + Randles-Libersky, contact, dx={(dx or 5e-5)*1e3:g} mm"}
    if name == "c1":
        return {"workload": f"ring impact, Gray-Monaghan SPH, dx={(dx or 1e-3)*1e3:g} mm"}
    raise SystemExit(f"unknown workload {name}")


def workload(name: str, dx: float | None, instances: int = 512):
    from mfree_iwf_gb300 import scenarios as S
    desc = workload_desc(name, dx, instances)
    if name in FAMILIES:
        return S.family_ensemble(name, instances), desc
    if name == "c4":
        return S.c4_ensemble(instances), desc
    if name == "c3":
        return S.c3_plate(dx=dx or 2e-5), desc
    if name == "c2":
        return S.c2_rings_tl(dx=dx or 5e-5), desc
    return S.c1_rings(dx=dx or 1e-3), desc


def job_throughput(dist, seconds: float, units: float, device: str = "cuda"):
    """Whole-job throughput of replicas: the units all ranks processed over the slowest
    rank's time.  Returns (max seconds over ranks, units per second)."""
    if dist is None:
        return seconds, units / seconds
    import torch
    t = torch.tensor([seconds], dtype=torch.float64, device=device)
    u = torch.tensor([units], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item()) / float(t.item())


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clock and throttle-reason samples during the timed region."""

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=10)

    def summary(self):
        sm, mx, reasons = [], None, set()
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx = float(f[2])
                except ValueError:
                    continue
                for name, v in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), f[5:9]):
                    if v.lower() == "active":
                        reasons.add(name)
        except OSError:
            pass
        finally:
            if self.path and os.path.exists(self.path):
                os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------- CPU baseline
def cpu_sample(workload_name: str, steps: int, warmup: int, procs: int):
    """The reference's CPU implementation of the step on a bounded sample of the
    workload (the same set-up at a coarser lattice), `procs` single-threaded copies at
    once (one per host core); returns particle-steps/s over all of them.

    The reference itself (its unmodified sources compiled by oracle/build_ref.sh) runs
    where it was built on this host; elsewhere the oracle port stands in for it.  On an
    x86 host where both ran, the reference ran at 0.92x the port's rate on the TL ring
    set-up and 0.73x on the Gray-Monaghan rings (same cases, one core each)."""
    import oracle
    from mfree_iwf_gb300 import scenarios as S
    if workload_name in FAMILIES:
        sc = S.family_ensemble(workload_name, 1)
        desc = f"one instance of the ensemble ({S.FAMILY_RING_SETUPS[workload_name]}(81))"
    elif workload_name == "c2":
        # at dx = 1 mm the workload's neighbour epsilon equals the reference's fixed 1e-6 m^2
        sc = S.c2_rings_tl(dx=1e-3)
        desc = "same ring-impact TL set-up at dx=1 mm"
    elif workload_name == "c3":
        sc = S.c3_plate(dx=5e-4)
        desc = "same weak-form plate set-up at dx=0.5 mm"
    else:
        sc = S.c1_rings(dx=1e-3)
        desc = "the ring workload at dx=1 mm"
    kind, binary = "port", oracle.build_oracle()
    if sc.nbh_eps == 1e-6 and os.access(oracle.REF, os.X_OK):
        kind, binary = "reference", oracle.REF
    n = sc.n_total
    with tempfile.TemporaryDirectory() as d:
        case = os.path.join(d, "c.case")
        S.write_case(case, sc, warmup + steps)
        t0 = time.time()
        if kind == "reference":  # the harness times every step; the warm-up steps are timed too
            cmds = [[binary, "run", case, os.path.join(d, f"o{k}.out")] for k in range(procs)]
        else:
            cmds = [[binary, case, os.path.join(d, f"o{k}.out"), str(warmup)] for k in range(procs)]
        ps = [subprocess.Popen(c, stdout=subprocess.DEVNULL, stderr=subprocess.PIPE) for c in cmds]
        rcs = [p.wait() for p in ps]
        wall = time.time() - t0
        secs = []
        for k in range(procs):
            r = S.read_result(os.path.join(d, f"o{k}.out"))
            secs.append(r.seconds)
    if any(rcs):
        raise RuntimeError(f"{kind} CPU run failed")
    timed = steps + (warmup if kind == "reference" else 0)
    span = max(secs)
    value = procs * n * timed / span
    what = ("the reference's own sources, compiled here" if kind == "reference" else
            "the oracle port of the reference (the reference's sources are not on this host)")
    return value, {"cores": procs, "kind": kind,
                   "sample": f"{what}; {desc}: {n} particles, {timed} timed steps, "
                             f"{procs} concurrent single-threaded runs ({wall:.1f} s wall)",
                   "n": n}


def reference_arm(args, cfg_desc):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    procs = os.cpu_count() or 1
    value, info = cpu_sample(args.workload, args.steps, args.warmup, procs)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * info["n"] * procs / value,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": cfg_desc,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": info["cores"], "kind": info["kind"],
                         "sample": info["sample"]},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ ours
# DRAM bytes (read + write) per row of one launch of the dominant kernel, from one ncu
# capture of that kernel alone (dram__bytes_read.sum + dram__bytes_write.sum) on a
# smaller case of the same workload; the bench scales it by its own rows per launch.
# (bytes per row, description of the capture)
MEASURED_TRAFFIC = {
    # k_tlB32r, stages 0-3 of one step at dx = 0.1 mm: (140.7 + 3 x 161.9) MB / 4 / 439,860 rows
    ("c2", "mixed", "TL pass B"): (356.0, "ncu, the run-walk pass B alone, the four stages of one step of the ring "
                                          "impact at dx = 0.1 mm (439,860 rows), mean per row, scaled by rows"),
    ("c3", "mixed", "weak TL Gauss-point pass"): (367.8, "ncu, the Gauss-point pass alone at dx = 0.1 mm "
                                                         "(800k Gauss points), scaled by Gauss points"),
}

# Idealised algorithmic bytes per particle-step (every per-particle value read or
# written once per stage, neighbour data served on chip, per-pair weights recomputed on
# chip): (method, mixed) -> bytes per particle-step.  The bench line reports the
# dominant kernel against it as "frac_survey_model".
IDEAL_BYTES = {("ul", False): 1344.0, ("ul", True): 992.0, ("tl", False): 896.0, ("tl", True): 768.0}


def rel_l2(pairs, floor=0.0):
    """Relative L2 of the first arrays against the second, the norm of the second
    floored at `floor`."""
    num = sum(float(np.sum((a - b) ** 2)) for a, b in pairs)
    den = max(sum(float(np.sum(b ** 2)) for _, b in pairs), floor ** 2)
    return (num / den) ** 0.5 if den > 0 else num ** 0.5


def field_errors(sc, got, want):
    """Relative L2 error of run `got` against run `want` (each: final states, stresses)
    per output field over all bodies: displacement (x - X0), velocity, density change
    (rho - rho_initial, where the method evolves it) and the stress the method
    evaluates (UL: the state's S; strong-form TL: the nominal stress P).  Density and
    stress norms are floored at those of a uniform 1e-6 strain (1e-6 rho0, 1e-6 E)."""
    import mfree_iwf_gb300 as M
    initial = [b.arrays for b in sc.bodies]
    n = sc.n_total
    (sg, pg), (sw, pw) = got, want
    res = {"x": rel_l2([(a[f] - b0[f], b[f] - b0[f]) for b0, a, b in zip(initial, sg, sw) for f in ("x", "y")]),
           "v": rel_l2([(a[f], b[f]) for a, b in zip(sg, sw) for f in ("vx", "vy")])}
    if sc.method == M.METHOD_UL:
        res["rho"] = rel_l2([(a["rho"] - b0["rho"], b["rho"] - b0["rho"]) for b0, a, b in zip(initial, sg, sw)],
                            1e-6 * sc.rho0 * n ** 0.5)
    else:
        res["rho"] = None  # not evolved by the method (constant, as in the reference)
    res["S"] = None if pg is None else rel_l2([(a[f], b[f]) for a, b in zip(pg, pw) for f in ("Pxx", "Pxy", "Pyx", "Pyy")],
                                              1e-6 * sc.E * (4 * n) ** 0.5)
    return res


def run_states(M, sc, precision, steps, device, graph, time_from=None):
    """Run `steps` steps of a fresh context; returns (final states, stresses) and, when
    `time_from` is given, particle-steps/s over the steps after that many (after
    autotuning; CUDA events on the library's stream, graph replay)."""
    import torch
    sim = M.from_scenario(sc, precision=precision, device=device, graph=graph)
    rate = None
    if time_from is None:
        sim.step(steps)
    else:
        sim.step(1)
        sim.autotune(1)
        sim.step(time_from - 1)
        sim.synchronize()
        st = torch.cuda.ExternalStream(sim.stream())
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        sim.step(steps - time_from)
        b.record(st)
        sim.synchronize()
        torch.cuda.synchronize()
        rate = sc.n_total * (steps - time_from) / (a.elapsed_time(b) / 1e3)
    out = [sim.get_state(k) for k in range(len(sc.bodies))]
    stress = None  # the UL and strong-form TL methods evaluate a per-particle stress
    if sc.method in (M.METHOD_UL, M.METHOD_TL):
        stress = [sim.get_stress(k) for k in range(len(sc.bodies))]
    sim.close()
    return (out, stress), rate


def timed_rate(M, sc, precision, steps, device, graph, tune=True):
    """particle-steps/s of `steps` timed steps (after set-up, autotuning and 3 warm-up
    steps) and the per-kernel CUDA-event statistics of two more eager steps."""
    import torch
    sim = M.from_scenario(sc, precision=precision, device=device, graph=graph)
    sim.step(1)
    if tune:
        sim.autotune(1)
    sim.step(3)
    sim.synchronize()
    st = torch.cuda.ExternalStream(sim.stream())
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(st)
    sim.step(steps)
    b.record(st)
    sim.synchronize()
    torch.cuda.synchronize()
    secs = a.elapsed_time(b) / 1e3
    sim.set_timing(True)
    sim.step(2)
    sim.synchronize()
    ks = {k: sim.kernel_stats(k) for k in range(6)}
    sim.close()
    return sc.n_total * steps / secs, secs / steps, ks


def weak_bytes(kind: int, n_p: int, n_g: int, e_g: int, e_t: int) -> float:
    """Unique bytes per row of the mixed weak TL passes (kind 5: per Gauss point, kind 2:
    per particle), stage-averaged over the four RK4 stages; the gathered records counted
    once (their unique bytes), as in algorithmic_bytes."""
    if kind == 5:  # Gauss-point pass
        return (2 + 12 * e_g / n_g      # count; per entry: index 4 + FP32 gradient pair 8
                + 16 + 4                # the point's own displacement (FP64 pair), body
                + 44 + 32               # RK4 of rho, S (FP32): reads stage, base, acc (stages 1-3); writes
                + 16                    # nominal stress for the particles
                + 32 * n_p / n_g)       # the particles' float-float displacement/velocity records
    return (2 + 12 * e_t / n_p          # count; per transposed entry: index 4 + gradient pair 8
            + 16 * n_g / n_p            # the Gauss points' nominal stress
            + 8 + 4 + 16                # m, body, contact force
            + 16 + 32 + 24 + 24 + 40)   # RK4 FP64 x y vx vy: stage v, base, acc (1-3), acc (0-2), stage/base


def algorithmic_bytes(kind: int, mixed: bool, nnz_per_row: float, tl: bool, family: str = "",
                      runs_per_row: float = 0.0) -> float:
    """Unique bytes per row of one launch: each row's own data once, the lists once, and
    neighbour records assumed served on chip (their unique bytes are the rows' own).
    runs_per_row > 0: the mixed TL run-walk passes (run words instead of per-pair
    entries; per row the reference position and the correction, 32 B, and h)."""
    if tl and mixed and runs_per_row > 0 and family not in ("corot", "potential"):
        if kind == 1:  # pass A
            return (2 + 4 * runs_per_row + 32 + 4  # run count and words; XF, G; h
                    + 16 + 16 + 16 + 4            # own displacement and velocity records, rho - rho0, S, body id
                    + 16 + 16)                    # writes: nominal stress P, rate terms
        if kind == 2:  # pass B
            return (2 + 4 * runs_per_row + 32     # run count and words; XF, G
                    + 64 + 16 + 16 + 24           # own record fields, rate terms, stage vx vy, fc and m
                    + 32 + 24 + 32 + 32 + 8       # RK4 FP64 x y vx vy
                    + 16 + 12 + 16 + 16 + 4       # RK4 FP32 rho S
                    + 24 + 64)                    # next-stage records
    if family in ("corot", "potential") and mixed:
        if kind == 1:  # pass A: index + qw-weighted gradient (+ X_j - X_i, corotational) per pair
            per_pair = 20 if family == "corot" else 12
            return 2 + per_pair * nnz_per_row + 16 + 16 + 12 + 8 + 4 + 16  # u, rotation, S, qw, body; writes P
        if kind == 2:  # pass B: index + gradient per pair (+ reverse gradient, potential)
            per_pair = 12 if family == "corot" else 20
            return (2 + per_pair * nnz_per_row + 80 + 24  # own records P R X V H, fc and m
                    + 112 + 32)                           # RK4 FP64 x y vx vy, rho/S carried to the next set
    if tl and mixed:
        if kind == 1:  # pass A
            return (2 + 12 * nnz_per_row  # count; per pair: index 4 + premultiplied gradient 8
                    + 16 + 16             # own displacement and velocity records
                    + 16 + 4              # rho - rho0, S (FP32), body id
                    + 16 + 16)            # writes: nominal stress P, rate terms
        if kind == 2:  # pass B (also writes the next stage's records)
            return (2 + 12 * nnz_per_row  # count; per pair: index 4 + mass-premultiplied gradient 8
                    + 64 + 16 + 16 + 24   # own record, rate terms, stage vx vy, fc and m
                    + 32 + 24 + 32 + 32 + 8   # RK4 FP64 x y vx vy: base, acc (stages 1-3), acc, next, base (stage 3)
                    + 16 + 12 + 16 + 16 + 4   # RK4 FP32 rho S: same pattern
                    + 24 + 64)            # next-stage records: reads X Y h m, writes displacement, x v hmrc
    if tl:
        if kind == 1:
            return 4 + 20 * nnz_per_row + 32 + 32 + 32 + 32 + 8
        return 4 + 20 * nnz_per_row + 32 + 32 + 8 + 8 + 8 + 8 + 32 + 32 + 16 + 128 + 64
    if kind == 0:  # UL pair: own record, perm/key/body, contact force, 4 accesses of the state vector
        return (80 + 12 + 16 + 4 * 48) if mixed else (128 + 12 + 16 + 4 * 64)
    return 0.0


def ours(args, cfg_desc):
    import torch
    import mfree_iwf_gb300 as M

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    sc, cfg = workload(args.workload, args.dx, args.instances)
    n = sc.n_total
    if args.workload in FP64_ONLY and args.precision == "mixed":
        args.precision = "fp64"
    tl = sc.method in (M.METHOD_TL, M.METHOD_TL_WEAK, M.METHOD_COROT, M.METHOD_POTENTIAL)
    sim = M.from_scenario(sc, precision=args.precision, device=local, graph=not args.no_graph)
    mixed = args.precision == "mixed"
    if args.tl_tiles:
        sim.set_option("tl_tiles", 1)
    if args.tl_runs is not None and sc.method == M.METHOD_TL and mixed:
        sim.set_option("tl_runs", args.tl_runs)
    sim.step(1)  # set-up (neighbour search, corrections)
    tune = sim.autotune(args.tune_steps) if not args.no_tune else "off"
    sim.step(args.warmup)
    sim.synchronize()
    stream = torch.cuda.ExternalStream(sim.stream())
    nnz = float(np.mean(sim.neighbor_counts(0))) if tl else 0.0
    runs_per_row = 0.0
    if sc.method == M.METHOD_TL and mixed and sim.get_option("tl_runs") and sim.get_option("tl_runs_built"):
        runs_per_row = sim.get_option("tl_run_words") / n

    # ---- device-resident timed region (graph replay of whole steps)
    l0 = sim.launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        e0.record(stream)
        sim.step(args.steps)
        e1.record(stream)
        sim.synchronize()
        torch.cuda.synchronize()
    if dist:
        dist.barrier()
    launches = sim.launch_count() - l0
    clocks = clk.summary()
    secs, value = job_throughput(dist, e0.elapsed_time(e1) / 1e3, n * args.steps)
    ms = secs * 1e3

    # ---- per-kernel CUDA-event times (eager launches: a graph replay carries no
    # per-launch events), same workload, right after the timed region
    sim.set_timing(True)
    sim.step(max(2, min(args.steps, 10)))
    sim.synchronize()
    kstats = {k: sim.kernel_stats(k) for k in range(8)}
    weak_lists = None
    if sc.method == M.METHOD_TL_WEAK:  # list sizes for the weak passes' byte model
        weak_lists = (sim.get_option("weak_gauss_points"), sim.get_option("weak_gp_entries"),
                      sim.get_option("weak_particle_entries"))
    sim.set_timing(False)

    # ---- end to end through the C ABI with host buffers: per step the state of all
    # bodies goes host -> device (pinned), one step runs, the state comes back into the
    # same host arrays (stream-ordered transfers: each field's host -> device copy of a
    # step waits for its device -> host copy of the step before; the two directions
    # overlap field by field); the timed region ends when the last state is on the host
    fields = ("x", "y", "vx", "vy", "rho", "Sxx", "Sxy", "Syy")
    host = {f: torch.empty(n, dtype=torch.float64).pin_memory().numpy() for f in fields}
    sim.get_state_all_into(host)
    k2 = max(3, min(args.steps, args.e2e_steps))
    # steps queue without a host synchronization each; the device status (errors, failed
    # bodies) is read by the synchronize that ends the timed region
    sim.set_option("async_steps", 1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    weak = sc.method in (M.METHOD_TL_WEAK, M.METHOD_UL_WEAK)  # (their transfers are synchronous)
    for _ in range(k2):
        if weak:
            sim.set_state_all(host)
            sim.step(1)
            sim.get_state_all_into(host)
        else:
            sim.set_state_all_async(host)
            sim.step(1)
            sim.get_state_all_async_into(host)
    sim.synchronize()
    wall = time.perf_counter() - t0
    _, e2e_value = job_throughput(dist, wall, n * k2)
    bytes_io = 8 * len(fields) * n

    sim.close()
    del sim

    # ---- the plain FP64 form on the same workload, same run, and the per-field error
    # of the mixed form against it after `err_steps` steps from the same initial state
    forms = None
    mixed_error = None
    if mixed and not args.no_compare:
        err_steps = args.error_steps
        want, v64 = run_states(M, sc, "fp64", err_steps, local, not args.no_graph, time_from=min(10, err_steps // 2))
        got, _ = run_states(M, sc, "mixed", err_steps, local, not args.no_graph)
        mixed_error = dict(field_errors(sc, got, want), steps=err_steps,
                           fields="relative L2 over all particles, mixed against FP64 from the same initial "
                                  "state: x = displacement, v = velocity, rho = density change (null: not evolved "
                                  "by the method), S = the stress the method evaluates (TL: nominal stress P); "
                                  "rho and S norms floored at a uniform 1e-6 strain")
        forms = {"mixed": value / world, "fp64": v64, "mixed_over_fp64": value / world / v64,
                 "fp64_steps": err_steps - min(10, err_steps // 2)}
        del want, got

    # ---- the batched ensemble (512 ring impacts, one launch per stage for all of
    # them): mixed against FP64 on the same ensemble, and the per-field error of the
    # mixed form after 1000 steps on its first 8 instances
    batched = None
    if args.workload == "c2" and not args.no_batched:
        from mfree_iwf_gb300 import scenarios as S
        sc4 = S.c4_ensemble(args.instances)
        vb, sb, ksb = timed_rate(M, sc4, "mixed", args.batched_steps, local, not args.no_graph)
        vb64, sb64, _ = timed_rate(M, sc4, "fp64", args.batched_steps, local, not args.no_graph)
        sub = S.c4_ensemble(8)
        pert = S.c4_ensemble(8)
        for b in pert.bodies:  # a 1-ulp change of the initial positions: the FP64 form's own spread
            b.arrays["x"] = np.nextafter(b.arrays["x"], np.inf)
        want, _ = run_states(M, sub, "fp64", args.error_steps, local, not args.no_graph)
        got, _ = run_states(M, sub, "mixed", args.error_steps, local, not args.no_graph)
        ulp, _ = run_states(M, pert, "fp64", args.error_steps, local, not args.no_graph)
        per_instance = []
        for k, b in enumerate(sub.bodies):
            per_instance.append({"particles": b.n, "dx_mm": b.params["dx"] * 1e3, "speed": b.params["speed"],
                                 "v": rel_l2([(got[0][k][f], want[0][k][f]) for f in ("vx", "vy")]),
                                 "fp64_1ulp_spread": rel_l2([(ulp[0][k][f], want[0][k][f]) for f in ("vx", "vy")])})
        well = [r for r in per_instance if r["fp64_1ulp_spread"] <= 1e-12]
        peaks, _ = measured_peaks()
        pms, pl, prow = ksb[0]
        pair = None
        if pl:
            t_launch = pms / pl / 1e3
            pair = {"avg_launch_ms": pms / pl,
                    "frac_survey_model": IDEAL_BYTES[("ul", True)] / 4 * (prow / pl) / t_launch / 1e9 / peaks["hbm_gbs"]}
        batched = {"workload": workload_desc("c4", None, args.instances)["workload"], "particles": sc4.n_total,
                   "instances": args.instances, "steps": args.batched_steps,
                   "mixed": vb, "fp64": vb64, "mixed_over_fp64": vb / vb64,
                   "ms_per_step": {"mixed": sb * 1e3, "fp64": sb64 * 1e3},
                   "step_frac_survey_model": IDEAL_BYTES[("ul", True)] * vb / 1e9 / peaks["hbm_gbs"],
                   "pair_kernel": pair,
                   "mixed_error": dict(field_errors(sub, got, want), steps=args.error_steps,
                                       instances=8, particles=sub.n_total, per_instance=per_instance,
                                       well_conditioned=len(well),
                                       v_max_well_conditioned=max((r["v"] for r in well), default=None),
                                       within_1e4=sum(r["v"] <= 1e-4 for r in per_instance),
                                       note="well conditioned: the FP64 velocities move by <= 1e-12 under a "
                                            "1-ulp change of the initial positions")}
        del want, got

    # ---- roofline of the dominant kernel
    peaks, peak_kind = measured_peaks()
    dom = max((k for k in kstats if k != 4), key=lambda k: kstats[k][0])  # kind 4 is a whole UL stage
    kms, klaunch, krows = kstats[dom]
    names = {0: "UL pair (+RK)", 1: "TL pass A", 2: "TL pass B", 3: "contact", 4: "UL stage (grid + gather + pair)",
             5: "weak"}
    if sc.method == M.METHOD_UL_WEAK:
        names.update({2: "weak UL particle pass", 5: "weak UL stress-point pass",
                      6: "weak UL neighbourhoods (ellipse + RKPM)"})
    elif sc.method == M.METHOD_TL_WEAK:
        names.update({2: "weak TL particle pass", 5: "weak TL Gauss-point pass"})
    elif sc.method in (M.METHOD_COROT, M.METHOD_POTENTIAL):
        names.update({1: "pass A", 2: "pass B"})
    roof = None
    # (no byte model for the weak UL passes, nor for the FP64 weak TL ones)
    weak_model = sc.method == M.METHOD_TL_WEAK and mixed and weak_lists is not None and dom in (2, 5)
    if klaunch and sc.method != M.METHOD_UL_WEAK and (sc.method != M.METHOD_TL_WEAK or weak_model):
        per_launch_rows = krows / klaunch
        if weak_model:
            abytes = weak_bytes(dom, n, weak_lists[0], weak_lists[1], weak_lists[2]) * per_launch_rows
        else:
            abytes = algorithmic_bytes(dom, mixed, nnz, tl, args.workload, runs_per_row) * per_launch_rows
        achieved = abytes / (kms / klaunch / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": names[dom], "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "traffic": None, "peak_source": peak_kind,
                "launches": klaunch, "avg_launch_ms": kms / klaunch,
                "algorithmic_bytes_per_launch": abytes,
                "byte_model": ("itemised: every byte the kernel must move (" +
                               ("run words per row, gradients recomputed on chip" if runs_per_row else
                                "lists and per-pair weights streamed") + ")")}
        fam = "tl" if sc.method == M.METHOD_TL else "ul" if sc.method == M.METHOD_UL else None
        if fam is not None:
            per_ps = IDEAL_BYTES[(fam, mixed)]
            # the survey's bytes of one stage (a quarter of a particle-step) per launch,
            # and of the whole step
            roof["survey_bytes_per_particle_step"] = per_ps
            roof["frac_survey_model"] = per_ps / 4 * per_launch_rows / (kms / klaunch / 1e3) / 1e9 / peaks["hbm_gbs"]
            roof["step_frac_survey_model"] = per_ps * value / world / 1e9 / peaks["hbm_gbs"]
        t = MEASURED_TRAFFIC.get((args.workload, args.precision, names[dom]))
        if t is not None and names[dom] == "TL pass B" and not runs_per_row:
            t = None  # (the capture is of the run-walk pass)
        if t is not None:
            roof["traffic"] = t[0] * per_launch_rows
            roof["traffic_source"] = t[1]
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            cv, info = cpu_sample(args.workload, args.cpu_steps, 1, 1)
            cpu = {"value": cv, "unit": UNIT, "cores": 1, "kind": info["kind"], "sample": info["sample"]}
        except Exception as e:  # noqa: BLE001
            cpu = {"value": None, "unit": UNIT, "cores": 1, "kind": "port", "sample": f"failed: {e}"}
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": {"mixed": "f32+f64", "fp64": "f64", "fp64_strict": "f64"}[args.precision],
            "data": "synthetic",
            "config": dict(cfg, particles=n, precision=args.precision, parallelism=f"replicas x{world}",
                           l2="inputs larger than L2 (state + neighbour lists of %d particles)" % n),
            "clocks": clocks, "gpu_launches": launches,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": bytes_io, "d2h_bytes_per_step": bytes_io,
                    "steps": k2, "status": "device status read once, by the synchronize ending the timed region"},
            "roofline": roof, "cpu_baseline": cpu,
            "kernels_ms": {names[k]: v[0] for k, v in kstats.items() if v[1]},
            "forms": forms, "mixed_error": mixed_error, "batched": batched, "autotune": tune,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c2", "c1", "c3", "c4", *FAMILIES])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64", "fp64_strict"])
    ap.add_argument("--dx", type=float, default=None)
    ap.add_argument("--cpu-steps", type=int, default=600)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=20)
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--tune-steps", type=int, default=3)
    ap.add_argument("--no-compare", action="store_true")
    ap.add_argument("--tl-tiles", action="store_true", help="mixed TL: the shared-memory halo-tile passes")
    ap.add_argument("--tl-runs", type=int, choices=[0, 1], default=None,
                    help="mixed TL: 1 = run-walk passes (gradients recomputed on chip), 0 = streamed lists")
    ap.add_argument("--instances", type=int, default=512, help="c4: ring impacts in the ensemble")
    ap.add_argument("--error-steps", type=int, default=1000, help="steps of the mixed-against-FP64 error runs")
    ap.add_argument("--batched-steps", type=int, default=20, help="timed steps of the batched ensemble block")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched ensemble block (c2 only)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    cfg_desc = workload_desc(args.workload, args.dx, args.instances)
    if args.impl == "reference":
        reference_arm(args, cfg_desc)
        return
    from __graft_entry__ import build
    build()
    ours(args, cfg_desc)


if __name__ == "__main__":
    main()
