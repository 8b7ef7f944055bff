"""Benchmark of the GB300 per-cell hot path (one JSON line on rank 0).

Workload (default, ``detonation_air_200k``): the 200,000-cell CH4/air
detonation tube on which the surrogate-vs-plain metric is quoted -- a 1 m
tube of 5 um cells, stoichiometric CH4/air at 1 atm, 300 K, a 1 cm driver at
3000 K / 30 atm holding the fresh mixture's TP-equilibrium products,
reflecting left wall, fixed-pressure outlet, WENO5-Z + HLLC + SSP-RK3, CFL
0.4, detailed GRI-Mech 3.0 chemistry (52 species and 323 reactions of the
C/H/O/N elements present) integrated per cell. ``detonation_o2_20k`` is the
20,000-cell, 50 um CH4/O2 tube; ``reactors`` the batch of 2^20 partially
reacted constant-volume reactors.

A step is one pass of the time loop body (calc_dt, three fluid stages,
chemistry, post-step) over the whole tube: "cell-steps" = cells x steps.
Exactly --warmup untimed steps, then exactly --steps timed steps.

value: device time of the timed steps through edyn_advance (CUDA graphs of
16 steps, state resident in HBM; the 200k tube's state, 358 MB, is larger
than L2; the 20k tube's is not, so L2 is flushed between graph launches).
e2e: the same steps through the C ABI with host buffers -- every step
uploads qf/Qc from pinned host memory, steps, and downloads qf/Qc/HRR.
--impl reference: the CPU restatement of the reference's algorithm (the
oracle; the Fortran code does not build here) on all host cores, timing the
same steps of the same tube.
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
METRIC = "cell-steps/s on 1 GB300: surrogate vs plain chemistry at ≤1e-3 species err"
UNIT = "cell-steps/s"
BYTES_CHEM_PER_CELL = 912   # chemistry launch: read qf (456 B) + write qf and Qc rows (456 B)
# one SSP-RK3 stage moves five rows of nequ doubles per cell: stage 1 reads
# qf, Qc and writes qf', Qc, Q0; stages 2-3 read qf, Qc, Q0 and write qf', Qc
STAGE_ROWSETS = 5
L2_BYTES = 129 << 20
# From ncu captures of the 200,000-cell tube at the timed steps
# (profiles/*_ch4_air_detonation_200000.md): DRAM bytes (read + write) of
# the chemistry launch's kernels per cell and step, and FP64 operations per
# step summed over one step's kernels (2 DFMA + DADD + DMUL thread
# instructions: stages 2.17e8, integrator pass 3.2e7, screen 1.3e6).
TRAFFIC_CHEM_PER_CELL = {"detonation_air_200k": 211.6e6 / 200000, "detonation_o2_20k": 1.93e6 / 4000,
                         "detonation_air_20k": None}
# DRAM read + write of one stage launch per cell (ncu, the 200k tube: 179.8 +
# 210.6 MB)
TRAFFIC_STAGE_PER_CELL = {"detonation_air_200k": (179.8e6 + 210.6e6) / 200000}
FP64_FLOPS_PER_STEP = {"detonation_air_200k": 2.50e8}

WORKLOADS = {
    "detonation_air_200k": dict(ncell=200000, length=1.0, oxidizer="air"),
    "detonation_o2_20k": dict(ncell=20000, length=1.0, oxidizer="O2"),
    # the first 10 cm of the 200k tube (the same 5 um cells): the small case
    # that ncu captures
    "detonation_air_20k": dict(ncell=20000, length=0.1, oxidizer="air"),
}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="detonation_air_200k",
                   choices=list(WORKLOADS) + ["reactors", "tubes", "flame", "spherical_flame"],
                   help="the tube of the headline metric (default), the 20k CH4/O2 tube, the reactor batch, "
                        "the uneven batch of --ntubes tubes in one context, the planar flame with transport, or "
                        "the spherical flame kernel (transport, chemistry, ignition energy)")
    p.add_argument("--flame-cells", type=int, default=None,
                   help="cells of --workload flame / spherical_flame (20 um each; 1000 / 2000 by default)")
    p.add_argument("--ntubes", type=int, default=256, help="tubes of --workload tubes")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-surrogate", action="store_true", help="skip the surrogate-vs-plain comparison")
    p.add_argument("--reactors", type=int, default=1 << 20, help="reactors in the batch of --workload reactors")
    p.add_argument("--prepared", type=int, default=1 << 16,
                   help="partially reacted states prepared for --workload reactors (each reused reactors/prepared "
                        "times with its own dt)")
    return p.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def max_over_ranks(t_local: float, world: int, device=None) -> float:
    """Max of a per-rank time over all ranks (the whole job ends with the
    slowest rank); the identity at world size 1."""
    if world == 1:
        return t_local
    import torch
    import torch.distributed as dist

    tt = torch.tensor([t_local], dtype=torch.float64, device=device)
    dist.all_reduce(tt, op=dist.ReduceOp.MAX)
    return float(tt.item())


def job_value(cells_per_rank: int, steps: int, world: int, t_max: float) -> float:
    """Whole-job cell-steps/s: every rank advances its own replica of the
    tube, so the units of all ranks count over the slowest rank's time."""
    return cells_per_rank * steps * world / t_max


def peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([c.strip() for c in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.3)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[j] for r in self.rows for j in range(4) if len(r) > 5 + j and r[5 + j] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def build_case(workload):
    from fortrancfd_gb300 import configs

    w = WORKLOADS[workload]
    return configs.detonation(ncell=w["ncell"], length=w["length"], oxidizer=w["oxidizer"])


def workload_config(case, args, world):
    """The `config` of both arms' JSON lines: what is simulated, not how."""
    return {"workload": case.name, "cells": case.ncell, "dx_m": case.dx,
            "mixture": "stoichiometric CH4/" + ("air" if "air" in case.name else "O2") + ", 1 atm, 300 K",
            "driver": "1 cm, 3000 K, 30 atm, TP-equilibrium products",
            "scheme": "WENO5-Z + HLLC + SSP-RK3, CFL 0.4, wall / fixed-p outlet",
            "chemistry": "GRI-Mech 3.0, per-cell stiff integration, rtol 1e-5, atol 1e-13",
            "timed_steps": f"steps {args.warmup + 1}..{args.warmup + args.steps} from the initial state",
            "parallelism": f"replicas x{world}"}


def oracle_tube(case):
    sys.path.insert(0, str(ROOT / "tests"))
    from oracle_ctypes import Oracle

    o = Oracle()
    qf0, qc0 = o.init_cells(case.T, case.p, case.u, case.X)
    t = o.tube(case.ncell, 3, [1, 2, 2, 2, 3, 0, 1, 1], [case.dx, 101325.0, 300.0, 0.0, 1e-5, 1e-13])
    t.set_interior(qf0, qc0)
    return o, t


def reference_arm(args, rank, world):
    """The reference's algorithm on the host cores: the oracle (a C
    restatement of the reference's CPU code; the Fortran code does not build
    here) on all cores, the same tube, the same steps as the GPU arm."""
    if rank != 0:
        return None
    if args.workload in ("reactors", "tubes"):
        print(json.dumps({"impl": "reference", "unavailable": f"the {args.workload} workload has no reference-arm "
                          "timing (the default workload carries the comparison)"}), flush=True)
        return None
    case = build_case(args.workload)
    o, t = oracle_tube(case)
    for _ in range(args.warmup):
        t.step(case.cfl)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t.step(case.cfl)
    el = time.perf_counter() - t0
    v = case.ncell * args.steps / el
    cores = o.L.or_num_threads()
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(case, args, world),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"steps {args.warmup + 1}..{args.warmup + args.steps} of the "
                                       f"{case.ncell}-cell tube, plain FP64 chemistry"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return line


def cpu_baseline(case, budget_s=15.0):
    """The oracle on the host cores over a bounded sample of the workload:
    the first steps of the same tube (one untimed)."""
    o, t = oracle_tube(case)
    t.step(case.cfl)
    n = 0
    t0 = time.perf_counter()
    while True:
        t.step(case.cfl)
        n += 1
        el = time.perf_counter() - t0
        if el > budget_s or n >= 64:
            break
    return {"value": case.ncell * n / el, "unit": UNIT, "cores": o.L.or_num_threads(), "kind": "port",
            "sample": f"steps 2..{n + 1} of the {case.ncell}-cell tube, {el:.1f} s"}


def fp64_peak(dev):
    """Measured FP64 peak of this GPU: cuBLAS DGEMM 4096^3, best of 5."""
    import torch

    a = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    b = torch.randn(4096, 4096, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    best = 1e30
    for _ in range(5):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1) / 1e3)
    return 2.0 * 4096 ** 3 / best / 1e12


def run_tube(tube, case, steps, warmup, stream, flush):
    """Exactly `warmup` untimed steps, then `steps` timed steps through
    edyn_advance. Returns (device seconds, graph launches). When the state
    fits in L2, it is flushed between 16-step graph launches, outside the
    timed events."""
    import torch

    t_sim, n = tube.advance(case.cfl, tend=1e9, time=0.0, max_steps=warmup) if warmup else (0.0, 0)
    assert n == warmup, (n, warmup)
    chunk = steps if flush is None else 16
    dev_ms, done, graphs = 0.0, 0, 0
    while done < steps:
        k = min(chunk, steps - done)
        if flush is not None:
            flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        t_sim, n = tube.advance(case.cfl, tend=1e9, time=t_sim, max_steps=k)
        e1.record(stream)
        e1.synchronize()
        assert n == k, (n, k)
        dev_ms += e0.elapsed_time(e1)
        done += k
        graphs += (k + 15) // 16
    return dev_ms / 1e3, graphs, t_sim


def species_err(a, b, floor=1e-6):
    """Largest relative difference of the mass fractions >= floor."""
    big = np.abs(b) >= floor
    return float(np.where(big, np.abs(a - b) / np.maximum(np.abs(b), floor), 0.0).max())


def surrogate_compare(case, args, stream, dev, plain_end, plain_value):
    """The learned surrogate in the tube's source step (chem_mode 1) against
    the plain chemistry on the same tube and the same steps. The network is
    trained first, on the GPU by the library's kernels, on pairs the plain
    integrator produces (rtol 1e-8) for exactly the cells a chem_mode 1 tube
    hands to it, harvested from 5 um CH4/air tubes over a seeded sweep of
    phi ~ U[0.7, 1.4] and driver T ~ U[2500, 3500] K. Then the same warm-up
    and timed steps run through edyn_advance with the network, and without
    it (the gated explicit increment, then the integrator); the species and
    peak-T errors are against the plain run's state after the same steps."""
    import torch

    from fortrancfd_gb300 import Reactors, Tube
    from fortrancfd_gb300 import surrogate as S

    t0 = time.perf_counter()
    rho, dt, y0, y1 = S.harvest_screened(S.tube_sweep(6, seed=0), nsteps=100)
    s = S.Surrogate(Reactors(rtol=1e-5, atol=1e-13), S.MLP(seed=0))
    hist = S.train(s, rho, dt, y0, y1, iters=3000, batch=4096, lr=2e-3, log_every=2999)
    t_train = time.perf_counter() - t0
    out = {"target": ">= 5x the plain integrator's cell-steps/s (not met)",
           "training": f"{len(rho)} pairs from 6 tubes x 100 steps, 3000 Adam steps of 4096 on the GPU, "
                       f"{t_train:.1f} s incl. harvest, final loss {hist[-1][1]:.3f}"}
    fl = case.flags
    for label, net in (("with_network", s), ("without_network", None)):
        tube = Tube(case.ncell, case.dx, flag_acu=2, flag_weno=fl["flag_weno"], flag_rbound=1, do_reaction=1,
                    strict_newton=0, rtol=1e-5, atol=1e-13, chem_mode=1)
        tube.set_stream(stream.cuda_stream)
        tube.set_surrogate(net)
        tube.init_cells(case.T, case.p, case.u, case.X)
        t_sim, n = tube.advance(case.cfl, tend=1e9, time=0.0, max_steps=args.warmup) if args.warmup else (0.0, 0)
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        t_sim, n = tube.advance(case.cfl, tend=1e9, time=t_sim, max_steps=args.steps)
        e1.record(stream)
        e1.synchronize()
        v = case.ncell * n / (e0.elapsed_time(e1) / 1e3)
        qf = tube.download()[0]
        out[label] = {"value": v, "speedup_vs_plain": v / plain_value, "last_step": tube.surrogate_stats(),
                      "species_err_vs_plain": species_err(qf[:, 3:], plain_end[:, 3:]),
                      "peak_T_err_vs_plain": float(abs(qf[:, 2].max() - plain_end[:, 2].max()) / plain_end[:, 2].max())}
        tube.close()
    out["value"] = out["with_network"]["value"]
    out["speedup"] = out["with_network"]["speedup_vs_plain"]
    return out


def gpu_arm(args, rank, world, local):
    import torch

    from fortrancfd_gb300 import Tube

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    case = build_case(args.workload)
    fl = case.flags
    # one non-default stream for the tube's kernels, the L2 flush and the
    # timing events (a NULL stream handle would leave the tube on its own
    # stream, unordered with torch's legacy default stream)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    tube = Tube(case.ncell, case.dx, flag_acu=2, flag_weno=fl["flag_weno"], flag_rbound=1, do_reaction=1,
                strict_newton=0, rtol=1e-5, atol=1e-13)
    tube.set_stream(stream.cuda_stream)
    tube.init_cells(case.T, case.p, case.u, case.X)
    state_bytes = 4 * case.ncell * tube.nequ * 8
    flush = None if state_bytes > L2_BYTES else torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        t_dev, graphs, t_sim = run_tube(tube, case, args.steps, args.warmup, stream, flush)
    torch.cuda.synchronize(dev)
    plain_end = tube.download()[0]
    t_max = max_over_ranks(t_dev, world, dev)
    value = job_value(case.ncell, args.steps, world, t_max)
    # per-launch kernel durations for the roofline: chemistry and one fluid step
    dt = tube.calc_dt(case.cfl)
    chem_ms, fluid_ms, rhs = [], [], []
    for _ in range(3):
        for which in ("fluid", "chem"):
            if flush is not None:
                flush.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            tube.solve_fluid(dt) if which == "fluid" else tube.solve_source(dt)
            b.record(stream)
            b.synchronize()
            (fluid_ms if which == "fluid" else chem_ms).append(a.elapsed_time(b))
        rhs.append(tube.chem_stats()["rhs"])
    chem_stats = tube.chem_stats()
    chem_s = statistics.median(chem_ms) / 1e3
    fluid_s = statistics.median(fluid_ms) / 1e3
    # end to end through the C ABI with pinned host buffers
    ne = tube.nequ
    qf_h = torch.empty((case.ncell, ne), dtype=torch.float64, pin_memory=True).numpy()
    qc_h = torch.empty((case.ncell, ne), dtype=torch.float64, pin_memory=True).numpy()
    hrr_h = torch.empty(case.ncell, dtype=torch.float64, pin_memory=True).numpy()
    from fortrancfd_gb300.edyn import _ptr, lib

    L = lib()
    L.edyn_download(tube._h, _ptr(qf_h), _ptr(qc_h), _ptr(hrr_h))
    e2e_steps = max(3, min(args.steps, 10))
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        tube.upload(qf_h, qc_h)
        tube.step(case.cfl)
        tube._check(L.edyn_download(tube._h, _ptr(qf_h), _ptr(qc_h), _ptr(hrr_h)))
    torch.cuda.synchronize(dev)
    e2e_el = time.perf_counter() - t0
    if rank != 0:
        return
    hbm, src = peaks()
    # the dominant kernel by time: the fluid stage (three launches a step)
    stage_s = fluid_s / 3.0
    stage_bytes = STAGE_ROWSETS * tube.nequ * 8 * case.ncell
    achieved = stage_bytes / stage_s / 1e9
    ts = TRAFFIC_STAGE_PER_CELL.get(args.workload)
    chem_ach = BYTES_CHEM_PER_CELL * case.ncell / chem_s / 1e9
    roof = {"bound": "hbm", "kernel": "k_stage (one of the three fluid stages of a step)", "achieved": achieved,
            "peak": hbm, "peak_source": src, "unit": "GB/s", "frac": achieved / hbm,
            "traffic": ts * case.ncell if ts else None, "algorithmic_bytes": stage_bytes,
            "launch_ms": stage_s * 1e3, "fluid_step_ms": fluid_s * 1e3,
            "note": "a stage moves five rows of nequ doubles per cell; in uniform regions it computes no faces, "
                    "and what remains is per-tile latency (window load, one QcToqf per run of equal columns)",
            "chemistry_launch": {"achieved": chem_ach, "frac": chem_ach / hbm, "launch_ms": chem_s * 1e3,
                                 "traffic": (TRAFFIC_CHEM_PER_CELL[args.workload] * case.ncell
                                             if TRAFFIC_CHEM_PER_CELL[args.workload] else None),
                                 "note": "lasts as long as its stiffest cells' sequential integrations (one SM "
                                         "each): latency, not bandwidth"}}
    p64 = fp64_peak(dev)
    fps = FP64_FLOPS_PER_STEP.get(args.workload)
    fp64 = {"bound": "fp64", "scope": "whole step", "peak": p64, "unit": "TFLOP/s",
            "peak_source": "cuBLAS DGEMM 4096^3, best of 5, this run", "rhs_launches": rhs}
    if fps:
        ach = fps * args.steps / t_max / 1e12
        fp64.update(achieved=ach, flops_per_step=fps, frac=ach / p64,
                    source="FP64 instructions of one step's kernels, ncu capture of the timed steps (profiles/)")
    cpu = None if args.no_cpu_baseline or world > 1 else cpu_baseline(case)
    surr = None
    if not args.no_surrogate and world == 1 and "air" in case.name:
        try:
            surr = surrogate_compare(case, args, stream, dev, plain_end, value)
        except Exception as ex:  # reported, not hidden: the headline line still prints
            surr = {"error": f"{type(ex).__name__}: {ex}"}
    # kernels per step: the loop test, the fluid stages, the chemistry
    # (counter clear + one pass; or, from 10,000 cells, counter clear, runs,
    # screening pass, followers, integrator pass, integrated followers and
    # the two team-pick kernels)
    per_step = 1 + 3 + (8 if case.ncell >= 10000 else 2)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(case, args, world),
            "impl": {"chemistry": "plain SDIRK4 (FP64 residual, FP32 analytic Jacobian/LU)",
                     "l2": ("state larger than L2" if flush is None else "L2 flushed between 16-step graphs"),
                     "stage_tile": "%d cells, %d threads per CTA" % tube.stage_tile(),
                     "chemistry_set": "%d species, %d reactions" % tube.chem_set(),
                     "simulated_time_s": t_sim},
            "clocks": clk.summary(),
            "e2e": {"value": case.ncell * e2e_steps / e2e_el, "unit": UNIT,
                    "h2d_bytes_per_step": 2 * case.ncell * ne * 8,
                    "d2h_bytes_per_step": (2 * case.ncell * ne + case.ncell) * 8, "steps": e2e_steps},
            "gpu_launches": graphs * 16 * per_step,
            "roofline": roof, "fp64": fp64,
            "cpu_baseline": cpu,
            "chem_launch": {"rhs_per_cell": chem_stats["rhs"] / max(1, chem_stats["cells"]),
                            "rejects": chem_stats["rejects"], "team_cells": chem_stats["team_cells"],
                            "precheck_cells": chem_stats["cells32"],
                            "identical_cells": chem_stats["cells_same"],
                            "failed": chem_stats["failed"]},
            "surrogate": surr}
    print(json.dumps(line), flush=True)


def reactors_arm(args, local):
    """Batched stiff chemistry: n constant-volume CH4/air reactors with
    T ~ U[900, 2500] K, p log-uniform in [1, 50] atm, phi ~ U[0.5, 2.0],
    dt log-uniform in [1e-8, 1e-6] s (configs.reactor_batch, seed 0), each
    first advanced by a seeded fraction U[0, 1] of its own ignition delay
    (the first time T rises 400 K above its start, found by the plain
    integrator in 50 us windows up to 2 ms; a reactor that does not ignite
    by then counts 2 ms). Preparing the states takes far longer than the
    timed steps, so `prepared` of them are made and each is reused for
    n / prepared reactors, every reactor keeping its own dt. A step is one
    batch call of the plain integrator (rtol 1e-5, atol 1e-13) over every
    reactor's dt, on states resident on the device and restored before each
    step."""
    import torch

    from fortrancfd_gb300 import Reactors, configs

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    n_all = args.reactors
    n = min(args.prepared, n_all)
    rho, _, yiT, _ = configs.reactor_batch(n, seed=0)
    _, dt_all, _, _ = configs.reactor_batch(n_all, seed=2)
    R = Reactors(rtol=1e-5, atol=1e-13)
    R.set_stream(stream.cuda_stream)
    rho_d = torch.tensor(rho, device=dev)
    t_prep = time.perf_counter()
    window, t_max = 50e-6, 2e-3
    y = torch.tensor(yiT, device=dev)
    T0 = y[:, -1].clone()
    tau = torch.full((n,), t_max, dtype=torch.float64, device=dev)
    found = torch.zeros(n, dtype=torch.bool, device=dev)
    w_d = torch.full((n,), window, dtype=torch.float64, device=dev)
    t = 0.0
    while t < t_max - 1e-12:
        # only reactors not yet ignited need the next window
        idx = torch.nonzero(~found).flatten()
        if idx.numel() == 0:
            break
        ys = y.index_select(0, idx).contiguous()
        rs = rho_d.index_select(0, idx).contiguous()
        ws = w_d[: idx.numel()].contiguous()
        R.integrate_device(idx.numel(), rs.data_ptr(), ws.data_ptr(), ys.data_ptr())
        t += window
        hit = (ys[:, -1] - T0.index_select(0, idx)) > 400.0
        tau[idx[hit]] = t
        found[idx[hit]] = True
        y[idx] = ys
        print(f"ignition window {t * 1e6:.0f} us: {idx.numel()} reactors, {time.perf_counter() - t_prep:.1f} s",
              file=sys.stderr, flush=True)
    # fresh mixtures advanced by frac * tau, in windows of at most 50 us
    frac = torch.tensor(np.random.default_rng(1).uniform(0.0, 1.0, n), device=dev)
    left = frac * tau
    y = torch.tensor(yiT, device=dev)
    while True:
        idx = torch.nonzero(left > 0).flatten()
        if idx.numel() == 0:
            break
        h = torch.clamp(left.index_select(0, idx), max=window).contiguous()
        ys = y.index_select(0, idx).contiguous()
        rs = rho_d.index_select(0, idx).contiguous()
        R.integrate_device(idx.numel(), rs.data_ptr(), h.data_ptr(), ys.data_ptr())
        y[idx] = ys
        left[idx] -= h
        left[left < 1e-15] = 0.0
    t_prep = time.perf_counter() - t_prep
    Tpre = y[:, -1].cpu().numpy()
    reps = (n_all + n - 1) // n
    y0 = y.repeat(reps, 1)[:n_all].contiguous()
    rho_d = rho_d.repeat(reps)[:n_all].contiguous()
    dt_d = torch.tensor(dt_all, device=dev)
    n_prep, n = n, n_all
    y = torch.empty_like(y0)
    stats = None
    for _ in range(args.warmup):
        y.copy_(y0)
        R.integrate_device(n, rho_d.data_ptr(), dt_d.data_ptr(), y.data_ptr())
    torch.cuda.synchronize(dev)
    ms = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            y.copy_(y0)  # n x 54 doubles (453 MB at 2^20): inputs larger than L2
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            stats = R.integrate_device(n, rho_d.data_ptr(), dt_d.data_ptr(), y.data_ptr())
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
    t_step = statistics.median(ms) / 1e3
    line = {"metric": "reactor-steps/s on 1 GB300 (batched stiff chemistry)", "value": n / t_step,
            "unit": "reactor-steps/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t_step * 1e3, "higher_is_better": True, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"ch4_air_reactors_{n}", "reactors": n,
                       "states": f"{n_prep} fresh CH4/air mixtures advanced by U[0,1] of their own ignition "
                                 f"delay, each reused for {n // n_prep} reactors with their own dt",
                       "chemistry": "plain SDIRK4 (FP64 residual, FP32 analytic Jacobian/LU), rtol 1e-5, atol 1e-13",
                       "l2": "inputs (453 MB at 2^20) larger than L2, restored before each step"},
            "clocks": clk.summary(), "gpu_launches": args.steps,
            "chem": {"rhs_per_reactor": stats["rhs"] / n, "steps_per_reactor": stats["steps"] / n,
                     "rejects": stats["rejects"], "failed": stats["failed"]},
            "preparation": {"seconds": t_prep, "ignited_within_2ms": float(found.float().mean().item()),
                            "T_pre_K": [float(np.percentile(Tpre, q)) for q in (0, 50, 100)]}}
    print(json.dumps(line), flush=True)


def tubes_arm(args, rank, world, local):
    """The uneven batch: --ntubes CH4/air detonation tubes (cells ~
    U[2000, 50000], lengths ~ U[0.1, 1] m, phi ~ U[0.7, 1.4], p ~ U[0.5, 5]
    atm, driver T ~ U[2500, 3500] K; configs.uneven_tubes, seed 0) in one
    context: one stage launch over every tube's tiles and one chemistry
    launch over every tube's cells per stage and step, each tube with its
    own dt, the steps in CUDA graphs. Under torchrun the tubes are split
    into contiguous cell-balanced ranges, one per rank (no exchange)."""
    import torch

    from fortrancfd_gb300 import Tubes, configs
    from fortrancfd_gb300.shard import my_range

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    cases = configs.uneven_tubes(args.ntubes, seed=0)
    a, b = my_range([c.ncell for c in cases], rank, world)
    mine = cases[a:b]
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    g = Tubes([c.ncell for c in mine], [c.dx for c in mine], p_outs=[c.flags["p_out"] for c in mine],
              do_reaction=1, strict_newton=0, rtol=1e-5, atol=1e-13)
    g.set_stream(stream.cuda_stream)
    g.init_cells(np.concatenate([c.T for c in mine]), np.concatenate([c.p for c in mine]),
                 np.concatenate([c.u for c in mine]), np.concatenate([c.X for c in mine]))
    t_sim, n = g.advance(0.4, tend=1e9, time=0.0, max_steps=args.warmup) if args.warmup else (0.0, 0)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        t_sim, n = g.advance(0.4, tend=1e9, time=t_sim, max_steps=args.steps)
        e1.record(stream)
        e1.synchronize()
    assert n == args.steps
    t_max = max_over_ranks(e0.elapsed_time(e1) / 1e3, world, dev)
    cells_all = sum(c.ncell for c in cases)
    chem = g.chem_stats()
    times, dts = g.times()
    if rank != 0:
        return
    line = {"metric": "cell-steps/s on 1 GB300: uneven tube batch, plain chemistry", "value": cells_all * args.steps / t_max,
            "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t_max / args.steps, "higher_is_better": True,
            "scaling": "strong" if world > 1 else "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": f"ch4_air_uneven_tubes_{args.ntubes}", "tubes": args.ntubes, "cells": cells_all,
                       "cells_range": [min(c.ncell for c in cases), max(c.ncell for c in cases)],
                       "scheme": "WENO5-Z + HLLC + SSP-RK3, CFL 0.4, wall / fixed-p outlet, per-tube dt",
                       "chemistry": "GRI-Mech 3.0, per-cell stiff integration, rtol 1e-5, atol 1e-13",
                       "parallelism": f"tubes split over {world} rank(s)",
                       "l2": "state (4 x 56 rows x cells doubles) larger than L2"},
            "clocks": clk.summary(), "gpu_launches": ((args.steps + 15) // 16) * 16 * 6,
            "chem_launch": {"rhs_per_cell": chem["rhs"] / max(1, chem["cells"]), "team_cells": chem["team_cells"]},
            "tube_dt_range_s": [float(dts.min()), float(dts.max())]}
    print(json.dumps(line), flush=True)


FLAME_METRICS = {"flame": "cell-steps/s on 1 GB300: planar CH4/air flame with transport and chemistry",
                 "spherical_flame": "cell-steps/s on 1 GB300: spherical CH4/air flame kernel with transport, "
                                    "chemistry and ignition energy"}


def flame_case(args):
    from fortrancfd_gb300 import configs

    if args.workload == "spherical_flame":
        return configs.spherical_flame(ncell=args.flame_cells or 2000)
    return configs.planar_flame(ncell=args.flame_cells or 1000)


def flame_config(case, args, world):
    sph = args.workload == "spherical_flame"
    return {"workload": case.name, "cells": case.ncell, "dx_m": case.dx,
            "mixture": ("stoichiometric CH4/O2/N2, 300 K, 1 atm, at rest" if sph else
                        "stoichiometric CH4/O2/N2, 1 atm; T erf profile 300 -> 2400 K at 1.4 cm, width 2 mm"),
            "scheme": ("spherical, MUSCL-minmod + HLLC + SSP-RK3, CFL 0.2, centre wall / outflow 1 atm" if sph else
                       "MUSCL-minmod + HLLC + SSP-RK3, CFL 0.5, inflow 300 K 1 m/s / outflow 1 atm"),
            "transport": "calc_flux_tran, TRANLIB mixture rules (MCAVIS, MCACON, MCADIF)",
            "chemistry": "GRI-Mech 3.0, per-cell stiff integration, rtol 1e-5, atol 1e-13",
            "sources": "ignition energy 0.5 mJ, 500 um, 100 us (Frendi et al.)" if sph else "none",
            "timed_steps": f"steps {args.warmup + 1}..{args.warmup + args.steps} from the initial state",
            "parallelism": f"replicas x{world}"}


def flame_oracle(case):
    sys.path.insert(0, str(ROOT / "tests"))
    from oracle_ctypes import Oracle

    o = Oracle()
    fl = case.flags
    qf0, qc0 = o.init_cells(case.T, case.p, case.u, case.X)
    t = o.tube(case.ncell, 2, [1, 2, 1, 2, 0, fl["flag_lbound"], fl["flag_rbound"], fl["do_reaction"]],
               [case.dx, fl["p_out"], fl.get("t_in", 300.0), fl.get("rho_u_in", 0.0), 1e-5, 1e-13],
               x_in=fl.get("x_in"))
    t.set_transport()
    if fl.get("is_spherical"):
        t.set_spherical()
    if fl.get("ignition"):
        t.set_sources(ignition=fl["ignition"])
    t.set_interior(qf0, qc0)
    return o, t


def flame_reference_arm(args, rank, world):
    """The oracle (the reference's algorithm, transport included) on all host
    cores, the same flame, the same steps as the GPU arm."""
    if rank != 0:
        return
    case = flame_case(args)
    o, t = flame_oracle(case)
    for _ in range(args.warmup):
        t.step(case.cfl)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t.step(case.cfl)
    el = time.perf_counter() - t0
    v = case.ncell * args.steps / el
    cores = o.L.or_num_threads()
    print(json.dumps({"impl": "reference", "metric": FLAME_METRICS[args.workload], "value": v, "unit": UNIT, "n_gpus": world,
                      "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps,
                      "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                      "data": "synthetic", "config": flame_config(case, args, world),
                      "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                                       "sample": f"steps {args.warmup + 1}..{args.warmup + args.steps} of the flame"},
                      "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}),
          flush=True)


def flame_arm(args, rank, world, local):
    """The planar flame with transport and chemistry (configs.planar_flame):
    steps in CUDA graphs through edyn_advance; the transport's share from
    the same tube's fluid step with and without it."""
    import torch

    from fortrancfd_gb300 import Tube

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    case = flame_case(args)
    fl = {k: v for k, v in case.flags.items() if k not in ("do_tran", "ignition", "strict_newton")}
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    tube = Tube(case.ncell, case.dx, do_tran=1, strict_newton=0, **fl)
    tube.set_stream(stream.cuda_stream)
    if case.flags.get("ignition"):
        tube.set_ignition(*case.flags["ignition"])
    tube.init_cells(case.T, case.p, case.u, case.X)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    with ClockSampler(local) as clk:
        t_dev, graphs, t_sim = run_tube(tube, case, args.steps, args.warmup, stream, flush)
    torch.cuda.synchronize(dev)
    t_max = max_over_ranks(t_dev, world, dev)
    # the fluid step with and without transport on the state reached
    qf, qc, _ = tube.download()
    inviscid = Tube(case.ncell, case.dx, strict_newton=0, **fl)
    inviscid.set_stream(stream.cuda_stream)
    inviscid.set_uniform_skip(False)
    dt = tube.calc_dt(case.cfl)
    ms = {"transport": [], "inviscid": []}
    for _ in range(3):
        for name, t in (("transport", tube), ("inviscid", inviscid)):
            t.upload(qf, qc)
            flush.zero_()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            t.solve_fluid(dt)
            b.record(stream)
            b.synchronize()
            ms[name].append(a.elapsed_time(b))
    fl_t, fl_i = statistics.median(ms["transport"]), statistics.median(ms["inviscid"])
    if rank != 0:
        return
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        o, t = flame_oracle(case)
        t.step(case.cfl)
        n, t0 = 0, time.perf_counter()
        while True:
            t.step(case.cfl)
            n += 1
            el = time.perf_counter() - t0
            if el > 15.0 or n >= 64:
                break
        cpu = {"value": case.ncell * n / el, "unit": UNIT, "cores": o.L.or_num_threads(), "kind": "port",
               "sample": f"steps 2..{n + 1} of the flame, {el:.1f} s"}
    # per step: the loop test, three (transport properties, transport flux,
    # stage) triples, the one-pass chemistry (counter clear + pass) and, with
    # an ignition energy, the source kernel
    per_step = 1 + 3 * 3 + 2 + (1 if case.flags.get("ignition") else 0)
    print(json.dumps({
        "metric": FLAME_METRICS[args.workload], "value": job_value(case.ncell, args.steps, world, t_max), "unit": UNIT,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_max / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": flame_config(case, args, world), "clocks": clk.summary(),
        "gpu_launches": graphs * 16 * per_step,
        "transport": {"fluid_step_ms": fl_t, "inviscid_fluid_step_ms": fl_i,
                      "transport_ms_per_stage": (fl_t - fl_i) / 3.0,
                      "note": "the same tube's fluid step with and without transport, L2 flushed"},
        "impl": {"l2": "L2 flushed between 16-step graphs", "simulated_time_s": t_sim},
        "cpu_baseline": cpu}), flush=True)


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        if args.workload in FLAME_METRICS:
            flame_reference_arm(args, rank, world)
            return
        reference_arm(args, rank, world)
        return
    if args.workload in FLAME_METRICS:
        flame_arm(args, rank, world, local)
        return
    if args.workload == "tubes":
        tubes_arm(args, rank, world, local)
        return
    if args.workload == "reactors":
        if rank == 0:
            reactors_arm(args, local)
        return
    gpu_arm(args, rank, world, local)


if __name__ == "__main__":
    main()
