"""Benchmark of the GB300 per-cell hot path (one JSON line on rank 0).

Workload (default): the CH4/O2 detonation tube of the reference's second
benchmark configuration -- 20,000 cells of 50 um on a 1 m tube, a 1 cm
driver at 3000 K / 30 atm, WENO5-Z + HLLC + SSP-RK3, CFL 0.4, detailed
GRI-Mech 3.0 chemistry (53 species, 325 reactions) integrated per cell by
the plain implicit integrator (FP64 residuals, FP32 Jacobian/LU).
A step is one pass of the time loop body (calc_dt, three fluid stages,
chemistry, post-step) over the whole tube: "cell-steps" = cells x steps.

value: device time of K steps with the state resident in HBM, CUDA events
on the library's stream (16-step CUDA-graph launches, L2 flushed between
launches). e2e: the same steps through the C ABI with host buffers -- every
step uploads qf/Qc from pinned host memory, steps, and downloads qf/Qc/HRR.
--impl reference: the CPU restatement of the reference's algorithm (the
oracle; the Fortran code does not build here) on all host cores.
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
BYTES_PER_CELL_STEP = 4544  # algorithmic: fluid RK3 3632 B + chemistry 912 B per cell-step
BYTES_CHEM_PER_CELL = 912   # chemistry launch: read qf (456 B) + write qf and Qc rows (456 B)
# DRAM bytes (read + write) of one chemistry launch per cell, from an ncu
# capture of the 4,000-cell tube (1.93 MB read, 0 B written), scaled by cells
TRAFFIC_CHEM_PER_CELL = 1.93e6 / 4000


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=32)
    p.add_argument("--warmup", type=int, default=16)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--cells", type=int, default=20000)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-surrogate", action="store_true", help="skip the surrogate-vs-plain chemistry comparison")
    p.add_argument("--workload", default="tube", choices=["tube", "reactors"],
                   help="tube: the detonation tube (default, the headline metric); reactors: the batch of "
                        "partially reacted constant-volume reactors")
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


def build_case(cells):
    from fortrancfd_gb300 import configs

    return configs.detonation(ncell=cells, length=cells * 50e-6)


def reference_arm(args, rank, world):
    """CPU restatement of the reference (oracle) on all host cores."""
    if rank != 0:
        return
    sys.path.insert(0, str(ROOT / "tests"))
    from oracle_ctypes import Oracle

    o = Oracle()
    case = build_case(args.cells)
    qf0, qc0 = o.init_cells(case.T, case.p, case.u, case.X)
    t = o.tube(case.ncell, 3, [1, 2, 2, 2, 3, 0, 1, 1], [case.dx, 101325.0, 300.0, 0.0, 1e-5, 1e-13])
    t.set_interior(qf0, qc0)
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
            "config": {"workload": case.name, "cells": case.ncell, "chemistry": "plain FP64 SDIRK4",
                       "scheme": "WENO5-Z + HLLC + SSP-RK3"},
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{args.steps} full steps of the {case.ncell}-cell tube after {args.warmup}"},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline(case, budget_s=12.0):
    """The oracle on the host cores over a bounded sample of the workload."""
    sys.path.insert(0, str(ROOT / "tests"))
    from oracle_ctypes import Oracle

    o = Oracle()
    qf0, qc0 = o.init_cells(case.T, case.p, case.u, case.X)
    t = o.tube(case.ncell, 3, [1, 2, 2, 2, 3, 0, 1, 1], [case.dx, 101325.0, 300.0, 0.0, 1e-5, 1e-13])
    t.set_interior(qf0, qc0)
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
            "sample": f"{n} full steps (after 1) of the {case.ncell}-cell tube, {el:.1f} s"}


def surrogate_compare(tube, case, dt, dev):
    """Surrogate-with-fallback chemistry against the plain implicit
    integrator on the same batch: the tube's cells after the timed steps,
    each advanced over the tube's step dt. The network is trained first, on
    the GPU, on pairs that the plain integrator produces along a 2,000-cell
    (10 cm) CH4/O2 detonation run; errors are against the FP64 reference
    integrator (rtol 1e-8, atol 1e-16). Wall-clock times, median of 3."""
    import numpy as np
    import torch

    from fortrancfd_gb300 import Reactors, configs
    from fortrancfd_gb300 import surrogate as S

    t0 = time.perf_counter()
    rho, dtt, y0, y1 = S.harvest_tube(configs.detonation(ncell=2000, length=0.1), nsteps=1200, every=20)
    s = S.Surrogate(Reactors(rtol=1e-5, atol=1e-13), S.MLP(seed=0))
    hist = S.train(s, rho, dtt, y0, y1, iters=3000, batch=4096, lr=2e-3, log_every=2999)
    t_train = time.perf_counter() - t0
    qf, _, _ = tube.download()
    yb = np.ascontiguousarray(np.concatenate([qf[:, 3:], qf[:, 2:3]], axis=1))
    rb = np.ascontiguousarray(qf[:, 0])
    db = np.full(len(rb), dt)
    ref = yb.copy()
    Reactors(rtol=1e-8, atol=1e-16).integrate(rb, db, ref)
    R = torch.tensor(rb, device=dev)
    D = torch.tensor(db, device=dev)

    def err(y):
        big = np.abs(ref[:, :-1]) >= 1e-6
        rel = np.where(big, np.abs(y[:, :-1] - ref[:, :-1]) / np.maximum(np.abs(ref[:, :-1]), 1e-6), 0.0)
        return float(rel.max()), float(abs(y[:, -1].max() - ref[:, -1].max()) / ref[:, -1].max())

    tp, ts, tz = [], [], []
    for _ in range(3):
        y = torch.tensor(yb, device=dev)
        with s:
            torch.cuda.synchronize(dev)
            a = time.perf_counter()
            pst = s.r.integrate_device(len(rb), R.data_ptr(), D.data_ptr(), y.data_ptr())
            tp.append(time.perf_counter() - a)
        ep = err(y.cpu().numpy())
        y = torch.tensor(yb, device=dev)
        torch.cuda.synchronize(dev)
        a = time.perf_counter()
        st = s.apply(R, D, y)
        ts.append(time.perf_counter() - a)
        es = err(y.cpu().numpy())
        y = torch.tensor(yb, device=dev)
        torch.cuda.synchronize(dev)
        a = time.perf_counter()
        st0 = s.apply(R, D, y, zero_net=True)
        tz.append(time.perf_counter() - a)
    n = len(rb)
    tp_, ts_, tz_ = statistics.median(tp), statistics.median(ts), statistics.median(tz)
    return {"batch": f"{n} cells of the bench tube after the timed steps, dt = its step ({dt:.3e} s)",
            "training": f"{len(rho)} pairs from a 2,000-cell detonation run, 3000 Adam steps of 4096, "
                        f"{t_train:.1f} s incl. harvest, final loss {hist[-1][1]:.3f}",
            "plain_cells_per_s": n / tp_, "surrogate_cells_per_s": n / ts_, "speedup": tp_ / ts_,
            "fallback_rate": st["fallback_rate"], "network_accepted": st["accepted_network"],
            "explicit_only_fallback_rate": st0["fallback_rate"], "explicit_only_cells_per_s": n / tz_,
            "plain_rhs": pst["rhs"], "fallback_rhs": st["integrator_rhs"],
            "species_err": {"plain": ep[0], "surrogate": es[0]}, "peak_T_err": {"plain": ep[1], "surrogate": es[1]}}


def gpu_arm(args, rank, world, local):
    import torch

    from fortrancfd_gb300 import Tube

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    case = build_case(args.cells)
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
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2
    per_graph = 16
    # warm-up (also captures the step graph)
    t_sim = 0.0
    done = 0
    while done < args.warmup:
        t_sim, n = tube.advance(case.cfl, tend=1e9, time=t_sim, max_steps=per_graph)
        done += n
    iters = max(1, (args.steps + per_graph - 1) // per_graph)
    steps = iters * per_graph
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize(dev)
    dev_ms = 0.0
    with ClockSampler(local) as clk:
        for _ in range(iters):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            t_sim, n = tube.advance(case.cfl, tend=1e9, time=t_sim, max_steps=per_graph)
            e1.record(stream)
            e1.synchronize()
            dev_ms += e0.elapsed_time(e1)
            assert n == per_graph
    torch.cuda.synchronize(dev)
    t_max = max_over_ranks(dev_ms / 1e3, world, dev)
    value = job_value(case.ncell, steps, world, t_max)
    # per-launch kernel durations for the roofline: chemistry and one fluid step
    dt = tube.calc_dt(case.cfl)
    chem_ms = []
    fluid_ms = []
    for _ in range(3):
        flush.zero_()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        tube.solve_fluid(dt)
        b.record(stream)
        b.synchronize()
        fluid_ms.append(a.elapsed_time(b))
        flush.zero_()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        tube.solve_source(dt)
        b.record(stream)
        b.synchronize()
        chem_ms.append(a.elapsed_time(b))
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
    e2e_steps = max(4, min(args.steps, 16))
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
    achieved = BYTES_CHEM_PER_CELL * case.ncell / chem_s / 1e9
    cpu = None if args.no_cpu_baseline or world > 1 else cpu_baseline(case)
    surr = None
    if not args.no_surrogate and world == 1:
        try:
            surr = surrogate_compare(tube, case, dt, dev)
        except Exception as ex:  # reported, not hidden: the headline line still prints
            surr = {"error": f"{type(ex).__name__}: {ex}"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t_max / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": case.name, "cells": case.ncell, "chemistry": "plain SDIRK4 (FP64 residual, "
                       "FP32 analytic Jacobian/LU)", "scheme": "WENO5-Z + HLLC + SSP-RK3, CFL 0.4",
                       "parallelism": f"replicas x{world}", "l2": "flushed between 16-step graph launches",
                       "tolerances": "rtol 1e-5, atol 1e-13",
                       "stage_tile": "%d cells, %d threads per CTA" % tube.stage_tile(),
                       "chemistry_set": "%d species, %d reactions" % tube.chem_set()},
            "clocks": clk.summary(),
            "e2e": {"value": case.ncell * e2e_steps / e2e_el, "unit": UNIT,
                    "h2d_bytes_per_step": 2 * case.ncell * ne * 8,
                    "d2h_bytes_per_step": (2 * case.ncell * ne + case.ncell) * 8},
            "gpu_launches": steps * 5,
            "roofline": {"bound": "hbm", "kernel": "k_tube_chem", "achieved": achieved, "peak": hbm,
                         "peak_source": src, "unit": "GB/s", "frac": achieved / hbm,
                         "traffic": TRAFFIC_CHEM_PER_CELL * case.ncell, "launch_ms": chem_s * 1e3, "fluid_step_ms": fluid_s * 1e3},
            "cpu_baseline": cpu,
            "chem_launch": {"rhs_per_cell": chem_stats["rhs"] / max(1, chem_stats["cells"]),
                            "rejects": chem_stats["rejects"], "team_cells": chem_stats["team_cells"],
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
    import numpy as np
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


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        reference_arm(args, rank, world)
        return
    if args.workload == "reactors":
        if rank == 0:
            reactors_arm(args, local)
        return
    gpu_arm(args, rank, world, local)


if __name__ == "__main__":
    main()
