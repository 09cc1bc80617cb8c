"""Benchmark of the GB300 VE Stokes PT path (2D VE Stokes, 2048^2 cells, 8 viscous inclusions).

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n 2048]

One step = one chunk of `ncheck` (= n/4) PT iterations (update_stress!, update_velocity!,
bc!(V), captured in a CUDA graph) followed by the on-device convergence measures of
examples/stokes_2d_inc_ve_T.jl:154-157 read back to the host.
Metric: effective memory throughput T_eff = A_eff * iterations / time (GB/s) with
A_eff = 16 arrays * n^2 * sizeof(T) per PT iteration (read+write V.x, V.y, P, tau.xx,
tau.yy, tau.xy; read tau_old x3, eta), the reference's T_eff convention
(examples/stokes_3d_inc_ve_T_mpi_perf.jl:209-213) for this field set.
Inputs are 16 arrays of 33.6 MB (FP64): larger than the 129 MB L2, so no flush is needed.

--impl reference times the CPU restatement of the same PT iterations (the reference itself
is Julia and is not available here) with all host threads on a bounded sample.
With torchrun (N > 1) every rank solves its own replica (the path has no data exchange on
one GPU); value = sum of the ranks' work / max time.
"""

from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
for _p in (ROOT / "chmy.jl_gb300", ROOT / "tests", ROOT / "oracle"):
    if str(_p) not in sys.path:
        sys.path.insert(0, str(_p))

import numpy as np  # noqa: E402

ARRAYS_PER_ITER = 16  # V(2) P tau(3) read+write = 12, tau_old(3) eta read = 4
STRESS_ARRAYS = 14  # update_stress: read V(2) tau(3) tau_old(3) P eta(inv) ; write tau(3) P
VEL_ARRAYS = 9  # update_velocity: read P tau(3) eta(inv) V(2) ; write V(2)


def _env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic(name: str):
    """DRAM bytes per launch from the committed ncu summary (profiles/<name>.txt, a line
    `dram_bytes_per_launch: <int>` scaled to this workload), or None."""
    p = ROOT / "profiles" / f"{name}.txt"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms in a background thread."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, device_index: int):
        self.dev = device_index
        self.samples = []
        self._stop = threading.Event()
        self._thr = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(
                    ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits"],
                    capture_output=True,
                    text=True,
                    timeout=5,
                ).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._thr = threading.Thread(target=self._run, daemon=True)
        self._thr.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._thr:
            self._thr.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no nvidia-smi samples"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for nm, v in zip(names, s[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {
            "sm_mhz": float(np.median(sm)) if sm else None,
            "sm_max_mhz": max(mx) if mx else None,
            "reasons": sorted(reasons),
            "samples": len(self.samples),
        }


def cpu_sample(n: int, seconds: float = 12.0, max_iters: int = 200):
    """Time the oracle's PT iterations (update_stress!, update_velocity!, bc!) on the host with
    all cores; returns (T_eff GB/s, iterations, seconds, threads)."""
    import ctypes as C

    from _oracle import NpField, bc_apply, lib, stokes_desc
    from chmy_gb300.configs import stokes2d_inclusions
    from chmy_gb300.grids import Center, Vertex

    threads = os.cpu_count() or 1
    lib().or_set_threads(threads)
    pb = stokes2d_inclusions(n)
    g = pb.grid
    Cl, Vl = Center(), Vertex()

    def mk(a, loc):
        f = NpField(g, loc)
        f.a[...] = a
        return f

    h = pb.host
    V = [mk(h["V"][0], (Vl, Cl)), mk(h["V"][1], (Cl, Vl))]
    tau = [mk(h["tau"][0], Cl), mk(h["tau"][1], Cl), mk(h["tau"][2], Vl)]
    tauo = [mk(h["tau_old"][0], Cl), mk(h["tau_old"][1], Cl), mk(h["tau_old"][2], Vl)]
    P = mk(h["P"], Cl)
    eta = mk(h["eta"], Cl)
    ieta = mk(1.0 / h["eta"], Cl)
    d = stokes_desc(V=V, P=P, tau=tau, tau_old=tauo, eta=eta, inv_eta=ieta)
    gd = g.desc()
    p = pb.params
    it = 0
    t0 = time.perf_counter()
    while True:
        lib().or_stokes_update_stress(C.byref(gd), C.byref(d), C.byref(p))
        lib().or_stokes_update_velocity(C.byref(gd), C.byref(d), C.byref(p))
        bc_apply(g, V, pb.bc_V)
        it += 1
        el = time.perf_counter() - t0
        if el >= seconds or it >= max_iters:
            break
    teff = ARRAYS_PER_ITER * n * n * 8 * it / el / 1e9
    return teff, it, el, threads


def run_reference(args, rank, world):
    if rank != 0:
        return
    teffs = []
    its = 0
    secs = 0.0
    threads = 1
    total = args.warmup + args.steps
    for s in range(total):
        teff, it, el, threads = cpu_sample(args.n, seconds=args.ref_seconds, max_iters=args.ref_iters)
        if s >= args.warmup:
            teffs.append(teff)
            its += it
            secs += el
    value = ARRAYS_PER_ITER * args.n * args.n * 8 * its / secs / 1e9
    line = {
        "impl": "reference",
        "metric": "T_eff GB/s",
        "value": value,
        "unit": "GB/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": 1e3 * secs / max(args.steps, 1),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic (seeded inclusions, seed 3)",
        "config": {"workload": f"2D VE Stokes {args.n}^2, 8 inclusions, PT iterations (update_stress!, update_velocity!, bc!)", "n": args.n},
        "cpu_baseline": {
            "value": value,
            "unit": "GB/s",
            "cores": threads,
            "kind": "port",
            "sample": f"{its} PT iterations over {args.steps} steps (C++ restatement of the reference CPU path, OpenMP)",
        },
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, dist):
    import torch

    from chmy_gb300 import Arch, GB300Backend
    from chmy_gb300.configs import stokes2d_inclusions
    from chmy_gb300.solvers import StokesSolver

    local = _env_int("LOCAL_RANK", 0)
    arch = Arch(GB300Backend(), device_id=local + 1)
    n = args.n
    pb = stokes2d_inclusions(n)
    solver = StokesSolver(arch, pb)
    solver.apply_bc()
    ncheck = pb.ncheck
    T = 8
    bytes_per_iter = ARRAYS_PER_ITER * n * n * T

    def barrier():
        if dist is not None:
            dist.barrier()

    def step():
        solver.iterate(ncheck)
        return solver.residual()  # host read of the step's result (blocks)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            err = step()
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    if dist is not None:
        t = torch.tensor([ms], device=arch.device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    iters = ncheck * args.steps
    value = bytes_per_iter * iters * world / (ms * 1e-3) / 1e9

    # e2e: public API with host buffers: every step uploads the initial state from pinned host
    # memory, runs the chunk and reads the residual measures back.
    pinned = {}
    h2d = 0
    for k, v in pb.host.items():
        if isinstance(v, list):
            pinned[k] = [torch.from_numpy(a).pin_memory() for a in v]
            h2d += sum(a.nbytes for a in v)
        else:
            pinned[k] = torch.from_numpy(v).pin_memory()
            h2d += v.nbytes
    d2h = 8 * (pb.grid.ndim + 1)

    def e2e_step():
        solver.upload(pinned)
        solver.apply_bc()
        return step()

    for _ in range(max(1, args.warmup // 2)):
        e2e_step()
    torch.cuda.synchronize()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1)
    if dist is not None:
        t = torch.tensor([ms_e2e], device=arch.device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_e2e = float(t.item())
    e2e_value = bytes_per_iter * iters * world / (ms_e2e * 1e-3) / 1e9

    # roofline of the dominant kernel (update_stress!), timed alone with CUDA events on the
    # launching stream, per-launch algorithmic bytes over average duration
    import ctypes

    reps = 50
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for _ in range(reps):
        arch.call("cg_stokes_update_stress", ctypes.byref(solver.grid_desc), ctypes.byref(solver.desc), ctypes.byref(pb.params))
    s1.record(stream)
    torch.cuda.synchronize()
    stress_ms = s0.elapsed_time(s1) / reps
    v0, v1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    v0.record(stream)
    for _ in range(reps):
        arch.call("cg_stokes_update_velocity", ctypes.byref(solver.grid_desc), ctypes.byref(solver.desc), ctypes.byref(pb.params))
    v1.record(stream)
    torch.cuda.synchronize()
    vel_ms = v0.elapsed_time(v1) / reps
    # update_stress! as called by the per-kernel API also writes divV (one more array)
    stress_bytes = (STRESS_ARRAYS + 1) * n * n * T
    achieved = stress_bytes / (stress_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = committed_traffic(f"stokes2d_stress_{n}")

    if rank == 0:
        cpu_teff, cpu_it, cpu_s, cpu_threads = cpu_sample(n, seconds=args.cpu_seconds, max_iters=args.ref_iters)
        line = {
            "metric": "T_eff GB/s",
            "value": value,
            "unit": "GB/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": args.warmup,
            "ms_per_step": ms / args.steps,
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f64",
            "data": "synthetic (seeded inclusions, seed 3)",
            "config": {
                "workload": f"2D VE Stokes {n}^2, 8 inclusions (log10 eta U[-3,3]), PT chunk of {ncheck} iterations + convergence check",
                "n": n,
                "iterations_per_step": ncheck,
                "arrays_per_iteration": ARRAYS_PER_ITER,
                "l2": "inputs larger than L2 (16 x 33.6 MB), no flush",
                "last_err": err,
            },
            "e2e": {"value": e2e_value, "unit": "GB/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": args.steps * (3 * ncheck + 2),
            "roofline": {
                "bound": "hbm",
                "kernel": "stress_kernel (update_stress!)",
                "achieved": achieved,
                "peak": peak,
                "unit": "GB/s",
                "frac": achieved / peak,
                "peak_kind": f"{peak_kind} (hbm_gbs)",
                "traffic": traffic,
                "kernel_ms": {"update_stress": stress_ms, "update_velocity": vel_ms},
            },
            "cpu_baseline": {
                "value": cpu_teff,
                "unit": "GB/s",
                "cores": cpu_threads,
                "kind": "port",
                "sample": f"{cpu_it} PT iterations of {n}^2 in {cpu_s:.1f} s (C++ restatement, OpenMP)",
            },
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    arch.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=2048)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-seconds", type=float, default=8.0)
    ap.add_argument("--ref-iters", type=int, default=200)
    args = ap.parse_args()
    world = _env_int("WORLD_SIZE", 1)
    rank = _env_int("RANK", 0)
    dist = None
    if world > 1 and args.impl == "ours":
        import torch
        import torch.distributed as tdist

        torch.cuda.set_device(_env_int("LOCAL_RANK", 0))
        tdist.init_process_group("nccl")
        dist = tdist
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, dist)
    if dist is not None:
        dist.barrier()
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
