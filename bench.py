"""Benchmark: 2D VE Stokes PT solve to 1e-8 (2048^2 cells, 8 viscous inclusions) on one GB300.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n 2048]

One step = one physical time step of examples/stokes_2d_inc_ve_T.jl:144-163 on the synthetic
inclusion problem: the PT solve from the initial state to residual 1e-8, with FP32 PT
iterations (one fused sm_103a kernel per iteration) inside an FP64 defect-correction loop.
The plain FP64 GPU solve of the same problem is timed once beside it (time_to_solution).

Metric: T_eff = A_eff x PT iterations / time (GB/s), the reference's effective-throughput
convention (examples/stokes_3d_inc_ve_T_mpi_perf.jl:209-213) for this field set:
A_eff = 19 arrays x n^2 x 4 B per FP32 PT iteration (read+write V.x V.y P tau.xx tau.yy
tau.xy = 12; read tau_old' x3, 1/eta, continuity forcing, momentum forcing x2 = 7); the
FP64 defect/update cycles (a handful per solve) are not counted.
The working set (32 FP64/FP32 arrays of 17-34 MB) exceeds the 129 MB L2: no flush needed.

--impl reference times the CPU restatement of the reference's FP64 PT iterations (Chmy is
Julia and cannot run here) with all host threads on a bounded sample; its T_eff counts
16 arrays x n^2 x 8 B per iteration (the FP64 form without forcing arrays).
With torchrun (N > 1) every rank solves its own replica (the path has no data exchange on one
GPU); value = the ranks' total work / the slowest rank's time.
"""

from __future__ import annotations

import argparse
import ctypes
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

A32 = 19  # arrays per FP32 PT iteration of the defect-correction solve
A64 = 16  # arrays per FP64 PT iteration (reference form, variable viscosity, no body force)
FUSED_ARRAYS = 18  # the timed fused kernel: no continuity forcing (public ping-pong entry)
# 3D: read/write V x3, tau x6, P; read tau_old x6, 1/eta, rho_g.z (the reference's T_eff set
# for 3D VE Stokes without the thermal arrays)
FUSED3_ARRAYS = 28


def _env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def reduce_over_ranks(dist, ms: float, work: float, device="cpu"):
    """The N > 1 replica aggregation: the slowest rank's time (max) and the ranks' total work
    (sum). With dist None (one rank) the inputs come back unchanged."""
    if dist is None:
        return float(ms), float(work)
    import torch

    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    w = torch.tensor([float(work)], dtype=torch.float64, device=device)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    return float(t.item()), float(w.item())


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_traffic(name: str):
    """DRAM bytes per launch (`dram_bytes_per_launch: <number>`) from profiles/<name>.md."""
    p = ROOT / "profiles" / f"{name}.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        line = line.strip().strip("`")
        if line.startswith("dram_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def committed_fp64_flops(unit: str):
    """FP64 FLOPs per cell of one unit (`fp64_flops_per_cell: <unit> <number>`) from
    profiles/fp64_kernels.md: 2 x DFMA + DADD + DMUL counted by ncu on the same kernels."""
    p = ROOT / "profiles" / "fp64_kernels.md"
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        parts = line.strip().split()
        if len(parts) == 3 and parts[0] == "fp64_flops_per_cell:" and parts[1] == unit:
            try:
                return float(parts[2])
            except ValueError:
                return None
    return None


def fp64_roofline(unit: str, cells: float, units: float, seconds: float, peak_flops: float):
    """The FP64-pipe roofline of an FP64-bound entry: FLOPs (per cell x cells x units) over its
    measured time, against the device's FP64 FMA peak measured live (cg_fp64_peak)."""
    fpc = committed_fp64_flops(unit)
    if fpc is None or seconds <= 0 or not peak_flops:
        return None
    achieved = fpc * cells * units / seconds
    return {"bound": "fp64", "achieved": achieved / 1e12, "peak": peak_flops / 1e12, "unit": "TFLOP/s",
            "frac": achieved / peak_flops, "flops_per_cell": fpc, "peak_kind": "measured (cg_fp64_peak)",
            "flops_source": "profiles/fp64_kernels.md (ncu DFMA/DADD/DMUL counts)"}


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

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None

        sm = [v for v in (num(s[1]) for s in self.samples) if v is not None]
        mx = [v for v in (num(s[2]) for s in self.samples) if v is not None]
        pw = [v for v in (num(s[3]) for s in self.samples) if v is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for nm, v in zip(names, s[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {
            "sm_mhz": float(np.median(sm)) if sm else None,
            "sm_max_mhz": max(mx) if mx else None,
            "power_w_max": max(pw) if pw else None,
            "reasons": sorted(reasons),
            "samples": len(self.samples),
        }


def cpu_sample(n: int, seconds: float, max_iters: int):
    """The oracle's FP64 PT iterations (update_stress!, update_velocity!, bc!) on all host
    cores: (T_eff GB/s, iterations, seconds, threads)."""
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
    bc_apply(g, V, pb.bc_V)
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
    return A64 * n * n * 8 * it / el / 1e9, it, el, threads


def workload_name(n):
    return (
        f"2D VE Stokes {n}^2, 8 circular inclusions (log10 eta U[-3,3], seed 3), pure shear, "
        "PT solve to residual 1e-8: FP32 PT in FP64 defect correction"
    )


def reference_workload_name(n):
    return (
        f"2D VE Stokes {n}^2, 8 circular inclusions (log10 eta U[-3,3], seed 3), pure shear: "
        "FP64 PT iterations (update_stress!, update_velocity!, bc!(V)), bounded sample; no solve"
    )


# PT iterations of the plain FP64 solve of the 2048^2 inclusion problem to residual 1e-8 with
# the PT parameters below (re_m = 4 pi, a check every n/4 iterations), as the FP64 GPU solve
# counts them (the GPU's FP64 iteration counts match the oracle's PT loop within 1 %). The
# reference arm cannot solve in its time budget; it extrapolates its time to solution with this
# count. Our arm measures the count itself on every run.
FP64_ITERATIONS_2048 = 96256


def run_reference(args, rank, world):
    if rank != 0:
        return
    its, secs, threads = 0, 0.0, 1
    for s in range(args.warmup + args.steps):
        teff, it, el, threads = cpu_sample(args.n, seconds=args.ref_seconds, max_iters=args.ref_iters)
        if s >= args.warmup:
            its += it
            secs += el
    value = A64 * args.n * args.n * 8 * its / secs / 1e9
    # the FP64 solve's iteration count scales with n (PT iterations per grid point are constant)
    iters_to_solve = int(round(FP64_ITERATIONS_2048 * args.n / 2048))
    tts_ref = secs / max(its, 1) * iters_to_solve
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
        "data": "synthetic (seeded inclusions)",
        "config": {"workload": reference_workload_name(args.n), "n": args.n,
                   "sample_per_step": f"{args.ref_seconds:.0f} s of FP64 PT iterations",
                   "bytes": "T_eff counts 16 arrays x n^2 x 8 B per FP64 PT iteration"},
        "time_to_solution_s": tts_ref,
        "time_to_solution": {"kind": "extrapolated", "fp64_iterations": iters_to_solve,
                             "note": "sampled seconds per FP64 PT iteration x the FP64 solve's iteration count"},
        "cpu_baseline": {
            "value": value,
            "unit": "GB/s",
            "cores": threads,
            "kind": "port",
            "sample": f"{its} FP64 PT iterations of {args.n}^2 over {args.steps} steps (C++ restatement of the reference CPU path, OpenMP)",
        },
        "e2e": {"value": value, "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args, rank, world, dist):
    import torch

    from chmy_gb300 import Arch, Field, GB300Backend, _abi
    from chmy_gb300.configs import stokes2d_inclusions
    from chmy_gb300.kernels import stokes_fields
    from chmy_gb300.solvers import StokesSolver

    local = _env_int("LOCAL_RANK", 0)
    arch = Arch(GB300Backend(), device_id=local + 1)
    n = args.n
    pb = stokes2d_inclusions(n)
    solver = StokesSolver(arch, pb)
    state_names = ("V", "P", "tau", "tau_old", "r_V", "divV")
    pristine = {}
    for k in state_names:
        v = solver.fields[k]
        pristine[k] = [f.data.clone() for f in v] if isinstance(v, list) else v.data.clone()

    def reset_device():
        for k in state_names:
            v = solver.fields[k]
            if isinstance(v, list):
                for f, src in zip(v, pristine[k]):
                    f.data.copy_(src)
            else:
                v.data.copy_(pristine[k])
        solver.apply_bc()

    def barrier():
        if dist is not None:
            dist.barrier()

    results = []

    def step():
        reset_device()
        r = solver.solve(precision=_abi.CG_F32, max_outer=12, inner_rtol=1e-5)
        if r.converged != 1:
            raise RuntimeError(f"solve did not converge: {list(r.err)} after {r.iterations} iterations")
        results.append(r)
        return r

    for _ in range(args.warmup):
        step()
    results.clear()
    torch.cuda.synchronize()
    barrier()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    iters = sum(r.iterations for r in results)
    ms, iters_all = reduce_over_ranks(dist, ms, iters, arch.device)
    bytes_per_iter = A32 * n * n * 4
    value = bytes_per_iter * iters_all / (ms * 1e-3) / 1e9
    # kernels in the timed solves: per PT iteration the fused kernel (bc!(V) folded into its
    # reads; one bc!(V) launch per chunk of ncheck iterations, or one per iteration with
    # CG_BC_FOLD=0); per check bc!(r_V), the max-norm and (inner checks) the constitutive
    # measure, or (outer checks) the FP64 defect; per correction the FP64 update and bc!(V);
    # one 1/eta conversion per solve
    nchunk = pb.ncheck + (pb.ncheck & 1)
    fold = os.environ.get("CG_BC_FOLD", "1")[:1] != "0"
    launches = sum(r.iterations + (r.iterations // nchunk if fold else r.iterations) + 3 * r.checks + 2 * r.outer + 1
                   for r in results)

    # e2e through the public API with host buffers: upload the initial state from pinned host
    # memory, solve, read the velocity and pressure back every step
    pinned = {}
    h2d = 0
    host_in = dict(pb.host)
    # 1/eta is an input of the kernels, prepared on the host (as StokesSolver does) and uploaded
    # with the other arrays: no device compute outside the library in the timed region
    host_in["inv_eta"] = 1.0 / np.asarray(pb.host["eta"])
    for k in state_names + ("eta", "inv_eta"):
        v = host_in[k]
        if isinstance(v, list):
            pinned[k] = [torch.from_numpy(a).pin_memory() for a in v]
            h2d += sum(a.nbytes for a in v)
        else:
            pinned[k] = torch.from_numpy(v).pin_memory()
            h2d += v.nbytes
    outs = [torch.empty(f.data.shape, dtype=f.data.dtype).pin_memory() for f in solver.fields["V"]]
    outs.append(torch.empty(solver.fields["P"].data.shape, dtype=solver.fields["P"].data.dtype).pin_memory())
    d2h = sum(o.numel() * o.element_size() for o in outs) + 8 * 3

    def e2e_step():
        solver.upload(pinned)
        solver.apply_bc()
        r = solver.solve(precision=_abi.CG_F32, max_outer=12, inner_rtol=1e-5)
        for o, f in zip(outs, list(solver.fields["V"]) + [solver.fields["P"]]):
            o.copy_(f.data, non_blocking=True)
        return r

    e2e_steps = max(1, min(args.steps, args.e2e_steps))
    e2e_step()
    torch.cuda.synchronize()
    barrier()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2e_iters = 0
    e0.record(stream)
    for _ in range(e2e_steps):
        e2e_iters += e2e_step().iterations
    e1.record(stream)
    torch.cuda.synchronize()
    ms_e2e = e0.elapsed_time(e1)
    ms_e2e, e2e_iters_all = reduce_over_ranks(dist, ms_e2e, e2e_iters, arch.device)
    e2e_value = bytes_per_iter * e2e_iters_all / (ms_e2e * 1e-3) / 1e9

    # roofline: the fused FP32 PT kernel timed alone (public ping-pong entry, no bc), CUDA events
    # on the launching stream, algorithmic bytes per launch over the mean launch time
    g = pb.grid
    da, db, _keep = fused_kernel_fields(arch, pb)
    gd = g.desc()
    reps = 200
    arch.call("cg_stokes_pt_iterations_pp", ctypes.byref(gd), ctypes.byref(da), ctypes.byref(db), ctypes.byref(pb.params), None, 20)
    torch.cuda.synchronize()
    k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    k0.record(stream)
    arch.call("cg_stokes_pt_iterations_pp", ctypes.byref(gd), ctypes.byref(da), ctypes.byref(db), ctypes.byref(pb.params), None, reps)
    k1.record(stream)
    torch.cuda.synchronize()
    fused_ms = k0.elapsed_time(k1) / reps
    fused_bytes = FUSED_ARRAYS * n * n * 4
    achieved = fused_bytes / (fused_ms * 1e-3) / 1e9
    peak, peak_kind = measured_peaks()
    traffic = committed_traffic(f"march2d_f32_{n}")

    # the 3D fused kernel on the 3D random-viscosity problem at 256^3, timed alone the same way
    stokes3d = None
    if not args.skip_3d:
        from chmy_gb300.configs import stokes3d_grf

        n3 = 256
        pb3 = stokes3d_grf(n3, dtype=np.float32)
        d3a, d3b, keep3 = fused3d_kernel_fields(arch, pb3)
        g3 = pb3.grid.desc()
        arch.call("cg_stokes_pt_iterations_pp", ctypes.byref(g3), ctypes.byref(d3a), ctypes.byref(d3b), ctypes.byref(pb3.params), None, 4)
        torch.cuda.synchronize()
        reps3 = 50
        k0.record(stream)
        arch.call("cg_stokes_pt_iterations_pp", ctypes.byref(g3), ctypes.byref(d3a), ctypes.byref(d3b), ctypes.byref(pb3.params), None, reps3)
        k1.record(stream)
        torch.cuda.synchronize()
        ms3 = k0.elapsed_time(k1) / reps3
        b3 = FUSED3_ARRAYS * n3**3 * 4
        stokes3d = {
            "workload": "3D VE Stokes 256^3, log-viscosity Gaussian random field (correlation length 0.1, std 1, seed 4), FP32 fused PT iteration",
            "kernel": "fused 3D PT iteration, the autotuner's choice of march3d_tma_kernel (inputs staged by TMA) and march3d_kernel",
            "kernel_ms": ms3,
            "algorithmic_bytes_per_launch": b3,
            "t_eff_gbs": b3 / (ms3 * 1e-3) / 1e9,
            "frac": b3 / (ms3 * 1e-3) / 1e9 / peak,
            "traffic": committed_traffic(f"march3d_f32_{n3}"),
        }
        del keep3, d3a, d3b
        torch.cuda.empty_cache()

    suite = None if args.skip_suite else config_suite(arch, stream, peak, fp64=not args.skip_fp64)

    # plain FP64 GPU solve of the same problem, once (time_to_solution comparison)
    fp64 = None
    err_vs_fp64 = None
    if not args.skip_fp64:
        dc_state = snapshot_state(solver)  # the last timed FP32-DC solve's converged state
        reset_device()
        r64 = solver.solve(precision=_abi.CG_F64)
        err_vs_fp64 = state_difference(dc_state, snapshot_state(solver), 2)
        fpk = ctypes.c_double()
        arch.call("cg_fp64_peak", ctypes.byref(fpk))
        fp64 = {"s": r64.seconds, "iterations": r64.iterations, "converged": r64.converged, "err": [r64.err[i] for i in range(3)],
                "t_eff_gbs": A64 * n * n * 8 * r64.iterations / r64.seconds / 1e9,
                "fp64_roofline": fp64_roofline("stokes_pt_iteration_2d", (n + 2) ** 2, r64.iterations, r64.seconds, fpk.value)}
    dc_s = np.array([r.seconds for r in results])
    tts = {
        "fp32_dc_s": float(np.median(dc_s)),
        "fp32_dc_iterations": int(np.median([r.iterations for r in results])),
        "fp32_dc_outer_cycles": int(np.median([r.outer for r in results])),
        "fp32_dc_err": [results[-1].err[i] for i in range(3)] + [results[-1].err_tau],
    }
    if fp64:
        tts.update({"fp64_s": fp64["s"], "fp64_iterations": fp64["iterations"], "fp64_err": fp64["err"],
                    "fp64_t_eff_gbs": fp64["t_eff_gbs"], "fp64_roofline": fp64["fp64_roofline"],
                    "speedup_fp32dc_vs_fp64": fp64["s"] / tts["fp32_dc_s"],
                    "err_vs_fp64": err_vs_fp64})

    if rank == 0:
        cpu_teff, cpu_it, cpu_s, cpu_threads = cpu_sample(n, seconds=args.cpu_seconds, max_iters=args.ref_iters)
        if tts.get("fp64_iterations"):
            tts["cpu_fp64_s_extrapolated"] = cpu_s / max(cpu_it, 1) * tts["fp64_iterations"]
            tts["speedup_vs_cpu_fp64"] = tts["cpu_fp64_s_extrapolated"] / tts["fp32_dc_s"]
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
            "dtype": "f32 PT + f64 defect correction",
            "data": "synthetic (seeded inclusions)",
            "config": {
                "workload": workload_name(n),
                "n": n,
                "eps": pb.eps,
                "ncheck": pb.ncheck,
                "re_m": "4 pi",
                "pt_constants": "examples/stokes_2d_inc_ve_T.jl:86-93 formulas with re_m = 4 pi (the example's 2.3 pi "
                "takes more iterations on this inclusion problem) and a check every n/4 iterations (the example: 2 nx); "
                "the reference's own constants are checked against the oracle in tests/test_gpu_solve.py",
                "arrays_per_iteration": A32,
                "l2": "working set larger than L2 (no flush)",
                "step": "one PT solve from the initial state to 1e-8",
            },
            "time_to_solution": tts,
            "time_to_solution_s": tts["fp32_dc_s"],
            "e2e": {"value": e2e_value, "unit": "GB/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "steps": e2e_steps},
            "gpu_launches": launches,
            "roofline": {
                "bound": "hbm",
                "kernel": "march2d_kernel<float> (update_stress! + update_velocity!, one launch per PT iteration)",
                "achieved": achieved,
                "peak": peak,
                "unit": "GB/s",
                "frac": achieved / peak,
                "peak_kind": f"{peak_kind} hbm_gbs",
                "traffic": traffic,
                "kernel_ms": fused_ms,
                "algorithmic_bytes_per_launch": fused_bytes,
            },
            "stokes3d": stokes3d,
            "configs": suite,
            "cpu_baseline": {
                "value": cpu_teff,
                "unit": "GB/s",
                "cores": cpu_threads,
                "kind": "port",
                "sample": f"{cpu_it} FP64 PT iterations of {n}^2 in {cpu_s:.1f} s (C++ restatement, OpenMP); "
                f"extrapolated FP64 time to solution {((tts.get('fp64_iterations') or 0) / max(cpu_it / cpu_s, 1e-9)):.0f} s",
            },
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    arch.close()


def snapshot_state(solver):
    """Device copies of a solver's V, tau and P (for solution comparisons outside timed regions)."""
    return {
        "V": [f.data.clone() for f in solver.fields["V"]],
        "tau": [f.data.clone() for f in solver.fields["tau"]],
        "P": solver.fields["P"].data.clone(),
    }


def state_difference(a, b, nd):
    """Max relative difference of two converged states per quantity: max|a - b| / max|b| over the
    interior for every V and tau component, and for P after subtracting each state's interior
    mean (normal velocity is prescribed on every side, so P is defined up to a constant)."""
    sl = (slice(2, -2),) * nd
    out = {}
    for name in ("V", "tau"):
        for k, (x, y) in enumerate(zip(a[name], b[name])):
            xi, yi = x[sl].double(), y[sl].double()
            out[f"{name}{k}"] = float((xi - yi).abs().max() / yi.abs().max().clamp_min(1e-300))
    pa, pb_ = a["P"][sl].double(), b["P"][sl].double()
    pa, pb_ = pa - pa.mean(), pb_ - pb_.mean()
    out["P_minus_mean"] = float((pa - pb_).abs().max() / pb_.abs().max().clamp_min(1e-300))
    out["max"] = max(out.values())
    return out


def _timed(fn, stream, reps=1):
    """CUDA-event time (ms) of `reps` calls of fn on `stream`, after one untimed call (which
    captures the call's CUDA graph)."""
    import torch

    fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for _ in range(reps):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def config_suite(arch, stream, peak, fp64=True):
    """The other configurations' hot loops, each timed with CUDA events on synthetic inputs of
    the configuration's shape: explicit diffusion 1024^2 (2000 steps), PT variable diffusion
    512^3 (a bounded sample of PT iterations, FP64 and FP32) and the SIA ensemble (64 members,
    1000 steps). T_eff counts the minimum unique traffic of one unit (step or PT iteration)."""
    import torch

    from chmy_gb300 import Field, _abi
    from chmy_gb300.bcs import Dirichlet, Neumann, to_cg_bc
    from chmy_gb300.configs import padded_mesh, ptdiff_params, sia_ensemble
    from chmy_gb300.grids import Center, UniformGrid, Vertex

    out = {}
    Cl, Vl = Center(), Vertex()
    fpk = ctypes.c_double()
    arch.call("cg_fp64_peak", ctypes.byref(fpk))
    fp64_peak = fpk.value
    out["fp64_peak_tflops"] = fp64_peak / 1e12

    # 2D explicit diffusion, FP64, 1024^2 over [-1, 1]^2, D = 1, dt = h^2/(4.1 D)
    n1 = 1024
    g1 = UniformGrid(origin=(-1.0, -1.0), extent=(2.0, 2.0), dims=(n1, n1), dtype=np.float64)
    x, y = padded_mesh(g1, Cl)
    C0 = np.exp(-(x * x + y * y) / 0.02) + np.random.default_rng(1).uniform(0.0, 1e-3, x.shape)
    A, B = Field(arch, g1, Cl, np.float64), Field(arch, g1, Cl, np.float64)
    A.from_numpy(C0)
    B.from_numpy(C0)
    bc1 = to_cg_bc(2, Neumann())
    h = float(g1.spacing()[0])
    dt1, steps1 = h * h / 4.1, 2000
    gd1 = g1.desc()
    ms1 = _timed(lambda: arch.call("cg_diffusion_run", ctypes.byref(gd1), ctypes.byref(A.desc()), ctypes.byref(B.desc()),
                                   1.0, dt1, ctypes.byref(bc1), steps1), stream)
    cells1 = n1 * n1
    out["diffusion2d"] = {
        "workload": "2D explicit diffusion 1024^2, FP64, Neumann, 2000 steps (fused flux + update + bc!, one launch per step)",
        "ms_per_run": ms1,
        "us_per_step": 1e3 * ms1 / steps1,
        "t_eff_gbs": 2 * cells1 * 8 * steps1 / (ms1 * 1e-3) / 1e9,
        "t_eff_gbs_7_arrays": 7 * cells1 * 8 * steps1 / (ms1 * 1e-3) / 1e9,
        "bytes": "2 arrays x n^2 x 8 B per step (read C, write C'); the reference's 7-array convention beside it",
        "l2": "L2-resident (2 x 8.4 MB): HBM fraction not meaningful",
        "fp64_roofline": fp64_roofline("diffusion_step_2d", (n1 + 2) ** 2, steps1, ms1 * 1e-3, fp64_peak),
    }
    del A, B

    # the same loop's gradient: dJ/dchi and dJ/dC0 of J = 1/2 |C^N|^2, host arrays in and out
    from chmy_gb300.adjoint import ExplicitDiffusion

    ed = ExplicitDiffusion(arch, g1, 1.0, dt1, bc1)

    def wall(fn):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = fn()
        torch.cuda.synchronize()
        return time.perf_counter() - t0, r

    wall(lambda: ed.run(C0, 8))
    wall(lambda: ed.gradient(C0, 8, lambda c: c))
    tf, _ = wall(lambda: ed.run(C0, steps1))
    tg, (gchi, _, _) = wall(lambda: ed.gradient(C0, steps1, lambda c: c))
    out["diffusion2d_adjoint"] = {
        "workload": "gradient of 1/2 |C^N|^2 over the 2000-step 1024^2 FP64 loop w.r.t. chi and C0 (taped forward, one reverse sweep), host arrays in and out",
        "forward_ms": tf * 1e3,
        "gradient_ms": tg * 1e3,
        "ratio": tg / tf,
        "tape_gb": ed.tape_bytes(steps1) / 1e9,
        "finite": bool(np.isfinite(gchi)),
    }
    del ed

    # the fused thermal step (advection-diffusion of T by V) and its vector-Jacobian product,
    # 2048^2 FP64, Neumann T, smooth random V
    from chmy_gb300.kernels import stokes_fields, stokes_params

    nt = 2048
    gt = UniformGrid(origin=(-1.0, -1.0), extent=(2.0, 2.0), dims=(nt, nt), dtype=np.float64)
    xt, yt = padded_mesh(gt, Cl)
    Tf = Field(arch, gt, Cl, np.float64)
    Tf.from_numpy(np.exp(-(xt * xt + yt * yt) / 0.05))
    To = Field(arch, gt, Cl, np.float64)
    To.from_numpy(np.exp(-(xt * xt + yt * yt) / 0.05))
    Vt = [Field(arch, gt, (Vl, Cl), np.float64), Field(arch, gt, (Cl, Vl), np.float64)]
    for d, v in enumerate(Vt):
        xv, yv = padded_mesh(gt, v.loc)
        v.from_numpy(np.sin(np.pi * (xv + 0.3 * d)) * np.cos(np.pi * yv))
    del xt, yt
    Tout = Field(arch, gt, Cl, np.float64)
    mu = Field(arch, gt, Cl, np.float64)
    mu.from_numpy(np.ones(Tout.data.shape))
    gTt, gTo = Field(arch, gt, Cl, np.float64), Field(arch, gt, Cl, np.float64)
    gVt = [Field(arch, gt, v.loc, np.float64) for v in Vt]
    ft = stokes_fields(V=Vt, T=Tf, T_old=To)
    pt = stokes_params(G=1.0, dt=1e-4, lambda_rhoCp=0.3)
    bct = to_cg_bc(2, Neumann())
    gdt = gt.desc()
    gVa = (_abi.cg_field * 3)(gVt[0].desc(), gVt[1].desc(), _abi.cg_field())
    reps = 50
    msf = _timed(lambda: arch.call("cg_stokes_thermal_step", ctypes.byref(gdt), ctypes.byref(ft), ctypes.byref(pt), ctypes.byref(bct),
                                   ctypes.byref(Tout.desc())), stream, reps)
    msa = _timed(lambda: arch.call("cg_stokes_thermal_step_adjoint", ctypes.byref(gdt), ctypes.byref(ft), ctypes.byref(pt),
                                   ctypes.byref(bct), ctypes.byref(mu.desc()), ctypes.byref(gTt.desc()), ctypes.byref(gTo.desc()),
                                   gVa, None), stream, reps)
    out["thermal_step_adjoint"] = {
        "workload": "fused thermal step (update_thermal_flux! + update_thermal!) at 2048^2 FP64 and its vector-Jacobian product "
                    "(dJ/dT, dJ/dT_old, dJ/dV; dJ/dlambda left out: it synchronises)",
        "forward_us": msf * 1e3,
        "adjoint_us": msa * 1e3,
        "ratio": msa / msf,
        "forward_t_eff_gbs": 5 * nt * nt * 8 / (msf * 1e-3) / 1e9,
        "adjoint_t_eff_gbs": 8 * nt * nt * 8 / (msa * 1e-3) / 1e9,
        "bytes": "forward: read T, T_old, V x2, write T (5 arrays); adjoint: read T, V x2, mu, write gT, gT_old, gV x2 (8 arrays)",
    }
    del Tf, To, Vt, Tout, mu, gTt, gTo, gVt

    # 3D PT variable diffusion at 512^3, a sample of PT iterations of one step
    n2, npt = 512, 100
    g2 = UniformGrid(origin=(-0.5,) * 3, extent=(1.0,) * 3, dims=(n2,) * 3, dtype=np.float64)
    rng = np.random.default_rng(2)
    gn = rng.standard_normal((n2 + 4,) * 3, dtype=np.float32)
    for _ in range(5):
        for ax in range(3):
            gn = (np.roll(gn, 1, ax) + gn + np.roll(gn, -1, ax)) / np.float32(3)
    D = np.exp(gn)
    del gn
    xs = padded_mesh(g2, Cl)
    Cb = np.exp(-(xs[0] * xs[0] + xs[1] * xs[1] + xs[2] * xs[2]) / 0.01)
    del xs
    bc2 = to_cg_bc(3, {"x": Dirichlet(0.0), "y": Neumann(), "z": Neumann()})
    p2 = ptdiff_params(g2, 1e-3, float(D.max()))
    gd2 = g2.desc()
    cfg2 = {}
    for T, name in ((np.float64, "fp64"), (np.float32, "fp32")):
        # FP32: one row pitch and plane height for every array (the fused single-pass kernel)
        lay = dict(pitch_align=128, plane_rows=n2 + 5, align_index=0) if T == np.float32 else {}
        fs = {k: Field(arch, g2, Cl, T, **lay) for k in ("C", "C_old", "D")}
        q = [Field(arch, g2, tuple(Vl if e == d else Cl for e in range(3)), T, **lay) for d in range(3)]
        fs["C"].from_numpy(Cb.astype(T))
        fs["D"].from_numpy(D.astype(T))
        f = _abi.cg_ptdiff_fields()
        f.C, f.C_old, f.D = fs["C"].desc(), fs["C_old"].desc(), fs["D"].desc()
        f.q = (_abi.cg_field * 3)(*[qq.desc() for qq in q])
        ms2 = _timed(lambda: arch.call("cg_ptdiff_run", ctypes.byref(gd2), ctypes.byref(f), ctypes.byref(p2), ctypes.byref(bc2), 1, npt),
                     stream)
        sz = np.dtype(T).itemsize
        teff = 10 * n2**3 * sz * npt / (ms2 * 1e-3) / 1e9
        cfg2[name] = {"ms_per_iteration": ms2 / npt, "t_eff_gbs": teff, "frac": teff / peak}
        if T == np.float64:
            cfg2[name]["fp64_roofline"] = fp64_roofline("ptdiff_pt_iteration_3d", (n2 + 2) ** 3, npt, ms2 * 1e-3, fp64_peak)
        del fs, q, f
        torch.cuda.empty_cache()
    # one implicit step: 500 FP64 PT iterations (the configuration's step), then the FP32 PT
    # solve inside FP64 defect correction to the residual those 500 iterations reach
    fs = {k: Field(arch, g2, Cl, np.float64) for k in ("C", "C_old", "D")}
    q = [Field(arch, g2, tuple(Vl if e == d else Cl for e in range(3)), np.float64) for d in range(3)]
    fs["D"].from_numpy(D.astype(np.float64))
    f = _abi.cg_ptdiff_fields()
    f.C, f.C_old, f.D = fs["C"].desc(), fs["C_old"].desc(), fs["D"].desc()
    f.q = (_abi.cg_field * 3)(*[qq.desc() for qq in q])

    def reset():
        fs["C"].from_numpy(Cb)
        arch.call("cg_bc_apply", ctypes.byref(gd2), 1, ctypes.byref(fs["C"].desc()), ctypes.byref(bc2))
        fs["C_old"].data.copy_(fs["C"].data)
        for qq in q:
            qq.data.zero_()

    def solve(prec, eps, max_iter, ncheck):
        # inner_rtol 1e-3: the FP32 measure of the correction bottoms out near 1e-5 of the
        # outer error here (eps_32 D dt / h^2 ~ 260 eps_32)
        o = _abi.cg_solve_opts()
        o.max_iter, o.ncheck, o.eps, o.precision, o.max_outer, o.inner_rtol = max_iter, ncheck, eps, prec, 20, 1e-3
        r = _abi.cg_solve_result()
        rc = arch.lib.cg_ptdiff_solve(arch.ctx, ctypes.byref(gd2), ctypes.byref(f), ctypes.byref(p2), ctypes.byref(bc2),
                                      ctypes.byref(o), ctypes.byref(r))
        if rc not in (0, _abi.CG_ERR_NOCONV):
            raise RuntimeError(f"cg_ptdiff_solve: {arch.lib.cg_last_error(arch.ctx)}")
        return r

    reset()
    r64 = solve(_abi.CG_F64, 1e-300, 500, 500)  # exactly 500 iterations, then the step's residual
    target = float(r64.err[0])
    times = []
    for _ in range(2):  # the first call captures the correction loop's graph and tunes its kernel
        reset()
        rdc = solve(_abi.CG_F32, target, 100000, 100)
        times.append(rdc.seconds)
    fp64_step_s = cfg2["fp64"]["ms_per_iteration"] * 500 * 1e-3
    # the configuration's 20 implicit steps (C_old <- C before each), every step solved by the
    # refined form to the residual 500 FP64 PT iterations reach in the first step; the FP64 run
    # of 20 x 500 iterations costs 20 times its measured step (its iteration count is fixed)
    import time as _time

    reset()
    torch.cuda.synchronize()
    t0 = _time.perf_counter()
    run_iters, run_cycles, run_err = 0, 0, 0.0
    for _ in range(20):
        fs["C_old"].data.copy_(fs["C"].data)
        rs = solve(_abi.CG_F32, target, 100000, 100)
        run_iters += int(rs.iterations)
        run_cycles += int(rs.outer)
        run_err = max(run_err, float(rs.err[0]))
    torch.cuda.synchronize()
    run_s = _time.perf_counter() - t0
    del fs, q, f, D, Cb
    torch.cuda.empty_cache()
    out["ptdiff3d"] = {
        "workload": f"3D PT variable diffusion 512^3, D = exp(box-smoothed Gaussian noise), Dirichlet x / Neumann y z; "
        f"per-iteration rates from one step of {npt} PT iterations; the step comparison solves one implicit step",
        "bytes": "10 arrays x n^3 x sizeof(T) per PT iteration (read/write C, q x3; read C_old, D)",
        **cfg2,
        "step": {
            "fp64_500_iterations": {"s": fp64_step_s, "err": target},
            "fp32_defect_correction": {"s": times[-1], "err": float(rdc.err[0]), "fp32_iterations": int(rdc.iterations),
                                       "fp64_cycles": int(rdc.outer), "converged": int(rdc.converged)},
            "speedup": fp64_step_s / times[-1],
            "err": "max |R| dt over the interior, R = -(C - C_old)/dt - divg(-lerp(D) grad C)",
        },
        "run_20_steps": {
            "fp32_defect_correction_s": run_s,
            "fp32_iterations": run_iters,
            "fp64_cycles": run_cycles,
            "max_err": run_err,
            "target": target,
            "fp64_20x500_s": 20 * fp64_step_s,
            "fp64_kind": "20 x the measured 500-iteration FP64 step",
            "speedup": 20 * fp64_step_s / run_s,
        },
    }

    # SIA ensemble, 64 members of 128^2..1024^2, FP64, 1000 steps in one batched run
    ens = sia_ensemble(members=64)
    keep, mem = [], (_abi.cg_sia_member * len(ens))()
    params = (_abi.cg_sia_params * len(ens))()
    cells5 = 0
    for k, (grid, hh, p) in enumerate(ens):
        H = Field(arch, grid, Cl, np.float64)
        Bf = Field(arch, grid, Cl, np.float64)
        H.from_numpy(hh["H"])
        Bf.from_numpy(hh["B"])
        qq = [Field(arch, grid, (Vl, Cl), np.float64), Field(arch, grid, (Cl, Vl), np.float64)]
        keep.append((H, Bf, qq))
        mem[k].grid = grid.desc()
        mem[k].H, mem[k].B = H.desc(), Bf.desc()
        mem[k].q[0], mem[k].q[1] = qq[0].desc(), qq[1].desc()
        params[k] = p
        cells5 += grid.dims[0] * grid.dims[1]
    ts = (ctypes.c_double * len(ens))()
    steps5 = 1000
    ms5 = _timed(lambda: arch.call("cg_sia_ensemble_run", len(ens), mem, params, steps5, ts), stream)
    teff5 = 3 * cells5 * 8 * steps5 / (ms5 * 1e-3) / 1e9
    out["sia_ensemble"] = {
        "workload": "SIA ensemble: 64 members of 128^2..1024^2 (seed 6), flux -Gamma H^5 |grad S|^2 grad S, ELA mass balance, FP64, 1000 steps, one batched run",
        "cells": cells5,
        "ms_per_run": ms5,
        "t_eff_gbs": teff5,
        "frac": teff5 / peak,
        "bytes": "3 arrays x cells x 8 B per step (read H, B; write H')",
        "fp64_roofline": fp64_roofline("sia_ensemble_step", cells5, steps5, ms5 * 1e-3, fp64_peak),
    }
    del keep
    torch.cuda.empty_cache()
    out["sia_adjoint"] = sia_adjoint_cost(arch)
    torch.cuda.empty_cache()
    out["stokes3d_adjoint"] = stokes3d_adjoint_cost(arch, fp64=fp64)
    torch.cuda.empty_cache()
    out["sia_ensemble_adjoint"] = sia_ensemble_adjoint_cost(arch)
    torch.cuda.empty_cache()
    return out


def sia_ensemble_adjoint_cost(arch, members=64, nsteps=1000):
    """The SIA ensemble configuration's gradient: per member, dJ/dGamma, dJ/dela and dJ/dH0 of
    J_m = 1/2 |H_m^N|^2 over the interior, for 64 members of 128^2..1024^2 (seed 6, FP64) over
    1000 steps, all members in each launch (SIAEnsemble: taped segments as large as half the free
    device memory holds, re-run from checkpoints). Wall clock from host arrays to host arrays,
    against the ensemble's forward run timed the same way."""
    import time

    import torch

    from chmy_gb300.adjoint import SIAEnsemble
    from chmy_gb300.configs import sia_ensemble

    ens_cfg = sia_ensemble(members=members)
    H0s = []
    for grid, hh, p in ens_cfg:  # a dome of ice on every member, so that every member flows
        H0s.append(hh["H"] + np.clip(0.35 - 0.25 * _dome_r2(grid), 0.0, None))
    ens = SIAEnsemble(arch, [(g, hh["B"], p) for g, hh, p in ens_cfg])

    def dJ(m, h):
        g = np.zeros_like(h)
        g[2:-2, 2:-2] = h[2:-2, 2:-2]
        return g

    def wall(f):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = f()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) * 1e3, r

    ens.run(H0s, 2)
    fwd, _ = wall(lambda: ens.run(H0s, nsteps))
    grad, r = wall(lambda: ens.gradient(H0s, nsteps, dJ))
    per_step = ens.tape_bytes(1) - ens.tape_bytes(0)
    free, _ = torch.cuda.mem_get_info()
    cells = sum(g.dims[0] * g.dims[1] for g, _, _ in ens_cfg)
    out = {
        "workload": f"SIA ensemble gradient: {members} members of 128^2..1024^2 ({cells} cells), {nsteps} steps, FP64, all members per launch",
        "forward_ms": fwd,
        "gradient_ms": grad,
        "ratio": grad / fwd,
        "tape_gb_per_step": per_step / 1e9,
        "finite": bool(all(np.isfinite(v) for v in r[0] + r[1])),
    }
    del ens
    return out


def _dome_r2(grid):
    """x^2 + y^2 at the padded Center points of a 2D grid on [-1, 1]^2, as a [y, x] array."""
    from chmy_gb300.configs import padded_mesh
    from chmy_gb300.grids import Center

    x, y = padded_mesh(grid, Center())
    return x * x + y * y


def stokes3d_adjoint_cost(arch, n=256, fp64=True):
    """The 3D VE Stokes configuration (n^3, random log-viscosity field, buoyant sphere): the
    forward solve to residual 1e-8 and the adjoint solve for dJ/d log(eta) of a misfit of Vz on
    the middle vertex plane (scaled so that max |dJ/dV| = 1), both in FP32 PT iterations inside
    FP64 defect correction. With `fp64`, the same forward and adjoint solves in plain FP64 PT
    (the configuration's precision) beside them: their times, and the FP32-DC results' errors
    against them. Wall clock around synchronised calls."""
    import time

    import torch

    from chmy_gb300 import _abi
    from chmy_gb300.configs import stokes3d_grf
    from chmy_gb300.solvers import StokesSolver

    pb = stokes3d_grf(n)
    sens = (n // 2 + 2, slice(2, n + 2), slice(2, n + 2))

    def run(precision):
        s = StokesSolver(arch, pb)
        s.apply_bc()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = s.solve(precision=precision)
        torch.cuda.synchronize()
        tf = time.perf_counter() - t0
        v = s.fields["V"][2].to_numpy()
        r = np.random.default_rng(3).standard_normal(v[sens].shape)
        dJ = np.zeros_like(v)
        dJ[sens] = r / np.abs(r).max()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        grad, ares = s.gradient_log_eta([None, None, dJ], precision=precision)
        torch.cuda.synchronize()
        ta = time.perf_counter() - t0
        state = snapshot_state(s)
        g = grad.data.clone()
        del s, grad
        torch.cuda.empty_cache()
        return res, tf, ares, ta, state, g

    res, tf, ares, ta, st_dc, g_dc = run(_abi.CG_F32)
    out = {
        "workload": f"3D VE Stokes {n}^3, log-viscosity Gaussian random field, forward solve and adjoint solve for dJ/d log(eta), FP32 PT in FP64 defect correction, residual 1e-8",
        "misfit": "1/2 |Vz - Vz_obs|^2 on the middle vertex plane z = n/2 (Vz on the top plane is a Dirichlet value, "
        "so its misfit has no sensitivity); Vz_obs - Vz = seeded normal noise scaled to max 1",
        "forward_s": tf,
        "forward_iterations": int(res.iterations),
        "forward_converged": int(res.converged),
        "adjoint_s": ta,
        "adjoint_iterations": int(ares.iterations),
        "adjoint_converged": int(ares.converged),
        "gradient_over_forward": (tf + ta) / tf,
    }
    if fp64:
        r64, tf64, a64, ta64, st64, g64 = run(_abi.CG_F64)
        sl = (slice(2, -2),) * 3
        gd, gr = g_dc[sl], g64[sl]
        out["fp64"] = {
            "forward_s": tf64,
            "forward_iterations": int(r64.iterations),
            "forward_converged": int(r64.converged),
            "adjoint_s": ta64,
            "adjoint_iterations": int(a64.iterations),
            "adjoint_converged": int(a64.converged),
            "speedup_fp32dc_forward": tf64 / tf,
            "speedup_fp32dc_gradient": (tf64 + ta64) / (tf + ta),
            "err_vs_fp64_forward": state_difference(st_dc, st64, 3),
            "err_vs_fp64_gradient": float((gd - gr).abs().max() / gr.abs().max().clamp_min(1e-300)),
        }
    return out


def sia_adjoint_cost(arch, n=1024, nsteps=1000):
    """Cost of the SIA gradient (dJ/dGamma, dJ/dela, dJ/dH0 of J = 1/2 |H^N|^2) over the
    forward run, on the largest member size of the ensemble configuration: n^2 cells, nsteps
    steps, FP64, from host arrays to host arrays. The taped reverse sweep (one segment when
    the tape fits half the free device memory) and the recomputing sweep with sqrt(N)
    checkpoints. Wall clock around synchronised calls, after one untimed run of each."""
    import math
    import time

    import torch

    from chmy_gb300 import _abi
    from chmy_gb300.adjoint import SIA
    from chmy_gb300.configs import gaussian_random_field, padded_mesh
    from chmy_gb300.grids import Center, UniformGrid

    T = np.float64
    grid = UniformGrid(origin=(T(-1), T(-1)), extent=(T(2), T(2)), dims=(n, n), dtype=T)
    x, y = padded_mesh(grid, Center())
    bed = 0.4 + 0.3 * gaussian_random_field(x.shape, 0.25, 2.0 / n, 7)
    H0 = np.clip(0.35 - 0.25 * (x * x + y * y), 0.0, None)
    p = _abi.cg_sia_params()
    p.Gamma, p.As, p.n, p.beta, p.ela, p.m_max, p.dt_max, p.cfl = 1.0, 0.0, 3, 0.5, 0.55, 0.25, 0.5, 4.1
    sia = SIA(arch, grid, bed, p)

    def dJ(h):
        return np.where(np.isfinite(h), h, 0.0)

    def wall(f):
        f()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        f()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) * 1e3

    fwd = wall(lambda: sia.run(H0, nsteps))
    taped = wall(lambda: sia.gradient(H0, nsteps, dJ))
    K = int(math.ceil(math.sqrt(nsteps)))
    recomp = wall(lambda: sia.gradient(H0, nsteps, dJ, tape=False, checkpoint_every=K))
    tape_gb = sia.tape_bytes(nsteps) / 1e9
    del sia
    return {
        "workload": f"SIA gradient w.r.t. Gamma, ela and H0: {n}^2 cells, {nsteps} steps, FP64, host arrays in and out",
        "forward_ms": fwd,
        "gradient_taped_ms": taped,
        "ratio_taped": taped / fwd,
        "tape_gb": tape_gb,
        "gradient_recomputing_ms": recomp,
        "ratio_recomputing": recomp / fwd,
        "recomputing_checkpoint_every": K,
    }


def fused_kernel_fields(arch, pb):
    """FP32 ping-pong field sets of the fused 2D PT kernel on the problem's grid (V from the
    initial state, 1/eta from eta, zero tau/P/tau_old/rho_g)."""
    import torch

    from chmy_gb300 import Field
    from chmy_gb300.grids import Center, Vertex
    from chmy_gb300.kernels import stokes_fields

    g = pb.grid
    Cl, Vl = Center(), Vertex()

    def f32(loc):
        # 128-byte row pitch: every array shares one row stride, as in the solver's work pool
        return Field(arch, g, loc, np.float32, pitch_align=128)

    A = dict(V=[f32((Vl, Cl)), f32((Cl, Vl))], P=f32(Cl), tau=[f32(Cl), f32(Cl), f32(Vl)])
    B = dict(V=[f32((Vl, Cl)), f32((Cl, Vl))], P=f32(Cl), tau=[f32(Cl), f32(Cl), f32(Vl)])
    extra = dict(tau_old=[f32(Cl), f32(Cl), f32(Vl)], inv_eta=f32(Cl), rho_g=[f32((Vl, Cl)), f32((Cl, Vl))])
    extra["inv_eta"].data.copy_(torch.from_numpy(1.0 / pb.host["eta"]).float())
    for lst in (A["V"], B["V"]):
        for f, a in zip(lst, pb.host["V"]):
            f.data.copy_(torch.from_numpy(a).float())
    keep = (A, B, extra)
    return stokes_fields(V=A["V"], P=A["P"], tau=A["tau"], **extra), stokes_fields(V=B["V"], P=B["P"], tau=B["tau"]), keep


def fused3d_kernel_fields(arch, pb, align_index=0):
    """FP32 ping-pong field sets of the fused 3D PT kernel on the problem's grid (1/eta from eta,
    rho_g from the problem, zero V/tau/P/tau_old). Every array shares its row and plane strides,
    as in the solver's work pool."""
    import torch

    from chmy_gb300 import Field
    from chmy_gb300.grids import Center, Vertex
    from chmy_gb300.kernels import stokes_fields

    g = pb.grid
    Cl, Vl = Center(), Vertex()
    rows = g.dims[1] + 5

    def f32(loc):
        # logical x index 0 of every row on a 128-byte boundary, as in the solver's 3D pool
        return Field(arch, g, loc, np.float32, pitch_align=128, plane_rows=rows, align_index=align_index)

    vl = [(Vl, Cl, Cl), (Cl, Vl, Cl), (Cl, Cl, Vl)]
    tl = [(Cl, Cl, Cl)] * 3 + [(Vl, Vl, Cl), (Vl, Cl, Vl), (Cl, Vl, Vl)]
    A = dict(V=[f32(l) for l in vl], P=f32(Cl), tau=[f32(l) for l in tl])
    B = dict(V=[f32(l) for l in vl], P=f32(Cl), tau=[f32(l) for l in tl])
    # buoyancy on the vertical component only, as in examples/stokes_3d_inc_ve_T.jl
    extra = dict(tau_old=[f32(l) for l in tl], inv_eta=f32(Cl), rho_g=[None, None, f32(vl[2])])
    extra["inv_eta"].data.copy_(torch.from_numpy(1.0 / pb.host["eta"]).float())
    extra["rho_g"][2].data.copy_(torch.from_numpy(pb.host["rho_g"][2]).float())
    keep = (A, B, extra)
    return stokes_fields(V=A["V"], P=A["P"], tau=A["tau"], **extra), stokes_fields(V=B["V"], P=B["P"], tau=B["tau"]), keep


def run_kernel_fp64(arch, args):
    """--kernel stokes64: `--reps` FP64 PT iterations of the 2D inclusion problem at n^2
    (cg_stokes_pt_iterations: stress_kernel, velocity_kernel and bc!(V) per iteration).
    --kernel ptdiff64: `--reps` FP64 PT-diffusion iterations at n^3 (ptdiff_q_kernel,
    ptdiff_C_kernel and bc!(C) per iteration). Timed with CUDA events after warm-up; the FP64
    FMA peak of the device (cg_fp64_peak) beside it."""
    import torch

    from chmy_gb300 import Field, _abi
    from chmy_gb300.bcs import Dirichlet, Neumann, to_cg_bc
    from chmy_gb300.configs import ptdiff_params, stokes2d_inclusions
    from chmy_gb300.grids import Center, UniformGrid, Vertex
    from chmy_gb300.solvers import StokesSolver

    n, reps = args.n, args.reps
    if args.kernel == "stokes64":
        s = StokesSolver(arch, stokes2d_inclusions(n))
        s.apply_bc()

        def run(k):
            s.iterate(k)
        cells = n * n
    else:
        T = np.float64
        g = UniformGrid(origin=(-0.5,) * 3, extent=(1.0,) * 3, dims=(n,) * 3, dtype=T)
        Cl, Vl = Center(), Vertex()
        rng = np.random.default_rng(2)
        fs = {k: Field(arch, g, Cl, T) for k in ("C", "C_old", "D")}
        q = [Field(arch, g, tuple(Vl if e == d else Cl for e in range(3)), T) for d in range(3)]
        fs["C"].from_numpy(rng.random(fs["C"].data.shape))
        D = np.exp(rng.uniform(-1, 1, fs["D"].data.shape))
        fs["D"].from_numpy(D)
        f = _abi.cg_ptdiff_fields()
        f.C, f.C_old, f.D = fs["C"].desc(), fs["C_old"].desc(), fs["D"].desc()
        f.q = (_abi.cg_field * 3)(*[qq.desc() for qq in q])
        p = ptdiff_params(g, 1e-3, float(D.max()))
        bc = to_cg_bc(3, {"x": Dirichlet(0.0), "y": Neumann(), "z": Neumann()})
        gd = g.desc()

        def run(k):
            arch.call("cg_ptdiff_run", ctypes.byref(gd), ctypes.byref(f), ctypes.byref(p), ctypes.byref(bc), 1, k)
        cells = n**3
    run(4)
    run(reps)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    run(reps)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    peak = ctypes.c_double()
    arch.call("cg_fp64_peak", ctypes.byref(peak))
    print(json.dumps({"kernel": args.kernel, "n": n, "cells": cells, "us_per_iteration": ms * 1e3,
                      "fp64_peak_tflops": peak.value / 1e12}))


def run_kernel_ptdiff(arch, args):
    """--kernel ptdiff3d: the fused FP32 PT-diffusion iteration on an n^3 grid (random C, q and
    D = exp(U[-1, 1]), Dirichlet x / Neumann y z), one step of `--reps` iterations timed with
    CUDA events."""
    import torch

    from chmy_gb300 import Field, _abi
    from chmy_gb300.bcs import Dirichlet, Neumann, to_cg_bc
    from chmy_gb300.configs import ptdiff_params
    from chmy_gb300.grids import Center, UniformGrid, Vertex

    n = args.n
    T = np.float32
    g = UniformGrid(origin=(-0.5,) * 3, extent=(1.0,) * 3, dims=(n,) * 3, dtype=T)
    Cl, Vl = Center(), Vertex()
    rng = np.random.default_rng(2)
    lay = dict(pitch_align=128, plane_rows=n + 5, align_index=0)
    fs = {k: Field(arch, g, Cl, T, **lay) for k in ("C", "C_old", "D")}
    q = [Field(arch, g, tuple(Vl if e == d else Cl for e in range(3)), T, **lay) for d in range(3)]
    fs["C"].from_numpy(rng.random(fs["C"].data.shape, dtype=T))
    D = np.exp(rng.uniform(-1, 1, fs["D"].data.shape)).astype(T)
    fs["D"].from_numpy(D)
    f = _abi.cg_ptdiff_fields()
    f.C, f.C_old, f.D = fs["C"].desc(), fs["C_old"].desc(), fs["D"].desc()
    f.q = (_abi.cg_field * 3)(*[qq.desc() for qq in q])
    p = ptdiff_params(g, 1e-3, float(D.max()))
    bc = to_cg_bc(3, {"x": Dirichlet(0.0), "y": Neumann(), "z": Neumann()})
    gd = g.desc()
    reps = args.reps

    def run(k):
        arch.call("cg_ptdiff_run", ctypes.byref(gd), ctypes.byref(f), ctypes.byref(p), ctypes.byref(bc), 1, k)

    run(4)
    run(reps)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    run(reps)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    byt = 10 * n**3 * 4
    print(json.dumps({"kernel": "ptd_march3d_kernel<float>", "n": n, "arrays": 10, "us_per_iteration": ms * 1e3,
                      "algorithmic_gbs": byt / (ms * 1e-3) / 1e9, "frac_of_measured_hbm": byt / (ms * 1e-3) / 1e9 / measured_peaks()[0]}))


def run_kernel_misc(arch, args):
    """--kernel sia_ensemble: `--members` members of the SIA ensemble (sizes --nmin..--nmax), `--reps`
    steps in one batched run. --kernel diffusion2d: the explicit diffusion step at n^2 (FP64,
    Neumann), `--reps` steps. Timed with CUDA events after one untimed run."""
    import torch

    from chmy_gb300 import Field, _abi
    from chmy_gb300.bcs import Neumann, to_cg_bc
    from chmy_gb300.configs import padded_mesh, sia_ensemble
    from chmy_gb300.grids import Center, UniformGrid, Vertex

    stream = torch.cuda.current_stream()
    Cl, Vl = Center(), Vertex()
    if args.kernel == "sia_ensemble":
        ens = sia_ensemble(members=args.members, nmin=args.nmin, nmax=args.nmax)
        keep, mem = [], (_abi.cg_sia_member * len(ens))()
        params = (_abi.cg_sia_params * len(ens))()
        cells = 0
        for k, (grid, hh, p) in enumerate(ens):
            H, Bf = Field(arch, grid, Cl, np.float64), Field(arch, grid, Cl, np.float64)
            H.from_numpy(hh["H"])
            Bf.from_numpy(hh["B"])
            qq = [Field(arch, grid, (Vl, Cl), np.float64), Field(arch, grid, (Cl, Vl), np.float64)]
            keep.append((H, Bf, qq))
            mem[k].grid = grid.desc()
            mem[k].H, mem[k].B = H.desc(), Bf.desc()
            mem[k].q[0], mem[k].q[1] = qq[0].desc(), qq[1].desc()
            params[k] = p
            cells += grid.dims[0] * grid.dims[1]
        ts = (ctypes.c_double * len(ens))()
        ms = _timed(lambda: arch.call("cg_sia_ensemble_run", len(ens), mem, params, args.reps, ts), stream)
        print(json.dumps({"kernel": "ens_D/q/H_kernel<double>", "members": len(ens), "cells": cells, "steps": args.reps,
                          "ms_per_step": ms / args.reps}))
        return
    n = args.n
    g = UniformGrid(origin=(-1.0, -1.0), extent=(2.0, 2.0), dims=(n, n), dtype=np.float64)
    x, y = padded_mesh(g, Cl)
    A, B = Field(arch, g, Cl, np.float64), Field(arch, g, Cl, np.float64)
    A.from_numpy(np.exp(-(x * x + y * y) / 0.02))
    B.from_numpy(np.exp(-(x * x + y * y) / 0.02))
    bc = to_cg_bc(2, Neumann())
    h = float(g.spacing()[0])
    gd = g.desc()
    ms = _timed(lambda: arch.call("cg_diffusion_run", ctypes.byref(gd), ctypes.byref(A.desc()), ctypes.byref(B.desc()), 1.0,
                                  h * h / 4.1, ctypes.byref(bc), args.reps), stream)
    print(json.dumps({"kernel": "diffusion_step_kernel<double,2>", "n": n, "steps": args.reps, "us_per_step": 1e3 * ms / args.reps}))


def run_kernel_sia_adjoint(arch, args):
    """--kernel sia_adjoint: the taped SIA gradient (dJ/dGamma, dJ/dela, dJ/dH0 of 1/2 |H^N|^2) on
    an n^2 grid over `--reps` steps, after one untimed run: the taped forward kernels and the
    reverse sweep's kernels, for launch lists and captures."""
    import time

    import torch

    from chmy_gb300 import _abi
    from chmy_gb300.adjoint import SIA
    from chmy_gb300.configs import gaussian_random_field, padded_mesh
    from chmy_gb300.grids import Center, UniformGrid

    n, nsteps = args.n, args.reps
    T = np.float64
    grid = UniformGrid(origin=(T(-1), T(-1)), extent=(T(2), T(2)), dims=(n, n), dtype=T)
    x, y = padded_mesh(grid, Center())
    bed = 0.4 + 0.3 * gaussian_random_field(x.shape, 0.25, 2.0 / n, 7)
    H0 = np.clip(0.35 - 0.25 * (x * x + y * y), 0.0, None)
    p = _abi.cg_sia_params()
    p.Gamma, p.As, p.n, p.beta, p.ela, p.m_max, p.dt_max, p.cfl = 1.0, 0.0, 3, 0.5, 0.55, 0.25, 0.5, 4.1
    sia = SIA(arch, grid, bed, p)

    def dJ(h):
        return np.where(np.isfinite(h), h, 0.0)

    sia.gradient(H0, nsteps, dJ)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sia.run(H0, nsteps)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    sia.gradient(H0, nsteps, dJ)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    print(json.dumps({"kernel": "SIA gradient (taped)", "n": n, "steps": nsteps, "forward_ms": (t1 - t0) * 1e3,
                      "gradient_ms": (t2 - t1) * 1e3, "ratio": (t2 - t1) / (t1 - t0)}))


def run_kernel_stokes3d_dc(arch, args):
    """--kernel stokes3d_dc: one forward solve of the 3D VE Stokes configuration at n^3 (random
    log-viscosity field, buoyant sphere, free slip) to residual 1e-8, FP32 PT inside FP64 defect
    correction; wall clock around the synchronised call, and the time per PT iteration."""
    import time

    import torch

    from chmy_gb300 import _abi
    from chmy_gb300.configs import stokes3d_grf
    from chmy_gb300.solvers import StokesSolver

    pb = stokes3d_grf(args.n)
    s = StokesSolver(arch, pb)
    s.apply_bc()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = s.solve(precision=_abi.CG_F32)
    torch.cuda.synchronize()
    t = time.perf_counter() - t0
    print(json.dumps({"kernel": "stokes3d_dc", "n": args.n, "converged": int(res.converged), "iterations": int(res.iterations),
                      "outer": int(res.outer), "s": t, "us_per_iteration": 1e6 * t / max(int(res.iterations), 1)}))


def run_kernel(args):
    """--kernel fused2d | fused3d: only the fused FP32 PT kernel (2D inclusions n^2, or 3D random
    viscosity n^3), `--reps` launches timed with CUDA events (the command the committed ncu
    summaries were captured with)."""
    import torch

    from chmy_gb300 import Arch, GB300Backend
    from chmy_gb300.configs import stokes2d_inclusions, stokes3d_grf

    arch = Arch(GB300Backend())
    if args.kernel == "ptdiff3d":
        run_kernel_ptdiff(arch, args)
        arch.close()
        return
    if args.kernel in ("stokes64", "ptdiff64"):
        run_kernel_fp64(arch, args)
        arch.close()
        return
    if args.kernel in ("sia_ensemble", "diffusion2d"):
        run_kernel_misc(arch, args)
        arch.close()
        return
    if args.kernel == "sia_adjoint":
        run_kernel_sia_adjoint(arch, args)
        arch.close()
        return
    if args.kernel == "stokes3d_dc":
        run_kernel_stokes3d_dc(arch, args)
        arch.close()
        return
    if args.kernel == "fused3d":
        pb = stokes3d_grf(args.n, dtype=np.float32)
        da, db, keep = fused3d_kernel_fields(arch, pb, args.align_index)
        name, arrays, cells = "fused 3D PT iteration (autotuner's choice)", FUSED3_ARRAYS, args.n**3
    else:
        pb = stokes2d_inclusions(args.n)
        da, db, keep = fused_kernel_fields(arch, pb)
        name, arrays, cells = "march2d_kernel<float>", FUSED_ARRAYS, args.n**2
    gd = pb.grid.desc()
    reps = args.reps + (args.reps & 1)

    def run(k):
        arch.call("cg_stokes_pt_iterations_pp", ctypes.byref(gd), ctypes.byref(da), ctypes.byref(db), ctypes.byref(pb.params), None, k)

    run(4)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(0) as clk:
        e0.record()
        run(reps)
        e1.record()
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    byt = arrays * cells * 4
    print(json.dumps({"kernel": name, "n": args.n, "arrays": arrays, "us_per_launch": ms * 1e3,
                      "algorithmic_gbs": byt / (ms * 1e-3) / 1e9, "frac_of_measured_hbm": byt / (ms * 1e-3) / 1e9 / measured_peaks()[0],
                      "clocks": clk.summary()}))
    arch.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--kernel", choices=["fused2d", "fused3d", "stokes3d_dc", "ptdiff3d", "sia_ensemble", "diffusion2d", "sia_adjoint", "stokes64",
                                         "ptdiff64"],
                    help="time one kernel alone (profiling driver)")
    ap.add_argument("--members", type=int, default=64, help="--kernel sia_ensemble: ensemble members")
    ap.add_argument("--nmin", type=int, default=128, help="--kernel sia_ensemble: smallest member size")
    ap.add_argument("--nmax", type=int, default=1024, help="--kernel sia_ensemble: largest member size")
    ap.add_argument("--reps", type=int, default=200)
    ap.add_argument("--align-index", type=int, default=0,
                    help="--kernel fused3d: the logical x index each padded row aligns to 128 bytes (-1: its first element)")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=2048)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-seconds", type=float, default=8.0)
    ap.add_argument("--ref-iters", type=int, default=400)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--skip-fp64", action="store_true", help="skip the one-off plain FP64 GPU solve")
    ap.add_argument("--skip-3d", action="store_true", help="skip the 3D fused-kernel measurement")
    ap.add_argument("--skip-suite", action="store_true", help="skip the other configurations' measurements")
    ap.add_argument("--suite-only", action="store_true", help="print only the other configurations' measurements")
    args = ap.parse_args()
    if args.kernel:
        run_kernel(args)
        return
    if args.suite_only:
        from chmy_gb300 import Arch, GB300Backend

        import torch

        arch = Arch(GB300Backend(), device_id=1)
        print(json.dumps({"configs": config_suite(arch, torch.cuda.current_stream(), measured_peaks()[0])}), flush=True)
        arch.close()
        return
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
