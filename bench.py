"""Benchmark of the per-timestep update on the 2-D shock-bubble workload.

Workload: water (stiffened gas, gamma 4.4, p_inf 6e8) with a Mach-1.5 shock
hitting an air bubble (radius 0.2, seeded centre), 1024 x 1024 cells,
max_grid_size 128 (64 boxes), MUSCL + BVD-THINC (beta 1.6), CFL 0.4. One
"step" is one full iteration of the reference's time loop (CFL reduction,
two RK stages, RK2 average, cleanUpAlpha) over all cells.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision mixed|fp64|fused64]
    python bench.py --impl reference ...   # the CPU reference arm

Prints one JSON line. `value` is cell-updates/s over the K timed steps
(device time, CUDA events on the library's stream, inputs resident in HBM);
`roofline` divides the stage kernel's algorithmic bytes by its mean launch
time, from CUDA events around every launch over a second run of K steps
right after the timed one (so that those events do not slow the timed run);
`e2e` is the same metric through the C ABI with the state copied in from
pinned host memory and back out every step. Under torchrun each rank runs an
independent replica (the update does not shard across GPUs in this build).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_CELLS = 1024
MAX_GRID = 128
METRIC = "cell-updates/s/GPU (FP32 vs FP64 at stated L1 err); adjoint/forward time ratio"
WORKLOAD = "2-D shock-bubble interface, water/air, 1024x1024, MUSCL+THINC beta 1.6, CFL 0.4, max_grid_size 128"


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(ms: float, device: str = "cuda") -> float:
    """Slowest rank's time (the job finishes when the last replica does)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return ms
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.file = None

    def __enter__(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.file:
            return None
        try:
            rows = [l.strip().split(",") for l in open(self.file.name) if l.strip()]
        except Exception:
            return None
        finally:
            try:
                os.unlink(self.file.name)
            except Exception:
                pass
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() in ("active", "1", "yes"):
                        reasons.add(n)
            except Exception:
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons), "samples": len(sm)}


def l2_flush_bytes():
    return 256 << 20  # larger than the 129 MB L2


def bench_config(args, ws):
    """The `config` object of the JSON line, the same for both arms."""
    return {"workload": WORKLOAD, "cells": N_CELLS * N_CELLS, "precision": args.precision,
            "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
            "l2": "state working set larger than L2 (three state buffers of >= 48 MB plus scratch per step)"}


def run_gpu_arm(args):
    import torch

    from tenjin_gb300 import build, cases
    from tenjin_gb300.host import FP64, FUSED64, MIXED, TenjinGPU

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    build.build()
    precision = {"mixed": MIXED, "fp64": FP64, "fused64": FUSED64}[args.precision]
    case = cases.shock_bubble_2d(n=N_CELLS, max_grid_size=MAX_GRID, max_steps=1 << 30)
    ncell = case.total_cells
    g = TenjinGPU(case, precision)
    lib = g.L
    sp = ctypes.c_void_p()
    lib.tj_get_stream(g.h, ctypes.byref(sp))
    stream = torch.cuda.ExternalStream(sp.value)

    # warm-up steps (untimed)
    g.run(args.warmup, 1e300)

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    barrier()
    torch.cuda.synchronize()
    l0 = g.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        with torch.cuda.stream(stream):
            ev0.record(stream)
        done, _ = g.run(args.steps, 1e300)
        with torch.cuda.stream(stream):
            ev1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = max_over_ranks(ev0.elapsed_time(ev1))
    launches = g.launch_count() - l0
    clocks = clk.summary()

    # dominant kernel: per-launch time from CUDA events recorded around each
    # launch, over a second run of the same number of steps right after the
    # timed one (the event nodes in the step graphs would otherwise add their
    # own latency to the timed region)
    lib.tj_set_profiling(g.h, 1)
    g.run(1, 1e300)  # capture with profiling, then reset totals
    lib.tj_set_profiling(g.h, 0)
    lib.tj_set_profiling(g.h, 1)
    g.run(args.steps, 1e300)
    torch.cuda.synchronize()
    kernels = {MIXED: ["tj_stage_mixed"], FUSED64: ["tj_stage_fused64"],
               FP64: ["tj_recon_fp64", "tj_flux_fp64", "tj_update_fp64", "tj_cfl_fp64"]}[precision]
    ktimes = {}
    for k in kernels:
        tot, cnt = ctypes.c_double(), ctypes.c_longlong()
        lib.tj_kernel_time(g.h, k.encode(), ctypes.byref(tot), ctypes.byref(cnt))
        if cnt.value:
            ktimes[k] = (tot.value, cnt.value)
    lib.tj_set_profiling(g.h, 0)
    dom = max(ktimes, key=lambda k: ktimes[k][0]) if ktimes else None
    peaks, peak_src = measured_peaks()
    roofline = None
    if dom:
        tot, cnt = ktimes[dom]
        per_launch_s = tot / cnt / 1e3
        if precision in (MIXED, FUSED64):
            # algorithmic bytes of one stage launch: the carried state (12 words
            # of 4 or 8 B) read and written once; stage 2 also reads U^n: 5
            # state passes per step spread over 2 launches
            bytes_per_launch = 2.5 * 12 * (4 if precision == MIXED else 8) * ncell
        else:
            bytes_per_launch = {"tj_recon_fp64": (7 + 2 * 14) * 8, "tj_flux_fp64": (2 * 14 + 9) * 8,
                                "tj_update_fp64": (2 * 9 + 2 * 15) * 8, "tj_cfl_fp64": 10 * 8}[dom] * ncell
        achieved = bytes_per_launch / per_launch_s / 1e9
        traffic = None
        try:
            with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
                tj = json.load(f)
            if tj.get("kernel") == dom:
                traffic = tj.get("dram_bytes_per_launch")
        except Exception:
            pass
        roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
                    "frac": round(achieved / peaks["hbm_gbs"], 4), "traffic": traffic, "kernel": dom,
                    "peak_source": peak_src, "launch_ms": round(tot / cnt, 4),
                    "kernel_ms": {k: round(v[0] / v[1], 4) for k, v in ktimes.items()}}

    # end to end through the C ABI: state in from pinned host memory, step,
    # state out, every step
    e2e = None
    if args.e2e_steps > 0:
        nc = g.ncomp
        host = torch.empty((nc, 1, N_CELLS, N_CELLS), dtype=torch.float64, pin_memory=True)
        host_np = host.numpy()
        lib.tj_download_domain(g.h, 0, host_np.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
        for _ in range(args.e2e_steps):
            p = host_np.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            lib.tj_upload_domain(g.h, 0, p)
            lib.tj_step(g.h, ctypes.c_double(1e300))
            lib.tj_download_domain(g.h, 0, p)
        with torch.cuda.stream(stream):
            e1.record(stream)
        torch.cuda.synchronize()
        e2e_ms = e0.elapsed_time(e1)
        wall = time.perf_counter() - t0
        from tenjin_gb300.host import carried_components
        # the upload copies the component planes of the carried state, the
        # download all Ncomp components of the AccessPattern
        up_bytes = len(carried_components(case)) * ncell * 8
        down_bytes = nc * ncell * 8
        e2e = {"value": ncell * args.e2e_steps / (max(e2e_ms / 1e3, wall)), "unit": "cell-updates/s",
               "h2d_bytes_per_step": up_bytes, "d2h_bytes_per_step": down_bytes, "steps": args.e2e_steps,
               "path": "tj_upload_domain + tj_step + tj_download_domain (AccessPattern layout, pinned host)"}
        e2e.update(e2e_breakdown(lib, g, host_np, up_bytes, down_bytes, max(e2e_ms, wall * 1e3) / args.e2e_steps))

    # accuracy and the FP64 speeds: the whole 2000-step workload (not part of
    # the timed region) in the three precisions, each timed on its own stream
    accuracy = None
    if precision == MIXED and args.fp64_compare:
        accuracy = accuracy_runs(case, args.accuracy_steps)
    # the second half of the metric: adjoint / forward time on the 2-D
    # interface problem at 512^2, 200 steps, checked against the tangent-linear
    # run (and, on request, against central differences)
    configs = other_configs() if args.other_configs and rank == 0 else None
    adjoint = None
    if args.adjoint_dirs >= 0 and rank == 0:
        from tenjin_gb300.adjoint import interface_problem_check
        adjoint = interface_problem_check(512, 200, 20, args.adjoint_dirs, background=args.adjoint_background,
                                          tlm_dirs=args.adjoint_tlm_dirs)
    g.close()
    value = ncell * args.steps * ws / (ms / 1e3)
    line = {
        "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": {MIXED: "f32 (compensated energy and pressure closure)", FUSED64: "f64 (fused kernels)",
                                        FP64: "f64"}[precision],
        "data": "synthetic (seeded shock-bubble initial condition)",
        "config": bench_config(args, ws),
        "gpu_launches": launches, "steps_done": done, "e2e": e2e, "roofline": roofline, "clocks": clocks,
        "accuracy": accuracy, "adjoint": adjoint, "other_configs": configs,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.cpu_seconds)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    if rank == 0:
        print(json.dumps(line), flush=True)


def _timed_run(g, steps):
    """Device time (ms) of g.run(steps) on the context's stream."""
    import torch

    sp = ctypes.c_void_p()
    g.L.tj_get_stream(g.h, ctypes.byref(sp))
    st = torch.cuda.ExternalStream(sp.value)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    with torch.cuda.stream(st):
        e0.record(st)
    done, _ = g.run(steps, 1e300)
    with torch.cuda.stream(st):
        e1.record(st)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1), done


def other_configs():
    """The two 3-D configurations, measured beside the headline: the batch of
    4096 uneven boxes (fused binary32 3-D kernel and the FP64 path, relative
    L1 density error after 5 steps) and the copper plate at 256^3 (FP64
    path: 5-wave solver, radial return, cleanUpV)."""
    from tenjin_gb300 import cases
    from tenjin_gb300.host import FP64, MIXED, TenjinGPU

    out = {}
    c = cases.uneven_boxes_3d()
    g64 = TenjinGPU(c, FP64)
    g64.run(2, 1e300)
    ms64, d64 = _timed_run(g64, 3)
    M = c.M
    sample = range(0, len(c.domains), 8)
    r64 = [g64.state(q)[M:2 * M].sum(axis=0) for q in sample]
    g64.close()
    g32 = TenjinGPU(c, MIXED)
    g32.run(5, 1e300)
    r32 = [g32.state(q)[M:2 * M].sum(axis=0) for q in sample]
    import numpy as np
    e = sum(float(np.abs(a - b).sum()) for a, b in zip(r32, r64)) / sum(float(np.abs(b).sum()) for b in r64)
    g32.run(3, 1e300)
    ms32, d32 = _timed_run(g32, 20)
    buf = ctypes.create_string_buffer(256)
    g32.L.tj_kernel_config(g32.h, buf, 256)
    g32.close()
    out["uneven_boxes_3d"] = {
        "workload": f"{len(c.domains)} independent 3-D boxes, edges log-uniform in [8, 64], {c.total_cells} cells, "
                    "water/air, MUSCL",
        "mixed": {"value": c.total_cells * d32 / (ms32 / 1e3), "unit": "cell-updates/s", "steps": d32,
                  "ms_per_step": ms32 / max(d32, 1), "kernel_config": buf.value.decode()},
        "fp64": {"value": c.total_cells * d64 / (ms64 / 1e3), "unit": "cell-updates/s", "steps": d64,
                 "ms_per_step": ms64 / max(d64, 1)},
        "l1_rel_density_err_after_5_steps": e, "sampled_boxes": len(sample),
        "whole_run": horizon("boxes", cases.uneven_boxes_3d(nbox=512), 100)}
    c = cases.copper_plate_3d(n=256)
    g = TenjinGPU(c, FP64)
    g.run(1, 1e300)
    ms, d = _timed_run(g, 2)
    r64 = g.state(0)[c.M:2 * c.M].sum(axis=0)
    g.close()
    g32 = TenjinGPU(c, MIXED)
    g32.run(1, 1e300)
    ms32, d32 = _timed_run(g32, 2)
    r32 = g32.state(0)[c.M:2 * c.M].sum(axis=0)
    g32.L.tj_kernel_config(g32.h, buf, 256)
    g32.run(3, 1e300)
    ms32b, d32b = _timed_run(g32, 5)
    g32.close()
    out["copper_plate_3d"] = {
        "workload": "copper plate impact, 256^3, Hugoniot Mie-Gruneisen, G 45 GPa, Y 90 MPa, plastic",
        "fp64": {"value": c.total_cells * d / (ms / 1e3), "unit": "cell-updates/s", "steps": d,
                 "ms_per_step": ms / max(d, 1)},
        "mixed": {"value": c.total_cells * d32b / (ms32b / 1e3), "unit": "cell-updates/s", "steps": d32b,
                  "ms_per_step": ms32b / max(d32b, 1), "kernel_config": buf.value.decode()},
        "l1_rel_density_err_after_3_steps": float(abs(r32 - r64).sum() / abs(r64).sum()),
        "whole_run": horizon("copper", cases.copper_plate_3d(n=64), 500)}
    return out


def horizon(name, case, steps):
    """Binary32 against the reference-ordered binary64 path over a whole run
    (relative L1 and Linf density difference every steps/10 steps), at a
    reduced size so that the binary64 run takes seconds."""
    from tenjin_gb300 import accuracy
    from tenjin_gb300.host import FP64, MIXED

    curves = accuracy.density_curves(case, {"fp64": (case, FP64), "mixed": (case, MIXED)}, [("mixed", "fp64")],
                                     steps, max(1, steps // 10))
    p = curves["pairs"]["mixed_vs_fp64"]
    return {"cells": case.total_cells, "steps": steps, "cfl": case.cfl, "curve_steps": curves["steps"],
            "l1_rel": p["l1"], "linf_rel": p["linf"], "l1_max": max(p["l1"])}


def accuracy_runs(case, steps):
    """The workload for `steps` steps from its initial state through the
    binary32 kernels (TJ_PRECISION_MIXED), the same fused kernels in binary64
    (TJ_PRECISION_FUSED64), the reference-ordered binary64 kernels
    (TJ_PRECISION_FP64), and the binary64 kernels from the initial state
    perturbed by 1e-14 and from it rounded to binary32 once: relative L1 and
    Linf density differences every 100 steps (tenjin_gb300.accuracy), the
    criterion along the run, each run's throughput, and the binary64 global
    conservation sums (tj_conservation_sums) at the start and the end."""
    from tenjin_gb300 import accuracy

    runs, pairs = accuracy.plan("bubble", case)
    curves = accuracy.density_curves(case, runs, pairs, steps, 100, sums=True)
    summ = accuracy.summarise(curves)
    sums = {k: curves["sums"][k] for k in ("fp64", "fused64", "mixed")}
    M = case.M
    rel = lambda a, b: abs(a - b) / abs(b)
    cons = {"layout": f"[alphaRho_0..{M - 1}, rhoU_x, rhoU_y, rhoU_z, E] x cell volume, binary64, fixed order",
            "runs": sums,
            "mixed_vs_fp64_end": {"mass": [rel(sums["mixed"]["end"][m], sums["fp64"]["end"][m]) for m in range(M)],
                                  "energy": rel(sums["mixed"]["end"][M + 3], sums["fp64"]["end"][M + 3])},
            "note": "the boundaries are transmissive (the shock enters at x = 0), so the sums change over the run "
                    "in every precision; their agreement between precisions is the check"}
    sec = curves["seconds"]
    speed = {k: {"value": case.total_cells * steps / sec[k], "unit": "cell-updates/s",
                 "ms_per_step": 1e3 * sec[k] / steps, "timing": "host wall time of the run blocks"}
             for k in ("mixed", "fused64", "fp64")}
    return {"steps": steps, "field": "density (sum of alphaRho)", "sampled_every": 100,
            "pairs": summ, "curve_steps": curves["steps"],
            "curves_l1": {k: v["l1"] for k, v in curves["pairs"].items()},
            "t_end": {k: v[-1] for k, v in curves["t"].items()}, "throughput": speed, "conservation": cons,
            "note": "fused64 vs fp64 and fp64_pert vs fp64 are the binary64 floor of this chaotic interface "
                    "flow; fp64_f32 vs fp64 is what one rounding of the state to binary32 grows to"}


def cpu_baseline(target_seconds=15.0):
    """The oracle port (oracle/port, FP64, OpenMP over all host threads) on a
    bounded sample of the same workload: the full 1024^2 domain for as many
    steps as fit in about target_seconds."""
    from oracle import port
    from tenjin_gb300 import cases

    port.build_port()
    case = cases.shock_bubble_2d(n=N_CELLS, max_grid_size=MAX_GRID, max_steps=1)
    sim = port.PortSim(case, omp=True)
    t0 = time.perf_counter()
    sim.run(max_steps=1)
    one = time.perf_counter() - t0
    steps = max(1, min(50, int(target_seconds / max(one, 1e-3))))
    t0 = time.perf_counter()
    sim.run(max_steps=steps)
    el = time.perf_counter() - t0
    return {"value": case.total_cells * steps / el, "unit": "cell-updates/s", "cores": port.threads(),
            "kind": "port", "sample": f"{steps} steps of the 1024x1024 workload after 1 untimed step, FP64"}


def run_reference_arm(args):
    """CPU reference arm: the oracle port (the reference itself cannot be built
    on the GPU host: it needs AMReX and its sources are not shipped there),
    with all host threads, on the same workload and metric; each step is one
    full time step of a bounded square sample of the domain."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    from oracle import port
    from tenjin_gb300 import cases

    port.build_port()
    nthr = port.threads()
    # size the sample so that (warmup + steps) stays within the time budget
    budget = args.ref_budget / max(1, args.steps + args.warmup)
    n = 256
    probe = cases.shock_bubble_2d(n=n, max_grid_size=MAX_GRID // 4, max_steps=1)
    sim = port.PortSim(probe, omp=True)
    t0 = time.perf_counter()
    sim.run(max_steps=1)
    rate = n * n / (time.perf_counter() - t0)
    side = int((budget * rate) ** 0.5) // 64 * 64
    side = max(64, min(N_CELLS, side))
    mgs = max(16, MAX_GRID * side // N_CELLS)
    case = cases.shock_bubble_2d(n=side, max_grid_size=mgs, max_steps=1 << 30)
    sim = port.PortSim(case, omp=True)
    sim.run(max_steps=args.warmup)
    t0 = time.perf_counter()
    sim.run(max_steps=args.steps)
    el = time.perf_counter() - t0
    value = case.total_cells * args.steps / el
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "cell-updates/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded shock-bubble initial condition)",
        "config": bench_config(args, ws),
        "cpu_baseline": {"value": value, "unit": "cell-updates/s", "cores": nthr, "kind": "port",
                         "sample": f"{args.steps} steps of a {side}x{side} sample of the workload "
                                   f"(max_grid_size {mgs}), FP64"},
        "e2e": {"value": value, "unit": "cell-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def e2e_breakdown(lib, g, host_np, up_bytes, down_bytes, ms_per_step, reps=10):
    """The end-to-end step's three calls timed apart (host wall clock around
    synchronised calls), and the host<->device link's own rate, measured by
    plain copies of page-locked buffers of the same sizes: the part of the
    end-to-end time the link alone needs."""
    import torch

    p = host_np.ctypes.data_as(ctypes.POINTER(ctypes.c_double))

    def timed(f):
        torch.cuda.synchronize()
        t = time.perf_counter()
        for _ in range(reps):
            f()
        torch.cuda.synchronize()
        return (time.perf_counter() - t) / reps * 1e3

    up = timed(lambda: lib.tj_upload_domain(g.h, 0, p))
    step = timed(lambda: (lib.tj_step(g.h, ctypes.c_double(1e300)), lib.tj_synchronize(g.h)))
    down = timed(lambda: lib.tj_download_domain(g.h, 0, p))
    hb = torch.empty(max(up_bytes, down_bytes) // 8, dtype=torch.float64, pin_memory=True)
    db = torch.empty_like(hb, device="cuda")
    nu, nd = up_bytes // 8, down_bytes // 8
    h2d = timed(lambda: db[:nu].copy_(hb[:nu], non_blocking=True))
    d2h = timed(lambda: hb[:nd].copy_(db[:nd], non_blocking=True))
    link_ms = h2d + d2h
    return {"phases_ms": {"upload": round(up, 4), "step": round(step, 4), "download": round(down, 4)},
            "link": {"h2d_gbs": round(up_bytes / h2d / 1e6, 1), "d2h_gbs": round(down_bytes / d2h / 1e6, 1),
                     "copy_ms_per_step": round(link_ms, 4),
                     "frac_of_step_time": round(link_ms / ms_per_step, 3),
                     "note": "page-locked copies of the step's upload and download sizes; the part of the "
                             "end-to-end step that the host link alone takes"}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64", "fused64"])
    ap.add_argument("--accuracy-steps", type=int, default=2000, help="steps of the precision comparison")
    ap.add_argument("--no-other-configs", dest="other_configs", action="store_false",
                    help="skip the 3-D configurations")
    ap.add_argument("--adjoint-dirs", type=int, default=0,
                    help="finite-difference directions of the adjoint check (-1: skip the adjoint)")
    ap.add_argument("--adjoint-tlm-dirs", type=int, default=64,
                    help="directions of the adjoint checked against the tangent-linear run")
    ap.add_argument("--adjoint-background", type=float, default=0.0,
                    help="smooth background of the adjoint problem's base state (0: the problem as stated)")
    ap.add_argument("--no-fp64-compare", dest="fp64_compare", action="store_false")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ref-budget", type=float, default=120.0, help="seconds for the whole reference arm")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference_arm(args)
    else:
        run_gpu_arm(args)


if __name__ == "__main__":
    main()
