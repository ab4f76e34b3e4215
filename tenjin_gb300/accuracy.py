"""Precision comparison of the density field along a whole run.

    python -m tenjin_gb300.accuracy bubble|copper|boxes [--steps N] [--every K] [--n SIZE]
                                    [--nbox B] [--out FILE]

Several contexts start from the same initial state and advance in lockstep,
each computing its own dt as the reference does (main.cpp:128-143). Every K
steps the density rho = sum of alphaRho_k of every domain is read back
(tj_download_component) and, for each pair of runs, the relative L1
difference sum|a - b| / sum|b| and the relative Linf difference
max|a - b| / max|b| are recorded.

Runs:
  fp64       TJ_PRECISION_FP64, the reference's evaluation order (bit for bit
             the reference on every golden fixture)
  mixed      TJ_PRECISION_MIXED, the binary32 kernels
  fused64    TJ_PRECISION_FUSED64, the fused 2-D kernels in binary64 (2-D only)
  fp64_pert  fp64 from an initial pressure multiplied by 1 + 1e-14 * xi, xi
             seeded uniform in [-1, 1]: a few units in the last place
  fp64_f32   fp64 from the initial primitive fields rounded to binary32 once:
             the state a binary32 run starts from, advanced in binary64

fp64_pert vs fp64 measures how fast the flow itself amplifies a last-bit
difference, and fused64 vs fp64 what a different but equally exact binary64
evaluation order gives: together they are the binary64 floor of any
comparison against the reference on this flow. fp64_f32 vs fp64 is what one
rounding of the state to binary32 grows to: a floor for any method that
stores the state in binary32. The workloads are the
benchmark's: the 2-D shock-bubble (1024^2, THINC, max_grid_size 128), the
copper plate (n^3, radial return) and the batch of uneven 3-D boxes.
"""
from __future__ import annotations

import argparse
import copy
import json
import time

import numpy as np

from . import cases
from .host import FP64, FUSED64, MIXED, TenjinGPU

PERTURBATION = 1e-14


def perturbed(case, eps: float = PERTURBATION, seed: int = 1234):
    """A copy of `case` whose initial pressure carries a seeded relative
    perturbation of size eps."""
    c = copy.deepcopy(case)
    rng = np.random.Generator(np.random.PCG64(seed))
    ip = 2 * c.M + 3  # alpha[M], rho_k[M], u[3], p in the primitive layout
    for d in c.domains:
        d.prim[ip] = d.prim[ip] * (1.0 + eps * rng.uniform(-1.0, 1.0, size=d.prim[ip].shape))
    return c


def rounded_to_binary32(case):
    """A copy of `case` whose initial primitive fields are rounded to binary32."""
    c = copy.deepcopy(case)
    for d in c.domains:
        d.prim = d.prim.astype(np.float32).astype(np.float64)
    return c


def _density(g, ndom):
    return np.concatenate([g.density(q).ravel() for q in range(ndom)])


def _diff(a, b):
    e = np.abs(a - b)
    return float(e.sum() / np.abs(b).sum()), float(e.max() / np.abs(b).max())


def density_curves(case, runs, pairs, steps: int, every: int, sums: bool = False):
    """Run each of `runs` ({name: (case, precision)}) for `steps` steps in
    blocks of `every`; after each block record the density differences of
    each pair (a, b) in `pairs`. Returns a dict of lists per pair; with
    `sums`, also each run's binary64 conservation sums at the start and the
    end (tj_conservation_sums)."""
    ctx = {k: TenjinGPU(c, p) for k, (c, p) in runs.items()}
    ndom = len(case.domains)
    out = {"steps": [], "t": {k: [] for k in runs}, "pairs": {f"{a}_vs_{b}": {"l1": [], "linf": []} for a, b in pairs},
           "seconds": {k: 0.0 for k in runs}}
    if sums:
        out["sums"] = {k: {"start": g.conservation_sums().tolist()} for k, g in ctx.items()}
    done = 0
    try:
        while done < steps:
            k = min(every, steps - done)
            dens = {}
            for name, g in ctx.items():
                t0 = time.perf_counter()
                g.run(k, 1e300)
                g.synchronize()
                out["seconds"][name] += time.perf_counter() - t0
                dens[name] = _density(g, ndom)
                out["t"][name].append(g.time()[0])
            done += k
            out["steps"].append(done)
            for a, b in pairs:
                l1, linf = _diff(dens[a], dens[b])
                out["pairs"][f"{a}_vs_{b}"]["l1"].append(l1)
                out["pairs"][f"{a}_vs_{b}"]["linf"].append(linf)
        if sums:
            for k, g in ctx.items():
                out["sums"][k]["end"] = g.conservation_sums().tolist()
    finally:
        for g in ctx.values():
            g.close()
    return out


def floor_gate(curves, run: str = "mixed_vs_fp64", floors=("fused64_vs_fp64", "fp64_pert_vs_fp64", "fp64_f32_vs_fp64"),
               tol: float = 1e-4, factor: float = 2.0):
    """The mixed-precision criterion along the curve: at every sample the L1
    difference of `run` is at most max(tol, factor x the binary64 floor),
    the floor being the largest of the `floors` pairs at that sample. Returns
    (passes, worst ratio of the L1 difference to its bound, sample index)."""
    l1 = np.asarray(curves["pairs"][run]["l1"])
    fl = np.zeros_like(l1)
    for f in floors:
        if f in curves["pairs"]:
            fl = np.maximum(fl, np.asarray(curves["pairs"][f]["l1"]))
    bound = np.maximum(tol, factor * fl)
    ratio = l1 / bound
    i = int(np.argmax(ratio))
    return bool(ratio[i] <= 1.0), float(ratio[i]), i


def workload(name: str, n: int = 0, nbox: int = 0):
    if name == "bubble":
        return cases.shock_bubble_2d(n=n or 1024, max_grid_size=128)
    if name == "copper":
        return cases.copper_plate_3d(n=n or 256)
    if name == "boxes":
        return cases.uneven_boxes_3d(nbox=nbox or 4096)
    raise ValueError(name)


def plan(name: str, case):
    runs = {"fp64": (case, FP64), "mixed": (case, MIXED), "fp64_pert": (perturbed(case), FP64),
            "fp64_f32": (rounded_to_binary32(case), FP64)}
    pairs = [("mixed", "fp64"), ("fp64_pert", "fp64"), ("fp64_f32", "fp64")]
    if name == "bubble":
        runs["fused64"] = (case, FUSED64)
        pairs += [("fused64", "fp64"), ("mixed", "fused64")]
    return runs, pairs


def summarise(curves):
    s = {}
    for k, v in curves["pairs"].items():
        l1 = np.asarray(v["l1"])
        s[k] = {"l1_final": float(l1[-1]), "l1_max": float(l1.max()), "linf_final": float(v["linf"][-1])}
    ok, ratio, i = floor_gate(curves)
    s["gate"] = {"criterion": "L1(mixed vs fp64) <= max(1e-4, 2 x binary64 floor) at every sample",
                 "passes": ok, "worst_ratio": ratio, "at_step": curves["steps"][i]}
    return s


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("config", choices=["bubble", "copper", "boxes"])
    ap.add_argument("--steps", type=int, default=0, help="default: the configuration's (2000 / 500 / 100)")
    ap.add_argument("--every", type=int, default=10)
    ap.add_argument("--n", type=int, default=0, help="cells per axis (bubble, copper)")
    ap.add_argument("--nbox", type=int, default=0, help="boxes (boxes)")
    ap.add_argument("--out", default="")
    a = ap.parse_args(argv)
    case = workload(a.config, a.n, a.nbox)
    steps = a.steps or {"bubble": 2000, "copper": 500, "boxes": 100}[a.config]
    runs, pairs = plan(a.config, case)
    curves = density_curves(case, runs, pairs, steps, a.every)
    res = {"config": a.config, "cells": case.total_cells, "steps_run": steps, "every": a.every,
           "perturbation": PERTURBATION, "summary": summarise(curves), "curves": curves}
    text = json.dumps(res)
    if a.out:
        with open(a.out, "w") as f:
            f.write(text)
    print(json.dumps({"config": a.config, "cells": case.total_cells, "summary": res["summary"],
                      "seconds": curves["seconds"]}))
    return res


if __name__ == "__main__":
    main()
