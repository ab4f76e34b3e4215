"""Run one of the synthetic workloads on the GPU path from the command line.

    python -m tenjin_gb300.run <builder> [key=value ...] [--precision fp64|mixed|fused64]
                               [--steps N] [--warmup W]

<builder> is a function of tenjin_gb300.cases (sod_1d, shock_bubble_2d,
copper_plate_3d, uneven_boxes_3d, solid_mixture_2d, reactive_charge, ...);
key=value pairs are its keyword arguments (ints, floats or Python literals).
The state is set up, W steps run untimed, then N steps are timed with CUDA
events on the context's stream. Prints one line: cells, steps, ms per step,
cell-updates/s and the kernel configuration the context chose.
"""
from __future__ import annotations

import argparse
import ast
import ctypes
import json

from . import cases
from .host import FP64, FUSED64, MIXED, TenjinGPU

_PREC = {"fp64": FP64, "mixed": MIXED, "fused64": FUSED64}


def _value(text: str):
    try:
        return ast.literal_eval(text)
    except (ValueError, SyntaxError):
        return text


def main(argv=None) -> dict:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("builder")
    ap.add_argument("kwargs", nargs="*", help="key=value arguments of the builder")
    ap.add_argument("--precision", default="mixed", choices=sorted(_PREC))
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    a = ap.parse_args(argv)
    kw = {}
    for item in a.kwargs:
        k, _, v = item.partition("=")
        kw[k] = _value(v)
    case = getattr(cases, a.builder)(**kw)
    g = TenjinGPU(case, _PREC[a.precision])
    g.run(a.warmup, 1e300)
    import torch

    sp = ctypes.c_void_p()
    g.L.tj_get_stream(g.h, ctypes.byref(sp))
    st = torch.cuda.ExternalStream(sp.value)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    done, _ = g.run(a.steps, 1e300)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    buf = ctypes.create_string_buffer(256)
    g.L.tj_kernel_config(g.h, buf, 256)
    out = {"builder": a.builder, "kwargs": kw, "precision": a.precision, "cells": case.total_cells,
           "steps": done, "ms_per_step": ms / max(done, 1),
           "cell_updates_per_s": case.total_cells * done / (ms / 1e3) if ms > 0 else None,
           "kernel_config": buf.value.decode()}
    print(json.dumps(out))
    g.close()
    return out


if __name__ == "__main__":
    main()
