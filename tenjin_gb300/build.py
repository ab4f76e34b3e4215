"""In-tree build of libtenjin_gpu.so for sm_103a with nvcc.

Each translation unit is compiled in parallel, then linked into
tenjin_gb300/_build/libtenjin_gpu.so. The FP64 reference-faithful unit is
compiled with -fmad=false so that no multiply-add is contracted (the reference
is compiled without contraction too).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(BUILD, "libtenjin_gpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE, "-I" + CSRC]
UNITS = {
    "tj_api.cu": [],
    "tj_fp64.cu": ["-fmad=false"],
    # binary32 bulk: approximate division / square root, denormals flushed;
    # the compensated energy sum uses explicit round-to-nearest intrinsics
    "tj_mixed.cu": ["-use_fast_math"],
    "tj_mixed3d.cu": ["-use_fast_math"],
    # binary32 general path: fast binary32 arithmetic; its binary64 closure and
    # yield projection need no bit-exactness
    "tj_fp32.cu": ["-use_fast_math"],
    "tj_noalloc.cu": ["-fmad=false"],
    # the adjoint's forward average must match the FP64 path bit for bit
    "tj_adjoint.cu": ["-fmad=false"],
    # tangent-linear runs: values bit for bit those of the FP64 path
    "tj_tangent.cu": ["-fmad=false"],
    # the general reverse mode differentiates the FP64 path's own arithmetic
    "tj_adjoint_gen.cu": ["-fmad=false"],
}

# The per-direction kernels, one object per (type, material count, direction)
# instance of tj_path_inst.cu; M = 0 / direction -1 is the generic instance.
_INST = [(1, 0), (1, 1), (1, 2), (2, 0), (2, 1), (2, 2), (0, -1)]
INSTANCES = {
    f"tj_path_{r}_m{m}_d{'g' if d < 0 else d}.o":
        ("tj_path_inst.cu", [f"-DTJ_INST_R={r}", f"-DTJ_INST_M={m}", f"-DTJ_INST_D={d}",
                             "-fmad=false" if r == 64 else "-use_fast_math"])
    for r in (64, 32) for m, d in _INST
}
# the tangent instance (tj_dual.cuh): two materials along x and y, and the
# generic instance for every other material count and direction
INSTANCES.update({
    f"tj_path_t_m{m}_d{'g' if d < 0 else d}.o":
        ("tj_path_inst.cu", ["-DTJ_INST_R=128", f"-DTJ_INST_M={m}", f"-DTJ_INST_D={d}", "-fmad=false"])
    for m, d in [(2, 0), (2, 1), (0, -1)]
})


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps_mtime() -> float:
    t = os.path.getmtime(os.path.abspath(__file__))
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


def _compile(obj_name: str, unit: str, extra) -> str:
    src = os.path.join(CSRC, unit)
    obj = os.path.join(BUILD, obj_name)
    cmd = [nvcc()] + ARCH + COMMON + extra + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {obj_name}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    jobs = [(u.replace(".cu", ".o"), u, f) for u, f in UNITS.items() if os.path.exists(os.path.join(CSRC, u))]
    jobs += [(o, u, f) for o, (u, f) in INSTANCES.items()]
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps_mtime():
        return LIB
    # the largest objects first, so that the parallel build ends together
    jobs.sort(key=lambda j: (not j[0].startswith("tj_path_"), j[0]))
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), max(2, os.cpu_count() or 2))) as ex:
        objs = list(ex.map(lambda j: _compile(*j), jobs))
    cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force=True, verbose=True)
