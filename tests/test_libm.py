"""The project-written binary64 transcendentals (exp, expm1, log, pow, cosh,
tanh) that the FP64 path and the oracle both use, over the argument ranges
the path feeds them:

* BVD-THINC (thinc.cpp:67-208): exp of theta*beta*(2C - 1) with beta up to
  1.61, cosh and tanh of beta;
* the Wilkins EOS (equationofstate.cpp:502-596): log of rho/rho0;
* the Romenskii EOS and cleanUpV: pow of rho/rho0 (exponents of a few units)
  and of det V (exponent -1/3); the reactive rate: pow of p/1e6 to 1.2.

Checked: the GPU build and the oracle's host build give the same bits (the
premise of the bit-exact FP64 parity), and both stay within 4 units in the
last place of the host libm and of CUDA's own functions -- except pow, which
is exp(y log x) without an extended-precision log: the log's rounding is
multiplied by |y ln x|, up to about 10 here, and pow stays within 8 units."""
import ctypes
import math
import os
import shutil
import subprocess

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
N = 20000
# (fn code, name, host libm function, x range, y range or None, log-uniform x,
#  largest distance in units in the last place)
CASES = [
    (0, "exp", math.exp, (-20.0, 20.0), None, False, 4),
    (5, "expm1", math.expm1, (-0.35, 0.35), None, False, 4),
    (1, "log", math.log, (1e-3, 1e3), None, True, 4),
    (2, "pow", math.pow, (0.3, 3.0), (-3.0, 5.0), False, 8),
    (2, "pow_reactive", math.pow, (1e-2, 1e4), (1.2, 1.2), True, 8),
    (3, "cosh", math.cosh, (1e-3, 5.0), None, False, 4),
    (4, "tanh", math.tanh, (-5.0, 5.0), None, False, 4),
]


def _args(xr, yr, logx, seed):
    rng = np.random.default_rng(seed)
    if logx:
        x = np.exp(rng.uniform(math.log(xr[0]), math.log(xr[1]), N))
    else:
        x = rng.uniform(xr[0], xr[1], N)
    y = rng.uniform(yr[0], yr[1], N) if yr else np.zeros(N)
    return np.ascontiguousarray(x), np.ascontiguousarray(y)


def ulp_diff(a, b):
    """|a - b| in units in the last place (ordered binary64 integers)."""
    ia = np.asarray(a, dtype=np.float64).view(np.int64).astype(np.int64)
    ib = np.asarray(b, dtype=np.float64).view(np.int64).astype(np.int64)
    ia = np.where(ia < 0, np.int64(-(2 ** 63)) - ia, ia)
    ib = np.where(ib < 0, np.int64(-(2 ** 63)) - ib, ib)
    return np.abs(ia - ib)


@pytest.fixture(scope="module")
def host_lib(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    out = str(tmp_path_factory.mktemp("libm") / "libtjm_host.so")
    subprocess.run([cc, "-O2", "-std=c99", "-ffp-contract=off", "-fno-builtin", "-shared", "-fPIC",
                    "-I" + os.path.join(ROOT, "oracle", "shims"), os.path.join(HERE, "libm", "libm_host.c"),
                    "-o", out, "-lm"], check=True)
    lib = ctypes.CDLL(out)
    lib.tjm_eval_host.restype = None
    return lib


def host_eval(lib, fn, x, y):
    out = np.empty_like(x)
    P = ctypes.POINTER(ctypes.c_double)
    lib.tjm_eval_host(fn, x.ctypes.data_as(P), y.ctypes.data_as(P), len(x), out.ctypes.data_as(P))
    return out


@pytest.mark.parametrize("case", CASES, ids=[c[1] for c in CASES])
def test_host_build_close_to_the_host_libm(host_lib, case):
    fn, name, ref, xr, yr, logx, ulp_max = case
    x, y = _args(xr, yr, logx, fn + 17)
    got = host_eval(host_lib, fn, x, y)
    want = np.array([ref(a, b) if yr else ref(a) for a, b in zip(x, y)])
    d = ulp_diff(got, want)
    assert d.max() <= ulp_max, f"{name}: max {d.max()} ulp at x={x[d.argmax()]!r}"


@pytest.fixture(scope="module")
def gpu_lib(tmp_path_factory):
    from tenjin_gb300 import build
    out = str(tmp_path_factory.mktemp("libm") / "libtjm_gpu.so")
    subprocess.run([build.nvcc(), "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-fmad=false", "-shared",
                    "-Xcompiler", "-fPIC", "-I" + os.path.join(ROOT, "tenjin_gb300", "csrc"),
                    "-I" + os.path.join(ROOT, "include"), os.path.join(HERE, "libm", "libm_harness.cu"), "-o", out],
                   check=True)
    lib = ctypes.CDLL(out)
    lib.tjm_eval_gpu.restype = ctypes.c_int
    return lib


@pytest.mark.gpu
@pytest.mark.parametrize("case", CASES, ids=[c[1] for c in CASES])
def test_gpu_build_equals_host_build_and_is_close_to_libm_and_cuda(gpu_lib, host_lib, case):
    fn, name, ref, xr, yr, logx, ulp_max = case
    x, y = _args(xr, yr, logx, fn + 17)
    ours, cuda = np.empty_like(x), np.empty_like(x)
    P = ctypes.POINTER(ctypes.c_double)
    rc = gpu_lib.tjm_eval_gpu(fn, x.ctypes.data_as(P), y.ctypes.data_as(P), len(x), ours.ctypes.data_as(P),
                              cuda.ctypes.data_as(P))
    assert rc == 0
    host = host_eval(host_lib, fn, x, y)
    assert np.array_equal(ours.view(np.int64), host.view(np.int64)), f"{name}: GPU and host builds differ"
    want = np.array([ref(a, b) if yr else ref(a) for a, b in zip(x, y)])
    d_libm = ulp_diff(ours, want)
    d_cuda = ulp_diff(ours, cuda)
    print(f"{name}: max {d_libm.max()} ulp from the host libm, {d_cuda.max()} from CUDA's")
    assert d_libm.max() <= ulp_max, f"{name}: {d_libm.max()} ulp from the host libm"
    assert d_cuda.max() <= ulp_max, f"{name}: {d_cuda.max()} ulp from CUDA's {name}"
