"""tj_compute_dt_noalloc: the time step for callers that cannot allocate
device memory (their GPU memory belongs to a host framework's pool, or they
may only use buffers handed to them). It must give what the context-based
tj_compute_dt gives on the same state, call after call, while allocating
nothing itself; the device buffer holding the state here is the caller's
(allocated by the test through torch)."""
import ctypes

import numpy as np
import pytest

from tenjin_gb300 import _lib, build, cases
from tenjin_gb300.host import FP64, TenjinGPU, make_params

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def noalloc_dt(L, case, dev_state, stream=None):
    p = make_params(case)
    d = case.domains[0]
    n = (ctypes.c_int * 3)(*d.n_cells)
    dl = (ctypes.c_double * 3)(*d.dim_l)
    dt = ctypes.c_double(-1.0)
    rc = L.tj_compute_dt_noalloc(ctypes.byref(p), n, dl, ctypes.c_void_p(dev_state.data_ptr()), ctypes.byref(dt),
                                 stream)
    assert rc == 0
    return dt.value


@pytest.mark.parametrize("builder,kw", [
    ("shock_bubble_2d", {"n": 64, "max_grid_size": 32, "max_steps": 4}),
    ("copper_plate_3d", {"n": 12, "max_grid_size": 6, "max_steps": 3}),
])
def test_noalloc_dt_matches_context_dt_twice(lib, builder, kw):
    torch = pytest.importorskip("torch")
    c = getattr(cases, builder)(**kw)
    g = TenjinGPU(c, FP64)
    for _ in range(2):  # before and after a few steps: two different states
        ref = g.getTimeStep()
        st = torch.from_numpy(g.state(0)).to("cuda")
        torch.cuda.synchronize()
        a = noalloc_dt(lib, c, st)
        b = noalloc_dt(lib, c, st)  # second call in a row on the shared array
        assert abs(a - ref) <= TOL * ref and abs(b - ref) <= TOL * ref, (a, b, ref)
        g.run(2, 1e300)


def test_noalloc_many_blocks_on_a_side_stream(lib):
    """A 1024^2 domain needs 512 first-pass blocks, more than the final pass
    has threads, so the final pass loops; the work is ordered on a torch
    stream other than the default one."""
    torch = pytest.importorskip("torch")
    c = cases.shock_bubble_2d(n=1024, max_grid_size=128, max_steps=2)
    g = TenjinGPU(c, FP64)
    g.run(1, 1e300)
    ref = g.getTimeStep()
    side = torch.cuda.Stream()
    with torch.cuda.stream(side):
        st = torch.from_numpy(g.state(0)).to("cuda", non_blocking=False)
    side.synchronize()
    got = [noalloc_dt(lib, c, st, ctypes.c_void_p(side.cuda_stream)) for _ in range(2)]
    g.close()
    assert all(abs(a - ref) <= TOL * ref for a in got), (got, ref)


@pytest.mark.parametrize("n_cells", [
    ((1 << 24) + 1, 1, 1),          # one axis beyond the maximum
    (1 << 12, 1 << 12, 2),          # a product just beyond it
    (2 ** 31 - 1, 2 ** 31 - 1, 2 ** 31 - 1),  # a product that overflows 64 bits if formed first
])
def test_noalloc_rejects_domains_beyond_the_maximum(lib, n_cells):
    c = cases.fluid_boxes_3d(n=4)
    p = make_params(c)
    n = (ctypes.c_int * 3)(*n_cells)
    dl = (ctypes.c_double * 3)(1.0, 1.0, 1.0)
    dt = ctypes.c_double(-1.0)
    dummy = ctypes.c_double(0.0)
    rc = lib.tj_compute_dt_noalloc(ctypes.byref(p), n, dl, ctypes.cast(ctypes.byref(dummy), ctypes.c_void_p),
                                   ctypes.byref(dt), None)
    assert rc == -1 and dt.value == -1.0
