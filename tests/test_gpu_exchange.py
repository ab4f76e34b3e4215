"""State exchange through the C ABI with page-locked host buffers.

On a device that reads host memory coherently (Grace + NVLink-C2C), a
page-locked buffer is converted in place by the exchange kernels instead of
being staged through device memory; pageable buffers (numpy arrays) take the
staged copy. Both must give the same bytes: whole-domain and per-box
downloads, ghost cells left as they were, and uploads that step identically.
"""
import numpy as np
import pytest

from tenjin_gb300 import build, cases
from tenjin_gb300.host import FP64, MIXED, TenjinGPU
from tenjin_gb300.output import variable_names

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def pinned(shape):
    return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()


def _ctx(precision, steps=3):
    c = cases.shock_bubble_2d(n=64, max_grid_size=24, max_steps=steps)
    g = TenjinGPU(c, precision)
    g.run(steps, 1e300)
    return c, g


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_pinned_domain_download_equals_pageable(precision):
    c, g = _ctx(precision)
    a = g.state(0)
    b = pinned(a.shape)
    b.fill(np.nan)
    g.state(0, out=b)
    np.testing.assert_array_equal(a, b)
    g.close()


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_pinned_fab_exchange_keeps_ghosts(precision):
    c, g = _ctx(precision)
    full = g.state(0)
    ng = 2
    rng = np.random.default_rng(5)
    for b, box in enumerate(c.domains[0].boxes):
        nx, ny = box[3] - box[0] + 1, box[4] - box[1] + 1
        fab = pinned((g.ncomp, 1, ny + 2 * ng, nx + 2 * ng))
        fab[...] = rng.standard_normal(fab.shape)
        ghosts = fab.copy()
        g.download_fab(0, b, fab, ng)
        np.testing.assert_array_equal(fab[:, :, ng:ng + ny, ng:ng + nx],
                                      full[:, :, box[1]:box[4] + 1, box[0]:box[3] + 1])
        mask = np.ones(fab.shape, bool)
        mask[:, :, ng:ng + ny, ng:ng + nx] = False
        np.testing.assert_array_equal(fab[mask], ghosts[mask])
        g.upload_fab(0, b, fab, ng)
    np.testing.assert_array_equal(g.state(0), full)
    g.close()


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_pinned_upload_steps_like_pageable(precision):
    c, g1 = _ctx(precision)
    _, g2 = _ctx(precision)
    st = g1.state(0)
    # a perturbed state: momenta and velocities 1 % larger
    comps = [i for i, nm in enumerate(variable_names(c)) if nm.startswith(("rhoU", "u0"))]
    assert comps
    st[comps] *= 1.01
    host = pinned(st.shape)
    host[...] = st
    g1.set_state(0, st)           # pageable: staged copy
    g2.set_state(0, host)         # page-locked: converted in place
    np.testing.assert_array_equal(g1.state(0), g2.state(0))
    for g in (g1, g2):
        g.run(2, 1e300)
    np.testing.assert_array_equal(g1.state(0), g2.state(0))
    g1.close()
    g2.close()


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_registered_buffer_exchange(precision):
    """Registered (cudaHostRegister) memory: read in place on upload, written
    through the staged copy on download (registered memory may be mapped
    read-only to the device); the same bytes as a pageable buffer."""
    c, g = _ctx(precision)
    ref = g.state(0)
    buf = np.empty(ref.shape)
    cudart = torch.cuda.cudart()
    torch.cuda.check_error(cudart.cudaHostRegister(buf.ctypes.data, buf.nbytes, 0))
    try:
        g.state(0, out=buf)
        np.testing.assert_array_equal(buf, ref)
        buf[...] = ref
        g.set_state(0, buf)
        g.run(2, 1e300)
        _, g2 = _ctx(precision)
        g2.set_state(0, ref.copy())
        g2.run(2, 1e300)
        np.testing.assert_array_equal(g.state(0), g2.state(0))
        g2.close()
    finally:
        torch.cuda.check_error(cudart.cudaHostUnregister(buf.ctypes.data))
    g.close()
