"""Binary32 per-direction kernels (the mixed precision of configurations the
fused kernels do not cover): solids with the 5-wave solver, plasticity and
cleanUpV, the 1-D shock tube, several 2-D domains. Against the FP64 path on
the same inputs: relative L1 density error <= 1e-4 (the pressure closure and
the pressure closure runs in binary64, the energy is a compensated pair)."""
import numpy as np
import pytest

from tenjin_gb300 import build, cases
from tenjin_gb300.host import FP64, MIXED, TenjinGPU

pytestmark = pytest.mark.gpu
L1_TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def density(g, c):
    return np.concatenate([g.state(q)[c.M:2 * c.M].sum(axis=0).ravel() for q in range(len(c.domains))])


def compare(c, steps):
    g64 = TenjinGPU(c, FP64)
    d64, t64 = g64.run(steps, c.final_t)
    g32 = TenjinGPU(c, MIXED)
    d32, t32 = g32.run(steps, c.final_t)
    buf = __import__("ctypes").create_string_buffer(256)
    g32.L.tj_kernel_config(g32.h, buf, 256)
    r64, r32 = density(g64, c), density(g32, c)
    assert d64 == d32, (d64, d32)
    assert np.all(np.isfinite(r32))
    return np.abs(r32 - r64).sum() / np.abs(r64).sum(), abs(t32 - t64) / t64, buf.value.decode()


def test_copper_plate_plastic():
    c = cases.copper_plate_3d(n=24, max_grid_size=12)
    l1, dt_rel, cfg = compare(c, 20)
    assert "binary32 per-direction" in cfg
    assert l1 <= L1_TOL, l1
    assert dt_rel <= 1e-5


@pytest.mark.parametrize("eos", [cases.EOS_WILKINS, cases.EOS_ROMENSKII, cases.EOS_HUGONIOT])
def test_solid_fluid_mixture_3d(eos):
    c = cases.solid_mixture_3d(eos=eos, n=12, max_grid_size=6, max_steps=8)
    l1, dt_rel, cfg = compare(c, 8)
    assert "binary32 per-direction" in cfg
    assert l1 <= L1_TOL, l1


@pytest.mark.parametrize("eos", [cases.EOS_WILKINS, cases.EOS_ROMENSKII, cases.EOS_HUGONIOT])
def test_solid_fluid_mixture_2d(eos):
    c = cases.solid_mixture_2d(eos=eos, n=24, max_steps=10)
    l1, dt_rel, _ = compare(c, 10)
    assert l1 <= L1_TOL, l1


def test_sod_1d_to_final_time():
    c = cases.sod_1d(ncells=1000, max_grid_size=125)
    l1, dt_rel, cfg = compare(c, 100000)
    assert l1 <= L1_TOL, l1


def test_several_2d_domains_with_thinc():
    c = cases.shock_bubble_2d(n=32, max_grid_size=16, max_steps=40)
    c.domains.append(cases.shock_bubble_2d(n=24, seed=1, max_grid_size=12).domains[0])
    l1, _, cfg = compare(c, 40)
    assert "binary32 per-direction" in cfg
    assert l1 <= L1_TOL, l1


@pytest.mark.parametrize("geom", ["spherical_1d", "cylindrical_2d", "cylindrical_plastic"])
def test_radial_source(geom):
    if geom == "spherical_1d":
        c = cases.sod_1d(ncells=400, max_grid_size=100, max_steps=300)
        c.lo_bc = [1, 0, 0]
    elif geom == "cylindrical_2d":
        c = cases.shock_bubble_2d(n=48, max_grid_size=24, max_steps=60, radius=0.3)
        c.lo_bc, c.hi_bc = [1, 1, 0], [1, 0, 0]
    else:
        c = cases.solid_mixture_2d(eos=cases.EOS_WILKINS, n=24, max_steps=10)
        c.lo_bc = [1, 0, 0]
    c.radial = 1
    l1, _, cfg = compare(c, c.max_steps)
    assert "binary32 per-direction" in cfg
    assert l1 <= L1_TOL, l1


@pytest.mark.parametrize("dim", [1, 2])
def test_mixture_and_reactive_update(dim):
    """MixtureEOS with the bisection closure in binary64 and the burn in binary32."""
    c = cases.reactive_charge(dim=dim, n=200 if dim == 1 else 48, max_grid_size=50 if dim == 1 else 16,
                              max_steps=120 if dim == 1 else 40)
    l1, _, cfg = compare(c, c.max_steps)
    assert "binary32 per-direction" in cfg
    assert l1 <= L1_TOL, l1
