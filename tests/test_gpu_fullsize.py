"""The benchmark workloads at their full sizes and over their full step
counts, checked through properties that do not need the oracle (which cannot
run them in seconds): agreement of the binary32 paths with the binary64 paths
on the same inputs, the same step count and time, finite states, and mass
conservation where no mass crosses the boundary.

The accuracy bar of the binary32 paths, along the whole run: at every sample
the relative L1 density difference against the reference-ordered binary64
path is at most 1e-4, or -- once the flow itself amplifies last-bit
differences beyond that -- at most twice the binary64 floor, the larger of
(a) the difference between two exact binary64 evaluation orders (fused64 vs
fp64) and (b) the difference that a 1e-14 relative perturbation of the
initial pressure grows to in the binary64 path."""
import numpy as np
import pytest

from tenjin_gb300 import accuracy, build, cases
from tenjin_gb300.host import FP64, FUSED64, MIXED, TenjinGPU

pytestmark = pytest.mark.gpu
L1_TOL = 1e-4


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def density(g, c):
    return np.concatenate([g.state(q)[c.M:2 * c.M].sum(axis=0).ravel() for q in range(len(c.domains))])


def l1(a, b):
    return np.abs(a - b).sum() / np.abs(b).sum()


def test_bubble_1024_mixed_against_fused64():
    """Config 2 workload, 1024^2 with THINC, 200 steps."""
    c = cases.shock_bubble_2d(n=1024, max_grid_size=128, max_steps=200)
    g64 = TenjinGPU(c, FUSED64)
    d64, t64 = g64.run(200, 1e300)
    g32 = TenjinGPU(c, MIXED)
    d32, t32 = g32.run(200, 1e300)
    assert d64 == d32 == 200
    assert abs(t32 - t64) <= 1e-5 * t64
    r32 = density(g32, c)
    assert np.all(np.isfinite(r32))
    assert l1(r32, density(g64, c)) <= L1_TOL


def test_bubble_1024_quiet_mass_conserved():
    """1024^2 with no shock and a pressure jump inside the domain: nothing
    reaches the transmissive boundary, each material's mass is conserved."""
    c = cases.shock_bubble_2d(n=1024, max_grid_size=128, max_steps=100, shock_x=-1.0)
    d = c.domains[0]
    d.prim[7] = np.where(d.prim[1] > 0.5, 3.0e5, d.prim[7])
    g = TenjinGPU(c, MIXED)
    s0 = g.state(0)
    g.run(100, 1e300)
    s1 = g.state(0)
    for m in range(c.M):
        assert abs(s1[c.M + m].sum() - s0[c.M + m].sum()) / abs(s0[c.M + m].sum()) < 1e-6


def _gate(curves):
    ok, ratio, i = accuracy.floor_gate(curves)
    assert ok, (f"L1 {curves['pairs']['mixed_vs_fp64']['l1'][i]:.3e} at step {curves['steps'][i]} is "
                f"{ratio:.2f} x its bound")


def test_bubble_512_whole_run_within_the_binary64_floor():
    """The config 2 setup at 512^2 over all 2000 steps, sampled every 50."""
    c = cases.shock_bubble_2d(n=512, max_grid_size=64)
    runs, pairs = accuracy.plan("bubble", c)
    curves = accuracy.density_curves(c, runs, pairs, 2000, 50)
    _gate(curves)


def test_uneven_boxes_whole_run_within_1e4():
    """The config 4 workload at 1024 boxes over all 100 steps, every 10."""
    c = cases.uneven_boxes_3d(nbox=1024)
    runs, pairs = accuracy.plan("boxes", c)
    curves = accuracy.density_curves(c, runs, pairs, 100, 10)
    assert max(curves["pairs"]["mixed_vs_fp64"]["l1"]) <= L1_TOL, curves["pairs"]["mixed_vs_fp64"]["l1"]
    _gate(curves)


def test_copper_128_whole_run_within_1e4():
    """The config 3 workload at 128^3 over all 500 steps, every 50."""
    c = cases.copper_plate_3d(n=128)
    runs, pairs = accuracy.plan("copper", c)
    curves = accuracy.density_curves(c, runs, pairs, 500, 50)
    assert max(curves["pairs"]["mixed_vs_fp64"]["l1"]) <= L1_TOL, curves["pairs"]["mixed_vs_fp64"]["l1"]


def test_uneven_boxes_4096_mixed_against_fp64():
    """Config 4 workload at its full size: 4096 boxes, 7.9e7 cells, 3 steps."""
    c = cases.uneven_boxes_3d()
    g64 = TenjinGPU(c, FP64)
    d64, t64 = g64.run(3, 1e300)
    sample = range(0, len(c.domains), 16)
    r64 = np.concatenate([g64.state(q)[c.M:2 * c.M].sum(axis=0).ravel() for q in sample])
    g64.close()
    g32 = TenjinGPU(c, MIXED)
    d32, t32 = g32.run(3, 1e300)
    r32 = np.concatenate([g32.state(q)[c.M:2 * c.M].sum(axis=0).ravel() for q in sample])
    assert d64 == d32 == 3
    assert abs(t32 - t64) <= 1e-5 * t64
    assert np.all(np.isfinite(r32))
    assert l1(r32, r64) <= L1_TOL


def test_copper_256_mixed_against_fp64():
    """Config 3 workload at its full size: copper plate 256^3, plastic, 3 steps."""
    c = cases.copper_plate_3d(n=256)
    g64 = TenjinGPU(c, FP64)
    d64, t64 = g64.run(3, 1e300)
    r64 = density(g64, c)
    g64.close()
    g32 = TenjinGPU(c, MIXED)
    d32, t32 = g32.run(3, 1e300)
    r32 = density(g32, c)
    assert d64 == d32 == 3
    assert abs(t32 - t64) <= 1e-5 * t64
    assert np.all(np.isfinite(r32))
    assert l1(r32, r64) <= L1_TOL
