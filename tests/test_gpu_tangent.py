"""Tangent-linear runs (tj_tangent): the FP64 path's per-direction kernels
instantiated with values that carry one direction.

* The values are the FP64 path's, bit for bit: against tj_forward on the 2-D
  THINC interface problem and against a plain FP64 run with the same dt
  schedule on the 3-D copper plate (5-wave solver, plastic radial return,
  cleanUpV).
* The directions are derivatives: against central differences of the same
  run on the copper plate (initial density and velocity fields, EOS
  parameters), and against the adjoint (tj_backward) on the interface
  problem, where <grad_state, dstate> = <grad_prim0, dprim0> + <grad_eos,
  deos> must hold to rounding for every direction -- also on the problem as
  stated, without the smooth background, where central differences cannot
  check the adjoint (the limiter and the THINC choice are not differentiable
  at exactly uniform states, but both runs take the same branches)."""
import numpy as np
import pytest
import torch

import fixtures as fx
from tenjin_gb300 import build, cases
from tenjin_gb300.adjoint import AdjointRun
from tenjin_gb300.host import FP64, TenjinGPU, carried_components

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def copper(n=12, steps=8):
    c = cases.copper_plate_3d(n=n, max_grid_size=n, max_steps=steps)
    return c


def smooth3(rng, n):
    """A seeded smooth field on an n^3 grid (mean of products of sines)."""
    x = (np.arange(n) + 0.5) / n
    Z, Y, X = np.meshgrid(x, x, x, indexing="ij")
    f = np.zeros((n, n, n))
    for _ in range(3):
        k = rng.integers(1, 4, 3)
        f += rng.standard_normal() * np.sin(2 * np.pi * (k[0] * X + rng.uniform())) * \
            np.sin(2 * np.pi * (k[1] * Y + rng.uniform())) * np.sin(2 * np.pi * (k[2] * Z + rng.uniform()))
    return f / 3


def copper_smooth(n=12, steps=8, seed=7):
    """The copper plate with a smooth background on the velocity and on V
    (relative 1e-3): no exactly uniform region, where the MUSCL limiter has no
    derivative and central differences of white-noise directions do not
    converge to one."""
    c = copper(n, steps)
    rng = np.random.default_rng(seed)
    p = c.domains[0].prim
    for r in range(3):
        p[2 + r] = p[2 + r] + 0.4 * smooth3(rng, n)
    for q in range(9):
        p[6 + q] = p[6 + q] + 1e-3 * smooth3(rng, n)
    return c


def plain_run(c, nsteps):
    g = TenjinGPU(c, FP64)
    dts = []
    for _ in range(nsteps):
        g.step()
        dts.append(g.time()[2])
    st = g.state(0)
    g.close()
    return st, np.array(dts)


def test_values_equal_a_plain_fp64_run_bitwise_copper():
    c = copper()
    st, dts = plain_run(c, 8)
    run = AdjointRun(c)
    prim = torch.from_numpy(np.ascontiguousarray(c.domains[0].prim)).cuda()
    val, dval = run.tangent(prim, None, run.eos_array(), None, dts, want_state=True)
    run.close()
    carried = carried_components(c)
    assert np.array_equal(val.cpu().numpy()[carried], st[carried])
    assert not dval.abs().sum().item()  # no direction, no derivative


def interface(n=48, background=1e-3):
    return cases.shock_bubble_2d(n=n, max_grid_size=24, thinc=1, background=background)


def test_values_equal_tj_forward_bitwise_interface():
    c = interface()
    run = AdjointRun(c)
    dts = run.dt_schedule(30)
    prim = torch.from_numpy(np.ascontiguousarray(c.domains[0].prim)).cuda()
    out = run.forward(prim, run.eos_array(), dts, 10).cpu().numpy()
    val, _ = run.tangent(prim, None, run.eos_array(), None, dts, want_state=True)
    run.close()
    carried = carried_components(c)
    assert np.array_equal(val.cpu().numpy()[carried], out[carried])


def test_tangent_matches_central_differences_copper():
    """A weighted sum of the final carried words along seeded smooth
    directions of the initial densities, velocities and V, and of the copper
    EOS parameters (rho0, c0, s, G0): central differences with relative step
    1e-6, on the copper plate with a smooth background."""
    c = copper_smooth(n=12, steps=8)
    _, dts = plain_run(c, 8)
    run = AdjointRun(c)
    prim0 = np.ascontiguousarray(c.domains[0].prim)
    prim = torch.from_numpy(prim0).cuda()
    eos = run.eos_array()
    rng = np.random.default_rng(3)
    n = c.domains[0].n_cells[0]
    carried = carried_components(c)
    w = np.zeros(run.shape_state)
    w[carried] = rng.standard_normal((len(carried),) + run.shape_state[1:])
    M = c.M
    errs = []
    for k in range(4):
        v = np.zeros_like(prim0)
        ve = np.zeros_like(eos)
        if k < 2:  # smooth directions of the densities, velocities and V
            for m in range(M):
                v[M + m] = smooth3(rng, n) * prim0[M + m] * 1e-2
            for r in range(3):
                v[2 * M + r] = smooth3(rng, n) * 10.0
            for q in range(9):
                v[2 * M + 4 + q] = smooth3(rng, n) * 1e-3
        else:  # rho0, c0, s, G0 of the Hugoniot EOS
            ve[:, 4:8] = rng.standard_normal((M, 4)) * eos[:, 4:8] * 1e-2
        _, ds = run.tangent(prim, torch.from_numpy(v).cuda(), eos, ve, dts)
        tl = float((w * ds.cpu().numpy()).sum())
        h = 1e-6
        sp, _ = run.tangent(torch.from_numpy(prim0 + h * v).cuda(), None, eos + h * ve, None, dts, want_state=True)
        sm, _ = run.tangent(torch.from_numpy(prim0 - h * v).cuda(), None, eos - h * ve, None, dts, want_state=True)
        fd = float((w * (sp.cpu().numpy() - sm.cpu().numpy())).sum()) / (2 * h)
        errs.append(abs(fd - tl) / max(abs(fd), abs(tl)))
    run.close()
    assert max(errs) <= 1e-5, errs


@pytest.mark.parametrize("background", [1e-3, 0.0], ids=["background", "as_stated"])
def test_adjoint_equals_tangent(background):
    c = interface(n=48, background=background)
    M = c.M
    run = AdjointRun(c)
    dts = run.dt_schedule(30)
    prim0 = np.ascontiguousarray(c.domains[0].prim)
    prim = torch.from_numpy(prim0).cuda()
    eos = run.eos_array()
    out = run.forward(prim, eos, dts, 10)
    rng = np.random.default_rng(5)
    gs = torch.zeros_like(out)
    gs[M:2 * M] = torch.from_numpy(rng.standard_normal((1,) + tuple(out.shape[1:]))).cuda()
    gp, ge = run.backward(gs)
    gp = gp.cpu().numpy()
    gsn = gs.cpu().numpy()
    errs = []
    for _ in range(6):
        v = np.zeros_like(prim0)
        for m in range(M):
            v[M + m, 0] = cases.smooth_field(rng, c.domains[0].n_cells[0]) * prim0[M + m, 0]
        v[2 * M:2 * M + 2] = rng.standard_normal(v[2 * M:2 * M + 2].shape)
        ve = np.zeros_like(eos)
        ve[:, 0:2] = rng.standard_normal((M, 2)) * eos[:, 0:2]
        _, ds = run.tangent(prim, torch.from_numpy(v).cuda(), eos, ve, dts)
        tl = float((gsn * ds.cpu().numpy()).sum())
        ad = float((gp * v).sum() + (ge * ve).sum())
        errs.append(abs(tl - ad) / max(abs(tl), abs(ad)))
    run.close()
    assert max(errs) <= 1e-9, errs


@pytest.mark.parametrize("name,precision,why", [
    ("uneven3d_4dom", "fp64", "one domain"),
    ("reactive_charge_1d", "fp64", "no mixtures"),
    ("copper12", "mixed", "runs the FP64 path"),
])
def test_tangent_refuses_what_it_does_not_cover(name, precision, why):
    from tenjin_gb300 import _lib
    from tenjin_gb300.host import MIXED
    c = fx.build_case(name)
    run = AdjointRun(c)
    if precision == "mixed":
        run.sim.close()
        run.sim = TenjinGPU(c, MIXED, set_initial=False)
    prim = torch.from_numpy(np.ascontiguousarray(c.domains[0].prim[:c.nprim - c.nmix])).cuda()
    with pytest.raises(_lib.TjError, match=why):
        run.tangent(prim, None, run.eos_array(), None, np.full(2, 1e-9))
    run.close()


def test_general_adjoint_refuses_thinc():
    from tenjin_gb300 import _lib
    c = fx.build_case("sod_thinc_1d")
    run = AdjointRun(c)
    prim = torch.from_numpy(np.ascontiguousarray(c.domains[0].prim)).cuda()
    with pytest.raises(_lib.TjError, match="BVD-THINC"):
        run.forward(prim, run.eos_array(), np.full(2, 1e-9), 1)
    run.close()
