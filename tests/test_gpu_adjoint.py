"""Adjoint pair tj_forward / tj_backward on the 2-D water/air interface
problem: the forward with a frozen dt schedule reproduces the FP64 path bit
for bit, the gradients are independent of the checkpoint stride, and they
match central finite differences of the same forward.

The base state carries a seeded smooth background variation (amplitude 1e-3):
at an exactly uniform state the MUSCL limiter has no derivative (the slope of
a perturbation v is minmod(dv), not linear in v), so finite differences there
measure something no adjoint returns. Directions are smooth seeded fields.
The directional derivative is linear in the direction, so each direction is
checked as the sum of its partial-density part and its EOS part, each with
its own step: central differences along the partial densities straddle the
limiter kinks (r = 1) of cells whose margin is below the step, an error that
falls with the step (1e-8 here); along the EOS parameters the state moves
smoothly and the step is the usual 1e-6 (smaller steps only add rounding).
"""
import numpy as np
import pytest
import torch

from tenjin_gb300 import build, cases
from tenjin_gb300.adjoint import AdjointRun, TenjinRun, density_misfit, eos_vector
from tenjin_gb300.host import FP64, TenjinGPU

pytestmark = pytest.mark.gpu
STEP_RHO = 1e-8   # relative step along the partial-density fields
STEP_EOS = 1e-6   # relative step along (gamma, p_ref)
FD_TOL = 1e-5


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def small_case(n=48, thinc=1, reflect=False, background=1e-3):
    c = cases.shock_bubble_2d(n=n, max_grid_size=n // 2, thinc=thinc, radius=0.25, background=background)
    if reflect:
        c.lo_bc, c.hi_bc = [1, 1, 0], [1, 1, 0]
    return c


def test_forward_is_the_fp64_path_bitwise():
    c = small_case(background=0.0)
    g = TenjinGPU(c, FP64)
    dts = []
    for _ in range(25):
        g.step()
        dts.append(g.time()[2])
    ref = g.state(0)
    run = AdjointRun(c)
    prim = torch.from_numpy(np.ascontiguousarray(c.domains[0].prim)).cuda()
    out = run.forward(prim, run.eos_array(), np.array(dts), 7).cpu().numpy()
    assert np.array_equal(out, ref)


def _setup(c, nsteps, stride, seed=3):
    run = AdjointRun(c)
    dts = run.dt_schedule(nsteps)
    prim = torch.from_numpy(np.ascontiguousarray(c.domains[0].prim)).cuda()
    out = run.forward(prim, run.eos_array(), dts, stride)
    M = c.M
    rng = np.random.default_rng(seed)
    rho = out[M:2 * M].sum(dim=0)
    target = rho * torch.from_numpy(1 + 0.01 * rng.standard_normal(tuple(rho.shape))).cuda()
    return run, dts, prim, target


def _J(run, prim, eos, dts, target, M, area):
    out = run.forward(prim, eos, dts, 1 << 20)
    return float(density_misfit(out, target, M, area))


def _fd_errors(c, nsteps, stride, kinds, ndir, seed=11):
    M = c.M
    d = c.domains[0]
    n = d.n_cells[0]
    area = (d.dim_l[0] / d.n_cells[0]) * (d.dim_l[1] / d.n_cells[1])
    run, dts, prim, target = _setup(c, nsteps, stride)
    eos = run.eos_array()
    # adjoint gradient through the autograd contract
    prim_t = prim.clone().requires_grad_(True)
    eos_t = torch.from_numpy(eos).requires_grad_(True)
    state = TenjinRun.apply(prim_t, eos_t, run, dts, stride)
    density_misfit(state, target, M, area).backward()
    gp = prim_t.grad.cpu().numpy()
    ge = eos_t.grad.numpy()
    rng = np.random.default_rng(seed)
    prim0 = prim.cpu().numpy()

    def central(v, ve, h):
        Jp = _J(run, torch.from_numpy(prim0 + h * v).cuda(), eos + h * ve, dts, target, M, area)
        Jm = _J(run, torch.from_numpy(prim0 - h * v).cuda(), eos - h * ve, dts, target, M, area)
        return (Jp - Jm) / (2 * h)

    errs = []
    for _ in range(ndir):
        fd = ad = 0.0
        if "rho_k" in kinds:
            v = np.zeros_like(prim0)
            for m in range(M):
                v[M + m, 0] = cases.smooth_field(rng, n) * prim0[M + m, 0]
            fd += central(v, np.zeros_like(eos), STEP_RHO)
            ad += float((gp * v).sum())
        if "eos" in kinds:
            ve = np.zeros_like(eos)
            ve[:, 0:2] = rng.standard_normal((M, 2)) * eos[:, 0:2]
            fd += central(np.zeros_like(prim0), ve, STEP_EOS)
            ad += float((ge * ve).sum())
        if "u" in kinds or "p" in kinds:
            v = np.zeros_like(prim0)
            if "u" in kinds:
                v[2 * M, 0] = 10 * cases.smooth_field(rng, n)
                v[2 * M + 1, 0] = 10 * cases.smooth_field(rng, n)
            if "p" in kinds:
                v[2 * M + 3, 0] = cases.smooth_field(rng, n) * prim0[2 * M + 3, 0]
            fd += central(v, np.zeros_like(eos), STEP_RHO)
            ad += float((gp * v).sum())
        errs.append(abs(fd - ad) / max(abs(fd), abs(ad)))
    run.close()
    return errs


@pytest.mark.parametrize("thinc,reflect", [(1, False), (0, True), (1, True)])
def test_gradient_matches_central_differences(thinc, reflect):
    # the inputs of the objective: initial partial densities and (gamma, p_ref)
    errs = _fd_errors(small_case(thinc=thinc, reflect=reflect), 30, 9, ("rho_k", "eos"), 4)
    assert max(errs) <= FD_TOL, errs


def test_velocity_and_pressure_gradients():
    # more kinks are crossed along u and p (HLLC side and wave-speed maxima of
    # near-equal face states); the bound is looser
    errs = _fd_errors(small_case(), 30, 9, ("u", "p"), 3)
    assert max(errs) <= 1e-4, errs


def test_gradient_independent_of_checkpoint_stride():
    c = small_case()
    nsteps = 30
    run, dts, prim, target = _setup(c, nsteps, 1)
    M = c.M
    res = []
    for stride in (1, 7, nsteps):
        out = run.forward(prim, run.eos_array(), dts, stride)
        rho = out[M:2 * M].sum(dim=0)
        gs = torch.zeros_like(out)
        gs[M:2 * M] = (rho - target).unsqueeze(0)
        gp, ge = run.backward(gs)
        res.append((gp.cpu().numpy(), ge))
    for gp, ge in res[1:]:
        assert np.array_equal(gp, res[0][0]) and np.array_equal(ge, res[0][1])


def test_gamma_pinf_gradient_through_torch():
    # EOS parameters keep a uniform state uniform: no background needed
    c = small_case(n=32, background=0.0)
    nsteps, M = 20, c.M
    d = c.domains[0]
    area = (d.dim_l[0] / d.n_cells[0]) ** 2
    run, dts, prim, target = _setup(c, nsteps, 5)
    gamma = torch.tensor([cases.WATER_GAMMA, cases.AIR_GAMMA], dtype=torch.float64, requires_grad=True)
    pinf = torch.tensor([cases.WATER_PINF, 0.0], dtype=torch.float64, requires_grad=True)
    rest = torch.tensor(run.eos_array()[:, 2:4])

    def J_of(g, p):
        e = eos_vector(g, p, rest)
        st = TenjinRun.apply(prim, e, run, dts, 5)
        return density_misfit(st, target, M, area)

    J_of(gamma, pinf).backward()
    with torch.no_grad():
        for which, vec, grad in (("gamma", gamma, gamma.grad), ("pinf", pinf, pinf.grad)):
            h = STEP_EOS * float(vec[0])
            e = torch.zeros_like(vec)
            e[0] = h
            Jp = float(J_of(gamma + e if which == "gamma" else gamma, pinf + e if which == "pinf" else pinf))
            Jm = float(J_of(gamma - e if which == "gamma" else gamma, pinf - e if which == "pinf" else pinf))
            fd = (Jp - Jm) / (2 * h)
            assert abs(fd - float(grad[0])) <= FD_TOL * max(abs(fd), 1e-300), (which, fd, float(grad[0]))
