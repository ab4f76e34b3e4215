"""The general reverse mode (tj_forward / tj_backward on configurations the
2-D fluid adjoint does not cover) against the tangent-linear run
(tj_tangent) of the same FP64 update: for seeded directions v of the initial
primitives and ve of the EOS parameters and a seeded objective gradient w on
the final carried words,

    <w, tangent(v, ve)> = <grad_prim0, v> + <grad_eos, ve>

must hold to rounding. Both differentiate the branches the FP64 run takes
(limiter, Riemann-solver sides, the yield test, clamps), so the identity is
exact whatever the directions -- white noise included. Cases: the 3-D copper
plate (5-wave solver, plastic radial return, cleanUpV, Hugoniot EOS), 2-D
solid/fluid mixtures with plasticity (Wilkins, Romenskii and Hugoniot
EOS), the 1-D shock tube, and the cylindrical and spherical radial source
with reflective axes."""
import numpy as np
import pytest
import torch

import fixtures as fx
from tenjin_gb300 import build, cases
from tenjin_gb300.adjoint import AdjointRun
from tenjin_gb300.host import carried_components

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


CASES = {
    "copper": (lambda: cases.copper_plate_3d(n=10, max_grid_size=10), 4, 2),
    "wilkins2d_plastic": (lambda: cases.solid_mixture_2d(eos=cases.EOS_WILKINS, n=16, max_steps=6), 6, 3),
    "sod_1d": (lambda: cases.sod_1d(ncells=120, max_grid_size=60), 12, 5),
    "wilkins2d_plastic_cylindrical": (lambda: fx.build_case("wilkins2d_plastic_cylindrical"), 5, 2),
    "sod_spherical_1d": (lambda: fx.build_case("sod_spherical_1d"), 10, 4),
    "romenskii2d_plastic": (lambda: fx.build_case("romenskii2d_plastic"), 5, 2),
    "hugoniot2d_plastic": (lambda: fx.build_case("hugoniot2d_plastic"), 5, 2),
    "romenskii3d_plastic_reflect": (lambda: fx.build_case("romenskii3d_plastic_reflect"), 4, 2),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_general_adjoint_equals_tangent(name):
    build_case, nsteps, stride = CASES[name]
    c = build_case()
    run = AdjointRun(c)
    dts = run.dt_schedule(nsteps)
    prim0 = np.ascontiguousarray(c.domains[0].prim)
    prim = torch.from_numpy(prim0).cuda()
    eos = run.eos_array()
    out = run.forward(prim, eos, dts, stride)
    rng = np.random.default_rng(11)
    carried = carried_components(c)
    w = np.zeros(run.shape_state)
    w[carried] = rng.standard_normal((len(carried),) + run.shape_state[1:])
    # scale each word's weight by its size so that every word counts
    scale = np.abs(out.cpu().numpy()).reshape(out.shape[0], -1).max(axis=1)
    w /= np.where(scale > 0, scale, 1.0)[:, None, None, None]
    gp, ge = run.backward(torch.from_numpy(w).cuda())
    gp = gp.cpu().numpy()
    errs = []
    for k in range(3):
        v = rng.standard_normal(prim0.shape) * np.abs(prim0) * 1e-3 + rng.standard_normal(prim0.shape) * 1e-6
        ve = np.zeros_like(eos)
        if k > 0:
            for m, mat in enumerate(c.materials):
                ve[m, :len(mat.params)] = rng.standard_normal(len(mat.params)) * np.abs(eos[m, :len(mat.params)]) * 1e-3
        _, ds = run.tangent(prim, torch.from_numpy(v).cuda(), eos, ve, dts)
        tl = float((w * ds.cpu().numpy()).sum())
        ad = float((gp * v).sum() + (ge * ve).sum())
        assert tl != 0.0 and np.isfinite(tl), tl
        errs.append(abs(tl - ad) / max(abs(tl), abs(ad)))
    run.close()
    assert np.count_nonzero(gp) > gp.size // 4
    assert max(errs) <= 1e-9, errs
