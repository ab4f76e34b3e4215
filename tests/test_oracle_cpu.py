"""The oracle (the CPU port of oracle/port/) against the golden fixtures made
by the reference's own sources, and against independent checks."""
import os

import numpy as np
import pytest

import fixtures as fx
import exact_riemann as er
from oracle import port, refio
from tenjin_gb300 import cases


@pytest.fixture(scope="module", autouse=True)
def _built():
    port.build_port()


@pytest.mark.parametrize("name", fx.names())
def test_fixture_inputs_are_reproducible(name):
    c = fx.build_case(name)
    assert fx.prim_sha(c) == fx.manifest()[name]["prim_sha256"]


@pytest.mark.parametrize("name", fx.names())
def test_port_bit_exact_against_reference_fixture(name):
    c = fx.build_case(name)
    gold = fx.load(name)
    out = port.run_port(c)
    np.testing.assert_array_equal(out["dts"], gold["dts"])
    for q, st in enumerate(out["states"]):
        got = st[gold["carried"]]
        assert fx.exact_fraction(got, gold["states"][q]) == 1.0, f"domain {q}: max rel diff {fx.rel_diff(got, gold['states'][q])}"


def test_sod_matches_exact_riemann_solution():
    gold = fx.load("sod1000_full")
    c = fx.build_case("sod1000_full")
    M = c.M
    rho = gold["states"][0][gold["carried"].index(3 * M)][0, 0]
    x = (np.arange(1000) + 0.5) / 1000
    re, ue, pe = er.sample(x, 0.2, 0.5, 1.0, 0.0, 1.0, 0.125, 0.0, 0.1)
    assert abs(float(np.sum(gold["dts"])) - 0.2) < 1e-14
    assert np.mean(np.abs(rho - re)) < 2e-3


def test_planted_mistake_is_caught():
    """A wrong CFL number in the oracle must break the bit-exact comparison."""
    c = fx.build_case("sod200_boxes")
    c.cfl = 0.5 * (1 + 1e-12)
    gold = fx.load("sod200_boxes")
    out = port.run_port(c)
    assert not np.array_equal(out["dts"], gold["dts"])


def test_mass_conservation_quiet_boundaries():
    """An over-pressured bubble in water at rest: until the waves reach the
    walls no mass crosses the boundary, so each total alphaRho is conserved to
    round-off (the interior update is conservative, hllc.cpp:493-523)."""
    c = cases.shock_bubble_2d(n=32, max_grid_size=16, max_steps=10, radius=0.2, shock_x=-1.0)
    d = c.domains[0]
    d.prim[7] = np.where(d.prim[1] > 0.5, 3.0e5, d.prim[7])
    sim = port.PortSim(c)
    st0 = sim.state(0)
    out = sim.run()
    st1 = out["states"][0]
    M = c.M
    for m in range(M):
        m0, m1 = st0[M + m].sum(), st1[M + m].sum()
        assert abs(m1 - m0) / abs(m0) < 1e-11


@pytest.mark.skipif(not refio.have_ref(2), reason="reference binaries are built only where the reference tree exists")
def test_port_matches_live_reference_random_inputs():
    rng = np.random.default_rng(7)
    c = cases.shock_bubble_2d(n=24, max_grid_size=9, max_steps=12, radius=0.25)
    d = c.domains[0]
    d.prim[7] *= 1.0 + 0.05 * rng.standard_normal(d.prim[7].shape)
    r = refio.run_reference(c)
    p = port.run_port(c)
    np.testing.assert_array_equal(r["dts"], p["dts"])
    assert fx.exact_fraction(p["states"][0], r["states"][0]) == 1.0


# Fixtures whose arithmetic needs no transcendental result whose last bit
# matters (no THINC jump, no pow/log in the EOS along their trajectory): the
# reference linked against the host's own libm reproduces them bit for bit, so
# the project-written exp/cosh/tanh/pow/log that both sides use for parity do
# not decide these results.
STOCK_EXACT = ["boxes3d_walls", "bubble32_muscl", "bubble3_tiny", "bubble4_reflect_boxes2", "copper10_reflect", "copper12",
               "fluid3d_boxes", "fluid3d_reflect", "hugoniot2d_plastic", "mixture_closed_form_2d", "sod1000_full",
               "sod200_boxes", "sod3_tiny", "sod_spherical_1d", "uneven3d_4dom", "wilkins2d_plastic_cylindrical"]


@pytest.mark.skipif(not refio.have_ref(3, stock=True),
                    reason="the stock-libm reference binaries are built only where the reference tree exists")
@pytest.mark.parametrize("name", STOCK_EXACT)
def test_stock_libm_reference_reproduces_fixture(name):
    c = fx.build_case(name)
    gold = fx.load(name)
    r = refio.run_reference(c, stock=True)
    np.testing.assert_array_equal(r["dts"], gold["dts"])
    for q, st in enumerate(r["states"]):
        assert fx.exact_fraction(st[gold["carried"]], gold["states"][q]) == 1.0


def _random_config(seed):
    """A small seeded configuration with random walls and a perturbed
    initial pressure, beyond the fixtures' settings: 3-D solid/gas mixtures,
    the copper plate, 2-D solids with the radial source, uneven 3-D boxes,
    THINC in 1-D and 2-D, the reactive MixtureEOS in 1-D (radial) and 2-D
    (THINC)."""
    rng = np.random.default_rng(100 + seed)
    walls = lambda: [int(x) for x in rng.integers(0, 2, 3)]
    if seed == 0:
        c = cases.solid_mixture_3d(eos=cases.EOS_ROMENSKII, n=6, max_grid_size=3, max_steps=4)
    elif seed == 1:
        c = cases.copper_plate_3d(n=8, max_grid_size=4, max_steps=4)
    elif seed == 2:
        c = cases.solid_mixture_2d(eos=cases.EOS_HUGONIOT, n=12, max_steps=6)
        c.radial = 1
    elif seed == 3:
        c = cases.uneven_boxes_3d(nbox=3, lo=5, hi=9, max_steps=4, seed=int(rng.integers(1000)))
    elif seed == 4:
        c = cases.shock_bubble_2d(n=20, max_grid_size=7, max_steps=10, radius=0.3)
    elif seed == 5:
        c = cases.sod_1d(ncells=60, max_grid_size=17, max_steps=40)
        c.thinc = 1
    elif seed == 6:
        c = cases.reactive_charge(dim=2, n=16, max_grid_size=6, max_steps=8, thinc=1)
    elif seed == 7:
        c = cases.reactive_charge(dim=1, n=60, max_grid_size=13, max_steps=30)
        c.radial = 1
    elif seed == 8:
        c = cases.solid_mixture_2d(eos=cases.EOS_ROMENSKII, n=12, max_steps=6)
        c.radial = 1
    else:
        c = cases.solid_mixture_3d(eos=cases.EOS_WILKINS, n=6, max_grid_size=4, max_steps=4)
    c.lo_bc, c.hi_bc = walls(), walls()
    if c.radial:
        c.lo_bc[0] = 1
    ip = 2 * c.M + 3
    for d in c.domains:
        d.prim[ip] *= 1.0 + 0.02 * rng.standard_normal(d.prim[ip].shape)
    return c


@pytest.mark.parametrize("seed", range(10))
def test_port_matches_live_reference_random_configs(seed):
    c = _random_config(seed)
    if not refio.have_ref(c.dim):
        pytest.skip("reference binaries are built only where the reference tree exists")
    r = refio.run_reference(c)
    p = port.run_port(c)
    np.testing.assert_array_equal(r["dts"], p["dts"])
    for q in range(len(c.domains)):
        assert fx.exact_fraction(p["states"][q], r["states"][q]) == 1.0
