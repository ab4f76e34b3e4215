"""FP64 GPU path (through the C ABI) against the reference: the golden
fixtures made by the reference's own sources, and the oracle port on seeded
inputs. Tolerance: the FP64 path keeps the reference's evaluation order, so
results agree to 1e-12 relative (most values bit for bit; cosh/tanh/exp/pow
may differ from the host libm in the last bit)."""
import numpy as np
import pytest

import fixtures as fx
from oracle import port
from tenjin_gb300 import build, cases
from tenjin_gb300.host import FP64, TenjinGPU, carried_components

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()
    port.build_port()


def run_gpu(c, precision=FP64):
    g = TenjinGPU(c, precision)
    done, t = g.run(c.max_steps, c.final_t)
    states = [g.state(q) for q in range(len(c.domains))]
    return g, done, t, states


@pytest.mark.parametrize("name", fx.names())
def test_fp64_matches_reference_fixture(name):
    c = fx.build_case(name)
    gold = fx.load(name)
    g, done, t, states = run_gpu(c)
    assert done == len(gold["dts"])
    assert abs(t - float(np.sum(gold["dts"]))) <= TOL * max(abs(t), 1e-300) * len(gold["dts"])
    for q, st in enumerate(states):
        got = st[gold["carried"]]
        rd = fx.rel_diff(got, gold["states"][q])
        assert rd <= TOL, f"{name} domain {q}: max rel diff {rd:.3e}, exact {fx.exact_fraction(got, gold['states'][q]):.6f}"
    assert g.launch_count() > 0


def test_fp64_matches_port_on_perturbed_inputs():
    rng = np.random.default_rng(11)
    c = cases.shock_bubble_2d(n=40, max_grid_size=13, max_steps=25, radius=0.27)
    d = c.domains[0]
    d.prim[7] *= 1.0 + 0.05 * rng.standard_normal(d.prim[7].shape)
    d.prim[4] += 5.0 * rng.standard_normal(d.prim[4].shape)
    ref = port.run_port(c)
    g, done, t, states = run_gpu(c)
    idx = carried_components(c)
    assert done == len(ref["dts"])
    assert fx.rel_diff(states[0][idx], ref["states"][0][idx]) <= TOL


def test_operators_match_port_one_by_one():
    """getTimeStep, advance, cleanUpAlpha as separate calls (the reference's
    main loop driven from the host) reproduce the fused step."""
    c = fx.build_case("bubble32_muscl")
    c.max_steps = 3
    g = TenjinGPU(c)
    ref = port.run_port(c)
    for n in range(3):
        dt = g.getTimeStep()
        if n < 5:
            dt *= 0.2
        assert abs(dt - ref["dts"][n]) <= TOL * dt
        g.advance(dt)
        g.cleanUpAlpha()
        assert not g.contains_nan()
    idx = carried_components(c)
    assert fx.rel_diff(g.state(0)[idx], ref["states"][0][idx]) <= TOL


@pytest.mark.parametrize("name", ["sod_spherical_1d", "wilkins2d_plastic_cylindrical"])
def test_radial_operators_one_by_one(name):
    """The loop of main.cpp:121-191 with RADIAL driven from the host:
    getTimeStep, advance, plasticUpdate, geometricSourceTerm, cleanUpV,
    cleanUpAlpha, against the fused steps of the port."""
    c = fx.build_case(name)
    c.max_steps = 6
    g = TenjinGPU(c)
    ref = port.run_port(c)
    for n in range(c.max_steps):
        dt = g.getTimeStep()
        if n < 5:
            dt *= 0.2
        assert abs(dt - ref["dts"][n]) <= TOL * dt
        g.advance(dt)
        if c.plastic:
            g.plasticUpdate(dt)
        g.geometricSourceTerm(dt)
        if c.solid:
            g.cleanUpV()
        g.cleanUpAlpha()
    idx = carried_components(c)
    assert fx.rel_diff(g.state(0)[idx], ref["states"][0][idx]) <= TOL


def test_reactive_operators_one_by_one():
    """getTimeStep, advance, reactiveUpdate, cleanUpAlpha as separate calls
    reproduce the port's steps on the MixtureEOS charge."""
    c = fx.build_case("reactive_charge_1d")
    c.max_steps = 8
    g = TenjinGPU(c)
    ref = port.run_port(c)
    for n in range(c.max_steps):
        dt = g.getTimeStep()
        if n < 5:
            dt *= 0.2
        assert abs(dt - ref["dts"][n]) <= TOL * dt
        g.advance(dt)
        g.reactiveUpdate(dt)
        g.cleanUpAlpha()
    idx = carried_components(c)
    assert fx.rel_diff(g.state(0)[idx], ref["states"][0][idx]) <= TOL


@pytest.mark.parametrize("name", ["bubble48_thinc_uneven", "copper12"])
def test_advance_stages_equal_advance(name):
    """tj_advance_stage(0) then (1) gives tj_advance bit for bit; the state
    after stage 0 differs from both."""
    c = fx.build_case(name)
    g1, g2 = TenjinGPU(c), TenjinGPU(c)
    dt = g1.getTimeStep() * 0.2
    g1.advance(dt)
    g2.advance_stage(0, dt)
    mid = g2.state(0)
    g2.advance_stage(1, dt)
    a, b = g1.state(0), g2.state(0)
    idx = carried_components(c)
    assert np.array_equal(a[idx], b[idx])
    assert not np.array_equal(mid[idx], a[idx])


def test_fab_exchange_roundtrip_keeps_ghosts():
    c = cases.shock_bubble_2d(n=24, max_grid_size=10, max_steps=1)
    g = TenjinGPU(c)
    full = g.state(0)
    ng = 2
    rng = np.random.default_rng(3)
    for b, box in enumerate(c.domains[0].boxes):
        nx, ny = box[3] - box[0] + 1, box[4] - box[1] + 1
        fab = rng.standard_normal((g.ncomp, 1, ny + 2 * ng, nx + 2 * ng))
        ghosts = fab.copy()
        g.download_fab(0, b, fab, ng)
        valid = fab[:, :, ng:ng + ny, ng:ng + nx]
        np.testing.assert_array_equal(valid, full[:, :, box[1]:box[4] + 1, box[0]:box[3] + 1])
        mask = np.ones(fab.shape, bool)
        mask[:, :, ng:ng + ny, ng:ng + nx] = False
        np.testing.assert_array_equal(fab[mask], ghosts[mask])
        g.upload_fab(0, b, fab, ng)
    np.testing.assert_array_equal(g.state(0), full)


def test_nan_injected_on_host_stops_the_loop():
    """A NaN written into the host state before upload (no device fault) is
    reported as TJ_ERR_NAN after the step, like main.cpp:183-187."""
    from tenjin_gb300._lib import TjError
    c = cases.shock_bubble_2d(n=16, max_grid_size=16, max_steps=4, thinc=0)
    g = TenjinGPU(c)
    st = g.state(0)
    st[3 * c.M + 8, 0, 8, 8] = np.nan   # pressure of one cell
    g.set_state(0, st)
    with pytest.raises(TjError) as e:
        g.run(4, 1e300)
    assert e.value.code == -3


def test_volume_fraction_error_is_reported():
    """alpha = (NaN, 0): the NaN is zeroed without being recorded (the
    reference cannot record material 0, boxaccesscellarray.cpp:553-556), the
    sum is 0 and the reference's 'Error in scaling volume fractions' exit
    (:583-588) becomes TJ_ERR_ALPHA."""
    from tenjin_gb300._lib import TjError
    c = cases.shock_bubble_2d(n=16, max_grid_size=16, max_steps=1, thinc=0)
    g = TenjinGPU(c)
    st = g.state(0)
    st[0, 0, 3, 3] = np.nan
    st[1, 0, 3, 3] = 0.0
    g.set_state(0, st)
    with pytest.raises(TjError) as e:
        g.cleanUpAlpha()
    assert e.value.code == -5


def test_cleanup_alpha_two_nans_quirk():
    """alpha = (NaN, NaN) with two materials is not an error in the reference:
    material 1 is recorded as the NaN one and set to 1 - sum = 1."""
    c = cases.shock_bubble_2d(n=16, max_grid_size=16, max_steps=1, thinc=0)
    g = TenjinGPU(c)
    st = g.state(0)
    st[0, 0, 3, 3] = np.nan
    st[1, 0, 3, 3] = np.nan
    st[0, 0, 5, 5] = -0.5
    st[1, 0, 5, 5] = 1.5
    g.set_state(0, st)
    g.cleanUpAlpha()
    out = g.state(0)
    assert out[0, 0, 3, 3] == 0.0 and out[1, 0, 3, 3] == 1.0
    tot = 1e-6 + 1.0
    assert out[0, 0, 5, 5] == 1e-6 * (1.0 / tot) and out[1, 0, 5, 5] == 1.0 * (1.0 / tot)
