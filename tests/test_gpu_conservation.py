"""Binary64 conservation sums on the device (tj_conservation_sums) and the
single-component download (tj_download_component).

The sums are checked against the same sums formed on the host from the
reference's own final states (golden fixtures) and from the oracle port; the
reduction order is fixed, so two calls on one state give the same bits; on a
problem whose boundaries no wave reaches, the total partial masses stay
constant to round-off over the run, in binary64 and in the binary32 path."""
import numpy as np
import pytest

import fixtures as fx
from oracle import port
from tenjin_gb300 import build, cases
from tenjin_gb300.host import FP64, MIXED, TenjinGPU

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()
    port.build_port()


def host_sums(c, states):
    """The sums of tj_conservation_sums from AccessPattern states on the host
    (alphaRho_k, rhoU, E are components M..2M-1, 3M+1..3M+3, 3M+7)."""
    M = c.M
    out = np.zeros(M + 4)
    for d, st in zip(c.domains, states):
        dv = float(np.prod([d.dim_l[k] / d.n_cells[k] for k in range(c.dim)]))
        for m in range(M):
            out[m] += st[M + m].sum() * dv
        for r in range(3):
            out[M + r] += st[3 * M + 1 + r].sum() * dv
        out[M + 3] += st[3 * M + 7].sum() * dv
    return out


def close(a, b, tol):
    scale = np.maximum(np.abs(b), 1e-300)
    # momentum sums of symmetric problems are near zero: compare them to the
    # size of the largest momentum component instead
    return np.all(np.abs(a - b) <= tol * np.maximum(scale, np.abs(b).max() * 1e-3))


@pytest.mark.parametrize("name", ["bubble64_thinc", "copper12", "uneven3d_4dom"])
def test_sums_match_reference_fixture_states(name):
    c = fx.build_case(name)
    gold = fx.load(name)
    g = TenjinGPU(c, FP64)
    g.run(c.max_steps, c.final_t)
    got = g.conservation_sums()
    again = g.conservation_sums()
    # the golden fixtures hold the carried components; expand them back into
    # AccessPattern planes for the host sums
    carried = gold["carried"]
    full = []
    for d, st in zip(c.domains, gold["states"]):
        a = np.zeros((g.ncomp,) + st.shape[1:])
        a[carried] = st
        full.append(a)
    ref = host_sums(c, full)
    g.close()
    assert np.array_equal(got, again), "the reduction order must be fixed"
    assert close(got, ref, 1e-13), (got, ref)


def test_sums_match_port_and_mixed_agrees():
    c = cases.shock_bubble_2d(n=96, max_grid_size=48, max_steps=30)
    ref = host_sums(c, port.run_port(c)["states"])
    g = TenjinGPU(c, FP64)
    g.run(c.max_steps, c.final_t)
    got = g.conservation_sums()
    g.close()
    assert close(got, ref, 1e-13), (got, ref)
    g32 = TenjinGPU(c, MIXED)
    g32.run(c.max_steps, c.final_t)
    got32 = g32.conservation_sums()
    g32.close()
    assert close(got32, ref, 1e-5), (got32, ref)


@pytest.mark.parametrize("precision,tol", [(FP64, 1e-12), (MIXED, 1e-6)])
def test_partial_masses_conserved_with_quiet_boundaries(precision, tol):
    """An over-pressured air bubble in water at rest, run for fewer steps than
    its waves need to reach the boundary: no mass crosses it."""
    c = cases.shock_bubble_2d(n=256, max_grid_size=128, max_steps=40, radius=0.15, shock_x=-1.0)
    d = c.domains[0]
    d.prim[7] = np.where(d.prim[1] > 0.5, 3.0e5, d.prim[7])
    g = TenjinGPU(c, precision)
    s0 = g.conservation_sums()
    g.run(c.max_steps, c.final_t)
    s1 = g.conservation_sums()
    g.close()
    M = c.M
    assert np.all(np.abs(s1[:M] - s0[:M]) <= tol * np.abs(s0[:M])), (s0[:M], s1[:M])
    assert abs(s1[M + 3] - s0[M + 3]) <= tol * abs(s0[M + 3])


@pytest.mark.parametrize("precision", [FP64, MIXED])
def test_component_download_equals_the_full_download(precision):
    c = cases.shock_bubble_2d(n=64, max_grid_size=32, max_steps=5)
    g = TenjinGPU(c, precision)
    g.run(c.max_steps, c.final_t)
    full = g.state(0)
    for comp in range(g.ncomp):
        assert np.array_equal(g.component(0, comp), full[comp]), comp
    assert np.array_equal(g.density(0), full[3 * c.M])
    g.close()
