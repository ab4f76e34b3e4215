"""Host-side helpers of the precision comparison and the adjoint, and the
case builders they use, without a GPU: the perturbation and binary32 rounding
of an initial state, the floor criterion on synthetic curves, the runs a
comparison plans, the stiffened-gas parameter rows and the density misfit of
the adjoint problem, and the 3-D solid/gas mixture builder."""
import numpy as np
import pytest
import torch

from tenjin_gb300 import accuracy, cases
from tenjin_gb300.adjoint import MAX_EOS, density_misfit, eos_vector


def test_perturbed_changes_only_the_pressure_by_at_most_eps():
    c = cases.shock_bubble_2d(n=16, max_grid_size=16)
    p = accuracy.perturbed(c, eps=1e-14, seed=3)
    a, b = c.domains[0].prim, p.domains[0].prim
    ip = 2 * c.M + 3
    others = [k for k in range(a.shape[0]) if k != ip]
    assert np.array_equal(a[others], b[others])
    rel = np.abs(b[ip] / a[ip] - 1.0)
    assert rel.max() <= 1e-14 * (1 + 1e-2) and rel.max() > 0
    # the original case is left as it was
    assert np.array_equal(c.domains[0].prim, cases.shock_bubble_2d(n=16, max_grid_size=16).domains[0].prim)


def test_rounded_to_binary32_is_exactly_representable():
    c = cases.copper_plate_3d(n=6, max_grid_size=6)
    r = accuracy.rounded_to_binary32(c)
    x = r.domains[0].prim
    assert np.array_equal(x, x.astype(np.float32).astype(np.float64))
    assert np.max(np.abs(x - c.domains[0].prim) / np.maximum(np.abs(c.domains[0].prim), 1e-300)) <= 2 ** -24


def curves(mixed, floors):
    pairs = {"mixed_vs_fp64": {"l1": mixed, "linf": mixed}}
    for k, v in floors.items():
        pairs[k] = {"l1": v, "linf": v}
    return {"steps": [100 * (i + 1) for i in range(len(mixed))], "pairs": pairs}


def test_floor_gate_takes_the_largest_floor_at_each_sample():
    c = curves([5e-5, 3e-4, 9e-4], {"fused64_vs_fp64": [1e-6, 2e-4, 3e-4], "fp64_pert_vs_fp64": [1e-6, 1e-4, 5e-4]})
    ok, ratio, i = accuracy.floor_gate(c)
    # bounds: max(1e-4, 2 x floor) = 1e-4, 4e-4, 1e-3
    assert ok and i == 2 and ratio == pytest.approx(0.9)
    c = curves([5e-5, 5e-4, 9e-4], {"fused64_vs_fp64": [1e-6, 2e-4, 3e-4]})
    ok, ratio, i = accuracy.floor_gate(c)
    # bounds 1e-4, 4e-4, 6e-4: ratios 0.5, 1.25, 1.5
    assert not ok and i == 2 and ratio == pytest.approx(1.5)
    # without any floor pair the bound is the absolute tolerance
    ok, ratio, i = accuracy.floor_gate(curves([2e-4], {}))
    assert not ok and ratio == pytest.approx(2.0)


def test_summarise_reports_every_pair_and_the_gate():
    c = curves([5e-5, 3e-4], {"fused64_vs_fp64": [1e-6, 2e-4]})
    s = accuracy.summarise(c)
    assert s["mixed_vs_fp64"]["l1_final"] == 3e-4 and s["mixed_vs_fp64"]["l1_max"] == 3e-4
    assert s["gate"]["passes"] and s["gate"]["at_step"] == 200


def test_plan_runs_and_pairs():
    c = cases.shock_bubble_2d(n=16, max_grid_size=16)
    runs, pairs = accuracy.plan("bubble", c)
    assert set(runs) == {"fp64", "mixed", "fp64_pert", "fp64_f32", "fused64"}
    assert ("fused64", "fp64") in pairs and ("mixed", "fused64") in pairs
    runs, pairs = accuracy.plan("copper", cases.copper_plate_3d(n=6, max_grid_size=6))
    assert "fused64" not in runs and ("mixed", "fp64") in pairs


def test_eos_vector_rows():
    g = torch.tensor([4.4, 1.4], dtype=torch.float64)
    pinf = torch.tensor([6e8, 0.0], dtype=torch.float64)
    rest = torch.tensor([[0.0, 1.0], [0.0, 1.0]], dtype=torch.float64)
    e = eos_vector(g, pinf, rest)
    assert e.shape == (2, MAX_EOS)
    assert torch.equal(e[:, 0], g) and torch.equal(e[:, 1], -g * pinf)
    assert torch.count_nonzero(e[:, 4:]) == 0


def test_density_misfit_and_its_gradient():
    M = 2
    state = torch.rand(26, 1, 4, 4, dtype=torch.float64, requires_grad=True)
    target = torch.rand(1, 4, 4, dtype=torch.float64)
    J = density_misfit(state, target, M, 0.25)
    rho = state[M:2 * M].sum(dim=0)
    assert J.detach().item() == pytest.approx(0.5 * float(((rho.detach() - target) ** 2).sum()) * 0.25)
    J.backward()
    g = state.grad
    assert torch.allclose(g[M], (rho - target).detach() * 0.25) and torch.allclose(g[M + 1], g[M])
    assert torch.count_nonzero(g[:M]) == 0 and torch.count_nonzero(g[2 * M:]) == 0


@pytest.mark.parametrize("eos", [cases.EOS_WILKINS, cases.EOS_ROMENSKII, cases.EOS_HUGONIOT])
def test_solid_mixture_3d_builder(eos):
    c = cases.solid_mixture_3d(eos=eos, n=8, max_grid_size=4)
    d = c.domains[0]
    assert c.dim == 3 and c.M == 2 and c.solid and c.plastic
    assert d.prim.shape == (c.nprim, 8, 8, 8)
    a = d.prim[0]
    assert np.all((a > 0) & (a < 1)) and np.allclose(d.prim[0] + d.prim[1], 1.0)
    V = d.prim[8:17].reshape(3, 3, 8, 8, 8)
    assert np.abs(V - np.eye(3)[:, :, None, None, None]).max() < 0.1
    assert len(d.boxes) == 8
    # seeded: the same call gives the same fields
    assert np.array_equal(d.prim, cases.solid_mixture_3d(eos=eos, n=8, max_grid_size=4).domains[0].prim)
