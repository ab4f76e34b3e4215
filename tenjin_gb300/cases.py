"""Synthetic workloads for the Tenjin per-timestep update.

Each builder returns a :class:`Case`: solver parameters (mirroring the fields
of the reference's ``ParameterStruct``, structdefinitions.h:105-144, and the
material list read by ``getMaterialParameters``, initialise.cpp:125-235) plus
one or more independent domains, each holding its box list and the initial
*primitive* state. The primitive fields are, in order:

    alpha[M], rho_k[M], u[3], p, V[9] (SOLID only), epsilon[M] (PLASTIC only)

which is exactly what ``initial_conditions`` writes before
``primitiveToConservative`` (initialise.cpp:20-109).

Equation-of-state parameter vectors follow ``getMaterialParameters``:
    MieGruneisen (stiffened form) : [gamma, pref, eref, CV]
    RomenskiiSolid                : [gamma, pref, eref, CV, rho0, K0, alpha, beta, G0]
    WilkinsSolid                  : [gamma, pref, eref, CV, rho0, e1..e5, G0]
    HugoniotSolid (copper; no reference class): [gamma, pref, eref, CV, rho0, c0, s, G0]
with the stiffened-gas mapping Gamma = gamma-1, pref = -gamma*p_inf, eref = 0.

The workloads are seeded synthetic stand-ins for the reference's benchmark
configurations (no external dataset is involved).
"""
from __future__ import annotations

import dataclasses
import math
from typing import List, Optional

import numpy as np

EOS_MIEGRUNEISEN = 0
EOS_ROMENSKII = 1
EOS_WILKINS = 2
EOS_HUGONIOT = 3
EOS_MIXTURE = 4   # two stiffened gases blended by the mass fraction lambda

PHASE_SOLID = 0
PHASE_FLUID = 1

BC_TRANSMISSIVE = 0
BC_REFLECTIVE = 1


@dataclasses.dataclass
class Material:
    phase: int
    eos: int
    params: List[float]
    yield_stress: float = 0.0


@dataclasses.dataclass
class Domain:
    n_cells: List[int]            # [nx, ny, nz] (unused dims = 1)
    dim_l: List[float]            # physical lengths
    boxes: List[List[int]]        # [[lox,loy,loz,hix,hiy,hiz], ...] in MFIter order
    prim: np.ndarray              # (nprim, nz, ny, nx) float64

    @property
    def ncells(self) -> int:
        return int(np.prod(self.n_cells))


@dataclasses.dataclass
class Case:
    name: str
    dim: int
    materials: List[Material]
    solid: int = 0
    thinc: int = 0
    plastic: int = 0
    muscl: int = 1
    radial: int = 0               # RADIAL: geometric source term, x the radius
    reactive: int = 0             # REACTIVE: reactiveUpdate of the mixture's mass fraction
    nghost: int = 2
    lo_bc: List[int] = dataclasses.field(default_factory=lambda: [0, 0, 0])
    hi_bc: List[int] = dataclasses.field(default_factory=lambda: [0, 0, 0])
    cfl: float = 0.5
    thinc_beta: float = 1.6
    final_t: float = 1e300
    max_steps: int = 1 << 30
    domains: List[Domain] = dataclasses.field(default_factory=list)

    @property
    def M(self) -> int:
        return len(self.materials)

    @property
    def nmix(self) -> int:
        """numberOfMixtures: the materials with the MixtureEOS (material 0 only)."""
        return sum(1 for m in self.materials if m.eos == EOS_MIXTURE)

    @property
    def nprim(self) -> int:
        """Primitive input rows: alpha[M], rho_k[M], u[3], p, V[9] (solid),
        epsilon[M] (plastic), lambda (mixture)."""
        return 2 * self.M + 4 + (9 if self.solid else 0) + (self.M if self.plastic else 0) + self.nmix

    @property
    def total_cells(self) -> int:
        return sum(d.ncells for d in self.domains)


# ---------------------------------------------------------------------------
# Box decomposition: AMReX BoxList::maxSize (power-of-two factoring, near-equal
# pieces chopped from the high end, one direction after another).
# ---------------------------------------------------------------------------

def max_size_boxes(n_cells, dim, max_grid_size):
    boxes = [[0, 0, 0, n_cells[0] - 1, n_cells[1] - 1, n_cells[2] - 1]]
    for d in range(dim):
        out = []
        for b in boxes:
            b = list(b)
            length = b[3 + d] - b[d] + 1
            if length > max_grid_size:
                ratio, bs, nlen = 1, max_grid_size, length
                while bs % 2 == 0 and nlen % 2 == 0:
                    ratio *= 2
                    bs //= 2
                    nlen //= 2
                numblk = nlen // bs + (1 if nlen % bs else 0)
                sz, ex = nlen // numblk, nlen % numblk
                for k in range(numblk - 1):
                    ksize = sz + 1 if k < ex else sz
                    pos = b[3 + d] - ksize * ratio + 1
                    upper = list(b)
                    upper[d] = pos
                    b[3 + d] = pos - 1
                    out.append(upper)
            out.append(b)
        boxes = out
    return boxes


def _stiffened(gamma, p_inf):
    return [gamma, -gamma * p_inf, 0.0, 1.0]


def _empty_prim(case: Case, n_cells):
    return np.zeros((case.nprim, n_cells[2], n_cells[1], n_cells[0]), dtype=np.float64)


# ---------------------------------------------------------------------------
# Config 1: 1-D two-material Sod tube.
# ---------------------------------------------------------------------------

def sod_1d(ncells: int = 1000, max_grid_size: int = 1000, final_t: float = 0.2,
           max_steps: int = 1 << 30, eps: float = 1e-6) -> Case:
    """Sod tube, ideal gas gamma=1.4 on both sides; alpha = (1-eps, eps) left of
    x=0.5 and (eps, 1-eps) right of it (exact 0/1 would divide by zero in
    rho_k = alphaRho/alpha, boxaccesscellarray.cpp:84; eps is the reference's
    own clamp value, boxaccesscellarray.cpp:566)."""
    mats = [Material(PHASE_FLUID, EOS_MIEGRUNEISEN, [1.4, 0.0, 0.0, 1.0]),
            Material(PHASE_FLUID, EOS_MIEGRUNEISEN, [1.4, 0.0, 0.0, 1.0])]
    c = Case("sod_1d", 1, mats, cfl=0.5, final_t=final_t, max_steps=max_steps)
    n = [ncells, 1, 1]
    prim = _empty_prim(c, n)
    x = (np.arange(ncells) + 0.5) / ncells
    left = x < 0.5
    prim[0, 0, 0] = np.where(left, 1 - eps, eps)
    prim[1, 0, 0] = np.where(left, eps, 1 - eps)
    prim[2, 0, 0] = np.where(left, 1.0, 0.125)
    prim[3, 0, 0] = np.where(left, 1.0, 0.125)
    prim[7, 0, 0] = np.where(left, 1.0, 0.1)
    c.domains = [Domain(n, [1.0, 1.0, 1.0], max_size_boxes(n, 1, max_grid_size), prim)]
    return c


# ---------------------------------------------------------------------------
# Config 2 / 5: 2-D water shock hitting an air bubble.
# ---------------------------------------------------------------------------

WATER_GAMMA, WATER_PINF, WATER_RHO = 4.4, 6.0e8, 1000.0
AIR_GAMMA, AIR_RHO = 1.4, 1.2
AMBIENT_P = 1.0e5


def stiffened_shock_state(mach, rho1, p1, gamma, p_inf):
    """Post-shock state behind a right-moving shock of Mach `mach` (relative to
    the quiescent pre-shock sound speed) in a stiffened gas: the ideal-gas
    Rankine-Hugoniot relations with p replaced by p + p_inf."""
    a1 = math.sqrt(gamma * (p1 + p_inf) / rho1)
    m2 = mach * mach
    p2 = (p1 + p_inf) * (1.0 + 2.0 * gamma / (gamma + 1.0) * (m2 - 1.0)) - p_inf
    rho2 = rho1 * (gamma + 1.0) * m2 / ((gamma - 1.0) * m2 + 2.0)
    s = mach * a1
    u2 = s * (1.0 - rho1 / rho2)
    return rho2, u2, p2


def smooth_field(rng, n: int, modes: int = 4) -> np.ndarray:
    """A seeded smooth field on an n x n grid: the mean of `modes` products of
    sines with wavenumbers 1..4 and random phases and amplitudes (order 1)."""
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x, indexing="xy")
    f = np.zeros((n, n))
    for _ in range(modes):
        kx, ky = rng.integers(1, 5, 2)
        f += rng.standard_normal() * np.sin(2 * np.pi * (kx * X + rng.uniform())) * \
            np.sin(2 * np.pi * (ky * Y + rng.uniform()))
    return f / modes


def shock_bubble_2d(n: int = 1024, seed: int = 0, max_grid_size: int = 128, max_steps: int = 2000,
                    thinc: int = 1, cfl: float = 0.4, beta: float = 1.6, eps: float = 1e-6,
                    radius: float = 0.2, shock_x: float = 0.2, mach: float = 1.5,
                    background: float = 0.0) -> Case:
    """background > 0 multiplies rho_k (both materials) and p by 1 + background
    * (a seeded smooth field), varies the air volume fraction by background *
    field * alpha_air * alpha_water (so that both fractions stay in (0, 1)) and
    adds 10 background m/s smooth fields to both velocity components: no
    region of the initial state is then exactly uniform (the MUSCL limiter is
    not differentiable at a uniform state; gradient checks need this
    variant)."""
    mats = [Material(PHASE_FLUID, EOS_MIEGRUNEISEN, _stiffened(WATER_GAMMA, WATER_PINF)),
            Material(PHASE_FLUID, EOS_MIEGRUNEISEN, _stiffened(AIR_GAMMA, 0.0))]
    c = Case("shock_bubble_2d", 2, mats, thinc=thinc, cfl=cfl, thinc_beta=beta, max_steps=max_steps)
    rng = np.random.Generator(np.random.PCG64(seed))
    cx, cy = 0.5 + rng.uniform(-0.05, 0.05, size=2)
    nn = [n, n, 1]
    prim = _empty_prim(c, nn)
    xc = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(xc, xc, indexing="xy")  # X[j, i] = x_i
    bubble = (X - cx) ** 2 + (Y - cy) ** 2 < radius * radius
    rho2, u2, p2 = stiffened_shock_state(mach, WATER_RHO, AMBIENT_P, WATER_GAMMA, WATER_PINF)
    shocked = X < shock_x
    a_air = np.where(bubble, 1.0 - eps, eps)
    prim[0, 0] = 1.0 - a_air
    prim[1, 0] = a_air
    prim[2, 0] = np.where(shocked, rho2, WATER_RHO)
    prim[3, 0] = AIR_RHO
    prim[4, 0] = np.where(shocked, u2, 0.0)
    prim[7, 0] = np.where(shocked, p2, AMBIENT_P)
    if background > 0.0:
        for q in (2, 3, 7):
            prim[q, 0] *= 1.0 + background * smooth_field(rng, n)
        # volume fractions: a variation proportional to alpha_air alpha_water
        # keeps both inside (0, 1)
        a_air = prim[1, 0] + background * smooth_field(rng, n) * prim[1, 0] * prim[0, 0]
        prim[1, 0], prim[0, 0] = a_air, 1.0 - a_air
        prim[4, 0] += 10.0 * background * smooth_field(rng, n)
        prim[5, 0] += 10.0 * background * smooth_field(rng, n)
    c.domains = [Domain(nn, [1.0, 1.0, 1.0], max_size_boxes(nn, 2, max_grid_size), prim)]
    return c


# ---------------------------------------------------------------------------
# Parity workload for the MixtureEOS and the reactive update: a condensed
# explosive (reactant/products mixture, material 0) next to air.
# ---------------------------------------------------------------------------

EXPL_REACTANT = [2.5, -2.5 * 1.0e7, 4.0e6, 1500.0]   # [gamma, pref, eref, CV]: stiffened, p_inf 1e7
EXPL_PRODUCTS = [1.4, 0.0, 0.0, 1000.0]
EXPL_RHO = 1600.0


def reactive_charge(dim: int = 1, n: int = 200, length: float = 0.1, max_grid_size: int = 64,
                    max_steps: int = 60, reactive: int = 1, thinc: int = 0, seed: int = 0,
                    eps: float = 1e-6, products: Optional[List[float]] = None, reactant: Optional[List[float]] = None,
                    ambient_p: float = 1.0e8, air_rho: float = 100.0) -> Case:
    """Explosive (MixtureEOS: reactant and products, lambda = reactant mass
    fraction) filling x < length/2 in 1-D (a disc of radius 0.3 length about the
    centre in 2-D), compressed air elsewhere, all at ambient_p (the
    pressure-based rate raises p to the power 1.2, reactive.cpp:19, so
    p must stay positive); a hot spot at 2 GPa (x < length/10, or a
    disc of radius 0.08 length) starts the pressure-based burn of
    reactive.cpp:3-26 when `reactive`. Lambda is 1 - 5e-4 except for a
    seeded partly-burnt patch (lambda in (0.2, 0.9)) that sends the closure
    through the bisection of equationofstate.cpp:274-376 from the first step."""
    mats = [Material(PHASE_FLUID, EOS_MIXTURE, list(reactant or EXPL_REACTANT) + list(products or EXPL_PRODUCTS)),
            Material(PHASE_FLUID, EOS_MIEGRUNEISEN, _stiffened(AIR_GAMMA, 0.0))]
    c = Case(f"reactive_charge_{dim}d", dim, mats, thinc=thinc, reactive=reactive, cfl=0.4, max_steps=max_steps)
    rng = np.random.Generator(np.random.PCG64(seed))
    nn = [n, n if dim > 1 else 1, 1]
    prim = _empty_prim(c, nn)
    xc = (np.arange(n) + 0.5) / n
    if dim == 1:
        X = xc[None, :]
        charge = X < 0.5
        hot = X < 0.1
        patch = (X > 0.2) & (X < 0.3)
    else:
        X, Y = np.meshgrid(xc, xc, indexing="xy")
        r2 = (X - 0.5) ** 2 + (Y - 0.5) ** 2
        charge = r2 < 0.09
        hot = r2 < 0.0064
        patch = (np.abs(X - 0.5) < 0.1) & (Y > 0.62) & (Y < 0.72)
    a0 = np.where(charge, 1.0 - eps, eps)
    prim[0, 0] = a0
    prim[1, 0] = 1.0 - a0
    prim[2, 0] = EXPL_RHO
    prim[3, 0] = air_rho
    prim[7, 0] = np.where(hot, 2.0e9, ambient_p)
    # unburnt lambda = 1 - 5e-4: at lambda = 1 exactly defineMixtureDensities
    # (equationofstate.cpp:390-396) gives rhomix_1 = 0/0 and the energy of the
    # reconstructed states NaN
    lam = np.full(a0.shape, 1.0 - 5e-4)
    lam[patch] = rng.uniform(0.2, 0.9, size=int(patch.sum()))
    prim[c.nprim - 1, 0] = lam
    L = [length, length if dim > 1 else 1.0, 1.0]
    c.domains = [Domain(nn, L, max_size_boxes(nn, dim, max_grid_size), prim)]
    return c


# ---------------------------------------------------------------------------
# Config 3: 3-D elastoplastic copper plate impact.
# ---------------------------------------------------------------------------

CU_RHO0, CU_C0, CU_S, CU_GAMMA0 = 8930.0, 3940.0, 1.49, 2.0
CU_G, CU_Y = 45.0e9, 90.0e6


def hugoniot_pressure(rho, rho0=CU_RHO0, c0=CU_C0, s=CU_S):
    eta = 1.0 - rho0 / rho
    return rho0 * c0 * c0 * eta / (1.0 - s * eta) ** 2


# CFL number of the 3-D workloads. The update is unsplit (every direction's
# flux difference is taken from the same stage-input state, hllc.cpp:579-695)
# and SSP-RK2 in time; where the limiter falls back to first order (at every
# local extremum, so for the odd-even mode of cell-to-cell noise) the scheme
# damps that mode only while the Courant numbers of the three directions sum
# to at most 1: with CFL * min(dx / (a + |u|)) that is CFL <= 1/3 in a region
# at rest. At 0.4 the batch of water/air boxes grows an odd-even pressure mode
# from its 1e4 Pa cell noise to +-8e6 Pa within 40 steps, in binary64.
CFL_3D = 0.3


def copper_plate_3d(n: int = 256, seed: int = 0, max_grid_size: int = 64, max_steps: int = 500,
                    cfl: float = CFL_3D, length: float = 0.01, u_flyer: float = 400.0, pert: float = 0.01) -> Case:
    mats = [Material(PHASE_SOLID, EOS_HUGONIOT, [CU_GAMMA0 + 1.0, 0.0, 0.0, 1.0, CU_RHO0, CU_C0, CU_S, CU_G],
                     yield_stress=CU_Y)]
    c = Case("copper_plate_3d", 3, mats, solid=1, plastic=1, cfl=cfl, max_steps=max_steps)
    rng = np.random.Generator(np.random.PCG64(seed))
    nn = [n, n, n]
    prim = _empty_prim(c, nn)
    rho = CU_RHO0 * (1.0 + pert * rng.standard_normal((n, n, n)))
    x = (np.arange(n) + 0.5) * length / n
    prim[0] = 1.0                                  # alpha
    prim[1] = rho                                  # rho_k
    prim[2] = np.where(x[None, None, :] < 0.5 * length, u_flyer, 0.0)
    prim[5] = hugoniot_pressure(rho)               # zero thermal part
    for r in range(3):                             # V = I
        prim[6 + 3 * r + r] = 1.0
    c.domains = [Domain(nn, [length] * 3, max_size_boxes(nn, 3, max_grid_size), prim)]
    return c


# ---------------------------------------------------------------------------
# Config 4: batch of independent uneven 3-D boxes.
# ---------------------------------------------------------------------------

def uneven_boxes_3d(nbox: int = 4096, seed: int = 0, lo: int = 8, hi: int = 64, dx: float = 1e-3,
                    max_steps: int = 100, cfl: float = CFL_3D, eps: float = 1e-6) -> Case:
    mats = [Material(PHASE_FLUID, EOS_MIEGRUNEISEN, _stiffened(WATER_GAMMA, WATER_PINF)),
            Material(PHASE_FLUID, EOS_MIEGRUNEISEN, _stiffened(AIR_GAMMA, 0.0))]
    c = Case("uneven_boxes_3d", 3, mats, cfl=cfl, max_steps=max_steps)
    rng = np.random.Generator(np.random.PCG64(seed))
    doms = []
    for _ in range(nbox):
        nn = [int(round(math.exp(rng.uniform(math.log(lo), math.log(hi))))) for _ in range(3)]
        prim = _empty_prim(c, nn)
        normal = rng.standard_normal(3)
        normal /= np.linalg.norm(normal)
        centre = rng.uniform(0.0, 1.0, size=3) * np.array(nn) * dx
        z, y, x = np.meshgrid(*[(np.arange(k) + 0.5) * dx for k in nn[::-1]], indexing="ij")
        dist = (x - centre[0]) * normal[0] + (y - centre[1]) * normal[1] + (z - centre[2]) * normal[2]
        a0 = 0.5 * (1.0 + np.tanh(dist / dx))
        a0 = eps + (1.0 - 2.0 * eps) * a0
        prim[0] = a0
        prim[1] = 1.0 - a0
        prim[2] = WATER_RHO
        prim[3] = AIR_RHO
        prim[7] = AMBIENT_P * (1.0 + 0.1 * rng.uniform(0.0, 1.0, size=(nn[2], nn[1], nn[0])))
        doms.append(Domain(nn, [k * dx for k in nn], [[0, 0, 0, nn[0] - 1, nn[1] - 1, nn[2] - 1]], prim))
    c.domains = doms
    return c


# ---------------------------------------------------------------------------
# Parity workload: 2-D solid/fluid mixture with plasticity (any solid EOS).
# ---------------------------------------------------------------------------

def solid_mixture_2d(eos: int = EOS_WILKINS, n: int = 20, max_steps: int = 8, seed: int = 1,
                     max_grid_size: int = 8, yield_stress: float = 3e8) -> Case:
    """Solid (left half) against an ideal gas (right half) with a shear
    perturbation of V and a moving flyer region; exercises the 5-wave solver,
    the Hencky closure, the radial return and cleanUpV."""
    if eos == EOS_WILKINS:
        K, r0 = 7.6e10, 2785.0
        prm = [3.0, 0.0, 0.0, 1.0, r0, 0.0, K / 2.0, 0.0, 0.0, 0.0, 2.76e10]
    elif eos == EOS_ROMENSKII:
        prm = [3.0, 0.0, 0.0, 1.0, 8930.0, 1.37e11, 1.0, 3.0, 4.6e10]
    else:
        prm = [CU_GAMMA0 + 1.0, 0.0, 0.0, 1.0, CU_RHO0, CU_C0, CU_S, CU_G]
    mats = [Material(PHASE_SOLID, eos, prm, yield_stress),
            Material(PHASE_FLUID, EOS_MIEGRUNEISEN, [1.4, 0.0, 0.0, 1.0])]
    c = Case(f"solid_mixture_2d_eos{eos}", 2, mats, solid=1, plastic=1, cfl=0.4, max_steps=max_steps)
    rng = np.random.Generator(np.random.PCG64(seed))
    prim = np.zeros((c.nprim, 1, n, n))
    a = np.full((n, n), 1 - 1e-6)
    a[:, n // 2:] = 1e-6
    prim[0, 0] = a
    prim[1, 0] = 1 - a
    prim[2, 0] = prm[4] * (1 + 0.01 * rng.standard_normal((n, n)))
    prim[3, 0] = 1.2
    prim[4, 0] = np.where(np.arange(n)[None, :] < n // 3, 300.0, 0.0)
    prim[5, 0] = 50.0 * rng.standard_normal((n, n))
    prim[7, 0] = 1e5 + 1e7 * rng.uniform(size=(n, n))
    V = np.eye(3)[:, :, None, None] + 0.01 * rng.standard_normal((3, 3, n, n))
    for r in range(3):
        for q in range(3):
            prim[8 + 3 * r + q, 0] = V[r, q]
    nn = [n, n, 1]
    c.domains = [Domain(nn, [0.01, 0.01, 1.0], max_size_boxes(nn, 2, max_grid_size), prim)]
    return c


def solid_mixture_3d(eos: int = EOS_WILKINS, n: int = 10, max_steps: int = 6, seed: int = 1,
                     max_grid_size: int = 5, yield_stress: float = 3e8, cfl: float = CFL_3D) -> Case:
    """The 2-D solid/gas mixture in 3-D: solid for x < L/2 against an ideal
    gas, a flyer region moving along x, random transverse velocities along y
    and z and a shear perturbation of V; two materials through the 5-wave
    solver, the Hencky closure, the radial return and cleanUpV along all
    three directions."""
    base = solid_mixture_2d(eos=eos, n=4, max_steps=max_steps, seed=seed, yield_stress=yield_stress)
    c = Case(f"solid_mixture_3d_eos{eos}", 3, base.materials, solid=1, plastic=1, cfl=cfl, max_steps=max_steps)
    prm = base.materials[0].params
    rng = np.random.Generator(np.random.PCG64(seed))
    prim = np.zeros((c.nprim, n, n, n))
    x = np.arange(n)[None, None, :]
    a = np.where(x < n // 2, 1 - 1e-6, 1e-6) * np.ones((n, n, n))
    prim[0] = a
    prim[1] = 1 - a
    prim[2] = prm[4] * (1 + 0.01 * rng.standard_normal((n, n, n)))
    prim[3] = 1.2
    prim[4] = np.where(x < n // 3, 300.0, 0.0) * np.ones((n, n, n))
    prim[5] = 50.0 * rng.standard_normal((n, n, n))
    prim[6] = 50.0 * rng.standard_normal((n, n, n))
    prim[7] = 1e5 + 1e7 * rng.uniform(size=(n, n, n))
    V = np.eye(3)[:, :, None, None, None] + 0.01 * rng.standard_normal((3, 3, n, n, n))
    for r in range(3):
        for q in range(3):
            prim[8 + 3 * r + q] = V[r, q]
    nn = [n, n, n]
    c.domains = [Domain(nn, [0.01, 0.01, 0.01], max_size_boxes(nn, 3, max_grid_size), prim)]
    return c


def fluid_boxes_3d(n: int = 12, max_grid_size: int = 5, max_steps: int = 5, seed: int = 0,
                   cfl: float = CFL_3D) -> Case:
    """One 3-D water/air domain split into several boxes (MUSCL only)."""
    c = uneven_boxes_3d(nbox=1, lo=n, hi=n, max_steps=max_steps, seed=seed, cfl=cfl)
    d = c.domains[0]
    d.boxes = max_size_boxes(d.n_cells, 3, max_grid_size)
    c.name = "fluid_boxes_3d"
    return c
