"""Host-side mirror of the reference's operator surface over libtenjin_gpu.so.

The reference drives its update from main.cpp:121-191 through free functions
and CellArray methods. :class:`TenjinGPU` exposes the same operators under the
same names, on state held on the GPU:

    reference (file:line)                                   here
    ------------------------------------------------------  ---------------------------
    TimeStep::getTimeStep(U1, parameters)  timestep.cpp:36   getTimeStep()
    advance(U, U1, U2, ...)                hllc.cpp:699      advance(dt)
    PlasticEOS::plasticUpdate(U1, ...)     plastic.cpp:227   plasticUpdate(dt)
    CellArray::cleanUpV()                  cellarray.h:27    cleanUpV()
    CellArray::cleanUpAlpha()              cellarray.h:28    cleanUpAlpha()
    CellArray::conservativeToPrimitive()   cellarray.h:25    conservativeToPrimitive()
    CellArray::primitiveToConservative()   cellarray.h:24    primitiveToConservative()
    CellArray::contains_nan()              cellarray.h:33    contains_nan()
    main.cpp time loop (one iteration)     main.cpp:121-191  step(t_end)

Errors the reference reports with Print + exit(1) raise :class:`TjError`.
State is exchanged in the reference's layout (AccessPattern component order,
component-major, i fastest).
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import _lib
from .cases import Case

FP64 = _lib.TJ_PRECISION_FP64
MIXED = _lib.TJ_PRECISION_MIXED
FUSED64 = _lib.TJ_PRECISION_FUSED64


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_params(case: Case, precision: int = FP64) -> _lib.TjParams:
    p = _lib.TjParams()
    p.dim, p.n_materials, p.n_mixtures = case.dim, case.M, case.nmix
    p.SOLID, p.THINC, p.RADIAL, p.PLASTIC, p.REACTIVE, p.MUSCL = (case.solid, case.thinc, case.radial,
                                                                  case.plastic, case.reactive, case.muscl)
    p.nghost = case.nghost
    for d in range(3):
        p.lo_bc[d], p.hi_bc[d] = case.lo_bc[d], case.hi_bc[d]
    p.CFL, p.THINCbeta, p.precision = case.cfl, case.thinc_beta, precision
    for m, mat in enumerate(case.materials):
        p.materials[m].phase, p.materials[m].eos = mat.phase, mat.eos
        p.materials[m].nparams = len(mat.params)
        for q, v in enumerate(mat.params):
            p.materials[m].params[q] = v
        p.materials[m].yield_stress = mat.yield_stress
    return p


class TenjinGPU:
    """One GPU context holding every domain of a :class:`Case`."""

    def __init__(self, case: Case, precision: int = FP64, set_initial: bool = True):
        self.L = _lib.load()
        self.case = case
        self.precision = precision
        self._p = make_params(case, precision)
        h = ctypes.c_void_p()
        rc = self.L.tj_create(ctypes.byref(self._p), ctypes.byref(h))
        if rc != 0:
            raise _lib.TjError(rc, "tj_create refused the parameters")
        self.h = h
        nd = len(case.domains)
        ncells = (ctypes.c_int * (3 * nd))(*[v for d in case.domains for v in d.n_cells])
        diml = (ctypes.c_double * (3 * nd))(*[v for d in case.domains for v in d.dim_l])
        self._check(self.L.tj_set_domains(self.h, nd, ncells, diml))
        for q, d in enumerate(case.domains):
            flat = [v for b in d.boxes for v in b]
            arr = (ctypes.c_int * len(flat))(*flat)
            self._check(self.L.tj_set_boxes(self.h, q, len(d.boxes), arr))
        self.ncomp = self.L.tj_ncomp(self.h)
        if set_initial:
            for q, d in enumerate(case.domains):
                self.set_primitive(q, d.prim)

    # -- plumbing -------------------------------------------------------------
    def _check(self, rc):
        if rc != 0:
            buf = ctypes.create_string_buffer(512)
            self.L.tj_last_error(self.h, buf, 512)
            raise _lib.TjError(rc, buf.value.decode())
        return rc

    def close(self):
        if getattr(self, "h", None):
            self.L.tj_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- state exchange ---------------------------------------------------------
    def set_primitive(self, q: int, prim: np.ndarray):
        prim = np.ascontiguousarray(prim, dtype=np.float64)
        self._check(self.L.tj_set_primitive(self.h, q, _dp(prim)))

    def state(self, q: int = 0, out: Optional[np.ndarray] = None) -> np.ndarray:
        """Domain q in AccessPattern layout (Ncomp planes of float64), into
        `out` when given (C-contiguous float64 of that shape, e.g. a
        page-locked buffer)."""
        d = self.case.domains[q]
        shape = (self.ncomp, d.n_cells[2], d.n_cells[1], d.n_cells[0])
        if out is None:
            out = np.empty(shape, dtype=np.float64)
        assert out.shape == shape and out.flags["C_CONTIGUOUS"] and out.dtype == np.float64
        self._check(self.L.tj_download_domain(self.h, q, _dp(out)))
        return out

    def component(self, q: int, comp: int) -> np.ndarray:
        """One AccessPattern component of domain q, shape (nz, ny, nx)."""
        d = self.case.domains[q]
        out = np.empty((d.n_cells[2], d.n_cells[1], d.n_cells[0]), dtype=np.float64)
        self._check(self.L.tj_download_component(self.h, q, comp, _dp(out)))
        return out

    def density(self, q: int = 0) -> np.ndarray:
        """rho = sum of alphaRho_k (the AccessPattern's RHO component)."""
        return self.component(q, 3 * self.case.M)

    def conservation_sums(self) -> np.ndarray:
        """Binary64 sums over all valid cells of alphaRho_k (M), rhoU (3) and
        E, each times the cell volume (deterministic reduction order)."""
        out = np.empty(self.case.M + 4, dtype=np.float64)
        self._check(self.L.tj_conservation_sums(self.h, _dp(out)))
        return out

    def set_state(self, q: int, st: np.ndarray):
        st = np.ascontiguousarray(st, dtype=np.float64)
        self._check(self.L.tj_upload_domain(self.h, q, _dp(st)))

    def upload_fab(self, q: int, box: int, fab: np.ndarray, ngrow: int):
        fab = np.ascontiguousarray(fab, dtype=np.float64)
        self._check(self.L.tj_upload_state(self.h, q, box, _dp(fab), self.ncomp, ngrow))

    def download_fab(self, q: int, box: int, fab: np.ndarray, ngrow: int):
        assert fab.flags["C_CONTIGUOUS"] and fab.dtype == np.float64
        self._check(self.L.tj_download_state(self.h, q, box, _dp(fab), self.ncomp, ngrow))

    # -- reference operators ----------------------------------------------------
    def getTimeStep(self) -> float:
        dt = ctypes.c_double()
        self._check(self.L.tj_compute_dt(self.h, ctypes.byref(dt)))
        return dt.value

    def advance(self, dt: float):
        self._check(self.L.tj_advance(self.h, float(dt)))

    def advance_stage(self, stage: int, dt: float):
        """One RK stage of advance (HLLCadvance, hllc.cpp:701-705), FP64 only."""
        self._check(self.L.tj_advance_stage(self.h, int(stage), float(dt)))

    def plasticUpdate(self, dt: float = 0.0):
        self._check(self.L.tj_plastic_update(self.h, float(dt)))

    def reactiveUpdate(self, dt: float):
        """reactiveUpdate (reactive.cpp:60-103) with parameters.dt = dt."""
        self._check(self.L.tj_reactive_update(self.h, float(dt)))

    def geometricSourceTerm(self, dt: float):
        """geometricSourceTerm (radial.cpp:37-54) with parameters.dt = dt."""
        self._check(self.L.tj_geometric_source(self.h, float(dt)))

    def cleanUpV(self):
        self._check(self.L.tj_cleanup_v(self.h))

    def cleanUpAlpha(self):
        self._check(self.L.tj_cleanup_alpha(self.h))

    def conservativeToPrimitive(self):
        self._check(self.L.tj_cons_to_prim(self.h))

    def primitiveToConservative(self):
        self._check(self.L.tj_prim_to_cons(self.h))

    def contains_nan(self) -> bool:
        f = ctypes.c_int()
        self._check(self.L.tj_contains_nan(self.h, ctypes.byref(f)))
        return bool(f.value)

    # -- time loop --------------------------------------------------------------
    def step(self, t_end: float = 1e300):
        self._check(self.L.tj_step(self.h, float(t_end)))

    def run(self, nsteps: Optional[int] = None, t_end: Optional[float] = None):
        nsteps = self.case.max_steps if nsteps is None else nsteps
        t_end = self.case.final_t if t_end is None else t_end
        done = ctypes.c_int()
        t = ctypes.c_double()
        self._check(self.L.tj_run(self.h, int(min(nsteps, 2**31 - 1)), float(t_end), ctypes.byref(done), ctypes.byref(t)))
        return done.value, t.value

    def time(self):
        t, n, dt = ctypes.c_double(), ctypes.c_int(), ctypes.c_double()
        self._check(self.L.tj_get_time(self.h, ctypes.byref(t), ctypes.byref(n), ctypes.byref(dt)))
        return t.value, n.value, dt.value

    def synchronize(self):
        self._check(self.L.tj_synchronize(self.h))

    def launch_count(self) -> int:
        n = ctypes.c_longlong()
        self._check(self.L.tj_launch_count(self.h, ctypes.byref(n)))
        return n.value


def carried_components(case: Case):
    """AccessPattern indices of the components that carry state from one step
    to the next (the rest -- sound speed, stress, Hencky strain, USTAR/VSTAR --
    are recomputed before use). HJ2 is carried for solids: the CFL sound speed
    of the solid EOS reads it; the mixture densities are carried for the
    MixtureEOS: the RK2 average leaves them in the state the CFL sound speed
    reads (equationofstate.cpp:208-220)."""
    M = case.M
    idx = list(range(0, 3 * M + 1))            # alpha, alphaRho, rho_k, rho
    base = 3 * M + 1
    idx += list(range(base, base + 3))         # rhoU
    idx += list(range(base + 3, base + 6))     # u
    idx += [base + 6, base + 7]                # E, p
    nmix = getattr(case, "nmix", 0)
    x0 = base + 8 + 1 + 1 + 9                  # after a, uStar, sigma
    idx += list(range(x0, x0 + 4 * nmix))      # rhomix (2), lambda, alphaRhoLambda
    if case.solid:
        v0 = x0 + 4 * nmix
        idx += list(range(v0, v0 + 9))         # V
        idx += [v0 + 27]                       # HenckyJ2
        if case.plastic:
            idx += list(range(v0 + 28, v0 + 28 + 2 * M))  # epsilon, alphaRhoEpsilon
    return idx
