"""ctypes front end of the CPU port (oracle/port/tenjin_port.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker, and by bench.py's CPU-baseline leg; never by the product.
The shared library is built by build_port() (called from
__graft_entry__.build()) into oracle/_build/.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "port", "tenjin_port.c")

MAX_MAT = 4
MAX_PARAMS = 16


class _Params(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int), ("M", ctypes.c_int), ("solid", ctypes.c_int), ("thinc", ctypes.c_int),
        ("plastic", ctypes.c_int), ("muscl", ctypes.c_int),
        ("lo_bc", ctypes.c_int * 3), ("hi_bc", ctypes.c_int * 3),
        ("cfl", ctypes.c_double), ("thinc_beta", ctypes.c_double),
        ("phase", ctypes.c_int * MAX_MAT), ("eos", ctypes.c_int * MAX_MAT),
        ("eos_params", (ctypes.c_double * MAX_PARAMS) * MAX_MAT),
        ("yield_stress", ctypes.c_double * MAX_MAT),
        ("radial", ctypes.c_int), ("nmix", ctypes.c_int), ("reactive", ctypes.c_int),
    ]


def lib_path(omp: bool) -> str:
    return os.path.join(BUILD_DIR, "libtenjin_port_omp.so" if omp else "libtenjin_port.so")


def build_port(force: bool = False) -> None:
    """Compile the port twice: serial (parity) and OpenMP (timed baseline)."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    for omp in (False, True):
        out = lib_path(omp)
        deps = [SRC, os.path.join(HERE, "port", "tenjin_port.h"), os.path.join(HERE, "shims", "tj_libm.h")]
        if not force and os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(f) for f in deps):
            continue
        cmd = ["gcc", "-O2", "-std=c99", "-ffp-contract=off", "-fPIC", "-shared", SRC, "-o", out, "-lm"]
        if omp:
            cmd.insert(1, "-fopenmp")
        subprocess.run(cmd, check=True)


_LIBS = {}


def _lib(omp: bool):
    if omp not in _LIBS:
        path = lib_path(omp)
        if not os.path.exists(path):
            build_port()
        L = ctypes.CDLL(path)
        L.tjp_create.restype = ctypes.c_void_p
        L.tjp_create.argtypes = [ctypes.POINTER(_Params), ctypes.c_int, ctypes.POINTER(ctypes.c_int),
                                 ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int),
                                 ctypes.POINTER(ctypes.c_int)]
        L.tjp_destroy.argtypes = [ctypes.c_void_p]
        L.tjp_ncomp.argtypes = [ctypes.POINTER(_Params)]
        L.tjp_set_primitive.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        L.tjp_get_state.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        L.tjp_set_state.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        L.tjp_run.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_double)]
        L.tjp_threads.restype = ctypes.c_int
        _LIBS[omp] = L
    return _LIBS[omp]


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def make_params(case) -> _Params:
    p = _Params()
    p.dim, p.M, p.solid, p.thinc, p.plastic, p.muscl = case.dim, case.M, case.solid, case.thinc, case.plastic, case.muscl
    for d in range(3):
        p.lo_bc[d], p.hi_bc[d] = case.lo_bc[d], case.hi_bc[d]
    p.cfl, p.thinc_beta = case.cfl, case.thinc_beta
    p.radial = getattr(case, "radial", 0)
    p.nmix = getattr(case, "nmix", 0)
    p.reactive = getattr(case, "reactive", 0)
    for m, mat in enumerate(case.materials):
        p.phase[m], p.eos[m] = mat.phase, mat.eos
        for q, v in enumerate(mat.params):
            p.eos_params[m][q] = v
        p.yield_stress[m] = mat.yield_stress
    return p


class PortSim:
    """The port's state for one Case (all domains)."""

    def __init__(self, case, omp: bool = False):
        self.case = case
        self.L = _lib(omp)
        self.p = make_params(case)
        nd = len(case.domains)
        ncells = (ctypes.c_int * (3 * nd))(*[v for d in case.domains for v in d.n_cells])
        diml = (ctypes.c_double * (3 * nd))(*[v for d in case.domains for v in d.dim_l])
        nbox = (ctypes.c_int * nd)(*[len(d.boxes) for d in case.domains])
        flat = [v for d in case.domains for b in d.boxes for v in b]
        boxes = (ctypes.c_int * len(flat))(*flat)
        self.h = self.L.tjp_create(ctypes.byref(self.p), nd, ncells, diml, nbox, boxes)
        if not self.h:
            raise ValueError("port rejected the parameters")
        self.ncomp = self.L.tjp_ncomp(ctypes.byref(self.p))
        for q, d in enumerate(case.domains):
            prim = np.ascontiguousarray(d.prim, dtype=np.float64)
            self.L.tjp_set_primitive(self.h, q, _dptr(prim))

    def __del__(self):
        if getattr(self, "h", None):
            self.L.tjp_destroy(self.h)
            self.h = None

    def state(self, q: int = 0) -> np.ndarray:
        d = self.case.domains[q]
        out = np.empty((self.ncomp, d.n_cells[2], d.n_cells[1], d.n_cells[0]), dtype=np.float64)
        self.L.tjp_get_state(self.h, q, _dptr(out))
        return out

    def set_state(self, q: int, st: np.ndarray) -> None:
        st = np.ascontiguousarray(st, dtype=np.float64)
        self.L.tjp_set_state(self.h, q, _dptr(st))

    def run(self, final_t=None, max_steps=None):
        final_t = self.case.final_t if final_t is None else final_t
        max_steps = self.case.max_steps if max_steps is None else max_steps
        cap = int(min(max_steps, 10_000_000))
        dts = np.zeros(max(cap, 1), dtype=np.float64)
        t = ctypes.c_double(0.0)
        n = self.L.tjp_run(self.h, float(final_t), cap, _dptr(dts), ctypes.byref(t))
        if n < 0:
            raise RuntimeError(f"port run failed with status {n}")
        return {"t": t.value, "dts": dts[:n].copy(), "states": [self.state(q) for q in range(len(self.case.domains))]}


def run_port(case, omp: bool = False):
    return PortSim(case, omp).run()


def threads() -> int:
    return _lib(True).tjp_threads()
