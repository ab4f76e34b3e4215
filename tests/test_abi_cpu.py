"""The C-ABI library builds, loads and exports every entry point that
include/tenjin_gpu.h declares; host-side argument checks (no GPU needed)."""
import ctypes
import os
import re
import subprocess

import pytest

from tenjin_gb300 import _lib, build, cases
from tenjin_gb300.host import make_params

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    build.build()
    return _lib.load()


def declared_symbols():
    with open(os.path.join(ROOT, "include", "tenjin_gpu.h")) as f:
        src = f.read()
    return sorted(set(re.findall(r"^int\s+(tj_\w+)\s*\(", src, flags=re.M)))


def test_every_declared_symbol_is_exported(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", build.LIB], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (tj_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    assert {name for name, _, _ in _lib.SIGNATURES} == set(declared_symbols())


def test_library_targets_sm_103a():
    """Every unit is compiled for sm_103a alone (no PTX for other targets, so
    a GPU of another architecture refuses the launches instead of running a
    JIT build); on a GB300 every -m gpu test then launches these images."""
    assert build.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


@pytest.mark.parametrize("mutate,why", [
    (lambda p: setattr(p, "dim", 4), "dim must be"),
    (lambda p: setattr(p, "n_mixtures", 1), "mixtures"),
    (lambda p: setattr(p, "precision", 7), "unknown precision"),
    (lambda p: setattr(p, "nghost", 1), "nghost"),
    (lambda p: setattr(p, "n_materials", 5), "n_materials"),
])
def test_create_rejects_unsupported_parameters(lib, capfd, mutate, why):
    p = make_params(cases.sod_1d(ncells=10))
    mutate(p)
    h = ctypes.c_void_p()
    assert lib.tj_create(ctypes.byref(p), ctypes.byref(h)) == -1
    assert not h.value
    assert why in capfd.readouterr().err


def test_create_rejects_radial_with_elastic_solids(lib, capfd):
    c = cases.solid_mixture_2d(n=8)
    c.plastic = 0
    c.radial = 1
    p = make_params(c)
    h = ctypes.c_void_p()
    assert lib.tj_create(ctypes.byref(p), ctypes.byref(h)) == -1
    assert "RADIAL with elastic solids" in capfd.readouterr().err


@pytest.mark.parametrize("mutate,why", [
    (lambda c: setattr(c, "materials", c.materials[::-1]), "material 0"),
    (lambda c: setattr(c, "solid", 1), "SOLID"),
])
def test_create_rejects_unsupported_mixtures(lib, capfd, mutate, why):
    c = cases.reactive_charge(dim=1, n=10)
    mutate(c)
    p = make_params(c)
    h = ctypes.c_void_p()
    assert lib.tj_create(ctypes.byref(p), ctypes.byref(h)) == -1
    assert why in capfd.readouterr().err


def test_create_rejects_two_mixtures(lib, capfd):
    p = make_params(cases.reactive_charge(dim=1, n=10))
    p.n_mixtures = 2
    h = ctypes.c_void_p()
    assert lib.tj_create(ctypes.byref(p), ctypes.byref(h)) == -1
    assert "n_mixtures must be 0 or 1" in capfd.readouterr().err


@pytest.mark.parametrize("case", ["sod", "plastic", "reactive"])
def test_create_accepts_radial_fluids_plastic_solids_and_mixtures(lib, capfd, case):
    c = (cases.sod_1d(ncells=10) if case == "sod" else cases.solid_mixture_2d(n=8) if case == "plastic"
         else cases.reactive_charge(dim=2, n=8))
    c.radial = 1
    p = make_params(c)
    h = ctypes.c_void_p()
    rc = lib.tj_create(ctypes.byref(p), ctypes.byref(h))
    if rc == 0:
        lib.tj_destroy(h)
    else:  # no device here: creation gets past the parameter checks and stops at the stream
        assert "no CUDA device" in capfd.readouterr().err


def test_create_rejects_thinc_in_3d(lib):
    c = cases.uneven_boxes_3d(nbox=1, lo=4, hi=4)
    c.thinc = 1
    p = make_params(c)
    h = ctypes.c_void_p()
    assert lib.tj_create(ctypes.byref(p), ctypes.byref(h)) == -1
