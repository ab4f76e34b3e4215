"""Finite-difference checks of the local adjoint operators on the host: each
reverse-mode operator of tenjin_gb300/csrc/tj_adjoint_local.h against central
differences of its forward operator, on seeded inputs away from branch
switches. The header is compiled here with g++ (the same source the CUDA
kernels include)."""
import ctypes
import os
import subprocess
import tempfile

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MM = 4
D = ctypes.POINTER(ctypes.c_double)


@pytest.fixture(scope="module")
def lib():
    out = os.path.join(tempfile.mkdtemp(prefix="tja_"), "libtja.so")
    src = os.path.join(ROOT, "tests", "adjoint_local_harness.cpp")
    inc = os.path.join(ROOT, "tenjin_gb300", "csrc")
    subprocess.run(["g++", "-O1", "-std=c++14", "-shared", "-fPIC", "-I" + inc, src, "-o", out], check=True)
    L = ctypes.CDLL(out)
    c_d, c_i = ctypes.c_double, ctypes.c_int
    L.h_thinc.argtypes = [D, c_i, c_d, c_d, c_d, D]
    L.h_thinc_rev.argtypes = [D, c_i, c_d, c_d, c_d, c_d, c_d, D]
    L.h_muscl.argtypes = [c_d, c_d, c_d, D]
    L.h_muscl_rev.argtypes = [c_d, c_d, c_d, c_d, c_d, D]
    return L


def p(a):
    return a.ctypes.data_as(D)


def eos(M, er=False, rng=None):
    e = np.zeros(3 * MM)
    G = [3.4, 0.4, 1.1, 2.0][:M]
    pr = [-4.4 * 6e8, 0.0, -1.4e7, 0.0][:M]
    e[:M] = G
    e[MM:MM + M] = pr
    if er:
        e[2 * MM:2 * MM + M] = [1.2e5, 3.0e4, 0.0, 5e4][:M]
    return e


def prim(M, rng):
    x = np.zeros(2 * MM + 3)
    a = rng.uniform(0.2, 0.8, M)
    x[:M] = a / a.sum() * rng.uniform(0.97, 1.03)
    x[MM:MM + M] = [1000.0, 1.2, 800.0, 50.0][:M] * rng.uniform(0.8, 1.2, M)
    x[2 * MM:2 * MM + 2] = rng.uniform(-60, 60, 2)
    x[2 * MM + 2] = rng.uniform(1e5, 3e8)
    return x


def fd_check(f, x, lam_out, lam_in_vec, scale, rng, h=1e-6, tol=2e-6, ndir=6):
    """lam_out . (f(x+hv) - f(x-hv)) / 2h == lam_in . v for random v."""
    for _ in range(ndir):
        v = rng.standard_normal(x.size) * scale
        fp, fm = f(x + h * v), f(x - h * v)
        fd = float(lam_out @ (fp - fm)) / (2 * h)
        ad = float(lam_in_vec @ v)
        ref = max(abs(fd), abs(ad), 1e-300)
        # round-off floor of the difference quotient: a few ulps of f over 2h
        floor = 8 * np.finfo(float).eps * float(np.abs(lam_out) @ np.abs(fp + fm)) / (2 * h)
        assert abs(fd - ad) <= tol * ref + floor, (fd, ad)


@pytest.mark.parametrize("M", [2, 3])
@pytest.mark.parametrize("clean", [0, 1])
@pytest.mark.parametrize("er", [False, True])
def test_face_state_rev(lib, M, clean, er):
    rng = np.random.default_rng(10 * M + clean + 100 * er)
    e = eos(M, er)
    for _ in range(4):
        x = prim(M, rng)

        def f(xx):
            o = np.zeros(2 * MM + 8)
            lib.h_face_state(M, p(e), p(np.ascontiguousarray(xx)), clean, p(o))
            return o

        lam = rng.standard_normal(2 * MM + 8)
        lam[M:MM] = 0.0
        lam[MM + M:2 * MM] = 0.0
        lx = np.zeros(2 * MM + 3)
        ge = np.zeros(3 * MM)
        lib.h_face_state_rev(M, p(e), p(x), clean, p(lam), p(lx), p(ge))
        mask = np.zeros_like(x)
        mask[:M] = 1
        mask[MM:MM + M] = 1
        mask[2 * MM:] = 1
        fd_check(f, x, lam, lx * mask, np.abs(x) * mask, rng)

        def fe(ee):
            o = np.zeros(2 * MM + 8)
            lib.h_face_state(M, p(np.ascontiguousarray(ee)), p(x), clean, p(o))
            return o

        emask = np.zeros_like(e)
        emask[:M] = 1
        emask[MM:MM + M] = 1
        emask[2 * MM:2 * MM + M] = 1
        fd_check(fe, e, lam, ge * emask, (np.abs(e) + 1.0) * emask, rng)


def face(lib, M, e, x, clean=1):
    o = np.zeros(2 * MM + 8)
    lib.h_face_state(M, p(e), p(x), clean, p(o))
    return o


@pytest.mark.parametrize("M", [2, 3])
@pytest.mark.parametrize("d", [0, 1])
def test_hllc_rev(lib, M, d):
    rng = np.random.default_rng(7 + M + 10 * d)
    e = eos(M)
    sides = set()
    for trial in range(12):
        xl, xr = prim(M, rng), prim(M, rng)
        # vary the sign of S* so that both sides of the face are exercised
        xl[2 * MM + d] = rng.uniform(-80, 80)
        xr[2 * MM + d] = rng.uniform(-80, 80)
        L, R = face(lib, M, e, xl), face(lib, M, e, xr)
        n = L.size

        def f(z):
            o = np.zeros(2 * MM + 4)
            lib.h_hllc(M, p(np.ascontiguousarray(z[:n])), p(np.ascontiguousarray(z[n:])), d, p(o))
            return o

        o = np.zeros(2 * MM + 4)
        sides.add(lib.h_hllc(M, p(L), p(R), d, p(o)))
        lam = rng.standard_normal(2 * MM + 4)
        lam[M:MM] = 0.0
        lam[MM + M:2 * MM] = 0.0
        lL, lR = np.zeros(n), np.zeros(n)
        lib.h_hllc_rev(M, p(L), p(R), d, p(lam), p(lL), p(lR))
        z = np.concatenate([L, R])
        mask = np.ones(n)
        mask[M:MM] = 0
        mask[MM + M:2 * MM] = 0
        mask2 = np.concatenate([mask, mask])
        fd_check(f, z, lam, np.concatenate([lL, lR]) * mask2, (np.abs(z) + 1e-3) * mask2, rng)
    assert sides == {0, 1}


@pytest.mark.parametrize("M", [2, 3])
def test_c2p_rev(lib, M):
    rng = np.random.default_rng(3 + M)
    e = eos(M, True)
    for _ in range(5):
        x = prim(M, rng)
        carried = np.zeros(3 * MM + 7)
        lib.h_p2c(M, p(e), p(x), p(carried))
        c = np.zeros(2 * MM + 3)
        c[:MM] = carried[:MM]
        c[MM:2 * MM] = carried[MM:2 * MM]
        c[2 * MM:2 * MM + 2] = carried[3 * MM + 1:3 * MM + 3]
        c[2 * MM + 2] = carried[3 * MM + 5]

        def f(cc):
            o = np.zeros(3 * MM + 7)
            lib.h_c2p(M, p(e), p(np.ascontiguousarray(cc)), p(o))
            return o

        lam = rng.standard_normal(3 * MM + 7)
        for blk in range(3):
            lam[blk * MM + M:(blk + 1) * MM] = 0.0
        mu = np.zeros(2 * MM + 3)
        ge = np.zeros(3 * MM)
        lib.h_c2p_rev(M, p(e), p(c), p(lam), p(mu), p(ge))
        mask = np.ones_like(c)
        mask[M:MM] = 0
        mask[MM + M:2 * MM] = 0
        fd_check(f, c, lam, mu * mask, (np.abs(c) + 1e-3) * mask, rng)

        def fe(ee):
            o = np.zeros(3 * MM + 7)
            lib.h_c2p(M, p(np.ascontiguousarray(ee)), p(c), p(o))
            return o

        emask = np.zeros_like(e)
        for blk in range(3):
            emask[blk * MM:blk * MM + M] = 1
        fd_check(fe, e, lam, ge * emask, (np.abs(e) + 1.0) * emask, rng)


@pytest.mark.parametrize("M", [2, 4])
def test_p2c_state_rev(lib, M):
    rng = np.random.default_rng(11 + M)
    e = eos(M, True)
    for _ in range(5):
        x = prim(M, rng)

        def f(xx):
            o = np.zeros(3 * MM + 7)
            lib.h_p2c(M, p(e), p(np.ascontiguousarray(xx)), p(o))
            return o

        lam = rng.standard_normal(3 * MM + 7)
        for blk in range(3):
            lam[blk * MM + M:(blk + 1) * MM] = 0.0
        lx = np.zeros(2 * MM + 3)
        ge = np.zeros(3 * MM)
        lib.h_p2c_rev(M, p(e), p(x), p(lam), p(lx), p(ge))
        mask = np.ones_like(x)
        mask[M:MM] = 0
        mask[MM + M:2 * MM] = 0
        fd_check(f, x, lam, lx * mask, np.abs(x) * mask, rng)

        def fe(ee):
            o = np.zeros(3 * MM + 7)
            lib.h_p2c(M, p(np.ascontiguousarray(ee)), p(x), p(o))
            return o

        emask = np.zeros_like(e)
        for blk in range(3):
            emask[blk * MM:blk * MM + M] = 1
        fd_check(fe, e, lam, ge * emask, (np.abs(e) + 1.0) * emask, rng)


@pytest.mark.parametrize("M", [2, 3])
def test_cleanup_rev(lib, M):
    rng = np.random.default_rng(5 + M)
    for _ in range(10):
        a = rng.uniform(0.05, 0.95, M)
        a[rng.integers(M)] *= rng.choice([1.0, -0.5, 3.0])  # exercise both clamps
        a = np.concatenate([a, np.zeros(MM - M)])

        def f(aa):
            o = np.zeros(MM)
            lib.h_cleanup(M, p(np.ascontiguousarray(aa)), p(o))
            return o[:M]

        lam = rng.standard_normal(M)
        li = np.zeros(MM)
        lib.h_cleanup_rev(M, p(a), p(np.concatenate([lam, np.zeros(MM - M)])), p(li))
        mask = np.zeros(MM)
        mask[:M] = 1
        fd_check(f, a, lam, li * mask, mask * 0.3, rng, h=1e-7)


@pytest.mark.parametrize("d", [0, 1])
def test_thinc_candidate_rev(lib, d):
    rng = np.random.default_rng(21 + d)
    done = 0
    for _ in range(200):
        # a smooth interface through the 3x3 stencil with a random normal
        ang = rng.uniform(0, 2 * np.pi)
        off = rng.uniform(-0.6, 0.6)
        ii, jj = np.meshgrid([-1, 0, 1], [-1, 0, 1], indexing="ij")
        s = 0.5 * (1 + np.tanh(1.3 * (np.cos(ang) * ii + np.sin(ang) * jj - off)))
        s = 1e-6 + (1 - 2e-6) * s
        s = s.reshape(-1).copy()
        LR = np.zeros(2)
        if not lib.h_thinc(p(s), d, 1.6, 1.0 / 512, 1.0 / 512, p(LR)):
            continue

        def f(ss):
            o = np.zeros(2)
            assert lib.h_thinc(p(np.ascontiguousarray(ss)), d, 1.6, 1.0 / 512, 1.0 / 512, p(o))
            return o

        lam = rng.standard_normal(2)
        ls = np.zeros(9)
        lib.h_thinc_rev(p(s), d, 1.6, 1.0 / 512, 1.0 / 512, lam[0], lam[1], p(ls))
        fd_check(f, s, lam, ls, np.full(9, 1e-3), rng, h=1e-6, tol=1e-5)
        done += 1
        if done >= 12:
            break
    assert done >= 12


def test_muscl_rev(lib):
    rng = np.random.default_rng(1)
    branches = set()
    for _ in range(40):
        u = rng.uniform(-1, 1, 3)
        lam = rng.standard_normal(2)
        out = np.zeros(3)
        lib.h_muscl_rev(u[0], u[1], u[2], lam[0], lam[1], p(out))

        def f(uu):
            o = np.zeros(2)
            lib.h_muscl(uu[0], uu[1], uu[2], p(o))
            return o

        r = (u[1] - u[0]) / (u[2] - u[1])
        branches.add(0 if r <= 0 else (1 if r < 1 else 2))
        fd_check(f, u, lam, out, np.ones(3), rng, h=1e-8, tol=1e-6)
    assert branches == {0, 1, 2}
