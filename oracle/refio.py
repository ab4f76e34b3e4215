"""Oracle I/O: runs the reference's own sources (built by oracle/Makefile into
oracle/_ref/tenjin_ref_<D>d) on a Case and reads back the state.

TEST INFRASTRUCTURE ONLY. It is imported by tests/ and by the fixture script
under tests/golden/, never by the product.

Input file: see oracle/ref_harness.cpp (magic 'ROJT'). Output: header, the
dt of every step, then for each domain all Ncomp components of U1 over the
valid cells in AccessPattern order (accesspattern.cpp:44-79), each component
a (nz, ny, nx) float64 block.
"""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")


def ref_binary(dim: int, omp: bool = False, stock: bool = False) -> str:
    """Path of a reference binary: serial with the pinned libm (parity),
    OpenMP (timing), or serial against the host's own libm (stock)."""
    kind = "omp_" if omp else "stock_" if stock else ""
    return os.path.join(REF_DIR, f"tenjin_ref_{kind}{dim}d")


def have_ref(dim: int = 1, stock: bool = False) -> bool:
    return os.path.exists(ref_binary(dim, stock=stock))


def write_input(case, path: str) -> None:
    with open(path, "wb") as f:
        w = f.write
        w(struct.pack("<i", 0x544A4F52))
        w(struct.pack("<7i", case.dim, case.M, case.solid, case.thinc, case.plastic, case.muscl, case.nghost))
        w(struct.pack("<3i", *case.lo_bc))
        w(struct.pack("<3i", *case.hi_bc))
        w(struct.pack("<3d", case.cfl, case.thinc_beta, case.final_t))
        w(struct.pack("<i", min(case.max_steps, 2**31 - 1)))
        for m in case.materials:
            w(struct.pack("<3i", m.phase, m.eos, len(m.params)))
            w(struct.pack(f"<{len(m.params)}d", *m.params))
            w(struct.pack("<d", m.yield_stress))
        w(struct.pack("<i", len(case.domains)))
        for d in case.domains:
            w(struct.pack("<3i", *d.n_cells))
            w(struct.pack("<3d", *d.dim_l))
            w(struct.pack("<i", len(d.boxes)))
            for b in d.boxes:
                w(struct.pack("<6i", *b))
            assert d.prim.shape[0] == case.nprim
            nmix = case.nmix
            w(np.ascontiguousarray(d.prim[:case.nprim - nmix], dtype="<f8").tobytes())
        # trailer: RADIAL, REACTIVE, numberOfMixtures, mixture flags, lambda rows
        w(struct.pack("<3i", int(case.radial), int(case.reactive), case.nmix))
        w(struct.pack(f"<{case.M}i", *[int(m.eos == 4) for m in case.materials]))
        for d in case.domains:
            if case.nmix:
                w(np.ascontiguousarray(d.prim[case.nprim - case.nmix:], dtype="<f8").tobytes())


def read_output(case, path: str):
    with open(path, "rb") as f:
        buf = f.read()
    magic, nsteps, nan_stop, ncomp = struct.unpack_from("<4i", buf, 0)
    assert magic == 0x544A4F55
    t, elapsed = struct.unpack_from("<2d", buf, 16)
    off = 32
    dts = np.frombuffer(buf, dtype="<f8", count=nsteps, offset=off).copy()
    off += 8 * nsteps
    states = []
    for d in case.domains:
        n = d.ncells * ncomp
        a = np.frombuffer(buf, dtype="<f8", count=n, offset=off).copy()
        off += 8 * n
        states.append(a.reshape(ncomp, d.n_cells[2], d.n_cells[1], d.n_cells[0]))
    return {"t": t, "dts": dts, "nan_stop": bool(nan_stop), "ncomp": ncomp, "elapsed": elapsed, "states": states}


def run_reference(case, omp: bool = False, threads: int | None = None, timeout: float = 3600.0,
                  stock: bool = False, gnuplot_dir: str | None = None):
    """Run the reference binary on `case`. With gnuplot_dir, the reference's
    PrintAllVarsTo1DGnuplotFile (print.cpp:33-43) also writes its 1-D dump of
    the first domain's final state there (picture 0)."""
    exe = ref_binary(case.dim, omp, stock)
    if not os.path.exists(exe):
        raise FileNotFoundError(f"{exe} missing: build it with `make -C oracle` where the reference tree exists")
    with tempfile.TemporaryDirectory() as td:
        fin, fout = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        write_input(case, fin)
        env = dict(os.environ)
        if threads is not None:
            env["OMP_NUM_THREADS"] = str(threads)
        argv = [exe, fin, fout] + ([gnuplot_dir] if gnuplot_dir else [])
        r = subprocess.run(argv, capture_output=True, text=True, timeout=timeout, env=env)
        if r.returncode != 0:
            raise RuntimeError(f"reference run failed ({r.returncode}): {r.stdout[-2000:]} {r.stderr[-2000:]}")
        out = read_output(case, fout)
        out["stdout"] = r.stdout
        return out
