"""Output of the device state in the reference's formats.

* ``write_plotfile``: an AMReX single-level plotfile, as the reference writes
  it with ``WriteSingleLevelPlotfile(pltfile, U1.data, variableNames, geom,
  t, n)`` (main.cpp:104-106, 173-180): a directory holding the text
  ``Header``, ``Level_0/Cell_H`` (the box list, per-box per-component minima
  and maxima) and ``Level_0/Cell_D_00000`` (one FAB per box: a text header
  line, then the component-major binary64 data, i fastest). Components and
  their names follow the AccessPattern (accesspattern.cpp:3-80), e.g.
  ``alpha0_00``, ``rhoU0_10``, ``sigma0_22``; the file name follows
  ``Concatenate(filename, n, 5)``.
* ``write_gnuplot``: the 1-D dump of print.cpp:3-43 (``PrintAllVarsTo1DGnuplotFile``):
  one text file per variable (rho, p, u, E, rhoU, alpha0) named
  ``<dir>/<var><picture, 2 digits>`` with one ``i value`` line per cell,
  boxes in box-list order.

``PictureSchedule`` says after which steps the reference writes a plotfile
(numberOfPictures over finalTime). ``read_plotfile`` reads such a plotfile
back (used by the tests, and handy to compare a GPU run with the reference's
own plotfiles).
"""
from __future__ import annotations

import os
import struct
from typing import Dict, List, Optional, Sequence

import numpy as np

from .cases import Case

# the binary64 little-endian real descriptor AMReX writes in FAB headers
_REAL_DESCRIPTOR = "((8, (64 11 52 0 1 12 0 1023)),(8, (1 2 3 4 5 6 7 8)))"


def variable_names(case: Case) -> List[str]:
    """Component names in AccessPattern order (accesspattern.cpp:44-80)."""
    M = case.M
    names: List[str] = []

    def add(base: str, mats: int = 1, rows: int = 1, cols: int = 1):
        for m in range(mats):
            for r in range(rows):
                for c in range(cols):
                    names.append(f"{base}{m}_{r}{c}")

    add("alpha", M)
    add("alphaRho", M)
    add("rho_k", M)
    add("rho")
    add("rhoU", 1, 3)
    add("u", 1, 3)
    add("E")
    add("p")
    add("a")
    add("uStar")
    add("sigma", 1, 3, 3)
    nmix = getattr(case, "nmix", 0)
    add("rhomix", nmix, 2)
    add("lambda", nmix)
    add("alpharholambda", nmix)
    if case.solid:
        add("V", 1, 3, 3)
        add("VStar", 1, 3, 3)
        add("devH", 1, 3, 3)
        add("HenckyJ2")
        if case.plastic:
            add("epsilon", M)
            add("alphaRhoEpsilon", M)
    return names


def _concatenate(base: str, n: int, digits: int) -> str:
    return f"{base}{n:0{digits}d}"


def _box3(b: Sequence[int], dim: int):
    lo = [b[k] if k < dim else 0 for k in range(3)]
    hi = [b[3 + k] if k < dim else 0 for k in range(3)]
    return lo, hi


def _fmt_box(lo, hi, dim: int) -> str:
    return "((" + ",".join(str(v) for v in lo[:dim]) + ") (" + ",".join(str(v) for v in hi[:dim]) + ") (" + \
        ",".join("0" for _ in range(dim)) + "))"


def write_plotfile(path: str, case: Case, state: np.ndarray, time: float, step: int, domain: int = 0) -> str:
    """Writes the state of one domain (``TenjinGPU.state(q)``: ncomp x nz x ny
    x nx) as the plotfile directory ``path``. Returns the directory."""
    d = case.domains[domain]
    dim = case.dim
    names = variable_names(case)
    ncomp = len(names)
    if state.shape[0] != ncomp:
        raise ValueError(f"state has {state.shape[0]} components, the AccessPattern {ncomp}")
    lev = os.path.join(path, "Level_0")
    os.makedirs(lev, exist_ok=True)
    dx = [d.dim_l[k] / d.n_cells[k] for k in range(3)]
    prob_lo = [0.0] * dim
    prob_hi = [d.dim_l[k] for k in range(dim)]
    dom_lo, dom_hi = [0, 0, 0], [d.n_cells[k] - 1 for k in range(3)]
    boxes = d.boxes
    # FAB data
    fab_offsets = []
    mins = np.zeros((len(boxes), ncomp))
    maxs = np.zeros((len(boxes), ncomp))
    with open(os.path.join(lev, "Cell_D_00000"), "wb") as f:
        for bi, b in enumerate(boxes):
            lo, hi = _box3(b, dim)
            fab_offsets.append(f.tell())
            blk = state[:, lo[2]:hi[2] + 1, lo[1]:hi[1] + 1, lo[0]:hi[0] + 1]
            f.write(f"FAB {_REAL_DESCRIPTOR}{_fmt_box(lo, hi, dim)} {ncomp}\n".encode())
            f.write(np.ascontiguousarray(blk, dtype="<f8").tobytes())
            flat = blk.reshape(ncomp, -1)
            mins[bi] = flat.min(axis=1)
            maxs[bi] = flat.max(axis=1)
    # FabArray header
    with open(os.path.join(lev, "Cell_H"), "w") as f:
        f.write("1\n1\n")
        f.write(f"{ncomp}\n0\n")
        f.write(f"({len(boxes)} 0\n")
        for b in boxes:
            lo, hi = _box3(b, dim)
            f.write(_fmt_box(lo, hi, dim) + "\n")
        f.write(")\n")
        f.write(f"{len(boxes)}\n")
        for off in fab_offsets:
            f.write(f"FabOnDisk: Cell_D_00000 {off}\n")
        f.write("\n")
        f.write(f"{len(boxes)},{ncomp}\n")
        for bi in range(len(boxes)):
            f.write("".join(f"{v:.17g}," for v in mins[bi]) + "\n")
        f.write("\n")
        f.write(f"{len(boxes)},{ncomp}\n")
        for bi in range(len(boxes)):
            f.write("".join(f"{v:.17g}," for v in maxs[bi]) + "\n")
    # plotfile header
    with open(os.path.join(path, "Header"), "w") as f:
        f.write("HyperCLaw-V1.1\n")
        f.write(f"{ncomp}\n")
        for nm in names:
            f.write(nm + "\n")
        f.write(f"{dim}\n")
        f.write(f"{time:.17g}\n")
        f.write("0\n")
        f.write(" ".join(f"{v:.17g}" for v in prob_lo) + "\n")
        f.write(" ".join(f"{v:.17g}" for v in prob_hi) + "\n")
        f.write("\n")
        f.write(_fmt_box(dom_lo, dom_hi, dim) + " \n")
        f.write(f"{step} \n")
        f.write(" ".join(f"{dx[k]:.17g}" for k in range(dim)) + " \n")
        f.write("0\n0\n")
        f.write(f"0 {len(boxes)} {time:.17g}\n")
        f.write(f"{step}\n")
        for b in boxes:
            lo, hi = _box3(b, dim)
            for k in range(dim):
                f.write(f"{lo[k] * dx[k]:.17g} {(hi[k] + 1) * dx[k]:.17g}\n")
        f.write("Level_0/Cell\n")
    return path


class PictureSchedule:
    """The reference's plotfile cadence (main.cpp:119-180). Its time loop is
    ``for (t = 0; t < finalT; t += dt, n++)``; after the update of each step it
    writes a plotfile of the new state, named and stamped with that step's
    loop values (t, n) -- the time and index at the START of the step -- when
    ``t > counter * finalT / numberOfPictures``, and then advances the counter
    (from 0). Step 0's initial state and the final state (stamped finalT and
    the final n) are always written (main.cpp:104-106, 196-199).

    ``due(t)`` is that test for the step that started at time t; call it once
    per step, in order."""

    def __init__(self, final_t: float, pictures: int):
        if pictures <= 0:
            raise ValueError("numberOfPictures must be positive")
        self.final_t = float(final_t)
        self.pictures = int(pictures)
        self.counter = 0

    @classmethod
    def from_settings(cls, cfg: Dict[str, object]) -> "PictureSchedule":
        """finalTime and numberOfPictures of a parsed settings file."""
        return cls(float(cfg["finalTime"]), int(cfg["numberOfPictures"]))

    def due(self, t: float) -> bool:
        if t > float(self.counter) * self.final_t / float(self.pictures):
            self.counter += 1
            return True
        return False


def plotfile_name(filename: str, step: int) -> str:
    """The reference's plotfile name: Concatenate(filename, n, 5) (main.cpp:104,176)."""
    return _concatenate(filename, step, 5)


def read_plotfile(path: str) -> Dict[str, object]:
    """Reads a single-level plotfile written as above: names, time, dim, dx
    and the full domain as an (ncomp, nz, ny, nx) array."""
    with open(os.path.join(path, "Header")) as f:
        lines = f.read().split("\n")
    ncomp = int(lines[1])
    names = lines[2:2 + ncomp]
    i = 2 + ncomp
    dim = int(lines[i])
    time = float(lines[i + 1])
    prob_hi = [float(v) for v in lines[i + 4].split()]
    dom = lines[i + 6]
    hi = [int(v) for v in dom.split(") (")[1].split(",")]
    dx = [float(v) for v in lines[i + 8].split()]
    n = [h + 1 for h in hi] + [1] * (3 - dim)
    out = np.full((ncomp, n[2], n[1], n[0]), np.nan)
    with open(os.path.join(path, "Level_0", "Cell_D_00000"), "rb") as f:
        data = f.read()
    pos = 0
    while pos < len(data):
        eol = data.index(b"\n", pos)
        head = data[pos:eol].decode()
        boxpart = head[head.rindex("((") :].rsplit(" ", 1)
        nc = int(boxpart[1])
        b = boxpart[0]
        lo = [int(v) for v in b[2:b.index(")")].split(",")] + [0] * (3 - dim)
        hib = [int(v) for v in b[b.index(") (") + 3:b.index(") (", b.index(") (") + 1)].split(",")] + [0] * (3 - dim)
        shape = (nc, hib[2] - lo[2] + 1, hib[1] - lo[1] + 1, hib[0] - lo[0] + 1)
        cnt = int(np.prod(shape))
        arr = np.frombuffer(data, dtype="<f8", count=cnt, offset=eol + 1).reshape(shape)
        out[:, lo[2]:hib[2] + 1, lo[1]:hib[1] + 1, lo[0]:hib[0] + 1] = arr
        pos = eol + 1 + 8 * cnt
    return {"names": names, "time": time, "dim": dim, "dx": dx, "prob_hi": prob_hi, "state": out}


def write_gnuplot(directory: str, case: Case, state: np.ndarray, picture: int, domain: int = 0) -> List[str]:
    """The 1-D dump of PrintAllVarsTo1DGnuplotFile (print.cpp:33-43): files
    rho, p, u, E, rhoU, alpha0 with the picture number in two digits, one
    'i value' line per cell, boxes in box-list order (MFIter order)."""
    M = case.M
    comp = {"rho": 3 * M, "p": 3 * M + 8, "u": 3 * M + 4, "E": 3 * M + 7, "rhoU": 3 * M + 1, "alpha0": 0}
    d = case.domains[domain]
    os.makedirs(directory, exist_ok=True)
    written = []
    for name, q in comp.items():
        fn = _concatenate(os.path.join(directory, name), picture, 2)
        with open(fn, "w") as f:
            for b in d.boxes:
                lo, hi = _box3(b, case.dim)
                for k in range(lo[2], hi[2] + 1):
                    for j in range(lo[1], hi[1] + 1):
                        for i in range(lo[0], hi[0] + 1):
                            f.write(f"{i} {_fmt_real(state[q, k, j, i])}\n")
        written.append(fn)
    return written


def _fmt_real(v: float) -> str:
    # std::ostream << double with the default precision (6 significant digits, %g)
    return f"{v:g}"
