"""Settings-file front end: the reference's input decks drive the GPU path.

The reference reads a libconfig file (libConfigInitialiseDataStructs,
initialise.cpp:271-385) plus three ParmParse inputs (max_grid_size, Nghost,
plotDirectory). ``parse`` reads the libconfig grammar (settings ``name = value;``
or ``name : value;``, groups ``{}``, lists ``()``, arrays ``[]``, strings,
integers, reals, booleans, ``#`` ``//`` ``/* */`` comments); ``to_case`` maps the
keys the reference reads onto a :class:`~tenjin_gb300.cases.Case`:

* scalars: finalTime, numberOfxCells/yCells/zCells, x/y/zdomainLength, CFL,
  materials, mixtures, states, interface, numberOfPictures, SOLID, THINC,
  RADIAL, PLASTIC, MUSCL, REACTIVE, THINCbeta, lowBoundary[], highBoundary[];
* listOfMaterials (getMaterialParameters, initialise.cpp:125-235): material
  ("solid"/"fluid"), EOS ("MieGruneisen", "RomenskiiSolid", "WilkinsSolid"),
  adiabaticIndex, pref, eref, CV, then rho0 K0 EOSalpha EOSbeta (Romenskii) or
  rho0 e1..e5 (Wilkins), G0 for solids, yieldStress when PLASTIC; a fluid with
  mixture = 1 is a MixtureEOS with adiabaticIndexmix, prefmix, erefmix, CVmix;
* listOfStates (getState, initialise.cpp:237-267): per material alpha, then
  rho (fluids), rhoa and lambda (the mixture) or F[9] (solids); then p, u, v,
  w.

The reference chooses the state of each cell with a hard-coded geometry
(chooseStateBasedOnInitialCondition, initialise.cpp:387-): ``to_case`` takes
that choice as a function ``chooser(i, j, k, x, y, z, cfg) -> state index``
(``planar_interface`` is the 1-D Riemann-problem choice). Initial pressure
gets the reference's non-thermal correction (initialise.cpp:104) and solid
states their deformation from F (initialise.cpp:26-45); solid F must be
isotropic here (F = f I, V = I and rho from F as the reference's
setRhoFromDeformationTensor does).
"""
from __future__ import annotations

import re
from typing import Any, Callable, Dict, List, Optional

import numpy as np

from . import cases
from .cases import Case, Domain, Material

_TOKEN = re.compile(r"""
    (?P<ws>\s+|\#[^\n]*|//[^\n]*|/\*.*?\*/)
  | (?P<str>"(?:[^"\\]|\\.)*")
  | (?P<hex>0[xX][0-9a-fA-F]+L{0,2})
  | (?P<num>[-+]?(?:\d+\.\d*|\.\d+|\d+)(?:[eE][-+]?\d+)?L{0,2})
  | (?P<name>[A-Za-z*][-A-Za-z0-9_*]*)
  | (?P<punct>[=:;,{}()\[\]])
""", re.VERBOSE | re.DOTALL)


class SettingsError(ValueError):
    pass


def _tokens(text: str):
    pos = 0
    out = []
    while pos < len(text):
        m = _TOKEN.match(text, pos)
        if not m:
            raise SettingsError(f"unexpected character at offset {pos}: {text[pos:pos + 20]!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        out.append((kind, m.group(kind)))
    return out


class _Parser:
    def __init__(self, toks):
        self.t = toks
        self.i = 0

    def peek(self):
        return self.t[self.i] if self.i < len(self.t) else (None, None)

    def take(self, val=None):
        k, v = self.peek()
        if val is not None and v != val:
            raise SettingsError(f"expected {val!r}, found {v!r}")
        self.i += 1
        return k, v

    def settings(self, end=None) -> Dict[str, Any]:
        out: Dict[str, Any] = {}
        while True:
            k, v = self.peek()
            if k is None or v == end:
                return out
            if k != "name":
                raise SettingsError(f"expected a setting name, found {v!r}")
            self.take()
            self.take("=") if self.peek()[1] == "=" else self.take(":")
            out[v] = self.value()
            if self.peek()[1] in (";", ","):
                self.take()

    def value(self):
        k, v = self.peek()
        if v == "{":
            self.take()
            g = self.settings("}")
            self.take("}")
            return g
        if v in ("(", "["):
            close = ")" if v == "(" else "]"
            self.take()
            items = []
            while self.peek()[1] != close:
                items.append(self.value())
                if self.peek()[1] == ",":
                    self.take()
            self.take(close)
            return items
        self.take()
        if k == "str":
            s = v[1:-1].encode().decode("unicode_escape")
            while self.peek()[0] == "str":  # adjacent strings concatenate
                s += self.take()[1][1:-1]
            return s
        if k == "hex":
            return int(v.rstrip("L"), 16)
        if k == "num":
            v = v.rstrip("L")
            return float(v) if any(c in v for c in ".eE") else int(v)
        if k == "name" and v.lower() in ("true", "false"):
            return v.lower() == "true"
        raise SettingsError(f"unexpected value {v!r}")


def parse(text: str) -> Dict[str, Any]:
    """The settings of a libconfig document as nested dicts and lists."""
    p = _Parser(_tokens(text))
    out = p.settings()
    if p.peek()[0] is not None:
        raise SettingsError(f"unexpected {p.peek()[1]!r}")
    return out


def read(path: str) -> Dict[str, Any]:
    with open(path) as f:
        return parse(f.read())


_EOS = {"MieGruneisen": cases.EOS_MIEGRUNEISEN, "RomenskiiSolid": cases.EOS_ROMENSKII,
        "WilkinsSolid": cases.EOS_WILKINS}


def materials(cfg: Dict[str, Any]) -> List[Material]:
    """getMaterialParameters (initialise.cpp:125-235) for every material."""
    out = []
    plastic = bool(cfg.get("PLASTIC", 0))
    for m, mat in enumerate(cfg["listOfMaterials"][:int(cfg["materials"])]):
        eos = mat.get("EOS")
        if eos not in _EOS:
            raise SettingsError(f"No valid EOS selected for material {m}")
        mix = int(mat.get("mixture", 0))
        prm = [float(mat["adiabaticIndex"]), float(mat["pref"]), float(mat["eref"]), float(mat["CV"])]
        if mix:
            if eos != "MieGruneisen" or mat.get("material") == "solid":
                raise SettingsError("Error: solid can't be a mixture (atm)")
            prm += [float(mat[k]) for k in ("adiabaticIndexmix", "prefmix", "erefmix", "CVmix")]
            out.append(Material(cases.PHASE_FLUID, cases.EOS_MIXTURE, prm, 0.0))
            continue
        if eos == "RomenskiiSolid":
            prm += [float(mat[k]) for k in ("rho0", "K0", "EOSalpha", "EOSbeta")]
        elif eos == "WilkinsSolid":
            prm += [float(mat[k]) for k in ("rho0", "e1", "e2", "e3", "e4", "e5")]
        phase = cases.PHASE_SOLID if mat.get("material") == "solid" else cases.PHASE_FLUID
        ys = 0.0
        if phase == cases.PHASE_SOLID:
            prm.append(float(mat["G0"]))
            if plastic:
                ys = float(mat["yieldStress"])
        out.append(Material(phase, _EOS[eos], prm, ys))
    return out


def planar_interface(i, j, k, x, y, z, cfg) -> int:
    """The reference's 1-D Riemann-problem choice (initialise.cpp:392-401):
    state 0 left of the interface, state 1 right of it."""
    n0 = int(cfg["numberOfxCells"])
    return 0 if i < int((float(cfg["interface"]) / float(cfg["xdomainLength"])) * n0) else 1


def to_case(cfg: Dict[str, Any], dim: int, max_grid_size: int,
            chooser: Callable[..., int] = planar_interface, nghost: int = 2) -> Case:
    """A Case from the settings (one domain of numberOf{x,y,z}Cells over
    {x,y,z}domainLength) with the cell states picked by `chooser`."""
    mats = materials(cfg)
    M = len(mats)
    c = Case("settings", dim, mats, solid=int(cfg.get("SOLID", 0)), thinc=int(cfg.get("THINC", 0)),
             plastic=int(cfg.get("PLASTIC", 0)), muscl=int(cfg.get("MUSCL", 1)), nghost=nghost,
             radial=int(cfg.get("RADIAL", 0)), reactive=int(cfg.get("REACTIVE", 0)),
             cfl=float(cfg["CFL"]), thinc_beta=float(cfg.get("THINCbeta", 1.6)),
             final_t=float(cfg["finalTime"]))
    if int(cfg.get("mixtures", 0)) != c.nmix:
        raise SettingsError("mixtures must equal the number of materials with mixture = 1")
    axes = "xyz"
    n = [int(cfg[f"numberOf{axes[d]}Cells"]) if d < dim else 1 for d in range(3)]
    L = [float(cfg[f"{axes[d]}domainLength"]) if d < dim else 1.0 for d in range(3)]
    lo, hi = list(cfg.get("lowBoundary", [0] * dim)), list(cfg.get("highBoundary", [0] * dim))
    c.lo_bc = [int(lo[d]) if d < dim else 0 for d in range(3)]
    c.hi_bc = [int(hi[d]) if d < dim else 0 for d in range(3)]
    states = cfg["listOfStates"][:int(cfg["states"])]
    prim = np.zeros((c.nprim, n[2], n[1], n[0]))
    dx = [L[d] / n[d] for d in range(3)]
    sel = np.zeros((n[2], n[1], n[0]), dtype=int)
    for k in range(n[2]):
        for j in range(n[1]):
            for i in range(n[0]):
                sel[k, j, i] = chooser(i, j, k, i * dx[0], j * dx[1], k * dx[2], cfg)
    for s, st in enumerate(states):
        msk = sel == s
        for m in range(M):
            sm = st["material"][m]
            prim[m][msk] = float(sm["alpha"])
            # getState (initialise.cpp:242-257): a mixture's density is
            # "rhoa", a fluid's "rho"; a solid's comes from F
            if mats[m].eos == cases.EOS_MIXTURE:
                rho = float(sm["rhoa"])
            elif mats[m].phase != cases.PHASE_SOLID:
                rho = float(sm["rho"])
            if mats[m].phase == cases.PHASE_SOLID:
                F = [float(v) for v in sm.get("F", [1, 0, 0, 0, 1, 0, 0, 0, 1])]
                Fm = np.array(F).reshape(3, 3)
                f = Fm[0, 0]
                if not np.allclose(Fm, f * np.eye(3)):
                    raise SettingsError("solid states need an isotropic deformation F = f I")
                rho = mats[m].params[4] / np.linalg.det(Fm)  # setRhoFromDeformationTensor
            prim[M + m][msk] = rho
        prim[2 * M][msk] = float(st["u"])
        prim[2 * M + 1][msk] = float(st.get("v", 0.0))
        prim[2 * M + 2][msk] = float(st.get("w", 0.0))
        prim[2 * M + 3][msk] = float(st["p"])
        if c.nmix:  # initialise.cpp:66-71, 245-248
            prim[c.nprim - 1][msk] = float(st["material"][0]["lambda"])
    if c.solid:
        for r in range(3):
            prim[2 * M + 4 + 3 * r + r] = 1.0
    # p += sum p_cold / sum alpha/G (initialise.cpp:104; V = I, so no shear part)
    pc = np.zeros(prim.shape[1:])
    ig = np.zeros(prim.shape[1:])
    for m, mat in enumerate(mats):
        a, rk, q = prim[m], prim[M + m], mat.params
        G = q[0] - 1.0
        if mat.eos == cases.EOS_MIXTURE:
            # rhomix = rho_k at this point (initialise.cpp:68-69), so the
            # density ratios of equationofstate.cpp:167-171 are 1
            lam = prim[c.nprim - 1]
            pc += (q[1] * a / (q[0] - 1.0)) * lam * rk / rk + (q[5] * a / (q[4] - 1.0)) * (1.0 - lam) * rk / rk
            ig += a / ((lam * q[0] * q[3] + (1.0 - lam) * q[4] * q[7]) / (lam * q[3] + (1.0 - lam) * q[7]) - 1.0)
            continue
        if mat.eos == cases.EOS_MIEGRUNEISEN:
            pc += q[1] * a / G
        elif mat.eos == cases.EOS_ROMENSKII:
            x = rk / q[4]
            pc += (a / G) * ((q[5] / q[6]) * x ** (q[6] + 1.0) * (x ** q[6] - 1.0))
        elif mat.eos == cases.EOS_WILKINS:
            x = rk / q[4]
            pc += (a / G) * (2.0 * q[6] * x ** 3 + q[7] * x * x - q[8] - q[9] * x)
        ig += a / G
    prim[2 * M + 3] += pc / ig
    c.domains = [Domain(n, L, cases.max_size_boxes(n, dim, max_grid_size), prim)]
    return c
