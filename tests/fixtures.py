"""Loading of the golden fixtures (tests/golden/*.npz, made by
tests/golden/make_golden.py from the reference's own sources)."""
import hashlib
import json
import os

import numpy as np

from tenjin_gb300 import cases

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def manifest():
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)["fixtures"]


def names():
    return sorted(manifest().keys())


def build_case(name):
    spec = manifest()[name]
    c = getattr(cases, spec["builder"])(**spec["kwargs"])
    for k, v in spec["overrides"].items():
        setattr(c, k, v)
    return c


def prim_sha(c):
    h = hashlib.sha256()
    for d in c.domains:
        h.update(np.ascontiguousarray(d.prim, dtype="<f8").tobytes())
    return h.hexdigest()


def load(name):
    z = np.load(os.path.join(GOLDEN, f"{name}.npz"))
    states = []
    q = 0
    while f"state_{q}" in z:
        states.append(z[f"state_{q}"])
        q += 1
    return {"dts": z["dts"], "carried": z["carried"].tolist(), "states": states}


def rel_diff(a, b):
    """Largest |a-b| / max(|b|, tiny) over entries, NaN-aware (NaN == NaN)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    d = np.abs(a - b) / np.maximum(np.abs(b), 1e-300)
    d[both_nan] = 0.0
    d[(a == b)] = 0.0
    return float(np.max(d)) if d.size else 0.0


def exact_fraction(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    eq = (a == b) | (np.isnan(a) & np.isnan(b))
    return float(np.mean(eq))
