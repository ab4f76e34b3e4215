"""Generate the golden fixtures of tests/golden/ by running the REFERENCE'S
OWN hot-path sources (compiled from the reference tree through oracle/Makefile
into oracle/_ref/) on seeded synthetic inputs.

Run where the reference tree exists:  python tests/golden/make_golden.py [name ...]
                                      python tests/golden/make_golden.py --gnuplot [name ...]
Each fixture stores the builder call that makes its input, a SHA-256 of the
initial primitive fields, the dt of every step and the final values of the
carried components (AccessPattern indices listed in the file).
"""
import hashlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from tenjin_gb300 import cases  # noqa: E402
from tenjin_gb300.host import carried_components  # noqa: E402
from oracle import refio  # noqa: E402

FIXTURES = {
    "sod1000_full": ("sod_1d", {}),
    "sod200_boxes": ("sod_1d", {"ncells": 200, "max_grid_size": 37, "max_steps": 60}),
    "sod_thinc_1d": ("sod_1d", {"ncells": 100, "max_grid_size": 30, "max_steps": 80}, {"thinc": 1}),
    "bubble48_thinc_uneven": ("shock_bubble_2d", {"n": 48, "max_grid_size": 20, "max_steps": 60, "radius": 0.3}),
    "bubble64_thinc": ("shock_bubble_2d", {"n": 64, "max_grid_size": 32, "max_steps": 40}),
    "bubble40_reflect": ("shock_bubble_2d", {"n": 40, "max_grid_size": 16, "max_steps": 40, "radius": 0.3},
                         {"lo_bc": [1, 1, 0], "hi_bc": [1, 0, 0]}),
    "bubble32_muscl": ("shock_bubble_2d", {"n": 32, "max_grid_size": 32, "max_steps": 30, "thinc": 0}),
    # the 3-D fixtures were made at CFL 0.4 (short runs, before the 3-D
    # workloads moved to cases.CFL_3D)
    "uneven3d_4dom": ("uneven_boxes_3d", {"nbox": 4, "lo": 6, "hi": 10, "max_steps": 8, "cfl": 0.4}),
    "fluid3d_boxes": ("fluid_boxes_3d", {"n": 12, "max_grid_size": 5, "max_steps": 5, "cfl": 0.4}),
    "copper12": ("copper_plate_3d", {"n": 12, "max_grid_size": 6, "max_steps": 8, "cfl": 0.4}),
    # 3-D reflective walls (reflect_odd of the normal velocity along z too)
    "copper10_reflect": ("copper_plate_3d", {"n": 10, "max_grid_size": 5, "max_steps": 6},
                         {"lo_bc": [1, 0, 1], "hi_bc": [0, 1, 1]}),
    "fluid3d_reflect": ("fluid_boxes_3d", {"n": 12, "max_grid_size": 5, "max_steps": 5},
                        {"lo_bc": [1, 1, 1], "hi_bc": [1, 0, 1]}),
    # several 3-D domains with reflective walls; a small 3-D mixture with walls
    "boxes3d_walls": ("uneven_boxes_3d", {"nbox": 3, "lo": 5, "hi": 9, "max_steps": 4},
                      {"hi_bc": [1, 0, 1]}),
    "mixture3d_walls": ("solid_mixture_3d", {"eos": cases.EOS_ROMENSKII, "n": 6, "max_grid_size": 3,
                                             "max_steps": 4}, {"lo_bc": [1, 1, 0], "hi_bc": [1, 0, 0]}),
    # two materials (solid and gas) through the 5-wave solver in 3-D
    "wilkins3d_plastic": ("solid_mixture_3d", {"eos": cases.EOS_WILKINS, "n": 10, "max_steps": 6}),
    "romenskii3d_plastic_reflect": ("solid_mixture_3d", {"eos": cases.EOS_ROMENSKII, "n": 8, "max_grid_size": 4,
                                                         "max_steps": 5}, {"lo_bc": [1, 0, 1], "hi_bc": [0, 1, 0]}),
    "wilkins2d_plastic": ("solid_mixture_2d", {"eos": cases.EOS_WILKINS, "n": 20, "max_steps": 10}),
    "romenskii2d_plastic": ("solid_mixture_2d", {"eos": cases.EOS_ROMENSKII, "n": 20, "max_steps": 10}),
    "hugoniot2d_plastic": ("solid_mixture_2d", {"eos": cases.EOS_HUGONIOT, "n": 16, "max_steps": 10}),
    # RADIAL: x is the radius, a reflective axis at x = 0
    "sod_spherical_1d": ("sod_1d", {"ncells": 200, "max_grid_size": 64, "max_steps": 80},
                         {"radial": 1, "lo_bc": [1, 0, 0]}),
    "bubble_cylindrical": ("shock_bubble_2d", {"n": 40, "max_grid_size": 16, "max_steps": 30, "radius": 0.3},
                           {"radial": 1, "lo_bc": [1, 1, 0], "hi_bc": [1, 0, 0]}),
    "wilkins2d_plastic_cylindrical": ("solid_mixture_2d", {"eos": cases.EOS_WILKINS, "n": 20, "max_steps": 10},
                                      {"radial": 1, "lo_bc": [1, 0, 0]}),
    # MixtureEOS (reactant/products, bisection closure) and the reactive update
    "reactive_charge_1d": ("reactive_charge", {"dim": 1, "n": 200, "max_steps": 120}),
    "reactive_charge_2d_thinc": ("reactive_charge", {"dim": 2, "n": 48, "max_grid_size": 16, "max_steps": 40,
                                                     "thinc": 1}),
    "mixture_closed_form_2d": ("reactive_charge", {"dim": 2, "n": 40, "max_grid_size": 16, "max_steps": 30,
                                                   "reactive": 0, "reactant": [2.5, 0.0, 4.0e6, 1500.0]}),
    "reactive_spherical_1d": ("reactive_charge", {"dim": 1, "n": 160, "max_grid_size": 40, "max_steps": 100},
                              {"radial": 1, "lo_bc": [1, 0, 0]}),
    # domains and boxes narrower than the stencils (2 ghost cells, the THINC
    # candidate's neighbours and the Youngs normal)
    "sod3_tiny": ("sod_1d", {"ncells": 3, "max_grid_size": 3, "max_steps": 6}),
    "bubble3_tiny": ("shock_bubble_2d", {"n": 3, "max_grid_size": 3, "max_steps": 6, "radius": 0.3}),
    "bubble4_reflect_boxes2": ("shock_bubble_2d", {"n": 4, "max_grid_size": 2, "max_steps": 6, "radius": 0.3},
                               {"lo_bc": [1, 1, 0], "hi_bc": [1, 1, 0]}),
}


def build_case(name):
    spec = FIXTURES[name]
    c = getattr(cases, spec[0])(**spec[1])
    for k, v in (spec[2] if len(spec) > 2 else {}).items():
        setattr(c, k, v)
    return c


def prim_sha(c):
    h = hashlib.sha256()
    for d in c.domains:
        h.update(np.ascontiguousarray(d.prim, dtype="<f8").tobytes())
    return h.hexdigest()


# fixtures whose final state the reference also dumps with its 1-D gnuplot
# writer (print.cpp:33-43), stored under gnuplot/<name>/
GNUPLOT_FIXTURES = ["sod200_boxes", "bubble4_reflect_boxes2"]


def _make_oracle():
    from __graft_entry__ import reference_tree
    ref = reference_tree()
    if not ref:
        raise RuntimeError("the reference tree is needed: set TENJIN_REFERENCE")
    subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "-j3", f"REF={ref}"], check=True)


def make_gnuplot(names=None):
    """The reference's own gnuplot dumps of the final states of
    GNUPLOT_FIXTURES (picture 0)."""
    for name in (names or GNUPLOT_FIXTURES):
        d = os.path.join(HERE, "gnuplot", name)
        os.makedirs(d, exist_ok=True)
        for f in os.listdir(d):
            os.remove(os.path.join(d, f))
        refio.run_reference(build_case(name), gnuplot_dir=d)
        print(f"{name}: gnuplot dump {sorted(os.listdir(d))}")


def main(names=None):
    """Regenerates the named fixtures (all when none are named); the manifest
    keeps the entries of the others."""
    _make_oracle()
    manifest = {}
    mpath = os.path.join(HERE, "manifest.json")
    if names and os.path.exists(mpath):
        with open(mpath) as f:
            manifest = json.load(f)["fixtures"]
    for name in (names or FIXTURES):
        c = build_case(name)
        out = refio.run_reference(c)
        if out["nan_stop"]:
            raise RuntimeError(f"{name}: reference stopped on NaN")
        idx = carried_components(c)
        arrs = {"dts": out["dts"], "carried": np.array(idx, dtype=np.int32)}
        for q, st in enumerate(out["states"]):
            arrs[f"state_{q}"] = st[idx]
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **arrs)
        spec = FIXTURES[name]
        manifest[name] = {"builder": spec[0], "kwargs": spec[1], "overrides": spec[2] if len(spec) > 2 else {},
                          "prim_sha256": prim_sha(c), "steps": int(len(out["dts"])), "t": out["t"]}
        print(f"{name}: {len(out['dts'])} steps, t={out['t']:.6g}")
    with open(os.path.join(HERE, "manifest.json"), "w") as f:
        json.dump({"generator": "reference sources through oracle/Makefile (serial, -O2 -ffp-contract=off)",
                   "fixtures": manifest}, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    if sys.argv[1:2] == ["--gnuplot"]:
        _make_oracle()
        make_gnuplot(sys.argv[2:])
    else:
        main(sys.argv[1:])
