"""Fused 3-D binary32 kernel over many independent domains (the batched
uneven-box workload, reduced): agreement with the FP64 path (relative L1
density error <= 1e-4), results independent of the tile shape the autotuner
picks, conservation with quiet boundaries, reflective walls."""
import os
import subprocess
import sys

import numpy as np
import pytest

from tenjin_gb300 import build, cases
from tenjin_gb300.host import FP64, MIXED, TenjinGPU

pytestmark = pytest.mark.gpu
L1_TOL = 1e-4
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


def density_all(g, c):
    return np.concatenate([g.state(q)[c.M:2 * c.M].sum(axis=0).ravel() for q in range(len(c.domains))])


def small_batch(nbox=24, seed=3, lo=6, hi=20):
    return cases.uneven_boxes_3d(nbox=nbox, seed=seed, lo=lo, hi=hi, max_steps=20)


@pytest.mark.parametrize("reflect", [False, True])
def test_mixed3d_against_fp64(reflect):
    c = small_batch()
    if reflect:
        c.lo_bc, c.hi_bc = [1, 1, 1], [1, 1, 1]
    g64 = TenjinGPU(c, FP64)
    d64, t64 = g64.run(20, 1e300)
    g32 = TenjinGPU(c, MIXED)
    d32, t32 = g32.run(20, 1e300)
    assert d64 == d32 == 20
    assert abs(t32 - t64) <= 1e-5 * t64
    r64, r32 = density_all(g64, c), density_all(g32, c)
    assert np.all(np.isfinite(r32))
    l1 = np.abs(r32 - r64).sum() / np.abs(r64).sum()
    assert l1 <= L1_TOL, l1


def test_mixed3d_quiet_state_conserves_mass():
    c = small_batch(nbox=8)
    for d in c.domains:
        d.prim[7] = cases.AMBIENT_P  # uniform pressure, fluid at rest: only the interface relaxes
    g = TenjinGPU(c, MIXED)
    m0 = density_all(g, c)
    g.run(10, 1e300)
    m1 = density_all(g, c)
    assert abs(m1.sum() - m0.sum()) / m0.sum() < 1e-6


_SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
from tenjin_gb300 import cases
from tenjin_gb300.host import MIXED, TenjinGPU
c = cases.uneven_boxes_3d(nbox=12, seed=5, lo=6, hi=20, max_steps=6)
g = TenjinGPU(c, MIXED)
g.run(6, 1e300)
np.save(sys.argv[2], np.concatenate([g.state(q).ravel() for q in range(len(c.domains))]))
"""


def test_mixed3d_result_independent_of_tile_shape(tmp_path):
    outs = []
    for shape in ("8x8x8", "8x8x4", "16x4x4", "4x4x4"):
        f = tmp_path / f"s{shape}.npy"
        env = dict(os.environ, TJ_TILE3D=shape)
        subprocess.run([sys.executable, "-c", _SCRIPT, ROOT, str(f)], check=True, env=env, timeout=600)
        outs.append(np.load(f))
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])


_CLASS_SCRIPT = r"""
import ctypes, sys, numpy as np
sys.path.insert(0, sys.argv[1])
from tenjin_gb300 import cases
from tenjin_gb300.host import MIXED, TenjinGPU
c = cases.uneven_boxes_3d(nbox=16, seed=7, lo=6, hi=44, max_steps=5)
g = TenjinGPU(c, MIXED)
g.run(5, 1e300)
buf = ctypes.create_string_buffer(1024)
g.L.tj_kernel_config(g.h, buf, 1024)
print(buf.value.decode())
np.save(sys.argv[2], np.concatenate([g.state(q).ravel() for q in range(len(c.domains))]))
"""


def test_mixed3d_size_classes_tuned_apart_give_the_pinned_result(tmp_path):
    """Boxes of all three size classes: the autotuner plans each class on its
    own (one launch per class and stage) and reports a tile per class; the
    state equals the one with a single pinned tile shape, bit for bit."""
    outs, cfg = [], []
    for shape in (None, "8x8x4"):
        f = tmp_path / f"s{shape}.npy"
        env = dict(os.environ)
        env.pop("TJ_TILE3D", None)
        if shape:
            env["TJ_TILE3D"] = shape
        r = subprocess.run([sys.executable, "-c", _CLASS_SCRIPT, ROOT, str(f)], check=True, env=env, timeout=600,
                           capture_output=True, text=True)
        cfg.append(r.stdout.strip().splitlines()[-1])
        outs.append(np.load(f))
    assert all(k in cfg[0] for k in ("small boxes", "medium boxes", "large boxes")), cfg[0]
    assert cfg[1].count("tile 8x8x4") == 3, cfg[1]
    assert np.array_equal(outs[0], outs[1])
