"""The front and back ends around the GPU path, against the reference's own
outputs: an input deck in the reference's keys driven through the settings
reader onto the GPU reproduces a golden fixture bit for bit, and the 1-D
gnuplot dump of the GPU's state equals, byte for byte, the dump the
reference's PrintAllVarsTo1DGnuplotFile (print.cpp:33-43) wrote for the same
fixture (tests/golden/gnuplot/)."""
import os

import numpy as np
import pytest

import fixtures as fx
import frontend
from tenjin_gb300 import build, output
from tenjin_gb300.host import FP64, TenjinGPU

pytestmark = pytest.mark.gpu
GOLDEN_GNUPLOT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gnuplot")


@pytest.fixture(scope="module", autouse=True)
def _built():
    build.build()


@pytest.mark.parametrize("name", ["sod1000_full", "sod200_boxes"])
def test_deck_through_settings_on_the_gpu_matches_the_fixture(name):
    c = frontend.deck_case(name)
    assert fx.prim_sha(c) == fx.manifest()[name]["prim_sha256"]
    gold = fx.load(name)
    g = TenjinGPU(c, FP64)
    done, t = g.run(c.max_steps, c.final_t)
    st = g.state(0)
    g.close()
    assert done == len(gold["dts"])
    assert fx.exact_fraction(st[gold["carried"]], gold["states"][0]) == 1.0


@pytest.mark.parametrize("name", sorted(os.listdir(GOLDEN_GNUPLOT)))
def test_gnuplot_dump_of_the_gpu_state_equals_the_reference_dump(tmp_path, name):
    c = fx.build_case(name)
    g = TenjinGPU(c, FP64)
    g.run(c.max_steps, c.final_t)
    st = g.state(0)
    g.close()
    files = output.write_gnuplot(str(tmp_path), c, st, 0)
    ref = os.path.join(GOLDEN_GNUPLOT, name)
    assert sorted(os.path.basename(f) for f in files) == sorted(os.listdir(ref))
    for f in files:
        with open(f, "rb") as a, open(os.path.join(ref, os.path.basename(f)), "rb") as b:
            assert a.read() == b.read(), os.path.basename(f)


def test_plotfile_of_the_gpu_state_round_trips(tmp_path):
    """The plotfile writer on a GPU state: the directory reads back to the
    same components, in the AccessPattern's order and names."""
    c = fx.build_case("bubble4_reflect_boxes2")
    g = TenjinGPU(c, FP64)
    done, t = g.run(c.max_steps, c.final_t)
    st = g.state(0)
    g.close()
    p = output.write_plotfile(str(tmp_path / output.plotfile_name("plt", done)), c, st, t, done)
    r = output.read_plotfile(p)
    assert r["names"] == output.variable_names(c)
    assert np.array_equal(r["state"], st)
