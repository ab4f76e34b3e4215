"""Plotfile and gnuplot output in the reference's formats (host side)."""
import os

import numpy as np
import pytest

from tenjin_gb300 import cases, output


def _state(case, seed=0):
    d = case.domains[0]
    n = len(output.variable_names(case))
    return np.random.default_rng(seed).standard_normal((n, d.n_cells[2], d.n_cells[1], d.n_cells[0]))


def test_variable_names_follow_the_access_pattern():
    fl = output.variable_names(cases.shock_bubble_2d(n=8))
    assert fl[:4] == ["alpha0_00", "alpha1_00", "alphaRho0_00", "alphaRho1_00"]
    assert fl[6] == "rho0_00" and fl[7:10] == ["rhoU0_00", "rhoU0_10", "rhoU0_20"]
    assert fl[-9:] == [f"sigma0_{r}{c}" for r in range(3) for c in range(3)]
    assert len(fl) == 26  # two fluids: the reference's Ncomp
    so = output.variable_names(cases.copper_plate_3d(n=4))
    assert len(so) == 53 and so[-2:] == ["epsilon0_00", "alphaRhoEpsilon0_00"]
    assert "HenckyJ20_00" in so


def test_plotfile_round_trip_2d(tmp_path):
    c = cases.shock_bubble_2d(n=24, max_grid_size=10)
    st = _state(c)
    p = output.write_plotfile(str(tmp_path / output.plotfile_name("plt", 7)), c, st, 1.25e-4, 7)
    assert p.endswith("plt00007")
    r = output.read_plotfile(p)
    assert r["names"] == output.variable_names(c)
    assert r["time"] == 1.25e-4 and r["dim"] == 2
    assert np.array_equal(r["state"], st)
    head = open(os.path.join(p, "Header")).read().split("\n")
    assert head[0] == "HyperCLaw-V1.1" and head[-2] == "Level_0/Cell"
    cell_h = open(os.path.join(p, "Level_0", "Cell_H")).read()
    assert cell_h.count("FabOnDisk: Cell_D_00000") == len(c.domains[0].boxes)


def test_plotfile_round_trip_3d_solid(tmp_path):
    c = cases.copper_plate_3d(n=10, max_grid_size=6)
    st = _state(c, 1)
    r = output.read_plotfile(output.write_plotfile(str(tmp_path / "plt00000"), c, st, 0.0, 0))
    assert np.array_equal(r["state"], st)


def test_gnuplot_dump(tmp_path):
    c = cases.sod_1d(ncells=40, max_grid_size=16)
    st = _state(c)
    files = output.write_gnuplot(str(tmp_path), c, st, 3)
    assert [os.path.basename(f) for f in files] == ["rho03", "p03", "u03", "E03", "rhoU03", "alpha003"]
    lines = open(files[0]).read().splitlines()
    # box-list (MFIter) order, one line per cell
    first = c.domains[0].boxes[0][0]
    assert len(lines) == 40 and int(lines[0].split()[0]) == first
    vals = {int(l.split()[0]): float(l.split()[1]) for l in lines}
    assert sorted(vals) == list(range(40))
    assert vals[5] == float(f"{st[3 * c.M, 0, 0, 5]:g}")


def test_picture_schedule_follows_the_reference_loop():
    # main.cpp:121-180 with exact binary steps: finalT 1, 4 pictures, dt 1/8;
    # the test t > counter * finalT / pictures fires at the steps that start
    # at t = 1/8, 3/8, 5/8, 7/8 (n = 1, 3, 5, 7)
    sch = output.PictureSchedule(1.0, 4)
    t, n, written = 0.0, 0, []
    while t < 1.0:
        if sch.due(t):
            written.append(n)
        t += 0.125
        n += 1
    assert written == [1, 3, 5, 7] and sch.counter == 4
    with pytest.raises(ValueError):
        output.PictureSchedule(1.0, 0)


def test_picture_schedule_from_settings():
    from tenjin_gb300 import settings
    cfg = settings.parse("finalTime = 0.2; numberOfPictures = 10;")
    sch = output.PictureSchedule.from_settings(cfg)
    assert sch.final_t == 0.2 and sch.pictures == 10
    assert not sch.due(0.0) and sch.due(1e-9) and not sch.due(0.02) and sch.due(0.0200001)


GOLDEN_GNUPLOT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "gnuplot")


def _same_files(files, ref_dir):
    for f in files:
        with open(f, "rb") as a, open(os.path.join(ref_dir, os.path.basename(f)), "rb") as b:
            if a.read() != b.read():
                return os.path.basename(f)
    return None


@pytest.mark.parametrize("name", ["sod200_boxes", "bubble4_reflect_boxes2", "bubble32_muscl", "copper12"])
def test_gnuplot_dump_equals_the_reference_writer(tmp_path, name):
    """write_gnuplot on the reference's own final state gives, byte for byte,
    the files the reference's PrintAllVarsTo1DGnuplotFile (print.cpp:33-43,
    compiled into the oracle harness) writes for that state."""
    from oracle import refio
    import fixtures as fx
    c = fx.build_case(name)
    if not refio.have_ref(c.dim):
        pytest.skip("reference binaries are built only where the reference tree exists")
    ref_dir = tmp_path / "ref"
    ref_dir.mkdir()
    r = refio.run_reference(c, gnuplot_dir=str(ref_dir))
    files = output.write_gnuplot(str(tmp_path / "mine"), c, r["states"][0], 0)
    assert sorted(os.path.basename(f) for f in files) == sorted(os.listdir(ref_dir))
    assert _same_files(files, str(ref_dir)) is None


@pytest.mark.parametrize("name", sorted(os.listdir(GOLDEN_GNUPLOT)) if os.path.isdir(GOLDEN_GNUPLOT) else [])
def test_gnuplot_golden_dumps_match_the_golden_states(tmp_path, name):
    """The committed dumps of the reference's writer agree with write_gnuplot
    on the committed golden state (carried components; the dumped variables
    rho, p, u, E, rhoU, alpha0 are all carried)."""
    import fixtures as fx
    c = fx.build_case(name)
    gold = fx.load(name)
    d = c.domains[0]
    st = np.zeros((len(output.variable_names(c)), d.n_cells[2], d.n_cells[1], d.n_cells[0]))
    st[gold["carried"]] = gold["states"][0]
    files = output.write_gnuplot(str(tmp_path), c, st, 0)
    assert _same_files(files, os.path.join(GOLDEN_GNUPLOT, name)) is None
