"""Settings-file front end: libconfig grammar and the mapping of the
reference's keys (initialise.cpp:125-385) onto a Case."""
import numpy as np
import pytest

from tenjin_gb300 import cases, settings

DECK = r"""
# a two-material shock tube in the reference's key names
finalTime = 0.2; numberOfxCells = 100; numberOfyCells = 1; numberOfzCells = 1;
xdomainLength = 1.0; ydomainLength = 1.0; zdomainLength : 1.0;
CFL = 0.5; materials = 2; mixtures = 0; states = 2; interface = 0.5;
numberOfPictures = 10;
SOLID = 0; THINC = 0; RADIAL = 0; PLASTIC = 0; MUSCL = 1; REACTIVE = 0;
THINCbeta = 1.6;
lowBoundary = [0, 0, 0]; highBoundary = [0, 0, 0];
/* materials */
listOfMaterials = (
  { material = "fluid"; mixture = 0; EOS = "MieGruneisen";
    adiabaticIndex = 4.4; pref = -2.64E9; eref = 0.0; CV = 1.0; },
  { material = "fluid"; mixture = 0; EOS = "MieGruneisen";
    adiabaticIndex = 1.4; pref = 0.0; eref = 0.0; CV = 1.0; }
);
listOfStates = (
  { material = ( { alpha = 0.999999; rho = 1000.0; }, { alpha = 0.000001; rho = 1.2; } );
    p = 1.0E9; u = 0.0; v = 0.0; w = 0.0; },
  { material = ( { alpha = 0.000001; rho = 1000.0; }, { alpha = 0.999999; rho = 1.2; } );
    p = 1.0E5; u = 0.0; v = 0.0; w = 0.0; }   // trailing comment
);
flags = { on = true; off = false; name = "a" "b"; hexv = 0x1F; };
"""


def test_parse_grammar():
    cfg = settings.parse(DECK)
    assert cfg["numberOfxCells"] == 100 and cfg["zdomainLength"] == 1.0
    assert cfg["lowBoundary"] == [0, 0, 0]
    assert cfg["listOfMaterials"][0]["pref"] == -2.64e9
    assert cfg["flags"] == {"on": True, "off": False, "name": "ab", "hexv": 31}
    assert cfg["listOfStates"][1]["material"][1]["alpha"] == 0.999999


def test_parse_errors():
    with pytest.raises(settings.SettingsError):
        settings.parse("a = ;")
    with pytest.raises(settings.SettingsError):
        settings.parse("a = 1; }")


def test_to_case_maps_keys_and_applies_the_pressure_correction():
    c = settings.to_case(settings.parse(DECK), dim=1, max_grid_size=50)
    assert c.M == 2 and c.cfl == 0.5 and c.final_t == 0.2 and c.muscl == 1
    assert c.materials[0].params == [4.4, -2.64e9, 0.0, 1.0]
    d = c.domains[0]
    assert d.n_cells == [100, 1, 1] and len(d.boxes) == 2
    p = d.prim[7, 0, 0]
    # left state: p + (pref alpha / G) / (sum alpha / G), initialise.cpp:104
    a0, a1 = 0.999999, 0.000001
    corr = (-2.64e9 * a0 / 3.4) / (a0 / 3.4 + a1 / 0.4)
    assert p[0] == pytest.approx(1.0e9 + corr, rel=1e-12)
    assert p[99] == pytest.approx(1.0e5 + (-2.64e9 * a1 / 3.4) / (a1 / 3.4 + a0 / 0.4), rel=1e-12)
    assert np.all(d.prim[0, 0, 0, :50] == a0) and np.all(d.prim[0, 0, 0, 50:] == a1)


def test_to_case_carries_radial():
    cfg = settings.parse(DECK)
    cfg["RADIAL"] = 1
    assert settings.to_case(cfg, 1, 50).radial == 1
    assert settings.to_case(settings.parse(DECK), 1, 50).radial == 0


def test_to_case_maps_a_mixture_and_reactive():
    cfg = settings.parse(DECK)
    cfg["mixtures"], cfg["REACTIVE"] = 1, 1
    m0 = cfg["listOfMaterials"][0]
    m0["mixture"] = 1
    m0.update({"adiabaticIndexmix": 1.4, "prefmix": 0.0, "erefmix": 0.0, "CVmix": 1000.0})
    for st, lam in zip(cfg["listOfStates"], (0.7, 0.999)):
        # a mixture's state names its density rhoa (initialise.cpp:245-248)
        st["material"][0]["lambda"] = lam
        st["material"][0]["rhoa"] = st["material"][0].pop("rho")
    c = settings.to_case(cfg, 1, 50)
    assert c.nmix == 1 and c.reactive == 1
    assert c.materials[0].eos == cases.EOS_MIXTURE
    assert c.materials[0].params == [4.4, -2.64e9, 0.0, 1.0, 1.4, 0.0, 0.0, 1000.0]
    d = c.domains[0]
    assert d.prim.shape[0] == c.nprim
    assert np.all(d.prim[-1, 0, 0, :50] == 0.7) and np.all(d.prim[-1, 0, 0, 50:] == 0.999)
    # initialise.cpp:104 with rhomix = rho_k: p += sum p_cold / sum alpha/Gamma
    assert np.all(d.prim[2, 0, 0, :50] == 1000.0) and np.all(d.prim[3, 0, 0, :50] == 1.2)
    a0, lam = 0.999999, 0.7
    g = (lam * 4.4 * 1.0 + (1 - lam) * 1.4 * 1000.0) / (lam * 1.0 + (1 - lam) * 1000.0) - 1.0
    pc = (-2.64e9 * a0 / 3.4) * lam
    assert d.prim[2 * 2 + 3, 0, 0, 0] == pytest.approx(1.0e9 + pc / (a0 / g + (1 - a0) / 0.4), rel=1e-12)


def test_to_case_rejects_what_the_path_does_not_cover():
    cfg = settings.parse(DECK)
    cfg["mixtures"] = 1  # no material has mixture = 1
    with pytest.raises(settings.SettingsError):
        settings.to_case(cfg, 1, 50)
    cfg = settings.parse(DECK)
    cfg["listOfMaterials"][0]["EOS"] = "Unknown"
    with pytest.raises(settings.SettingsError):
        settings.materials(cfg)


@pytest.mark.parametrize("name", ["sod1000_full", "sod200_boxes"])
def test_deck_reproduces_the_fixture_input_and_the_oracle_result(name):
    """A deck written in the reference's keys yields the fixture's initial
    state bit for bit, and the oracle run from it the fixture's result."""
    import fixtures as fx
    import frontend
    from oracle import port
    c = frontend.deck_case(name)
    assert fx.prim_sha(c) == fx.manifest()[name]["prim_sha256"]
    gold = fx.load(name)
    out = port.run_port(c)
    assert np.array_equal(out["dts"], gold["dts"])
    assert fx.exact_fraction(out["states"][0][gold["carried"]], gold["states"][0]) == 1.0
