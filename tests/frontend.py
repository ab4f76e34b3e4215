"""Test helper: a libconfig input deck, in the reference's key names
(initialise.cpp:271-385), for the two-material Sod tube of the golden
fixtures `sod1000_full` and `sod200_boxes` (cases.sod_1d). Every number is
written with repr(), so the parsed deck holds the same binary64 values."""

SOD_DECK = """
# two-material Sod tube (alpha = 1 - 1e-6 / 1e-6 on either side of x = 0.5)
finalTime = {final_t!r}; numberOfxCells = {n}; numberOfyCells = 1; numberOfzCells = 1;
xdomainLength = 1.0; ydomainLength = 1.0; zdomainLength = 1.0;
CFL = 0.5; materials = 2; mixtures = 0; states = 2; interface = 0.5; numberOfPictures = 1;
SOLID = 0; THINC = 0; RADIAL = 0; PLASTIC = 0; MUSCL = 1; REACTIVE = 0; THINCbeta = 1.6;
lowBoundary = [0]; highBoundary = [0];
listOfMaterials = (
  {{ material = "fluid"; mixture = 0; EOS = "MieGruneisen"; adiabaticIndex = 1.4; pref = 0.0; eref = 0.0; CV = 1.0; }},
  {{ material = "fluid"; mixture = 0; EOS = "MieGruneisen"; adiabaticIndex = 1.4; pref = 0.0; eref = 0.0; CV = 1.0; }}
);
listOfStates = (
  {{ material = ( {{ alpha = {a_hi!r}; rho = 1.0; }}, {{ alpha = {a_lo!r}; rho = 1.0; }} );
    p = 1.0; u = 0.0; v = 0.0; w = 0.0; }},
  {{ material = ( {{ alpha = {a_lo!r}; rho = 0.125; }}, {{ alpha = {a_hi!r}; rho = 0.125; }} );
    p = 0.1; u = 0.0; v = 0.0; w = 0.0; }}
);
"""


def sod_deck(n: int, final_t: float = 0.2, eps: float = 1e-6) -> str:
    return SOD_DECK.format(final_t=final_t, n=n, a_hi=1.0 - eps, a_lo=eps)


def deck_case(name: str):
    """The fixture's case rebuilt from its deck through the settings front
    end, with the fixture's step limit (the reference's loop has none; the
    fixtures that stop early name theirs in the manifest)."""
    import fixtures as fx
    from tenjin_gb300 import settings

    spec = fx.manifest()[name]
    kw = spec["kwargs"]
    c = settings.to_case(settings.parse(sod_deck(kw.get("ncells", 1000))), dim=1,
                         max_grid_size=kw.get("max_grid_size", 1000))
    c.max_steps = kw.get("max_steps", 1 << 30)
    return c
