"""Deck reader (fiesta_gb300/deck.py): the Lua subset, the keys FIESTA's input
stage reads (src/input.cpp:136-284) with their defaults and required-key
errors, and the per-cell initial-condition call (src/input.cpp:453-515)."""
import glob
import math
import os

import numpy as np
import pytest

from fiesta_gb300 import abi, deck

DECK_3D = """
fiesta.title = "mixing box"
fiesta.eos.R = 8.314462
fiesta.viscosity.enabled = true
fiesta.advection_scheme = "weno5"
fiesta.species = {
    {name="N2", gamma=1.4, M=0.028, mu=1.8e-5},
    {name="SF6", gamma=1.1, M=0.146, mu=1.5e-5},
}
fiesta.time.dt = 1e-7
fiesta.time.nt = 2e3
Lx, Ly, Lz = 1.0, 0.5, 0.25
fiesta.grid.type = "cartesian"
fiesta.grid.ndim = 3
fiesta.grid.ni = {32, 16, 8}
fiesta.grid.dx = {Lx/fiesta.grid.ni[1], Ly/fiesta.grid.ni[2], Lz/fiesta.grid.ni[3]}
fiesta.mpi.procs = {1, 1, 1}
fiesta.bc.xperiodic = true
fiesta.bc.ymin = "No-Slip"
fiesta.bc.ymax = "reflective"
fiesta.bc.zmin = "hydro_static"
fiesta.bc.zmax = "OUTFLOW"
fiesta.buoyancy.enabled = true
fiesta.buoyancy.acceleration = 9.81
fiesta.ceq.enabled = true
fiesta.ceq.epsilon = 0.5
fiesta.ceq.alpha = 20
fiesta.ceq.beta = 0
fiesta.ceq.betae = 0
fiesta.gb300 = {mode = "mixed"}

function fiesta.initial_conditions(x, y, z, v)
    local p = 1e5 * (1 + 0.1*math.exp(-((x-0.5)^2 + (y-0.25)^2)/0.01))
    if v == 3 then return p/(1.4-1)
    elseif v == 4 then return 1.2*(1-z)
    elseif v == 5 then return 0.1*z
    else return 0 end
end
"""


def test_deck_keys_and_config():
    d = deck.load(text=DECK_3D)
    assert d.title == "mixing box"
    assert d.ndim == 3 and d.ni == [32, 16, 8]
    assert d.dx == [1.0 / 32, 0.5 / 16, 0.25 / 8]
    assert d.nt == 2000 and d.dt == 1e-7
    assert [s["M"] for s in d.species] == [0.028, 0.146]
    assert d.visc and d.ceq and d.buoyancy
    assert d.kap == 1.23456  # the reference's default for fiesta.ceq.kappa
    assert (d.eps, d.alpha) == (0.5, 20.0)
    assert d.periodic == (True, False, False)
    assert d.bcs == (0, 0, abi.BC_NOSLIP, abi.BC_REFLECTIVE, abi.BC_HYDROSTATIC, abi.BC_OUTFLOW)
    assert d.mode == abi.MODE_MIXED
    assert d.noise_params() is None
    dn = deck.load(text=DECK_3D + "\nfiesta.noise.enabled=true\nfiesta.noise.dh=1e-5\n"
                   "fiesta.noise.eta=1e-3\nfiesta.noise.coff=0.05\n")
    np_ = dn.noise_params()
    assert (np_.dh, np_.eta, np_.coff, np_.nt, np_.mode) == (1e-5, 1e-3, 0.05, 1, 1)
    cfg = d.config()
    assert (cfg.nci, cfg.ncj, cfg.nck, cfg.ns) == (32, 16, 8, 2)
    assert cfg.dz == 0.25 / 8 and cfg.g_accel == 9.81 and cfg.xper == 1
    assert cfg.bc_ymin == abi.BC_NOSLIP and cfg.mode == abi.MODE_MIXED


def test_deck_initial_conditions_at_cell_centres():
    d = deck.load(text=DECK_3D)
    cfg = d.config()
    U = d.initial_conditions(cfg)
    assert U.shape == abi.dims(cfg)
    ng = 3
    i, j, k = 5, 7, 4
    x, y, z = (i + 0.5) / 32, 0.5 / 16 * (j + 0.5), 0.25 / 8 * (k + 0.5)
    p = 1e5 * (1 + 0.1 * math.exp(-((x - 0.5) ** 2 + (y - 0.25) ** 2) / 0.01))
    assert U[i + ng, j + ng, k + ng, 3] == pytest.approx(p / 0.4, rel=1e-15)
    assert U[i + ng, j + ng, k + ng, 4] == pytest.approx(1.2 * (1 - z), rel=1e-15)
    assert np.all(U[:ng] == 0) and np.all(U[..., 6:] == 0)  # ghosts, C-variables


def test_reference_quirks_of_the_reader():
    base = DECK_3D.replace('fiesta.eos.R = 8.314462', 'fiesta.R = 1.0')
    d = deck.load(text=base)
    assert d.R == 8.314462           # only fiesta.eos.R is read
    d = deck.load(text=base.replace("fiesta.viscosity.enabled = true",
                                    "fiesta.viscosity.enabled = 0"))
    assert d.visc                    # lua_toboolean(0) is true
    d = deck.load(text=base.replace("fiesta.time.nt = 2e3", "fiesta.time.nt = 2.5"))
    assert d.nt == 0                 # lua_tointegerx of a non-integral number


def test_required_keys_and_errors():
    with pytest.raises(deck.DeckError, match="fiesta.time.dt"):
        deck.load(text=DECK_3D.replace("fiesta.time.dt = 1e-7", ""))
    with pytest.raises(deck.DeckError, match="fiesta.ceq.epsilon"):
        deck.load(text=DECK_3D.replace("fiesta.ceq.epsilon = 0.5", ""))
    with pytest.raises(deck.DeckError, match="Unknown boundary condition 'wall'"):
        deck.load(text=DECK_3D.replace('"reflective"', '"wall"'))
    with pytest.raises(deck.DeckError, match="fiesta.bc.xmin"):
        deck.load(text=DECK_3D.replace("fiesta.bc.xperiodic = true", ""))
    with pytest.raises(deck.DeckError, match="unknown fiesta.grid.type"):
        deck.load(text=DECK_3D.replace('"cartesian"', '"curvy"'))
    with pytest.raises(deck.DeckError, match="periodic"):
        deck.load(text=DECK_3D.replace('"cartesian"', '"generalized"')
                  .replace('mode = "mixed"', 'mode = "plain"'))
    with pytest.raises(deck.DeckError, match="plain FP64"):
        deck.load(text=DECK_3D.replace('"cartesian"', '"generalized"')
                  .replace('mode = "mixed"', 'mode = "hybrid"'))
    d = deck.load(text=DECK_3D.replace('"weno5"', '"centered4"'))
    assert d.config().scheme == abi.SCHEME_CENTERED4  # the 3D modules ignore it
    d = deck.load(text=DECK_3D.replace('"weno5"', '"upwind"'))
    assert d.config().scheme == abi.SCHEME_WENO5      # unknown names leave WENO5
    with pytest.raises(deck.DeckError, match="mode"):
        deck.load(text=DECK_3D.replace('mode = "mixed"', 'mode = "fast"'))
    with pytest.raises(deck.DeckError):
        deck.load(text="fiesta.title = ")


def test_lua_subset_semantics():
    d = deck.load(text=DECK_3D + """
a = 7 // 2; b = 7 / 2; c = 2^10; e = -7 % 3; f = 1 .. "x"
g = nil or "dflt"; h = false and 1; s = 0
for i = 1, 10, 3 do s = s + i end
local t = {10, 20, 30, n = "x"}
n = #t
w = 0
while w < 5 do w = w + 2 end
function fact(n) if n <= 1 then return 1 end return n * fact(n - 1) end
q = fact(6)
r = math.max(3, 9, 4) + math.floor(2.7) + math.sqrt(16)
""")
    G = d.lua.g.vars
    assert G["a"] == 3 and isinstance(G["a"], int)
    assert G["b"] == 3.5 and G["c"] == 1024.0 and G["e"] == 2
    assert G["f"] == "1x" and G["g"] == "dflt" and G["h"] is False
    assert G["s"] == 1 + 4 + 7 + 10 and G["n"] == 3 and G["w"] == 6
    assert G["q"] == 720 and G["r"] == 9 + 2 + 4.0


# the reference's sample decks, staged by oracle/ref_build.sh next to the
# reference checker it builds
SAMPLES = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle",
                       "_ref", "samples")


@pytest.mark.skipif(not os.path.isdir(SAMPLES), reason="reference sample decks not staged")
def test_reference_sample_decks():
    """The decks written for the current reader load; the legacy flat-global
    decks fail on their first required key, as with the reference."""
    ok, legacy = 0, 0
    for p in sorted(glob.glob(os.path.join(SAMPLES, "*", "fiesta.lua"))):
        text = open(p).read()
        if "fiesta.title" in text:
            d = deck.load(p)
            cfg = d.config()
            assert cfg.nci == d.ni[0] and cfg.ns == len(d.species) >= 1
            ok += 1
        else:
            with pytest.raises(deck.DeckError, match="fiesta.title"):
                deck.load(p)
            legacy += 1
    assert ok >= 5 and legacy >= 1


DECK_GEN2D = """
fiesta.title = "wavy channel"
fiesta.species = {{name="air", gamma=1.4, M=0.02897, mu=2.928e-5}}
fiesta.time.dt = 1e-6
fiesta.grid.type = "generalized"
fiesta.grid.ndim = 2
fiesta.grid.ni = {6, 5}
fiesta.grid.dx = {0.5, 0.5}
fiesta.advection_scheme = "quick"
fiesta.bc.xmin = "outflow"
fiesta.bc.xmax = "outflow"
fiesta.bc.ymin = "reflective"
fiesta.bc.ymax = "outflow"
fiesta.mpi.procs = {1, 1}
function fiesta.initialize_grid(i, j, k, v)
    local x = i * 10 / 6
    local dh = 0.3 * math.sin(x * 2.0)
    if v == 0 then return x end
    return dh + (10 - dh) * (j * 10 / 5) / 10
end
function fiesta.initial_conditions(x, y, z, v)
    if v == 2 then return 1e5 + x + 10 * y end
    if v == 3 then return 1.0 end
    return 0
end
"""


def test_generalized_deck_grid_and_cell_centres():
    d = deck.load(text=DECK_GEN2D)
    cfg = d.config()
    assert cfg.grid_type == abi.GRID_GENERALIZED and cfg.scheme == abi.SCHEME_QUICK
    assert (cfg.dx, cfg.dy) == (1.0, 1.0)  # computational space
    X = d.grid_nodes(cfg)
    assert X.shape == (7, 6, 1, 3) and np.all(X[..., 2] == 0)
    i, j = 4, 2
    x = i * 10 / 6
    assert X[i, j, 0, 0] == x
    assert X[i, j, 0, 1] == pytest.approx(0.3 * math.sin(2 * x) + (10 - 0.3 * math.sin(2 * x)) * j / 5,
                                          rel=1e-15)
    U = d.initial_conditions(cfg, X)
    ci, cj = 3 + 2, 3 + 1  # cell (2, 1): the mean of its four nodes
    xc = (X[2, 1, 0, 0] + X[2, 2, 0, 0] + X[3, 1, 0, 0] + X[3, 2, 0, 0]) / 4.0
    yc = (X[2, 1, 0, 1] + X[2, 2, 0, 1] + X[3, 1, 0, 1] + X[3, 2, 0, 1]) / 4.0
    assert U[ci, cj, 0, 2] == pytest.approx(1e5 + xc + 10 * yc, rel=1e-15)
    assert U[ci, cj, 0, 3] == 1.0 and np.all(U[:3] == 0)
    bad = DECK_GEN2D.replace("return 0\nend", "end")
    with pytest.raises(deck.DeckError, match="should return a number"):
        deck.load(text=bad).initial_conditions(cfg, X)


DECK_TERRAIN = """
fiesta.title = "valley"
fiesta.species = {{name="air", gamma=1.4, M=0.02897, mu=1.8e-5}}
fiesta.time.dt = 1e-4
fiesta.grid.type = "terrain"
fiesta.grid.ndim = 3
fiesta.grid.ni = {6, 5, 4}
fiesta.grid.dx = {1, 1, 1}
fiesta.tdx = 10.0
fiesta.tdy = 12.5
fiesta.h = 100.0
fiesta.bc.xmin = "outflow"
fiesta.bc.xmax = "outflow"
fiesta.bc.ymin = "outflow"
fiesta.bc.ymax = "outflow"
fiesta.bc.zmin = "reflective"
fiesta.bc.zmax = "outflow"
fiesta.mpi.procs = {1, 1, 1}
function fiesta.initial_conditions(x, y, z, v)
    if v == 3 then return 2.5e5 end
    if v == 4 then return 1.2 end
    return 0
end
"""


def test_terrain_deck_and_nodes():
    d = deck.load(text=DECK_TERRAIN)
    cfg = d.config()
    assert cfg.grid_type == abi.GRID_GENERALIZED and (cfg.dx, cfg.dy, cfg.dz) == (1.0, 1.0, 1.0)
    assert (d.tdx, d.tdy, d.h) == (10.0, 12.5, 100.0)
    with pytest.raises(deck.DeckError, match="ground heights"):
        d.grid_nodes(cfg)
    hgt = np.fromfunction(lambda i, j: 3.0 * i + 0.5 * j * j, (7, 6))
    X = d.grid_nodes(cfg, height=hgt)
    i, j, k = 5, 4, 3
    assert X[i, j, k, 0] == 10.0 * i and X[i, j, k, 1] == 12.5 * j
    assert X[i, j, k, 2] == hgt[i, j] + (100.0 - hgt[i, j]) / 4 * k
    U = d.initial_conditions(cfg, X)
    assert U[3, 3, 3, 3] == 2.5e5 and np.all(U[..., 0] == 0)
    with pytest.raises(deck.DeckError, match="fiesta.tdx"):
        deck.load(text=DECK_TERRAIN.replace("fiesta.tdx = 10.0", ""))
    with pytest.raises(deck.DeckError, match="ndim must be equal to 3"):
        deck.load(text=DECK_TERRAIN.replace("fiesta.grid.ndim = 3", "fiesta.grid.ndim = 2")
                  .replace("{6, 5, 4}", "{6, 5}"))
