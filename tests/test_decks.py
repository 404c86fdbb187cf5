"""DL_POLY 2 decks (CONTROL, FIELD, CONFIG) of the reference read into the GB300 path's
inputs (mbx/decks.py): exact round trips of positions, velocities and cell, the vmbpol and
Ewald settings, the FIELD units applied to tt68 dispersion parameters, the Ewald precision
rule of SOURCE/simdef_cmd.f:1270-1290, and the errors of inconsistent decks."""
import math

import numpy as np
import pytest

from mbx import decks, systems


def test_deck_round_trip_matches_systems():
    box = systems.config0()
    vdw = [("OW", "OW", 600.0, 3.2, 0.0, 0.0), ("HW", "OW", 200.0, 3.6, 0.0, 0.0), ("HW", "HW", 60.0, 3.9, 0.0, 0.0)]
    d = decks.read_deck(*decks.write_deck(box, vdw=vdw))
    assert d["nw"] == box.nw and d["natms"] == box.natms and d["imcon"] == box.imcon
    np.testing.assert_array_equal(d["xyz"], box.xyz)
    np.testing.assert_array_equal(d["vel"], box.vel)
    np.testing.assert_array_equal(d["cell"], np.asarray(box.cell, np.float64))
    polr, polr2 = systems.polarizabilities(box.nw)
    np.testing.assert_array_equal(d["polr"], polr)
    np.testing.assert_array_equal(d["polr2"], polr2)
    want = systems.polar_params(alpha=0.3, rcut=9.0, kmax=(8, 8, 8), toler_debye=1e-8)
    np.testing.assert_allclose(d["polar_prm"], want, rtol=1e-15, atol=0)
    # dispersion: types by first appearance (OW 1, HW 2, MW 3, M without partners -> 0)
    lt, mol = systems.water_types(box)
    np.testing.assert_array_equal(np.where(d["ltype"] > 0, d["ltype"], 0), np.where(lt == 3, 0, lt))
    np.testing.assert_array_equal(d["molecule"], mol)
    nt, pp = d["disp"]
    assert nt == 3
    np.testing.assert_allclose(pp[0], [600.0 * 418.4, 3.2, 0.0, 0.0], rtol=1e-15)   # OW-OW
    np.testing.assert_allclose(pp[1], [200.0 * 418.4, 3.6, 0.0, 0.0], rtol=1e-15)   # HW-OW
    np.testing.assert_allclose(pp[2], [60.0 * 418.4, 3.9, 0.0, 0.0], rtol=1e-15)    # HW-HW


def test_units_and_control_keywords():
    box = systems.box_for(32, seed=3)
    c, f, g = decks.write_deck(box, units="kj", vdw=[("OW", "OW", 1.0, 2.0, 3.0, 4.0)],
                               control_extra="aspc_omega 0.5\nascc 0.3\nascd 0.35\neps 2.0")
    c = c.replace("ewald sum 0.3 8 8 8", "ewald sum 0.35 7 6 5").replace("iter 1.0e-8", "iter 2.0d-9")
    d = decks.read_deck(c, f, g)
    p = d["polar_prm"]
    assert (p[0], p[11], p[12], p[13]) == (0.35, 7, 6, 5)
    assert p[2] == 2.0 and p[4] == 0.5 and (p[8], p[9]) == (0.3, 0.35)
    assert p[3] == 2.0e-9 / decks.EATD
    np.testing.assert_array_equal(d["disp"][1][0], [100.0, 2.0, 300.0, 4.0])


@pytest.mark.parametrize("lines, want", [
    ("", None),
    ("aspc", (4, 6, 6.0 / 11.0)),
    ("aspc_k 2", None),                                   # sets k, ASPC still off
    ("aspc\naspc_k 2", (2, 4, 4.0 / 7.0)),
    ("aspc_k 2\naspc", (4, 6, 6.0 / 11.0)),               # `aspc` afterwards restores k 4
    ("aspc\naspc_k 2\naspc_omega 0.5", (2, 4, 0.5)),
    ("aspc\naspc_k 3", (3, 6, 6.0 / 11.0)),               # other k keep the weight and step count
])
def test_aspc_keywords(lines, want):
    """`aspc`, `aspc_k`, `aspc_omega` in the order given, as SOURCE/simdef_cmd.f:742-788."""
    box = systems.box_for(32, seed=3)
    c, f, g = decks.write_deck(box, control_extra=lines)
    d = decks.read_deck(c, f, g)
    if want is None:
        assert d["aspc"] is None
    else:
        assert d["aspc"] == want[:2] and d["polar_prm"][4] == want[2]


def test_ewald_precision_rule():
    cell = [19.73, 0, 0, 0, 21.0, 0, 0, 0, 23.5]
    alpha, km = decks.ewald_from_precision(cell, 9.0, 1e-6)
    # the rule restated: tol = sqrt|ln(eps rc)|, alpha = sqrt|ln(eps rc tol)| / rc,
    # tol1 = sqrt(-ln(eps rc (2 tol alpha)^2)), kmax = nint(0.25 + L alpha tol1 / pi)
    eps, rc = 1e-6, 9.0
    tol = math.sqrt(abs(math.log(eps * rc)))
    a = math.sqrt(abs(math.log(eps * rc * tol))) / rc
    tol1 = math.sqrt(-math.log(eps * rc * (2 * tol * a) ** 2))
    assert alpha == a
    assert km == [int(math.floor(0.25 + L * a * tol1 / math.pi + 0.5)) for L in (19.73, 21.0, 23.5)]
    box = systems.box_for(32, seed=4)
    c, f, g = decks.write_deck(box)
    d = decks.read_deck(c.replace("ewald sum 0.3 8 8 8", "ewald precision 1.0e-6"), f, g)
    a2, k2 = decks.ewald_from_precision(box.cell, 9.0, 1e-6)
    assert d["polar_prm"][0] == a2 and list(d["polar_prm"][11:14]) == k2


def test_inconsistent_decks_are_refused():
    box = systems.box_for(32, seed=5)
    c, f, g = decks.write_deck(box)
    with pytest.raises(ValueError):
        decks.read_deck(c, f.replace("units kcal", "units furlongs"), g)
    short = "\n".join(g.splitlines()[:-3]) + "\n"   # one atom short
    with pytest.raises(ValueError):
        decks.read_deck(c, f, short)
    with pytest.raises(ValueError):
        decks.read_deck(c.replace("ewald sum 0.3 8 8 8", ""), f, g)
