"""A deck written for the reference (CONTROL, FIELD, CONFIG), read with mbx.decks, drives
mbx_water_step to the same results as the synthetic box it was written from."""
import numpy as np
import pytest

from mbx import capi, decks, systems

pytestmark = pytest.mark.gpu


def test_deck_drives_water_step():
    box = systems.config0()
    vdw = [("OW", "OW", 600.0, 3.2, 0.0, 0.0), ("HW", "OW", 200.0, 3.6, 0.0, 0.0), ("HW", "HW", 60.0, 3.9, 0.0, 0.0)]
    d = decks.read_deck(*decks.write_deck(box, vdw=vdw))
    prm = systems.polar_params(alpha=0.3, rcut=9.0, kmax=(8, 8, 8), toler_debye=1e-8)
    ctx = capi.Context(0)
    try:
        # the deck's dispersion table (types OW, HW, MW) and the synthetic one agree on every
        # interacting pair; the M sites carry no dispersion in either
        ctx.disp_setup(d["disp"][1], rcut=9.0, delr=1.0)
        got = ctx.water_step(box, d["polar_prm"], precision=capi.FP64, disp=(d["ltype"], d["molecule"]))
        ctx.disp_setup(systems.DISP_PARAMS_SYNTHETIC, rcut=9.0, delr=1.0)
        want = ctx.water_step(box, prm, precision=capi.FP64, disp=systems.water_types(box))
    finally:
        ctx.close()
    for key in ("forces", "atomic_energy", "dipoles"):
        g, w = got[key], want[key]
        assert np.abs(g - w).max() <= 1e-10 * np.abs(w).max(), key
    assert np.abs(got["scalars"] - want["scalars"]).max() <= 1e-10 * np.abs(want["scalars"]).max()
