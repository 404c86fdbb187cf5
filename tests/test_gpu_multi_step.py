"""Many boxes per call (mbx_water_step_multi): each box's results are those of
mbx_water_step on that box alone, for FP64 and mixed, with dispersion and heat current;
a box whose dipoles do not converge is reported in its own status."""
import numpy as np
import pytest

from mbx import capi, systems

pytestmark = pytest.mark.gpu


def _boxes():
    boxes = [systems.box_for(nw, seed=(77, b)) for b, nw in enumerate((48, 32, 64, 32, 40))]
    prms = [systems.polar_params_for(b.cell) for b in boxes]
    for p in prms:
        p[3] = systems.polar_params(toler_debye=1e-10)[3]
    return boxes, prms


def _disp(boxes):
    lt, mol = zip(*(systems.water_types(b) for b in boxes))
    return np.concatenate(lt), np.concatenate(mol)


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
def test_multi_step_matches_single_boxes(precision):
    boxes, prms = _boxes()
    rng = np.random.default_rng(3)
    dip0 = [rng.normal(0, 0.05, size=(b.natms, 3)) for b in boxes]
    for d, b in zip(dip0, boxes):
        d[3 * b.nw:] = 0.0
    ctx = capi.Context(0)
    try:
        ctx.disp_setup(systems.DISP_PARAMS_SYNTHETIC, rcut=4.5, delr=0.3)
        ctx.set_lanes(3)
        got = ctx.water_step_multi(boxes, prms, precision=precision, dip0=np.concatenate(dip0), disp=_disp(boxes))
        # the same boxes one at a time on another context
        one = capi.Context(0)
        try:
            one.disp_setup(systems.DISP_PARAMS_SYNTHETIC, rcut=4.5, delr=0.3)
            want = [one.water_step(b, p, precision=precision, dip0=d, disp=systems.water_types(b))
                    for b, p, d in zip(boxes, prms, dip0)]
        finally:
            one.close()
    finally:
        ctx.close()
    assert got["status"] == 0 and not got["box_status"].any()
    tol = 1e-12 if precision == capi.FP64 else 1e-9
    o = 0
    for b, (w, sc) in enumerate(zip(want, got["scalars"])):
        n = boxes[b].natms
        for key in ("forces", "atomic_energy", "dipoles", "chge", "sites"):
            g, r = got[key][o:o + n], w[key]
            assert np.abs(g - r).max() <= tol * np.abs(r).max(), (b, key, np.abs(g - r).max())
        assert np.abs(sc - w["scalars"]).max() <= tol * np.abs(w["scalars"]).max(), b
        o += n


def test_multi_step_reports_each_box():
    boxes, prms = _boxes()
    prms[2] = prms[2].copy()
    prms[2][14] = 2    # maxit: box 2 cannot converge
    ctx = capi.Context(0)
    try:
        got = ctx.water_step_multi(boxes, prms, precision=capi.FP64, check=False)
        assert got["status"] == capi.ERR_CONVERGE
        assert list(got["box_status"]) == [0, 0, capi.ERR_CONVERGE, 0, 0]
        # the other boxes' results are complete
        single = ctx.water_step(boxes[0], prms[0], precision=capi.FP64)
        n0 = boxes[0].natms
        assert np.abs(got["forces"][:n0] - single["forces"]).max() <= 1e-12 * np.abs(single["forces"]).max()
        # an empty call and a bad box are handled on the host
        assert ctx.water_step_multi([], [], precision=capi.FP64)["status"] == 0
        bad = [p.copy() for p in prms]
        bad[1][4] = 1.5
        with pytest.raises(capi.MbxError):
            ctx.water_step_multi(boxes, bad, precision=capi.FP64)
    finally:
        ctx.close()
