"""i-PI driver mode on the GPU (mbx_ipi_run): the forces, energy, virial and water dipoles
a loopback i-PI server receives equal mbx_water_step on the same configuration, converted
with the reference's unit factors (SOURCE/ipi.f90:72-77); a replica's second frame starts
from its first frame's dipoles."""
import numpy as np
import pytest

from mbx import capi, systems
from mbx.ipi_loopback import FakeIpiServer

pytestmark = pytest.mark.gpu

BOHR = np.float64(np.float32(0.52917721067))
E_AU = np.float64(np.float32(3.8087989e-06))
RATIO = np.float64(np.float32(np.float64(np.float32(418.6799938)) / 418.4))


def _moldip(step, nw):
    """per water: DMS charges x positions (H imaged next to O) + its sites' dipoles, Debye"""
    x, q, d = step["sites"], step["chge"], step["dipoles"]
    L = np.array([step["cell"][0], step["cell"][4], step["cell"][8]])
    out = np.zeros((nw, 3))
    for w in range(nw):
        o, m = 3 * w, 3 * nw + w
        mu = q[m] * x[m]
        for h in (o + 1, o + 2):
            dd = x[o] - x[h]
            dd -= L * np.round(dd / L)
            mu = mu + q[h] * (x[o] - dd)
        mu = mu + d[o] + d[o + 1] + d[o + 2] + d[m]
        out[w] = mu * 4.803239
    return out


def test_ipi_run_matches_water_step():
    box = systems.config0()
    nw = box.nw
    h = np.array(box.cell, np.float64) / BOHR          # the client multiplies by BOHR again
    hinv = np.linalg.inv(h.reshape(3, 3)).ravel()
    pos0 = box.xyz[:3 * nw] / BOHR
    pos1 = pos0 + 0.0002 * box.vel[:3 * nw] / BOHR
    srv = FakeIpiServer([(0, h, hinv, pos0), (0, h, hinv, pos1)])
    ctx = capi.Context(0)
    try:
        steps = ctx.ipi_run(srv.address, precision=capi.FP64)
        iters_second = ctx.polar_iterations()
    finally:
        ctx.close()
    srv.join()
    assert srv.error is None, srv.error
    assert steps == 2
    # the same evaluations directly (positions as the client converts them)
    cell = np.array([h[b + 3 * a] for b in range(3) for a in range(3)]) * BOHR
    prm = capi.polar_params_for_cell(cell)
    ref = capi.Context(0)
    try:
        dip = None
        for k, pos in enumerate((pos0, pos1)):
            b = systems.box_for(nw, seed=1)
            b.cell = cell
            b.imcon = 2
            b.xyz = np.zeros((4 * nw, 3))
            b.xyz[:3 * nw] = pos * BOHR
            st = ref.water_step(b, prm, precision=capi.FP64, dip0=dip, heat=False)
            st["cell"] = cell
            dip = st["dipoles"]
            if k == 1:
                iters_ref = ref.polar_iterations()
            sc = st["scalars"]
            nb, be = capi.NSCALARS, capi.NWATERSCALARS
            e = sc[0] + sc[1] + sc[nb] + sc[nb + 14] + sc[be]
            stress = sc[3:12] + sc[nb + 2:nb + 11] + sc[nb + 16:nb + 25] + sc[be + 2:be + 11]
            r = srv.replies[k]
            assert abs(r["energy"] - e * E_AU * RATIO) <= 1e-12 * abs(e * E_AU * RATIO)
            f = st["forces"][:3 * nw] * E_AU * BOHR * RATIO
            assert np.abs(r["forces"] - f).max() <= 1e-12 * np.abs(f).max()
            vir = np.array([stress[b_ + 3 * a] for b_ in range(3) for a in range(3)]) * E_AU * RATIO
            assert np.abs(r["virial"] - vir).max() <= 1e-12 * np.abs(vir).max()
            md = np.array([float(t) for t in r["text"].split()]).reshape(nw, 3)
            want = _moldip(st, nw)
            assert np.abs(md - want).max() <= 1e-10 * np.abs(want).max()
    finally:
        ref.close()
    assert iters_second == iters_ref
