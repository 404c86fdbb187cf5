"""The SPME oracle (oracle/spme_oracle.py) on the CPU.

* Its SPME for charges and dipoles, with the dipoles at zero, equals the line-by-line
  restatement of the reference's charge SPME (SOURCE/ewald_spme.f, bspgen.f, bspcoe.f,
  spme_for.f): energy, stress and forces to 1e-12.
* Forces, fields and potentials are the exact derivatives of its energy (central
  differences; the forces up to the removed mean).
* It converges to the explicit Ewald sum (the reference's ewald1p k space, restated in
  numpy) as the grid is refined: every quantity, the heat-current term included.
* The explicit Ewald sum's fields, potentials and forces are the derivatives of its energy.
"""
import numpy as np
import pytest

import spme_oracle as so
from mbx import systems


def _case(n=96, seed=0, L=19.73, tric=False):
    rng = np.random.default_rng(seed)
    cell = np.array([L, 0, 0, 0, L, 0, 0, 0, L], np.float64)
    if tric:
        cell = np.array([L, 0, 0, 0.2 * L, L, 0, 0.1 * L, -0.15 * L, L], np.float64)
    s = rng.uniform(-0.5, 0.5, (n, 3))
    xyz = s @ cell.reshape(3, 3)
    q = rng.normal(size=n)
    q -= q.mean()
    mu = rng.normal(scale=0.1, size=(n, 3))
    v = rng.normal(scale=0.01, size=(n, 3))
    return xyz, q, mu, v, cell


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / np.abs(np.asarray(b)).max())


@pytest.mark.parametrize("tric", [False, True])
def test_charge_spme_equals_reference_restatement(tric):
    xyz, q, _, _, cell = _case(tric=tric)
    alpha, K, p = 0.35, (24, 30, 24), 6
    e_ref, st_ref, f_ref = so.ewald_spme_charges(xyz, q, cell, alpha, K, p)
    got = so.spme_kspace(xyz, q, cell, alpha, K, p)
    engsic = -so.R4PIE0 * alpha * np.sum(q ** 2) / np.sqrt(np.pi)
    # the only difference is the Nyquist plane, which the reference gives to m = -K/2 and
    # the SPME path leaves out: its Gaussian factor exp(-k^2 / 4 alpha^2) is 1e-13 at K = 24
    # on this 19.73 A cell (1e-9 at K = 20, where the two differ by ~1e-9 in the stress)
    tol = 1e-12
    assert abs(got["eng"] - (e_ref - engsic)) <= tol * abs(e_ref - engsic)
    assert abs(got["engc"] - got["eng"]) <= 1e-14 * abs(got["eng"])
    assert _rel(got["stress"], st_ref) <= tol
    assert _rel(got["forces"], f_ref) <= tol


def test_spme_derivatives_are_exact():
    xyz, q, mu, _, cell = _case(n=48, seed=1, tric=True)
    alpha, K, p = 0.4, (20, 20, 24), 6
    ref = so.spme_kspace(xyz, q, cell, alpha, K, p, dip=mu)
    E = lambda x_, q_, m_: so.spme_kspace(x_, q_, cell, alpha, K, p, dip=m_)["eng"]
    h = 1e-5
    fmean = None
    for j in (3, 17):
        for c in range(3):
            xp, xm = xyz.copy(), xyz.copy()
            xp[j, c] += h
            xm[j, c] -= h
            mp, mm = mu.copy(), mu.copy()
            mp[j, c] += h
            mm[j, c] -= h
            fd_f = -(E(xp, q, mu) - E(xm, q, mu)) / (2 * h)
            fd_e = -(E(xyz, q, mp) - E(xyz, q, mm)) / (2 * h)
            scale = np.abs(ref["field"]).max()
            assert abs(fd_e - ref["field"][j, c]) <= 1e-6 * scale
            # the forces carry the removed mean (the SPME drift)
            drift = fd_f - ref["forces"][j, c]
            fmean = drift if fmean is None else fmean
            assert abs(drift) <= 1e-3 * np.abs(ref["forces"]).max()
        qp, qm = q.copy(), q.copy()
        qp[j] += h
        qm[j] -= h
        fd_p = (E(xyz, qp, mu) - E(xyz, qm, mu)) / (2 * h)
        assert abs(fd_p - ref["pot"][j]) <= 1e-6 * np.abs(ref["pot"]).max()


def test_spme_converges_to_ewald():
    xyz, q, mu, v, cell = _case(n=96, seed=2)
    alpha = 0.35
    ew = so.ewald_kspace(xyz, q, cell, alpha, (14, 14, 14), dip=mu, vel=v)
    errs = []
    for K in ((20, 20, 20), (24, 24, 24), (32, 32, 32)):
        sp = so.spme_kspace(xyz, q, cell, alpha, K, 6, dip=mu, vel=v)
        e = max(abs(sp["eng"] - ew["eng"]) / abs(ew["eng"]), abs(sp["engc"] - ew["engc"]) / abs(ew["engc"]),
                *(_rel(sp[k], ew[k]) for k in ("stress", "jpot", "forces", "field", "pot")))
        errs.append(e)
    # order-6 interpolation: the error falls steeply with the spacing (1.0, 0.82, 0.62 A)
    assert errs[0] > errs[1] > errs[2]
    assert errs[1] <= 1e-4
    assert errs[2] <= 1e-5


def test_ewald_derivatives_are_exact():
    xyz, q, mu, _, cell = _case(n=32, seed=4, L=12.0)
    alpha, kmax = 0.5, (8, 8, 8)
    ref = so.ewald_kspace(xyz, q, cell, alpha, kmax, dip=mu)
    E = lambda x_, q_, m_: so.ewald_kspace(x_, q_, cell, alpha, kmax, dip=m_)["eng"]
    h = 1e-5
    j = 7
    for c in range(3):
        xp, xm = xyz.copy(), xyz.copy()
        xp[j, c] += h
        xm[j, c] -= h
        mp, mm = mu.copy(), mu.copy()
        mp[j, c] += h
        mm[j, c] -= h
        fd_f = -(E(xp, q, mu) - E(xm, q, mu)) / (2 * h)
        fd_e = -(E(xyz, q, mp) - E(xyz, q, mm)) / (2 * h)
        # the exact Ewald forces sum to zero: the mean removal changes nothing
        assert abs(fd_f - ref["forces"][j, c]) <= 1e-6 * np.abs(ref["forces"]).max()
        assert abs(fd_e - ref["field"][j, c]) <= 1e-6 * np.abs(ref["field"]).max()
    qp, qm = q.copy(), q.copy()
    qp[j] += h
    qm[j] -= h
    assert abs((E(xyz, qp, mu) - E(xyz, qm, mu)) / (2 * h) - ref["pot"][j]) <= 1e-6 * np.abs(ref["pot"]).max()


def test_spme_on_water_box_matches_ewald():
    """DMS-like charges on a water box (O, H, H, M) with dipoles: SPME at the config-1 grid
    rule (spacing <= 0.78 A; 18^3 here) within 3e-5 of the Ewald sum, the heat term included,
    and 1e-4 for the stress (a sum with cancellations; 6e-5 measured)."""
    box = systems.box_for(64, seed=3)
    n = 4 * box.nw
    rng = np.random.default_rng(5)
    xyz = np.array(box.xyz[:n], np.float64)
    o = xyz[:3 * box.nw:3]
    xyz[3 * box.nw:] = o + 0.2 * (xyz[1:3 * box.nw:3] + xyz[2:3 * box.nw:3] - 2 * o) / 2
    q = np.zeros(n)
    q[1:3 * box.nw:3] = 0.55
    q[2:3 * box.nw:3] = 0.55
    q[3 * box.nw:] = -1.1
    mu = rng.normal(scale=0.05, size=(n, 3))
    mu[3 * box.nw:] = 0.0
    v = rng.normal(scale=0.01, size=(n, 3))
    K = tuple([_smooth_even(box.L / 0.7766)] * 3)   # the grid rule of mbx_spme_grid_for_cell
    alpha = 0.35
    ew = so.ewald_kspace(xyz, q, box.cell, alpha, (12, 12, 12), dip=mu, vel=v)
    sp = so.spme_kspace(xyz, q, box.cell, alpha, K, 6, dip=mu, vel=v)
    for k, tol in (("stress", 1e-4), ("jpot", 3e-5), ("forces", 3e-5), ("field", 3e-5), ("pot", 3e-5)):
        assert _rel(sp[k], ew[k]) <= tol, (k, _rel(sp[k], ew[k]))
    assert abs(sp["eng"] - ew["eng"]) <= 2e-5 * abs(ew["eng"])


def _smooth_even(x):
    k = max(2, int(np.ceil(x - 1e-9)))
    while True:
        if k % 2 == 0:
            m = k
            for p in (2, 3, 5):
                while m % p == 0:
                    m //= p
            if m == 1:
                return k
        k += 1
