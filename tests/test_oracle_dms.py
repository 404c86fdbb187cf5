"""Oracle M sites and DMS charges (SOURCE/qdetermine.f90): neutrality and dq/dr by finite differences."""
import numpy as np

from mbx import systems

GAMMA = 0.426706882


def _p12(q, nw, i, gamma=GAMMA):
    f = gamma / 2.0 / (1.0 - gamma)
    qh1, qh2 = q[3 * i + 1], q[3 * i + 2]
    s = (qh1 + qh2) / (1.0 + 2.0 * f)
    return 0.5 * (s + (qh1 - qh2)), 0.5 * (s - (qh1 - qh2))


def test_msites_and_neutrality(oracle_lib):
    b = systems.config0()
    xyz, q, dp, worst = oracle_lib.msites_dms(b)
    assert worst <= 1e-12
    nw = b.nw
    O, H1, H2 = b.xyz[0:3 * nw:3], b.xyz[1:3 * nw:3], b.xyz[2:3 * nw:3]
    M = O + GAMMA / 2.0 * ((H1 - O) + (H2 - O))
    assert np.max(np.abs(xyz[3 * nw:] - M)) <= 1e-12
    assert np.all(q[1:3 * nw:3] > 0.4) and np.all(q[3 * nw:] < -0.8)


def test_dms_derivatives_match_finite_differences(oracle_lib):
    b = systems.box_for(8, seed=2)
    _, _, dp, _ = oracle_lib.msites_dms(b)
    h = 1e-6
    for i in range(3):
        O, H1 = b.xyz[3 * i], b.xyz[3 * i + 1]
        u = (H1 - O) / np.linalg.norm(H1 - O)
        ps = []
        for s in (+1, -1):
            bb = systems.WaterBox(b.nw, b.L, b.xyz.copy(), b.vel, 0)
            bb.xyz[3 * i + 1] = H1 + s * h * u     # changes r1 only
            _, q, _, _ = oracle_lib.msites_dms(bb)
            ps.append(_p12(q, b.nw, i))
        d1 = (ps[0][0] - ps[1][0]) / (2 * h)
        d2 = (ps[0][1] - ps[1][1]) / (2 * h)
        assert abs(d1 - dp[i, 0]) <= 1e-6 * max(abs(dp[i, 0]), 1e-3)
        assert abs(d2 - dp[i, 2]) <= 1e-6 * max(abs(dp[i, 2]), 1e-3)
