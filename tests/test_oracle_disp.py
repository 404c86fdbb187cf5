"""The dispersion oracle (vdw type 12 of the reference): Tang-Toennies damping, tables,
forces as the gradient, energy partition, virial; and the library's host-side
long-range correction against the oracle's."""
import math

import numpy as np
import pytest

from mbx import systems

PRM = systems.DISP_PARAMS_SYNTHETIC


def _tt_closed(n, x):
    return 1.0 - math.exp(-x) * sum(x ** k / math.factorial(k) for k in range(n + 1))


@pytest.mark.parametrize("n", [6, 8])
def test_tang_toennies(oracle_lib, n):
    for x in (0.5, 1.0, 3.0, 10.0, 30.0):
        assert abs(oracle_lib.lib.orc_tang_toennies(n, x) - _tt_closed(n, x)) <= 1e-13
    # below ~1e-8 the reference switches to the series exp(-x) sum_{k>n} x^k/k!
    for x in (1e-3, 1e-2, 0.05):
        series = math.exp(-x) * sum(x ** k / math.factorial(k) for k in range(n + 1, n + 40))
        assert abs(oracle_lib.lib.orc_tang_toennies(n, x) - series) <= 1e-8 * series


def test_tables_match_the_formula(oracle_lib):
    import ctypes as C
    mxgrid, rcut = 1004, 9.0
    dl = rcut / (mxgrid - 4)
    v = np.zeros(mxgrid)
    g = np.zeros(mxgrid)
    p = np.ascontiguousarray(PRM[0])
    D = C.POINTER(C.c_double)
    oracle_lib.lib.orc_disp_tables(1, p.ctypes.data_as(D), mxgrid, dl, v.ctypes.data_as(D), g.ctypes.data_as(D))
    for i in (150, 500, 999):   # r >= 1.4 A: no cancellation in 1 - exp(-x) sum(...)
        r = (i + 1) * dl
        ref = -p[0] * _tt_closed(6, p[1] * r) / r ** 6
        assert abs(v[i] - ref) <= 1e-12 * abs(ref)
        h = 1e-6   # gg12 = -r dV/dr
        dv = (-p[0] * _tt_closed(6, p[1] * (r + h)) / (r + h) ** 6 + p[0] * _tt_closed(6, p[1] * (r - h)) / (r - h) ** 6) / (2 * h)
        assert abs(g[i] + r * dv) <= 1e-6 * abs(g[i])


def _small_box():
    return systems.box_for(64, seed=3)


def test_forces_are_minus_gradient(oracle_lib):
    box = _small_box()
    lt, mol = systems.water_types(box)
    out = oracle_lib.dispersion(box, lt, mol, PRM, rcut=5.5)
    f = out["forces"]
    rng = np.random.default_rng(0)
    for atom in rng.choice(3 * box.nw, 5, replace=False):
        for c in range(3):
            h = 1e-4
            e = []
            for s in (+1, -1):
                b = systems.WaterBox(box.nw, box.L, box.xyz.copy(), box.vel, box.seed)
                b.xyz[atom, c] += s * h
                e.append(oracle_lib.dispersion(b, lt, mol, PRM, rcut=5.5, velocities=False)["eng"])
            fd = -(e[0] - e[1]) / (2 * h)
            assert abs(fd - f[atom, c]) <= 1e-5 * max(abs(f[atom, c]), 1.0), (atom, c, fd, f[atom, c])


def test_partition_momentum_virial(oracle_lib):
    box = _small_box()
    lt, mol = systems.water_types(box)
    out = oracle_lib.dispersion(box, lt, mol, PRM, rcut=6.0)
    assert out["npairs"] > 0
    assert abs(out["atomic_energy"].sum() - out["eng"]) <= 1e-12 * abs(out["eng"])
    assert np.max(np.abs(out["forces"].sum(0))) <= 1e-9 * np.max(np.abs(out["forces"]))
    # stress = sum d (x) f and virial = -sum d . f over the pairs
    assert abs(out["stress"][0] + out["stress"][4] + out["stress"][8] + out["vir"]) <= 1e-10 * abs(out["vir"])
    # M sites and intramolecular pairs carry nothing
    assert np.all(out["forces"][3 * box.nw:] == 0.0)


def test_library_lrc_matches_oracle(oracle_lib):
    """mbx_disp_lrc runs on the host (no GPU): the library's restatement of lrcorrect
    against the oracle's, with the reference's factorial."""
    import ctypes as C
    from mbx import capi
    lib = capi.load()
    prm = np.ascontiguousarray(PRM.ravel())
    numtyp = np.array([256, 512, 256], dtype=np.int32)
    e = C.c_double(0)
    v = C.c_double(0)
    rc = lib.mbx_disp_lrc(3, prm.ctypes.data_as(C.POINTER(C.c_double)), numtyp.ctypes.data_as(C.POINTER(C.c_int)),
                          9.0, 19.73 ** 3, C.byref(e), C.byref(v))
    assert rc == 0
    eo, vo = oracle_lib.disp_lrc(PRM, numtyp, 9.0, 19.73 ** 3)
    assert eo < 0.0
    assert abs(e.value - eo) <= 1e-12 * abs(eo) and abs(v.value - vo) <= 1e-12 * abs(vo)
