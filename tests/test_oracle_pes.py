"""Self-consistency of the oracle's 1-body Partridge-Schwenke PES (SOURCE/ps_type_couple.f90)."""
import numpy as np
import pytest

from mbx import systems


@pytest.fixture(scope="module")
def box():
    return systems.box_for(32, seed=8)


def test_pes_forces_are_minus_gradient(oracle_lib, box):
    out = oracle_lib.angfrc_ps(box, velocities=False)
    h = 1e-6
    for atom in (0, 1, 5):
        for c in range(3):
            e = []
            for s in (+1, -1):
                b = systems.WaterBox(box.nw, box.L, box.xyz.copy(), box.vel, 0)
                b.xyz[atom, c] += s * h
                e.append(oracle_lib.angfrc_ps(b, velocities=False)["engang"])
            fd = -(e[0] - e[1]) / (2 * h)
            f = out["forces"][atom, c]
            assert abs(fd - f) <= 2e-6 * max(abs(f), 1.0), (atom, c, fd, f)


def test_pes_energy_partition_and_momentum(oracle_lib, box):
    out = oracle_lib.angfrc_ps(box)
    assert abs(out["atomic_energy"].sum() - out["engang"]) <= 1e-12 * abs(out["engang"])
    assert np.max(np.abs(out["forces"].sum(0))) <= 1e-9 * np.max(np.abs(out["forces"]))


def test_pes_virial_is_sum_r_dot_f(oracle_lib, box):
    # angfrc's vterm is the virial of the intramolecular forces: sum over bonds of r.f
    out = oracle_lib.angfrc_ps(box, velocities=False)
    m = oracle_lib.image_monomers(box)
    f = out["forces"]
    w = np.zeros_like(f[:3 * box.nw])
    w[:] = m.reshape(-1, 3)
    vir = -np.sum(w * f[:3 * box.nw])
    assert abs(vir - out["virang"]) <= 1e-8 * abs(out["virang"])


def test_pes_coupling_term_bend_minimum(oracle_lib):
    # ps_type_couple is the angle/coupling part of the Partridge-Schwenke PES (the O-H
    # stretches are separate bond terms); at r = r_e its bend minimum is near theta_e
    import ctypes as C
    D = C.POINTER(C.c_double)

    def V(th_deg):
        th = np.radians(th_deg)
        f = np.zeros(6)
        p = C.c_double()
        v = C.c_double()
        oracle_lib.lib.orc_ps_couple(0.958649, 1.0, 0.0, 0.0, 0.958649, np.cos(th), np.sin(th), 0.0, th,
                                     C.byref(p), f.ctypes.data_as(D), C.byref(v))
        return p.value

    assert V(104.3475) < V(100.0) and V(104.3475) < V(109.0)
