"""Self-consistency of the oracle's mbpol_forces restatement (SOURCE/mbpol.f90:98-1361)."""
import numpy as np
import pytest

from mbx import systems


@pytest.fixture(scope="module")
def small_box():
    return systems.box_for(64, seed=3)


@pytest.fixture(scope="module")
def tiny_box():
    return systems.box_for(24, seed=5)


def _brute_lists(box):
    m = box.monomers()
    O = m[:, 0:3]
    d = O[:, None, :] - O[None, :, :]
    d = d - box.L * np.round(d * (1.0 / box.L))
    r2 = (d[..., 0] ** 2 + d[..., 1] ** 2) + d[..., 2] ** 2
    nw = box.nw
    pairs = [(i, j) for i in range(nw) for j in range(i + 1, nw) if not r2[i, j] > 6.5 ** 2]
    e = (np.sqrt(r2) <= 4.5).astype(int)
    tri = []
    for i in range(nw):
        for j in range(i + 1, nw):
            for k in range(j + 1, nw):
                if (e[i, j] + e[i, k] + e[j, k]) >= 2:
                    tri.append((i, j, k))
    return np.array(pairs), np.array(tri)


def test_lists_match_brute_force(oracle_lib, small_box):
    out = oracle_lib.mbpol_forces(small_box, lists=True)
    p, t = _brute_lists(small_box)
    assert np.array_equal(out["pairs"], p)
    assert np.array_equal(out["trimers"], t)


def test_atomic_energies_sum_to_total(oracle_lib, small_box):
    out = oracle_lib.mbpol_forces(small_box)
    tot = out["eng2"] + out["eng3"]
    assert abs(out["atomic_energy"].sum() - tot) <= 1e-12 * abs(tot)


def test_forces_are_minus_energy_gradient(oracle_lib, tiny_box):
    small_box = tiny_box
    out = oracle_lib.mbpol_forces(small_box, velocities=False)
    h = 1e-5
    rng = np.random.default_rng(0)
    for atom in rng.choice(3 * small_box.nw, 2, replace=False):
        for c in range(3):
            e = []
            for s in (+1, -1):
                b = systems.WaterBox(small_box.nw, small_box.L, small_box.xyz.copy(), small_box.vel, 0)
                b.xyz[atom, c] += s * h
                o = oracle_lib.mbpol_forces(b, velocities=False)
                e.append(o["eng2"] + o["eng3"])
            fd = -(e[0] - e[1]) / (2 * h)
            f = out["forces"][atom, c]
            assert abs(fd - f) <= 1e-5 * max(abs(f), 10.0)


def test_total_force_vanishes(oracle_lib, small_box):
    out = oracle_lib.mbpol_forces(small_box)
    f = out["forces"]
    assert np.max(np.abs(f.sum(0))) <= 1e-9 * np.max(np.abs(f))


def test_dense_force_matrix_heat_flux_equals_fused(oracle_lib, small_box):
    dense = oracle_lib.mbpol_forces(small_box, dense=True)
    fused = oracle_lib.mbpol_forces(small_box, dense=False)
    assert np.max(np.abs(dense["jpot"] - fused["jpot"])) <= 1e-10 * np.max(np.abs(dense["jpot"]))


@pytest.mark.parametrize("ranks", [2, 3])
def test_replicated_data_ranks_sum_to_serial(oracle_lib, small_box, ranks):
    # bead_rank/bead_size striding of the pair and triple loops (SOURCE/mbpol.f90:215-226, :311-314)
    a = oracle_lib.mbpol_forces(small_box)
    b = oracle_lib.mbpol_forces(small_box, nthreads=ranks)
    # the ranks re-image their own monomer copies, so absolute coordinates (and the
    # virial's w.g terms) differ by lattice shifts at rounding level
    for k in ("eng2", "eng3", "vir"):
        assert abs(a[k] - b[k]) <= 1e-10 * abs(a[k])
    assert np.max(np.abs(a["forces"] - b["forces"])) <= 1e-11 * np.max(np.abs(a["forces"]))
    assert np.max(np.abs(a["jpot"] - b["jpot"])) <= 1e-11 * np.max(np.abs(a["jpot"]))


def test_empty_and_tiny_systems(oracle_lib):
    for nw in (1, 2):
        b = systems.water_box(nw, 12.0, seed=1, lattice=2)
        out = oracle_lib.mbpol_forces(b, lists=True)
        assert out["ntrip"] == 0
        assert np.all(np.isfinite(out["forces"]))
