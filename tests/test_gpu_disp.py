"""Dispersion (vdw type 12) on the GPU against the oracle: FP64 parity 1e-10 on a small
box (all-pairs list), the 4096-water box (cell list) and an orthorhombic box; the Verlet
list is kept while atoms move less than half the skin and rebuilt after."""
import numpy as np
import pytest

from conftest import rel_err
from mbx import capi, systems

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
PRM = systems.DISP_PARAMS_SYNTHETIC


def _ortho():
    b = systems.water_box(216, 19.5, seed=9, lattice=6)
    b.xyz[:, 1] *= 1.05
    b.xyz[:, 2] *= 0.97
    b.cell = np.array([19.5, 0, 0, 0, 19.5 * 1.05, 0, 0, 0, 19.5 * 0.97])
    b.imcon = 2
    return b


def _check(got, ref):
    assert abs(got["eng"] - ref["eng"]) <= TOL64 * abs(ref["eng"])
    assert abs(got["vir"] - ref["vir"]) <= TOL64 * abs(ref["vir"])
    assert rel_err(got["stress"], ref["stress"]) <= TOL64
    assert rel_err(got["forces"], ref["forces"]) <= TOL64
    assert rel_err(got["atomic_energy"], ref["atomic_energy"]) <= TOL64
    assert rel_err(got["jpot"], ref["jpot"]) <= TOL64


def _triclinic():
    b = systems.water_box(216, 19.5, seed=13, lattice=6)
    L = b.L
    H = np.array([[L, 0.1 * L, 0.05 * L], [0.0, L, 0.08 * L], [0.0, 0.0, L]])
    b.xyz = (b.xyz / L) @ H.T
    b.cell = np.ascontiguousarray(H.T.ravel())
    b.imcon = 3
    return b


@pytest.mark.parametrize("name", ["cfg0_256", "cfg1_4096", "ortho_imcon2", "triclinic_imcon3"])
def test_dispersion_matches_oracle(oracle_lib, name):
    box = {"cfg0_256": systems.config0, "cfg1_4096": systems.config1, "ortho_imcon2": _ortho,
           "triclinic_imcon3": _triclinic}[name]()
    lt, mol = systems.water_types(box)
    ctx = capi.Context(0)
    try:
        ctx.disp_setup(PRM, rcut=9.0, delr=1.0)
        got = ctx.dispersion(box, lt, mol)
    finally:
        ctx.close()
    ref = oracle_lib.dispersion(box, lt, mol, PRM, rcut=9.0)
    _check(got, ref)


def test_verlet_list_kept_within_half_skin_and_rebuilt_after(oracle_lib):
    box = systems.config0()
    lt, mol = systems.water_types(box)
    rng = np.random.default_rng(1)
    ctx = capi.Context(0)
    try:
        ctx.disp_setup(PRM, rcut=8.0, delr=1.0)
        ctx.dispersion(box, lt, mol)
        assert ctx.disp_list_builds() == 1
        small = systems.WaterBox(box.nw, box.L, box.xyz + rng.uniform(-0.25, 0.25, box.xyz.shape), box.vel, 0)
        got = ctx.dispersion(small, lt, mol)
        assert ctx.disp_list_builds() == 1          # every atom moved < delr / 2: list kept
        _check(got, oracle_lib.dispersion(small, lt, mol, PRM, rcut=8.0))
        big = systems.WaterBox(box.nw, box.L, small.xyz.copy(), box.vel, 0)
        big.xyz[5] += np.array([0.6, 0.0, 0.0])     # one atom beyond half the skin
        got = ctx.dispersion(big, lt, mol)
        assert ctx.disp_list_builds() == 2
        _check(got, oracle_lib.dispersion(big, lt, mol, PRM, rcut=8.0))
        # other molecules with the same number of atoms: the list is rebuilt
        mol2 = mol.copy()
        mol2[0:3], mol2[3:6] = mol[3:6], mol[0:3]
        ctx.dispersion(big, lt, mol2)
        assert ctx.disp_list_builds() == 3
    finally:
        ctx.close()


def test_dispersion_rejects_use_before_setup():
    ctx = capi.Context(0)
    try:
        box = systems.box_for(32, seed=2)
        lt, mol = systems.water_types(box)
        with pytest.raises(capi.MbxError):
            ctx.dispersion(box, lt, mol)
    finally:
        ctx.close()
