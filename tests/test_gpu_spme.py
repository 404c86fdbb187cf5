"""SPME k space on the GPU (mbx_spme.cu).

* The hand-written 3D FFT against numpy (FP64, both signs, mixed radices 2/3/4/5).
* mbx_spme_kspace (charges + induced point dipoles: energies, stress, heat term, forces,
  fields, potentials) against the numpy restatement (oracle/spme_oracle.py) to 1e-9; that
  restatement's charge part equals the reference's ewald_spme (tests/test_oracle_spme.py).
* Whole electrostatics solves with SPME against the explicit Ewald sum at the same alpha
  and converged kmax (the reference's method): the difference is the SPME discretisation
  error, bounded per quantity below; mixed SPME against FP64 SPME within the mixed budget.
"""
import numpy as np
import pytest

import spme_oracle as so
from mbx import capi, systems

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("shape", [(64, 64, 64), (20, 24, 30), (10, 12, 8), (50, 6, 4)])
def test_fft3d_matches_numpy(mbx_ctx, shape):
    n3, n2, n1 = shape
    rng = np.random.default_rng(sum(shape))
    a = rng.normal(size=(2, n3, n2, n1)) + 1j * rng.normal(size=(2, n3, n2, n1))
    fwd = mbx_ctx.fft3d(a, sign=1)
    bwd = mbx_ctx.fft3d(a, sign=-1)
    N = n1 * n2 * n3
    ref_f = np.fft.ifftn(a, axes=(1, 2, 3)) * N   # sum_g a(g) exp(+2 pi i m.g / n)
    ref_b = np.fft.fftn(a, axes=(1, 2, 3))
    assert _rel(fwd, ref_f) <= 1e-13
    assert _rel(bwd, ref_b) <= 1e-13


def _sites_case(orc, box, seed):
    sites, q, _, _ = orc.msites_dms(box)
    n = sites.shape[0]
    rng = np.random.default_rng(seed)
    dip = rng.normal(0.0, 0.05, size=(n, 3))
    dip[3 * box.nw:] = 0.0
    vel = np.array(box.vel[:n], np.float64)
    vel[3 * box.nw:] = rng.normal(0.0, 0.01, size=(box.nw, 3))
    return sites, q, dip, vel


@pytest.mark.parametrize("which", ["config0", "triclinic"])
def test_spme_kspace_matches_oracle(mbx_ctx, oracle_lib, which):
    if which == "config0":
        box = systems.config0()
        grid, order, alpha = (24, 24, 24), 6, 0.35
    else:
        box = systems.box_for(64, seed=9)
        L = box.L
        box.cell = np.array([L, 0, 0, 0.2 * L, L, 0, 0.1 * L, -0.15 * L, L], dtype=np.float64)
        box.imcon = 3
        grid, order, alpha = (20, 24, 30), 5, 0.5
    sites, q, dip, vel = _sites_case(oracle_lib, box, 3)
    got = mbx_ctx.spme_kspace(sites, box.cell, box.imcon, q, alpha, grid, order=order, dip=dip, vel=vel)
    ref = so.spme_kspace(sites, q, box.cell, alpha, grid, order, dip=dip, vel=vel)
    for key in ("engc", "eng"):
        assert abs(got[key] - ref[key]) <= 1e-10 * abs(ref[key]), (key, got[key], ref[key])
    for key in ("stress", "jpot", "forces", "field", "pot"):
        assert _rel(got[key], ref[key]) <= 1e-9, (key, _rel(got[key], ref[key]))


def _polar_case(orc, box, alpha, kmax, toler=1e-10):
    sites, q, dp, _ = orc.msites_dms(box)
    polr, polr2 = systems.polarizabilities(box.nw)
    prm = systems.polar_params(alpha=alpha, rcut=9.0, kmax=kmax, toler_debye=toler)
    return sites, q, dp, polr, polr2, prm


# SPME (order 6, ~0.8 A spacing, alpha 0.35) against the converged Ewald sum: measured
# differences on the 256-water box are ~1e-6 of the total energy and a few 1e-6 of the
# largest force; the bounds leave a factor of ~10
SPME_TOL = {"engcpe": 2e-5, "forces": 5e-5, "dipoles": 5e-5, "atomic_energy": 5e-5, "jpot": 2e-4, "jkin": 5e-5,
            "stress": 5e-5}


def test_spme_solve_matches_ewald(oracle_lib):
    box = systems.config0()
    sites, q, dp, polr, polr2, prm = _polar_case(oracle_lib, box, 0.35, (13, 13, 13))
    ctx = capi.Context(0)
    try:
        ew = ctx.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, vel=box.vel)
        ctx.set_spme(6, grid=(24, 24, 24))
        sp = ctx.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, vel=box.vel)
        assert ctx.spme_last_grid() == (24, 24, 24)
        mixed = ctx.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, vel=box.vel,
                          precision=capi.MIXED)
    finally:
        ctx.close()
    errs = {"engcpe": abs(sp["engcpe"] - ew["engcpe"]) / abs(ew["engcpe"])}
    for key in ("forces", "dipoles", "atomic_energy", "jpot", "jkin", "stress"):
        errs[key] = _rel(sp[key], ew[key])
    print("SPME vs Ewald:", {k: "%.2e" % v for k, v in errs.items()})
    for key, tol in SPME_TOL.items():
        assert errs[key] <= tol, (key, errs[key])
    # mixed SPME against FP64 SPME: the mixed path's budget
    frms = np.sqrt(np.mean((mixed["forces"] - sp["forces"]) ** 2)) / np.sqrt(np.mean(sp["forces"] ** 2))
    print("mixed vs FP64 SPME: force rms %.2e, jpot %.2e, energy %.2e" %
          (frms, _rel(mixed["jpot"], sp["jpot"]), abs(mixed["engcpe"] - sp["engcpe"]) / abs(sp["engcpe"])))
    assert frms <= 1e-6
    assert _rel(mixed["jpot"], sp["jpot"]) <= 1e-6
    assert _rel(mixed["jkin"], sp["jkin"]) <= 1e-6
    assert abs(mixed["engcpe"] - sp["engcpe"]) <= 1e-8 * abs(sp["engcpe"])


def test_water_step_spme_4096():
    """Config 1's box and k space (4096 H2O, SPME 64^3, order 6, alpha 0.35): the whole FP64
    force evaluation against the same evaluation with the converged Ewald sum (kmax 27,
    exp(-k^2 / 4 alpha^2) < 1e-13 beyond it), and mixed SPME against FP64 SPME."""
    box = systems.config1()
    prm = systems.polar_params(alpha=0.35, rcut=9.0, kmax=(27, 27, 27), toler_debye=1e-10)
    ctx = capi.Context(0)
    try:
        ew = ctx.water_step(box, prm, precision=capi.FP64)
        ctx.set_spme(6, spacing=49.70 / 64)
        sp = ctx.water_step(box, prm, precision=capi.FP64)
        assert ctx.spme_last_grid() == (64, 64, 64)
        mixed = ctx.water_step(box, prm, precision=capi.MIXED)
    finally:
        ctx.close()
    nws = capi.NWATERSCALARS

    def heat(r):
        v = r["scalars"]
        j = v[12:15] + v[15:18] + v[capi.NSCALARS + 11:capi.NSCALARS + 14] + v[capi.NSCALARS + 25:capi.NSCALARS + 28]
        return j + v[nws + 16:nws + 19] + v[nws + 19:nws + 22]

    errs = {"engcpe": abs(sp["scalars"][nws] - ew["scalars"][nws]) / abs(ew["scalars"][nws]),
            "forces": _rel(sp["forces"], ew["forces"]), "dipoles": _rel(sp["dipoles"], ew["dipoles"]),
            "atomic_energy": _rel(sp["atomic_energy"], ew["atomic_energy"]),
            "heat": float(np.linalg.norm(heat(sp) - heat(ew)) / np.linalg.norm(heat(ew)))}
    print("4096 H2O, SPME 64^3 vs Ewald:", {k: "%.2e" % v for k, v in errs.items()})
    for key, tol in (("engcpe", 2e-5), ("forces", 5e-5), ("dipoles", 5e-5), ("atomic_energy", 5e-5),
                     ("heat", 5e-5)):
        assert errs[key] <= tol, (key, errs[key])
    frms = np.sqrt(np.mean((mixed["forces"] - sp["forces"]) ** 2)) / np.sqrt(np.mean(sp["forces"] ** 2))
    herr = float(np.linalg.norm(heat(mixed) - heat(sp)) / np.linalg.norm(heat(sp)))
    print("4096 H2O mixed vs FP64 (SPME): force rms %.2e, heat %.2e" % (frms, herr))
    assert frms <= 1e-5
    assert herr <= 1e-6


def test_spme_dipoles_under_the_ewald_equations(oracle_lib):
    """induced_error of the SPME solve's dipoles under the oracle's Ewald fields (same alpha,
    converged kmax): the residual is the SPME field error, below 1e-4 of the dipoles."""
    box = systems.config0()
    sites, q, dp, polr, polr2, prm = _polar_case(oracle_lib, box, 0.35, (13, 13, 13))
    ctx = capi.Context(0)
    try:
        ctx.set_spme(6, grid=(24, 24, 24))
        sp = ctx.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm)
    finally:
        ctx.close()
    pol = polr2 > 1e-6
    l2, _ = oracle_lib.induced_error(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, sp["dipoles"])
    rms_mu = float(np.sqrt(np.mean(sp["dipoles"][pol] ** 2)))
    rel = l2 / np.sqrt(3 * pol.sum()) / rms_mu
    print("SPME dipoles: Ewald residual rms / dipole rms = %.2e" % rel)
    assert rel <= 1e-4


@pytest.mark.parametrize("spme", [True, False])
def test_overlapped_step_matches_sequential(spme):
    """mbx_set_overlap: the MB-pol terms on a second stream beside the dipole solve give the
    sequential step's results up to the order of FP64 atomic additions.  That order can move
    a CG stopping decision, and the converged dipoles then differ within the dipole
    tolerance (measured: forces 3e-8 relative), so the bound is 2e-7; a lost or doubled
    force update would show at 1e-3 and above."""
    box = systems.box_for(512, seed=11)
    prm = systems.polar_params(alpha=0.35, rcut=9.0, kmax=(12, 12, 12), toler_debye=1e-8)
    ctx = capi.Context(0)
    try:
        if spme:
            ctx.set_spme(6, spacing=0.78)
        seq = ctx.water_step(box, prm, precision=capi.MIXED)
        ctx.set_overlap(True)
        ovl = ctx.water_step(box, prm, precision=capi.MIXED)
        ctx.set_overlap(True, dimer_warps=3)
        ov3 = ctx.water_step(box, prm, precision=capi.MIXED)
    finally:
        ctx.close()
    for got in (ovl, ov3):
        assert got["status"] == 0
        for key in ("forces", "atomic_energy", "dipoles", "scalars"):
            assert _rel(got[key], seq[key]) <= 2e-7, (key, _rel(got[key], seq[key]))


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
def test_overlapped_terms_match_sequential(precision):
    """mbx_set_overlap_terms: the 1-body and dispersion terms on a third stream beside the
    electrostatics (and with the MB-pol overlap as well) give the sequential step's results
    up to the order of FP64 atomic additions (FP64: 1e-11; mixed: 2e-7, the bound of the
    MB-pol overlap, for a CG stopping decision moved by that order); a lost or doubled
    force update would show at 1e-3 and above."""
    box = systems.box_for(512, seed=11)
    prm = systems.polar_params(alpha=0.35, rcut=9.0, kmax=(12, 12, 12), toler_debye=1e-8)
    lt, mol = systems.water_types(box)
    ctx = capi.Context(0)
    try:
        ctx.set_spme(6, spacing=0.78)
        ctx.disp_setup(systems.DISP_PARAMS_SYNTHETIC, rcut=9.0, delr=1.0)
        seq = ctx.water_step(box, prm, precision=precision, disp=(lt, mol))
        ctx.set_overlap_terms(True)
        got = [ctx.water_step(box, prm, precision=precision, disp=(lt, mol))]
        if precision == capi.MIXED:
            ctx.set_overlap(True)
            got.append(ctx.water_step(box, prm, precision=precision, disp=(lt, mol)))
    finally:
        ctx.close()
    tol = 1e-11 if precision == capi.FP64 else 2e-7
    for g in got:
        assert g["status"] == 0
        for key in ("forces", "atomic_energy", "dipoles", "scalars"):
            assert _rel(g[key], seq[key]) <= tol, (key, _rel(g[key], seq[key]))


def _jtotal(v):
    """The step's total heat current: the MB-pol block's jpot + jkin, the 1-body and
    dispersion jpot, and the electrostatics' jpot + jkin (include/mbx.h scalar layout)."""
    ns, nw = capi.NSCALARS, capi.NWATERSCALARS
    j = v[12:15] + v[15:18] + v[ns + 11:ns + 14] + v[ns + 25:ns + 28]
    return j + v[nw + 16:nw + 19] + v[nw + 19:nw + 22]


@pytest.mark.parametrize("spme", [True, False])
def test_final_fp64_pass(spme):
    """mbx_set_final_fp64: the mixed step with its electrostatics' final pass in FP64.  The
    dipoles converge to the same tolerance as the FP64 method's, so the electrostatics'
    heat current (jpot + jkin) and forces match the FP64 step's to the dipole tolerance
    (measured on the 64 uneven boxes: 3e-9 to 1.8e-8 of the total heat current, against
    up to 1.5e-6 with the FP32 final pass); the total heat current stays within the 1e-6
    budget (its remaining error is the FP32 3B term's)."""
    box = systems.box_for(256, seed=5)
    prm = systems.polar_params(alpha=0.35, rcut=8.0, kmax=(10, 10, 10), toler_debye=1e-8)
    ctx = capi.Context(0)
    try:
        if spme:
            ctx.set_spme(6, spacing=0.78)
        ref = ctx.water_step(box, prm, precision=capi.FP64)
        ctx.set_final_fp64(True)
        got = ctx.water_step(box, prm, precision=capi.MIXED)
        ctx.set_final_fp64(False)
        dflt = ctx.water_step(box, prm, precision=capi.MIXED)
    finally:
        ctx.close()
    nw = capi.NWATERSCALARS
    jr = _jtotal(ref["scalars"])
    jel = lambda v: v[nw + 16:nw + 19] + v[nw + 19:nw + 22]
    assert got["status"] == 0 and dflt["status"] == 0
    assert np.linalg.norm(jel(got["scalars"]) - jel(ref["scalars"])) <= 1e-7 * np.linalg.norm(jr)
    assert np.linalg.norm(_jtotal(got["scalars"]) - jr) <= 1e-6 * np.linalg.norm(jr)
    assert _rel(got["dipoles"], ref["dipoles"]) <= 1e-6
    # the MB-pol terms are the mixed method's in both mixed calls
    assert _rel(got["forces"], ref["forces"]) <= 1e-5
    assert _rel(got["forces"], dflt["forces"]) <= 1e-5
