"""GPU parity of the TTM4-F electrostatics (mbx_polar_forces) against the oracle.

FP64 path: energies, virial, stress, site forces, converged dipoles, per-site energies and
the heat-current terms within 1e-10 relative (vectors relative to their largest entry),
the same number of dipole iterations.
"""
import numpy as np
import pytest

from mbx import capi, systems

pytestmark = pytest.mark.gpu

TOL = 1e-10


def _case(orc, box, prm):
    sites, q, dp, _ = orc.msites_dms(box)
    polr, polr2 = systems.polarizabilities(box.nw)
    return sites, q, dp, polr, polr2, prm


def _compare(got, ref):
    assert got["iterations"] == ref["iterations"], (got["iterations"], ref["iterations"])
    for key in ("engcpe", "vircpe", "eng_polar", "eng_kspace", "eng_real"):
        assert abs(got[key] - ref[key]) <= TOL * abs(ref[key]), (key, got[key], ref[key])
    smax = np.abs(ref["stress"]).max()
    assert np.abs(got["stress"] - ref["stress"]).max() <= TOL * smax
    for key in ("forces", "dipoles", "atomic_energy", "jpot", "jkin"):
        r = ref[key]
        assert np.abs(got[key] - r).max() <= TOL * np.abs(r).max(), (key, np.abs(got[key] - r).max(), np.abs(r).max())


@pytest.mark.parametrize("which", ["small", "config0", "triclinic"])
def test_polar_matches_oracle(mbx_ctx, oracle_lib, which):
    if which == "small":
        box = systems.box_for(32, seed=5)
        prm = systems.polar_params(alpha=0.6, rcut=4.5, kmax=(8, 8, 8), toler_debye=1e-12)
    elif which == "config0":
        box = systems.config0()
        prm = systems.polar_params(alpha=0.3, rcut=9.0, kmax=(8, 8, 8), toler_debye=1e-12)
    else:
        box = systems.box_for(64, seed=9)
        L = box.L
        # a sheared cell (imcon 3) of the same volume: the box's waters imaged into it
        box.cell = np.array([L, 0, 0, 0.2 * L, L, 0, 0.1 * L, -0.15 * L, L], dtype=np.float64)
        box.imcon = 3
        prm = systems.polar_params(alpha=0.55, rcut=5.0, kmax=(7, 7, 7), toler_debye=1e-11)
    sites, q, dp, polr, polr2, prm = _case(oracle_lib, box, prm)
    ref = oracle_lib.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, vel=box.vel)
    assert ref["status"] == 0
    got = mbx_ctx.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, vel=box.vel)
    _compare(got, ref)


def test_polar_warm_start_and_no_heat(mbx_ctx, oracle_lib):
    box = systems.box_for(32, seed=6)
    prm = systems.polar_params(alpha=0.6, rcut=4.5, kmax=(6, 6, 6), toler_debye=1e-12)
    sites, q, dp, polr, polr2, prm = _case(oracle_lib, box, prm)
    first = mbx_ctx.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm)
    rng = np.random.default_rng(1)
    dip0 = first["dipoles"] + rng.normal(0, 1e-4, size=first["dipoles"].shape)
    dip0[3 * box.nw:] = 0.0
    ref = oracle_lib.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, dip0=dip0)
    got = mbx_ctx.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, dip0=dip0)
    assert got["iterations"] < first["iterations"]
    assert not got["jpot"].any() and not got["jkin"].any()
    ref["jpot"] = got["jpot"]
    ref["jkin"] = got["jkin"]
    _compare(got, ref)


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
def test_aspc_steps_match_the_oracle(oracle_lib, precision):
    """ASPC (mbx_set_aspc, k 2, 4 converged steps): an MD sequence of 8 steps with the
    positions advancing by v dt, against the oracle's restatement of aspc_predict /
    aspc_set and the loop branch of SOURCE/forces.f:334-366 (AspcDriver).  Steps 1-4 iterate
    to toler with SOR weight 0.3; steps 5-8 start from the prediction and make one
    iteration.  FP64: every result within 1e-10 at every step; mixed: the converged steps
    within the dipole tolerance, the one-iteration steps' dipoles within 1e-9."""
    import copy

    import oracle
    box0 = systems.box_for(32, seed=5)
    prm = systems.polar_params(alpha=0.6, rcut=4.5, kmax=(8, 8, 8), toler_debye=1e-12, omega=4.0 / 7.0)
    polr, polr2 = systems.polarizabilities(box0.nw)
    ctx = capi.Context(0)
    try:
        with pytest.raises(capi.MbxError):
            ctx.set_aspc(3)
        ctx.set_aspc(2, 4)
        assert ctx.aspc_step() == 0
        drv = oracle.AspcDriver(2, 4)
        dg = dr = None
        for step in range(1, 9):
            box = copy.copy(box0)
            box.xyz = box0.xyz + (step - 1) * 0.0005 * box0.vel
            sites, q, dp, _ = oracle_lib.msites_dms(box)
            ref = drv.step(oracle_lib, sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, dip0=dr,
                           vel=box.vel)
            got = ctx.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, dip0=dg, vel=box.vel,
                            precision=precision)
            assert ctx.aspc_step() == step
            assert ref["status"] == (0 if step <= 4 else 1)
            if step > 4:
                assert got["iterations"] == 1
            if precision == capi.FP64:
                _compare(got, ref)
            else:
                m = np.abs(ref["dipoles"]).max()
                assert np.abs(got["dipoles"] - ref["dipoles"]).max() <= 1e-9 * m, step
                f, fr = got["forces"], ref["forces"]
                assert np.sqrt(np.mean((f - fr) ** 2)) <= 1e-6 * np.sqrt(np.mean(fr ** 2)), step
            dg, dr = got["dipoles"], ref["dipoles"]
        # a restart (an image change): the next step is step 1 again and iterates to toler
        ctx.aspc_restart()
        assert ctx.aspc_step() == 0
        got = ctx.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, dip0=dg, precision=precision)
        assert ctx.aspc_step() == 1 and got["iterations"] > 1
        ctx.set_aspc(0, 0)
    finally:
        ctx.close()


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
def test_dipole_guess_changes_iterations_not_results(oracle_lib, precision):
    """mbx_set_dipole_guess: on an MD sequence (positions advancing by v dt, dipoles carried
    over) the extrapolated start needs fewer iterations than the warm start, and every step's
    results agree with the warm-started ones within the dipole tolerance."""
    import copy
    box0 = systems.box_for(32, seed=5)
    prm = systems.polar_params(alpha=0.6, rcut=4.5, kmax=(8, 8, 8), toler_debye=1e-11)
    polr, polr2 = systems.polarizabilities(box0.nw)
    runs = {}
    for order in (0, 2):
        ctx = capi.Context(0)
        try:
            ctx.set_dipole_guess(order)
            dip, out = None, []
            for step in range(7):
                box = copy.copy(box0)
                box.xyz = box0.xyz + step * 0.0005 * box0.vel
                sites, q, dp, _ = oracle_lib.msites_dms(box)
                got = ctx.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, dip0=dip, vel=box.vel,
                                precision=precision)
                inner = ctx.polar_inner_sweeps() if precision == capi.MIXED else got["iterations"]
                out.append((got, inner))
                dip = got["dipoles"]
        finally:
            ctx.close()
        runs[order] = out
    # the mixed path's FP32 pair forces round differently for dipoles a tolerance apart
    ftol = 1e-8 if precision == capi.FP64 else 1e-6
    for (g0, _), (g2, _) in zip(runs[0], runs[2]):
        assert np.abs(g2["dipoles"] - g0["dipoles"]).max() <= 1e-8 * np.abs(g0["dipoles"]).max()
        assert np.abs(g2["forces"] - g0["forces"]).max() <= ftol * np.abs(g0["forces"]).max()
    # steps 4..7 start from the quadratic extrapolation
    assert sum(i for _, i in runs[2][3:]) < sum(i for _, i in runs[0][3:])


def test_polar_not_converged_status(mbx_ctx, oracle_lib):
    box = systems.box_for(32, seed=5)
    prm = systems.polar_params(alpha=0.6, rcut=4.5, kmax=(6, 6, 6), toler_debye=1e-12, maxit=3)
    sites, q, dp, polr, polr2, prm = _case(oracle_lib, box, prm)
    got = mbx_ctx.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, check=False)
    assert got["status"] == capi.ERR_CONVERGE and got["iterations"] == 3
    ref = oracle_lib.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm)
    assert ref["status"] == 1
    np.testing.assert_allclose(got["dipoles"], ref["dipoles"], rtol=0, atol=1e-12)
    # bad parameters are refused before any work
    bad = prm.copy()
    bad[4] = 1.5
    with pytest.raises(capi.MbxError):
        mbx_ctx.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, bad)


def test_msite_redistribute(mbx_ctx):
    import ctypes as C
    nw = 5
    rng = np.random.default_rng(2)
    f = rng.normal(size=(3, 4 * nw))
    g = 0.426706882
    want = f.copy()
    for w in range(nw):
        m = want[:, 3 * nw + w].copy()
        want[:, 3 * w] += (1 - g) * m
        want[:, 3 * w + 1] += m * g / 2
        want[:, 3 * w + 2] += m * g / 2
    P = C.POINTER(C.c_double)
    assert mbx_ctx.lib.mbx_msite_redistribute(nw, g, f[0].ctypes.data_as(P), f[1].ctypes.data_as(P),
                                              f[2].ctypes.data_as(P)) == 0
    # the host compiler may contract f + w * m into one FMA (aarch64): 1 ulp
    np.testing.assert_allclose(f, want, rtol=1e-15, atol=1e-15)


@pytest.mark.parametrize("which", ["small", "config0"])
def test_polar_mixed_refinement(mbx_ctx, oracle_lib, which):
    """MBX_MIXED solves the same dipole equations (FP32 corrections under FP64 refinement):
    its results are those of the FP64 oracle within the dipole tolerance."""
    if which == "small":
        box = systems.box_for(32, seed=5)
        prm = systems.polar_params(alpha=0.6, rcut=4.5, kmax=(8, 8, 8), toler_debye=1e-12)
    else:
        box = systems.config0()
        prm = systems.polar_params(alpha=0.3, rcut=9.0, kmax=(8, 8, 8), toler_debye=1e-8)
    sites, q, dp, polr, polr2, prm = _case(oracle_lib, box, prm)
    ref = oracle_lib.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, vel=box.vel)
    got = mbx_ctx.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, vel=box.vel,
                        precision=capi.MIXED)
    assert got["deltadip"] <= prm[3]
    assert mbx_ctx.polar_inner_sweeps() > 0 and got["iterations"] < ref["iterations"]
    assert abs(got["engcpe"] - ref["engcpe"]) <= 1e-8 * abs(ref["engcpe"])
    f, fr = got["forces"], ref["forces"]
    assert np.sqrt(np.mean((f - fr) ** 2)) <= 1e-6 * np.sqrt(np.mean(fr ** 2))
    # the heat-current budget of the mixed path: 1e-6 relative (its k-space force and
    # per-site energy gathers run in FP32 with FP64 tile sums)
    for key in ("jpot", "jkin"):
        assert np.linalg.norm(got[key] - ref[key]) <= 1e-6 * np.linalg.norm(ref[key]), key


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
def test_water_step_is_the_sum_of_its_terms(oracle_lib, precision):
    """mbx_water_step = M sites/DMS + electrostatics + 1-body + dispersion + MB-pol, then the
    M-site redistribution, in one host call; the same results as the separate entry points."""
    box = systems.config0()
    prm = systems.polar_params(alpha=0.3, rcut=9.0, kmax=(8, 8, 8), toler_debye=1e-10)
    lt, mol = systems.water_types(box)
    polr, polr2 = systems.polarizabilities(box.nw)
    ctx = capi.Context(0)
    try:
        ctx.disp_setup(systems.DISP_PARAMS_SYNTHETIC, rcut=9.0, delr=1.0)
        step = ctx.water_step(box, prm, precision=precision, disp=(lt, mol))
        parts = ctx.water_forces(box, precision=precision, dispersion=True)
        sites, q, dp = ctx.msites_dms(box)
        pol = ctx.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, vel=box.vel,
                        precision=precision)
    finally:
        ctx.close()
    tol = 1e-11 if precision == capi.FP64 else 1e-8
    nw = box.nw
    f = parts["forces"] + pol["forces"]
    g = prm[10]
    fm = f[3 * nw:].copy()
    f[0:3 * nw:3] += (1 - g) * fm
    f[1:3 * nw:3] += 0.5 * g * fm
    f[2:3 * nw:3] += 0.5 * g * fm
    assert np.abs(step["forces"] - f).max() <= tol * np.abs(f).max()
    ae = parts["atomic_energy"] + pol["atomic_energy"]
    assert np.abs(step["atomic_energy"] - ae).max() <= tol * np.abs(ae).max()
    np.testing.assert_allclose(step["sites"][3 * nw:], sites[3 * nw:], rtol=0, atol=1e-12)
    np.testing.assert_allclose(step["chge"], q, rtol=0, atol=1e-14)
    assert np.abs(step["dipoles"] - pol["dipoles"]).max() <= tol * np.abs(pol["dipoles"]).max()
    sc = step["scalars"]
    nws = capi.NWATERSCALARS
    assert np.abs(sc[:nws] - parts["scalars"]).max() <= tol * np.abs(parts["scalars"]).max()
    assert abs(sc[nws] - pol["engcpe"]) <= tol * abs(pol["engcpe"])
    assert np.abs(sc[nws + 16:nws + 19] - pol["jpot"]).max() <= tol * np.abs(pol["jpot"]).max()
    assert np.abs(sc[nws + 19:nws + 22] - pol["jkin"]).max() <= tol * np.abs(pol["jkin"]).max()


def test_polar_phase_timings(mbx_ctx, oracle_lib):
    box = systems.box_for(32, seed=5)
    prm = systems.polar_params(alpha=0.6, rcut=4.5, kmax=(6, 6, 6), toler_debye=1e-10)
    sites, q, dp, polr, polr2, prm = _case(oracle_lib, box, prm)
    mbx_ctx.set_profiling(True)
    try:
        for prec in (capi.FP64, capi.MIXED):
            mbx_ctx.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, vel=box.vel, precision=prec)
            ms, kv = mbx_ctx.polar_timings()
            assert kv > 0 and (ms >= 0).all() and ms.sum() > 0
    finally:
        mbx_ctx.set_profiling(False)


def test_polar_mixed_preconditioner_settings(mbx_ctx, oracle_lib):
    """The mixed solve's preconditioner (mbx_set_precond_sweeps: 0 automatic, 1 diagonal, 3,
    5; mbx_set_precond_block: the per-water block inverse) changes the iteration count, not
    the converged results beyond the mixed budgets; even counts (not positive definite in
    general) are refused."""
    box = systems.config0()
    prm = systems.polar_params(alpha=0.3, rcut=9.0, kmax=(8, 8, 8), toler_debye=1e-8)
    sites, q, dp, polr, polr2, prm = _case(oracle_lib, box, prm)
    ref = oracle_lib.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, vel=box.vel)
    with pytest.raises(capi.MbxError):
        mbx_ctx.set_precond_sweeps(2)
    sweeps = {}
    try:
        for p in (0, 1, 3, 5, "block"):
            mbx_ctx.set_precond_block(p == "block")
            mbx_ctx.set_precond_sweeps(1 if p == "block" else p)
            got = mbx_ctx.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, vel=box.vel,
                                precision=capi.MIXED)
            sweeps[p] = mbx_ctx.polar_inner_sweeps()
            assert got["deltadip"] <= prm[3]
            assert abs(got["engcpe"] - ref["engcpe"]) <= 1e-8 * abs(ref["engcpe"])
            f, fr = got["forces"], ref["forces"]
            assert np.sqrt(np.mean((f - fr) ** 2)) <= 1e-6 * np.sqrt(np.mean(fr ** 2))
    finally:
        mbx_ctx.set_precond_block(True)   # the default
        mbx_ctx.set_precond_sweeps(0)
    assert min(sweeps.values()) > 0
    assert sweeps[0] == sweeps[3]   # automatic with the Ewald sum: the 3-sweep polynomial
    # the per-water block inverse takes fewer sweeps than the diagonal
    assert sweeps["block"] < sweeps[1], sweeps


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
def test_gpu_dipoles_solve_the_oracle_equations(mbx_ctx, oracle_lib, precision):
    """induced_error (SOURCE/induced_error.f90) of the GPU's converged dipoles under the
    ORACLE's fields: whatever the iteration path (the reference's SOR, or FP32 corrections
    under FP64 refinement), the dipoles solve the reference's dipole equations to the
    tolerance."""
    box = systems.config0()
    prm = systems.polar_params(alpha=0.3, rcut=9.0, kmax=(8, 8, 8), toler_debye=1e-10)
    sites, q, dp, polr, polr2, prm = _case(oracle_lib, box, prm)
    got = mbx_ctx.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, precision=precision)
    l2, linf = oracle_lib.induced_error(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, got["dipoles"])
    npol = int((polr2 > 1e-6).sum())
    assert l2 / np.sqrt(3 * npol) <= prm[3] / (1.0 - prm[4]), (l2, prm[3])
    assert linf <= 20 * prm[3]


def _brute_pairs(sites, cell, nw, rcut):
    """Site pairs i < j of different waters within rcut (the Verlet pairs of SOURCE/parlst.f
    with exclude_ttm's intramolecular exclusions), by brute force with the nearest image."""
    n = sites.shape[0]
    mol = np.concatenate([np.arange(3 * nw) // 3, np.arange(nw)])
    h = np.asarray(cell, np.float64).reshape(3, 3)        # rows: the cell vectors
    hinv = np.linalg.inv(h)
    out = []
    for i in range(n - 1):
        d = sites[i] - sites[i + 1:]
        s = d @ hinv
        s -= np.round(s)
        r2 = np.sum((s @ h) ** 2, 1)
        j = np.nonzero((r2 < rcut * rcut) & (mol[i + 1:] != mol[i]))[0] + i + 1
        out.extend((i, int(k)) for k in j)
    return set(out)


@pytest.mark.parametrize("which", ["config0", "triclinic"])
def test_pair_list_is_the_verlet_set(oracle_lib, which):
    """The electrostatics' site pair list (kept with a skin) is exactly the set of site pairs
    of different waters within rcut."""
    if which == "config0":
        box = systems.config0()
        prm = systems.polar_params(alpha=0.3, rcut=9.0, kmax=(8, 8, 8), toler_debye=1e-8)
    else:
        box = systems.box_for(64, seed=9)
        L = box.L
        box.cell = np.array([L, 0, 0, 0.2 * L, L, 0, 0.1 * L, -0.15 * L, L], dtype=np.float64)
        box.imcon = 3
        prm = systems.polar_params(alpha=0.55, rcut=5.0, kmax=(7, 7, 7), toler_debye=1e-8)
    sites, q, dp, polr, polr2, prm = _case(oracle_lib, box, prm)
    ctx = capi.Context(0)
    try:
        ctx.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm)
        got = set(map(tuple, ctx.polar_last_pairs().tolist()))
    finally:
        ctx.close()
    want = _brute_pairs(sites, box.cell, box.nw, prm[1])
    assert got == want, (len(got), len(want), len(got ^ want))


def test_skin_list_reuse_matches_rebuilding(oracle_lib):
    """Along a trajectory (atoms moved by v dt, the fastest 0.06 A per step, so that a skin
    of 0.3 A runs out after a few steps) the electrostatics with the kept skin list equal those with the
    list rebuilt at every call (the same pairs, summed in another order), and the list is
    rebuilt only when a site moved more than half the skin."""
    box = systems.config0()
    prm = systems.polar_params(alpha=0.3, rcut=9.0, kmax=(8, 8, 8), toler_debye=1e-10)
    polr, polr2 = systems.polarizabilities(box.nw)
    kept, fresh = capi.Context(0), capi.Context(0)
    try:
        kept.set_polar_skin(0.3)
        fresh.set_polar_skin(0.0)
        x0 = box.xyz.copy()
        steps = 8
        dt = 0.06 / np.abs(box.vel).max()                # the fastest atom moves 0.06 A per step
        for k in range(steps):
            box.xyz = x0 + k * dt * box.vel
            sites, q, dp, _ = oracle_lib.msites_dms(box)
            a = kept.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, vel=box.vel)
            b = fresh.polar(sites, box.cell, box.imcon, box.nw, q, dp, polr, polr2, prm, vel=box.vel)
            assert a["iterations"] == b["iterations"]
            assert abs(a["engcpe"] - b["engcpe"]) <= 1e-12 * abs(b["engcpe"])
            for key in ("forces", "dipoles", "atomic_energy", "jpot", "jkin"):
                assert np.abs(a[key] - b[key]).max() <= 1e-11 * np.abs(b[key]).max(), key
        assert fresh.polar_list_builds() == steps
        assert 1 < kept.polar_list_builds() < steps
    finally:
        kept.close()
        fresh.close()
