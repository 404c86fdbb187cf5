"""GPU parity of libmbx against the oracle (FP64: 1e-10; mixed: the stated budgets)."""
import ctypes as C

import numpy as np
import pytest

from conftest import rel_err
from mbx import capi, systems

pytestmark = pytest.mark.gpu

# FP64 path tolerance (relative to the array's largest magnitude)
TOL64 = 1e-10
# mixed path budgets at 4096 H2O: force RMS error and heat-current error, relative
TOL_MIXED_FORCE_RMS = 1e-5
TOL_MIXED_HEAT = 1e-6
# small boxes carry fewer trimers per unit of heat current: their heat budget is 3e-6
TOL_MIXED_HEAT_SMALL = 3e-6


def _as_set(a):
    return set(map(tuple, np.asarray(a).tolist()))


def _boxes():
    return {
        "cfg0_256": systems.config0(),
        "small_64_allpairs": systems.box_for(64, seed=5),
        "ortho_imcon2": _ortho(),
        "shuffled_layout": _shuffled(),
        "triclinic_imcon3": _triclinic(),
    }


def _triclinic():
    """The 216-water box sheared into a parallelepiped (imcon 3): r = H s."""
    b = systems.water_box(216, 19.5, seed=13, lattice=6)
    L = b.L
    H = np.array([[L, 0.1 * L, 0.05 * L], [0.0, L, 0.08 * L], [0.0, 0.0, L]])   # columns = cell vectors
    s = b.xyz / L
    b.xyz = s @ H.T
    b.cell = np.ascontiguousarray(H.T.ravel())   # cell(1:3) = a, cell(4:6) = b, cell(7:9) = c
    b.imcon = 3
    return b


def _ortho():
    b = systems.water_box(216, 19.5, seed=9, lattice=6)
    b.xyz[:, 1] *= 1.05
    b.xyz[:, 2] *= 0.97
    b.cell = np.array([19.5, 0, 0, 0, 19.5 * 1.05, 0, 0, 0, 19.5 * 0.97])
    b.imcon = 2
    return b


def _shuffled():
    b = systems.box_for(128, seed=21)
    rng = np.random.default_rng(2)
    perm = rng.permutation(b.nw)
    w = b.xyz[:3 * b.nw].reshape(b.nw, 3, 3)[perm].reshape(-1, 3)
    v = b.vel[:3 * b.nw].reshape(b.nw, 3, 3)[perm].reshape(-1, 3)
    b.xyz[:3 * b.nw] = w
    b.vel[:3 * b.nw] = v
    # molecules also wrapped into the box by O (atoms may straddle the boundary)
    shift = np.floor(b.xyz[0:3 * b.nw:3] / b.L) * b.L
    b.xyz[:3 * b.nw] -= np.repeat(shift, 3, axis=0)
    return b


BOXES = _boxes()


@pytest.fixture(scope="module")
def refs(oracle_lib):
    return {k: oracle_lib.mbpol_forces(b, lists=True) for k, b in BOXES.items()}


@pytest.mark.parametrize("name", list(BOXES))
def test_fp64_matches_oracle(mbx_ctx, refs, name):
    box = BOXES[name]
    ref = refs[name]
    got = mbx_ctx.mbpol_forces(box, precision=capi.FP64)
    pairs, trip = mbx_ctx.last_lists()
    assert _as_set(pairs) == _as_set(ref["pairs"])
    assert _as_set(np.sort(trip, axis=1)) == _as_set(ref["trimers"])
    assert len(trip) == len(ref["trimers"])
    for k in ("eng2", "eng3", "vir"):
        assert abs(got[k] - ref[k]) <= TOL64 * abs(ref[k]), k
    assert rel_err(got["stress"], ref["stress"]) <= TOL64
    assert rel_err(got["forces"], ref["forces"]) <= TOL64
    assert rel_err(got["atomic_energy"], ref["atomic_energy"]) <= TOL64
    assert rel_err(got["jpot"], ref["jpot"]) <= TOL64
    assert rel_err(got["jkin"], ref["jkin"]) <= TOL64
    # accumulate semantics of the mbpol_forces interface
    assert abs(got["engsrp"] - (ref["eng2"] + ref["eng3"])) <= TOL64 * abs(ref["eng2"] + ref["eng3"])


@pytest.mark.parametrize("name", ["cfg0_256", "shuffled_layout"])
def test_mixed_within_budget(mbx_ctx, refs, name):
    box = BOXES[name]
    ref = refs[name]
    got = mbx_ctx.mbpol_forces(box, precision=capi.MIXED)
    f, fr = got["forces"], ref["forces"]
    rms = np.sqrt(np.mean((f - fr) ** 2) / np.mean(fr ** 2))
    assert rms <= TOL_MIXED_FORCE_RMS, rms
    jt = got["jpot"] + got["jkin"]
    jr = ref["jpot"] + ref["jkin"]
    assert np.linalg.norm(jt - jr) <= TOL_MIXED_HEAT_SMALL * np.linalg.norm(jr)
    # total energy: the 3B energy carries the FP32 rounding (~5e-6 of E3), the total
    # stays within 2e-6 (measured 2e-7 at 4096 waters, ~1e-6 on the 128-water box)
    e, er = got["eng2"] + got["eng3"], ref["eng2"] + ref["eng3"]
    assert abs(e - er) <= 2e-6 * abs(er)


def test_models_fp64_and_mixed_vs_reference_golden(mbx_ctx, golden):
    W2 = golden["W2"]
    E, g1, g2 = mbx_ctx.poly2b_batch(W2[:, 0], W2[:, 1], precision=capi.FP64)
    scale = np.maximum(np.abs(golden["E2"]), 1.0)
    assert np.all(np.abs(E - golden["E2"]) <= 1e-10 * scale)
    G = np.concatenate([g1, g2], 1)
    GR = golden["G2"].reshape(len(W2), 18)
    assert np.all(np.abs(G - GR).max(1) <= 1e-10 * np.maximum(np.abs(GR).max(1), 1.0))
    W3 = golden["W3"]
    E3, h1, h2, h3 = mbx_ctx.poly3b_batch(W3[:, 0], W3[:, 1], W3[:, 2], precision=capi.FP64)
    assert np.all(np.abs(E3 - golden["E3"]) <= 1e-10 * np.maximum(np.abs(golden["E3"]), 1.0))
    G3 = np.concatenate([h1, h2, h3], 1)
    GR3 = golden["G3"].reshape(len(W3), 27)
    assert np.all(np.abs(G3 - GR3).max(1) <= 1e-10 * np.maximum(np.abs(GR3).max(1), 1.0))
    # mixed: FP32 per cluster
    # FP32 shifted 3B polynomial (the mixed path's 3B term): per-trimer budget
    E3m, *_ = mbx_ctx.poly3b_batch(W3[:, 0], W3[:, 1], W3[:, 2], precision=capi.MIXED)
    assert np.all(np.abs(E3m - golden["E3"]) <= 1e-4 * np.maximum(np.abs(golden["E3"]), 1.0))


def test_3b_batch_accumulates_into_gradients(mbx_ctx, golden):
    W3 = golden["W3"][:8]
    g0 = [np.full((8, 9), 0.25) for _ in range(3)]
    E, a, b, c = mbx_ctx.poly3b_batch(W3[:, 0], W3[:, 1], W3[:, 2], g=g0)
    assert np.allclose(np.concatenate([a, b, c], 1) - 0.25, golden["G3"][:8].reshape(8, 27), rtol=0, atol=1e-9)


def test_dropin_symbols(golden):
    lib = capi.load()
    D = C.POINTER(C.c_double)
    w1 = np.ascontiguousarray(golden["W2"][0, 0])
    w2 = np.ascontiguousarray(golden["W2"][0, 1])
    e = C.c_double(0)
    g1 = np.zeros(9)
    g2 = np.zeros(9)
    fm = np.zeros(108)
    lib.mbpol_2b_poly_(w1.ctypes.data_as(D), w2.ctypes.data_as(D), C.byref(e), g1.ctypes.data_as(D),
                       g2.ctypes.data_as(D), fm.ctypes.data_as(D))
    assert abs(e.value - golden["E2"][0]) <= 1e-10 * max(abs(golden["E2"][0]), 1.0)
    r = C.c_double(0)
    lib.mbpol_2b_cutoff_(C.byref(r))
    assert r.value == 6.5
    lib.mbpol_3b_cutoff_(C.byref(r))
    assert r.value == 4.5
    W = [np.ascontiguousarray(golden["W3"][0, q]) for q in range(3)]
    g = [np.zeros(9) for _ in range(3)]
    lib.mbpol_3b_poly_(*(w.ctypes.data_as(D) for w in W), C.byref(e), *(a.ctypes.data_as(D) for a in g),
                       np.zeros(243).ctypes.data_as(D))
    assert abs(e.value - golden["E3"][0]) <= 1e-10 * max(abs(golden["E3"][0]), 1.0)


@pytest.mark.parametrize("nw", [0, 1, 2, 3])
def test_tiny_systems(mbx_ctx, oracle_lib, nw):
    box = systems.water_box(max(nw, 1), 12.0, seed=4, lattice=2)
    if nw == 0:
        box = systems.WaterBox(0, 12.0, np.zeros((0, 3)), np.zeros((0, 3)), 0)
    got = mbx_ctx.mbpol_forces(box)
    if nw == 0:
        assert got["eng2"] == 0 and got["eng3"] == 0
        return
    ref = oracle_lib.mbpol_forces(box)
    assert abs(got["eng2"] - ref["eng2"]) <= TOL64 * max(abs(ref["eng2"]), 1.0)
    assert abs(got["eng3"] - ref["eng3"]) <= TOL64 * max(abs(ref["eng3"]), 1.0)


def test_invalid_arguments_rejected(mbx_ctx):
    box = systems.box_for(8, seed=1)
    box.imcon = 7
    with pytest.raises(capi.MbxError):
        mbx_ctx.mbpol_forces(box)
    box.imcon = 1
    with pytest.raises(capi.MbxError):
        mbx_ctx.mbpol_forces(box, precision=5)


def test_repeatable_and_lists_stable(mbx_ctx):
    box = systems.config0(seed=77)
    a = mbx_ctx.mbpol_forces(box)
    pa, ta = mbx_ctx.last_lists()
    b = mbx_ctx.mbpol_forces(box)
    pb, tb = mbx_ctx.last_lists()
    assert np.array_equal(pa, pb) and np.array_equal(ta, tb)
    assert abs(a["eng3"] - b["eng3"]) <= 1e-13 * abs(a["eng3"])


def test_full_size_properties_4096(mbx_ctx):
    """cfg1 (4096 H2O): mixed vs FP64 budgets, energy partition and momentum conservation."""
    box = systems.config1()
    d = mbx_ctx.mbpol_forces(box, precision=capi.FP64)
    m = mbx_ctx.mbpol_forces(box, precision=capi.MIXED)
    e = d["eng2"] + d["eng3"]
    assert abs(d["atomic_energy"].sum() - e) <= 1e-10 * abs(e)
    assert np.max(np.abs(d["forces"].sum(0))) <= 1e-8 * np.max(np.abs(d["forces"]))
    rms = np.sqrt(np.mean((m["forces"] - d["forces"]) ** 2) / np.mean(d["forces"] ** 2))
    assert rms <= TOL_MIXED_FORCE_RMS, rms
    jd = d["jpot"] + d["jkin"]
    jm = m["jpot"] + m["jkin"]
    assert np.linalg.norm(jm - jd) <= TOL_MIXED_HEAT * np.linalg.norm(jd)
    _, (nd, nt, _, _, _) = mbx_ctx.last_timings()
    assert nd > 0 and nt > 0


def test_mixed_handoff_limits(mbx_ctx, refs):
    """A vanishing limit hands every cluster to the FP64 kernels: the mixed call then equals FP64."""
    box = BOXES["small_64_allpairs"]
    ref = refs["small_64_allpairs"]
    try:
        mbx_ctx.set_mixed_limits(1e-30, 1e-30)
        got = mbx_ctx.mbpol_forces(box, precision=capi.MIXED)
        _, (nd, nt, _, hd, ht) = mbx_ctx.last_timings()
        assert hd == nd and ht == nt
        assert rel_err(got["forces"], ref["forces"]) <= TOL64
        mbx_ctx.set_mixed_limits(1e9, 1e9)
        mbx_ctx.mbpol_forces(box, precision=capi.MIXED)
        _, (_, _, _, hd, ht) = mbx_ctx.last_timings()
        assert hd == 0 and ht == 0
    finally:
        mbx_ctx.set_mixed_limits(0.0, 3.4e38)


@pytest.mark.parametrize("name", ["cfg0_256", "ortho_imcon2", "shuffled_layout", "triclinic_imcon3"])
def test_ps_pes_fp64_matches_oracle(mbx_ctx, oracle_lib, name):
    box = BOXES[name]
    ref = oracle_lib.angfrc_ps(box)
    got = mbx_ctx.ps_pes(box)
    assert abs(got["engang"] - ref["engang"]) <= TOL64 * abs(ref["engang"])
    assert abs(got["virang"] - ref["virang"]) <= TOL64 * abs(ref["virang"])
    assert rel_err(got["stress"], ref["stress"]) <= TOL64
    assert rel_err(got["forces"], ref["forces"]) <= TOL64
    assert rel_err(got["atomic_energy"], ref["atomic_energy"]) <= TOL64
    assert rel_err(got["jpot"], ref["jpot"]) <= TOL64


@pytest.mark.parametrize("name", ["cfg0_256", "ortho_imcon2", "shuffled_layout", "triclinic_imcon3"])
def test_msites_dms_match_oracle(mbx_ctx, oracle_lib, name):
    box = BOXES[name]
    rx, rq, rdp, _ = oracle_lib.msites_dms(box)
    gx, gq, gdp = mbx_ctx.msites_dms(box)
    nw = box.nw
    assert np.max(np.abs(gx[3 * nw:] - rx[3 * nw:])) <= 1e-12 * max(box.L, 1.0)
    assert rel_err(gq, rq) <= TOL64
    assert rel_err(gdp, rdp) <= TOL64


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
def test_fused_kernel_matches_separate_kernels(precision):
    """The persistent 2B+3B kernel and the two separate kernels run the same
    per-cluster arithmetic.  FP64 (unfused operations) agrees to the order of the FP64
    sums; the FP32 model code is compiled into two different kernels, where the compiler
    may contract different FP32 multiply-adds, so mixed results agree to FP32 rounding."""
    tol = 1e-11 if precision == capi.FP64 else 1e-6
    box = systems.config0()
    ctx = capi.Context(0)
    try:
        fused = ctx.mbpol_forces(box, precision=precision)
        ctx.set_fused(False)
        sep = ctx.mbpol_forces(box, precision=precision)
    finally:
        ctx.close()
    for k in ("eng2", "eng3", "vir"):
        assert abs(fused[k] - sep[k]) <= tol * abs(sep[k]), k
    for k in ("forces", "atomic_energy", "stress", "jpot", "jkin"):
        assert rel_err(fused[k], sep[k]) <= tol, k


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
def test_water_forces_one_call_matches_the_separate_calls(precision):
    """mbx_water_forces = 1-body + dispersion + MB-pol through the separate entry points;
    jkin sees every term's per-atom energy."""
    box = systems.config0()
    lt, mol = systems.water_types(box)
    ctx = capi.Context(0)
    try:
        ctx.disp_setup(systems.DISP_PARAMS_SYNTHETIC, rcut=9.0, delr=1.0)
        one = ctx.water_forces(box, precision=precision, dispersion=True)
        pes = ctx.ps_pes(box)
        disp = ctx.dispersion(box, lt, mol)
        mb = ctx.mbpol_forces(box, precision=precision)
    finally:
        ctx.close()
    tol = 1e-11
    # the mixed whole evaluation takes the dispersion's mixed form (FP32 pair terms, FP64
    # sums): against the FP64 entry point its forces and per-atom energies within 2e-7 of
    # their largest entries, its energy and heat terms within 1e-6
    tol_a = tol if precision == capi.FP64 else 2e-7
    tol_s = tol if precision == capi.FP64 else 1e-6
    ref_f = pes["forces"] + disp["forces"] + mb["forces"]
    assert rel_err(one["forces"], ref_f) <= tol_a
    ref_ae = pes["atomic_energy"] + disp["atomic_energy"] + mb["atomic_energy"]
    assert rel_err(one["atomic_energy"], ref_ae) <= tol_a
    sc = one["scalars"]
    assert abs(sc[capi.S_ENG3] - mb["eng3"]) <= tol * abs(mb["eng3"])
    assert abs(sc[capi.NSCALARS] - pes["engang"]) <= tol * abs(pes["engang"])
    assert abs(sc[capi.NSCALARS + 14] - disp["eng"]) <= tol_s * abs(disp["eng"])
    assert rel_err(sc[capi.NSCALARS + 25:capi.NSCALARS + 28], disp["jpot"]) <= tol_s
    nw3 = 3 * box.nw
    m, v = box.mass[:nw3], box.vel[:nw3]
    eng = 0.5 * m * (v * v).sum(1) + ref_ae[:nw3]
    assert rel_err(sc[capi.S_JKIN:capi.S_JKIN + 3], (eng[:, None] * v).sum(0)) <= tol_a


def _offdiag(nsite):
    m = np.ones((nsite, nsite, 3), bool)
    for i in range(nsite):
        m[i, i, :] = False
    return m.ravel()


def test_force_matrices_match_reference_golden(mbx_ctx, golden):
    """The force matrices of the per-cluster entry points (read by the reference's
    HEAT_STRESS build) against the reference's own C++ on the golden clusters: every
    entry its reader uses (the off-diagonal ones), 1e-10 of max(|entry|, 1); 3B leaves its
    diagonal as given, 2B writes 0 there; dimers beyond the cutoff are left untouched."""
    lib = mbx_ctx.lib
    D = C.POINTER(C.c_double)
    W2 = np.ascontiguousarray(golden["W2"])
    n2 = len(W2)
    w1, w2 = np.ascontiguousarray(W2[:, 0]), np.ascontiguousarray(W2[:, 1])
    fm = np.zeros((n2, 108))
    assert lib.mbx_2b_force_matrix_batch(mbx_ctx.h, n2, w1.ctypes.data_as(D), w2.ctypes.data_as(D),
                                         fm.ctypes.data_as(D)) == 0
    ref = golden["FM2"]
    off = _offdiag(6)
    scale = np.maximum(np.abs(ref[:, off]).max(1), 1.0)
    assert np.all(np.abs(fm[:, off] - ref[:, off]).max(1) <= 1e-10 * scale)
    assert not fm[:, ~off].any()
    # the O-O entries carry the switch: the rows of a dimer sum to its gradient (row
    # sums of the 6 x 6 block, X sites redistributed) -- a check of the bookkeeping
    G = golden["G2"].reshape(n2, 18)
    rows = fm.reshape(n2, 6, 6, 3).sum(2).reshape(n2, 18)
    inside = golden["E2"] != 0
    assert np.abs(rows[inside] - G[inside]).max() <= 1e-9 * np.abs(G).max()
    W3 = np.ascontiguousarray(golden["W3"])
    n3 = len(W3)
    v = [np.ascontiguousarray(W3[:, q]) for q in range(3)]
    fm3 = np.zeros((n3, 243))
    assert lib.mbx_3b_force_matrix_batch(mbx_ctx.h, n3, *(a.ctypes.data_as(D) for a in v),
                                         fm3.ctypes.data_as(D)) == 0
    ref3 = golden["FM3"]
    scale3 = np.maximum(np.abs(ref3).max(1), 1.0)
    assert np.all(np.abs(fm3 - ref3).max(1) <= 1e-10 * scale3)
    # through the drop-in symbol, as the reference's Fortran calls it
    e = C.c_double(0)
    g1, g2 = np.zeros(9), np.zeros(9)
    k = int(np.argmax(inside))
    a, b = np.ascontiguousarray(W2[k, 0]), np.ascontiguousarray(W2[k, 1])
    f1 = np.zeros(108)
    lib.mbpol_2b_poly_(a.ctypes.data_as(D), b.ctypes.data_as(D), C.byref(e), g1.ctypes.data_as(D),
                       g2.ctypes.data_as(D), f1.ctypes.data_as(D))
    assert np.abs(f1[off] - ref[k, off]).max() <= 1e-10 * max(np.abs(ref[k, off]).max(), 1.0)
