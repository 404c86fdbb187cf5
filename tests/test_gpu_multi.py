"""Many boxes in one evaluation (mbx_mbpol_multi*): parity per box.

Each box of a packed set must give what it gives alone: against the oracle (FP64,
1e-10 relative, the 1-body PES term included), and against the single-box entry points
of libmbx (FP64 and mixed; the same per-cluster arithmetic, so only the order of the
FP64 atomic sums differs: 1e-11).  The CUDA-graph replay must match a direct launch
and must read new positions written into the same device arrays.
"""
import numpy as np
import pytest

from conftest import rel_err
from mbx import capi, systems

pytestmark = pytest.mark.gpu

TOL64 = 1e-10          # against the oracle
TOL_SAME = 1e-11       # against libmbx's own single-box path (summation order only)


def _per_box_context(ctx, box, precision):
    """1-body + MB-pol of one box through the single-box host entry points."""
    one = ctx.ps_pes(box)
    two = ctx.mbpol_forces(box, precision=precision)
    return one, two


def _check_box(got_f, got_ae, sc, box, one, two, tol):
    ref_f = one["forces"] + two["forces"]
    assert rel_err(got_f, ref_f) <= tol
    assert rel_err(got_ae, one["atomic_energy"] + two["atomic_energy"]) <= tol
    mb = sc[:capi.NSCALARS]
    pes = sc[capi.NSCALARS:]
    for k, slot in (("eng2", capi.S_ENG2), ("eng3", capi.S_ENG3), ("vir", capi.S_VIR)):
        assert abs(mb[slot] - two[k]) <= tol * abs(two[k]), k
    assert rel_err(mb[capi.S_STRESS:capi.S_STRESS + 9], two["stress"]) <= tol
    assert rel_err(mb[capi.S_JPOT:capi.S_JPOT + 3], two["jpot"]) <= tol
    assert abs(pes[0] - one["engang"]) <= tol * abs(one["engang"])
    assert abs(pes[1] - one["virang"]) <= tol * abs(one["virang"])
    assert rel_err(pes[2:11], one["stress"]) <= tol
    assert rel_err(pes[11:14], one["jpot"]) <= tol
    # jkin of the multi-box step runs after the 1-body and MB-pol energies are in place
    nw3 = 3 * box.nw
    m, v = box.mass[:nw3], box.vel[:nw3]
    eng = 0.5 * m * (v * v).sum(1) + one["atomic_energy"][:nw3] + two["atomic_energy"][:nw3]
    assert rel_err(mb[capi.S_JKIN:capi.S_JKIN + 3], (eng[:, None] * v).sum(0)) <= tol


def test_multi_fp64_matches_oracle(oracle_lib):
    boxes = [systems.box_for(64, seed=31), systems.box_for(96, seed=32), systems.box_for(128, seed=33),
             systems.box_for(200, seed=34)]
    bs = systems.BoxSet(boxes)
    ctx = capi.Context(0)
    try:
        got = ctx.mbpol_multi(bs, precision=capi.FP64)
        _, counts = ctx.last_timings()
    finally:
        ctx.close()
    fs, aes = bs.split(got["forces"]), bs.split(got["atomic_energy"])
    npairs = ntrip = 0
    for b, box in enumerate(boxes):
        one = oracle_lib.angfrc_ps(box)
        two = oracle_lib.mbpol_forces(box)
        npairs += two["npairs"]
        ntrip += two["ntrip"]
        _check_box(fs[b], aes[b], got["scalars"][b], box, one, two, TOL64)
    assert counts[0] == npairs and counts[1] == ntrip


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
def test_beads_match_single_box_path(precision):
    beads = systems.beads_from(systems.config0(), 8, 0.05, seed=77)
    bs = systems.BoxSet(beads)
    ctx = capi.Context(0)
    try:
        got = ctx.mbpol_multi(bs, precision=precision)
        fs, aes = bs.split(got["forces"]), bs.split(got["atomic_energy"])
        for b, box in enumerate(beads):
            one, two = _per_box_context(ctx, box, precision)
            _check_box(fs[b], aes[b], got["scalars"][b], box, one, two, TOL_SAME)
    finally:
        ctx.close()


def test_uneven_boxes_match_single_box_path():
    boxes = systems.config3(seed=5, nbox=10)
    bs = systems.BoxSet(boxes)
    ctx = capi.Context(0)
    try:
        got = ctx.mbpol_multi(bs, precision=capi.FP64)
        fs, aes = bs.split(got["forces"]), bs.split(got["atomic_energy"])
        for b, box in enumerate(boxes):
            one, two = _per_box_context(ctx, box, capi.FP64)
            _check_box(fs[b], aes[b], got["scalars"][b], box, one, two, TOL_SAME)
    finally:
        ctx.close()


def test_dense_boxes_regrow_lists():
    """Compressed water (2.7x density) outgrows the default trimer capacity: the step
    is repeated with larger lists and still matches the single-box path."""
    boxes = []
    for k, nw in enumerate((96, 128)):
        b = systems.box_for(nw, seed=50 + k)
        s = 1.0 / 1.4
        b.xyz = b.xyz * s
        b.L *= s
        b.cell = b.cell * s
        boxes.append(b)
    bs = systems.BoxSet(boxes)
    ctx = capi.Context(0)
    try:
        got = ctx.mbpol_multi(bs, precision=capi.FP64)
        assert np.all(np.isfinite(got["forces"]))
        fs, aes = bs.split(got["forces"]), bs.split(got["atomic_energy"])
        for b, box in enumerate(boxes):
            one, two = _per_box_context(ctx, box, capi.FP64)
            _check_box(fs[b], aes[b], got["scalars"][b], box, one, two, TOL_SAME)
    finally:
        ctx.close()


def test_graph_replay_matches_direct_and_sees_new_positions():
    torch = pytest.importorskip("torch")
    beads = systems.beads_from(systems.box_for(128, seed=90), 4, 0.05, seed=91)
    bs = systems.BoxSet(beads)
    n = bs.natms
    f64 = dict(dtype=torch.float64, device="cuda")
    x = [torch.tensor(np.ascontiguousarray(bs.xyz[:, k]), **f64) for k in range(3)]
    v = [torch.tensor(np.ascontiguousarray(bs.vel[:, k]), **f64) for k in range(3)]
    m = torch.tensor(bs.mass, **f64)

    def run(ctx, precision):
        f = torch.zeros((3, n), **f64)
        ae = torch.zeros(n, **f64)
        torch.cuda.synchronize()   # the context works on its own stream
        sc = ctx.mbpol_multi_device(precision, bs, [t.data_ptr() for t in x], [f[k].data_ptr() for k in range(3)],
                                    [t.data_ptr() for t in v], m.data_ptr(), ae.data_ptr())
        torch.cuda.synchronize()
        return f.cpu().numpy(), ae.cpu().numpy(), sc

    direct = capi.Context(0)
    graph = capi.Context(0)
    try:
        direct.set_graphs(False)
        for precision in (capi.FP64, capi.MIXED):
            ref = run(direct, precision)
            before = graph.graph_launches()
            # a replay needs the same arrays: keep the outputs across calls
            f = torch.zeros((3, n), **f64)
            ae = torch.zeros(n, **f64)

            def replay():
                f.zero_()
                ae.zero_()
                torch.cuda.synchronize()
                sc = graph.mbpol_multi_device(precision, bs, [t.data_ptr() for t in x],
                                              [f[k].data_ptr() for k in range(3)], [t.data_ptr() for t in v],
                                              m.data_ptr(), ae.data_ptr())
                torch.cuda.synchronize()
                return f.cpu().numpy(), ae.cpu().numpy(), sc

            for _ in range(3):
                g = replay()
                for a, b in zip(g, ref):
                    assert rel_err(a, b) <= TOL_SAME
            assert graph.graph_launches() - before == 3
            assert direct.graph_launches() == 0
            # new positions written into the same device arrays: the replay must see them
            saved = [t.clone() for t in x]
            rng = np.random.default_rng(3 + precision)
            moved = bs.xyz + rng.normal(scale=0.01, size=bs.xyz.shape)
            for k in range(3):
                x[k].copy_(torch.tensor(np.ascontiguousarray(moved[:, k]), **f64))
            torch.cuda.synchronize()
            ref_moved = run(direct, precision)
            assert rel_err(ref_moved[0], ref[0]) > 1e-6   # the move changes the forces
            g = replay()
            for a, b in zip(g, ref_moved):
                assert rel_err(a, b) <= TOL_SAME
            for k in range(3):
                x[k].copy_(saved[k])
            torch.cuda.synchronize()
    finally:
        direct.close()
        graph.close()


def test_multi_rejects_bad_arguments():
    ctx = capi.Context(0)
    try:
        bs = systems.BoxSet([systems.box_for(64, seed=1)])
        bs.nw_box[0] = -1
        with pytest.raises(capi.MbxError):
            ctx.mbpol_multi(bs)
        bs = systems.BoxSet([systems.box_for(64, seed=1)])
        with pytest.raises(capi.MbxError):
            ctx.mbpol_multi(bs, precision=7)
    finally:
        ctx.close()


@pytest.mark.parametrize("precision", [capi.FP64, capi.MIXED])
def test_multi_fused_matches_separate_kernels(precision):
    # FP64: summation order only; mixed: FP32 rounding (the FP32 model code is compiled
    # into two kernels, whose multiply-add contraction may differ)
    tol = TOL_SAME if precision == capi.FP64 else 1e-6
    bs = systems.BoxSet(systems.config3(seed=9, nbox=6))
    ctx = capi.Context(0)
    try:
        a = ctx.mbpol_multi(bs, precision=precision)
        ctx.set_fused(False)
        b = ctx.mbpol_multi(bs, precision=precision)
    finally:
        ctx.close()
    assert rel_err(a["forces"], b["forces"]) <= tol
    assert rel_err(a["atomic_energy"], b["atomic_energy"]) <= tol
    for k in range(bs.nbox):
        assert rel_err(a["scalars"][k], b["scalars"][k]) <= tol
