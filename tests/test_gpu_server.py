"""The continuous-batching server: each result is the same alone and in a concurrent mix."""
import numpy as np
import pytest

from mbx import capi, systems

pytestmark = pytest.mark.gpu


def _boxes():
    sizes = [64, 128, 256, 512, 96, 200, 384, 64]
    return [systems.box_for(n, seed=100 + k) for k, n in enumerate(sizes)]


@pytest.mark.parametrize("precision,tol", [(capi.FP64, 1e-12), (capi.MIXED, 1e-10)])
def test_results_same_alone_and_in_mix(precision, tol):
    boxes = _boxes()
    solo = capi.Server(slots=1)
    try:
        alone = [solo.wait(solo.submit(b, precision)) for b in boxes]
    finally:
        solo.close()
    srv = capi.Server(slots=4, budget_bytes=16e9)
    try:
        ids = [srv.submit(b, precision) for b in boxes]
        mixed = [srv.wait(i) for i in ids]
    finally:
        srv.close()
    for a, m in zip(alone, mixed):
        scale = np.max(np.abs(a["forces"]))
        assert np.max(np.abs(a["forces"] - m["forces"])) <= tol * scale
        assert np.max(np.abs(a["scalars"] - m["scalars"])) <= tol * np.max(np.abs(a["scalars"]))


def test_server_matches_context_api(mbx_ctx):
    box = systems.box_for(150, seed=7)
    srv = capi.Server(slots=2)
    try:
        got = srv.wait(srv.submit(box, capi.FP64))
    finally:
        srv.close()
    one = mbx_ctx.ps_pes(box)
    two = mbx_ctx.mbpol_forces(box, precision=capi.FP64)
    ref = one["forces"] + two["forces"]
    assert np.max(np.abs(got["forces"] - ref)) <= 1e-12 * np.max(np.abs(ref))
    assert abs(got["scalars"][capi.NSCALARS] - one["engang"]) <= 1e-12 * abs(one["engang"])


def test_tiny_budget_still_serves_everything():
    boxes = _boxes()[:4]
    srv = capi.Server(slots=4, budget_bytes=1.0)   # every request exceeds it: runs alone
    try:
        ids = [srv.submit(b, capi.MIXED) for b in boxes]
        out = [srv.wait(i) for i in ids]
    finally:
        srv.close()
    assert all(np.all(np.isfinite(o["forces"])) for o in out)


@pytest.mark.parametrize("precision,tol", [(capi.FP64, 1e-10), (capi.MIXED, 1e-8)])
def test_step_results_same_alone_and_in_mix(precision, tol):
    """Whole force evaluations with the electrostatics: one client per box, so every request
    starts from zero dipoles; alone (one slot) and in a concurrent mix the same."""
    boxes = _boxes()[:6]
    solo = capi.Server(slots=1)
    try:
        alone = [solo.wait_step(solo.submit_step(b, client=k, precision=precision)) for k, b in enumerate(boxes)]
    finally:
        solo.close()
    srv = capi.Server(slots=4, budget_bytes=64e9)
    try:
        ids = [srv.submit_step(b, client=k, precision=precision) for k, b in enumerate(boxes)]
        mixed = [srv.wait_step(i) for i in ids]
    finally:
        srv.close()
    for a, m in zip(alone, mixed):
        scale = np.max(np.abs(a["forces"]))
        assert np.max(np.abs(a["forces"] - m["forces"])) <= tol * scale
        nws = capi.NWATERSCALARS
        assert abs(a["scalars"][nws] - m["scalars"][nws]) <= tol * abs(a["scalars"][nws])   # engcpe
        assert np.max(np.abs(a["dipoles"] - m["dipoles"])) <= tol * np.max(np.abs(a["dipoles"])) + 1e-14


def test_step_server_matches_context_and_warm_starts(mbx_ctx):
    """The server's step = mbx_water_step with the same settings; a client's second request
    starts from the dipoles of its first."""
    box = systems.box_for(128, seed=11)
    moved = systems.box_for(128, seed=11)
    moved.xyz = box.xyz + 0.0002 * box.vel
    prm = systems.polar_params_for(box.cell)
    srv = capi.Server(slots=2)
    try:
        first = srv.wait_step(srv.submit_step(box, client=7, precision=capi.FP64))
        second = srv.wait_step(srv.submit_step(moved, client=7, precision=capi.FP64))
    finally:
        srv.close()
    ref1 = mbx_ctx.water_step(box, prm, precision=capi.FP64)
    ref2 = mbx_ctx.water_step(moved, prm, precision=capi.FP64, dip0=ref1["dipoles"])
    for got, ref in ((first, ref1), (second, ref2)):
        assert np.max(np.abs(got["forces"] - ref["forces"])) <= 1e-11 * np.max(np.abs(ref["forces"]))
        assert np.max(np.abs(got["dipoles"] - ref["dipoles"])) <= 1e-11 * np.max(np.abs(ref["dipoles"]))
        assert np.max(np.abs(got["scalars"] - ref["scalars"])) <= 1e-11 * np.max(np.abs(ref["scalars"]))
