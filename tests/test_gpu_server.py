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
