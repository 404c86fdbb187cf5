"""mbx_mbpol_forces_noalloc against the allocating device entry point.

Callers that cannot allocate device memory where they need forces (inside a CUDA
stream capture, under a foreign memory pool, in a driver that forbids allocation
after start-up) use mbx_mbpol_forces_noalloc, which keeps its intermediates in one
static device array.  This file runs last; it checks the no-allocation entry point
through the C ABI against mbx_mbpol_forces_device on the same device inputs, on two
calls in a row (the shared array keeps the previous call's contents).
"""
import ctypes as C

import numpy as np
import pytest

from mbx import capi, systems

pytestmark = pytest.mark.gpu

TOL64 = 1e-10        # same tolerance as the FP64 parity tests
TOL_MIXED = 1e-10    # the two entry points run the same mixed kernels


def _device_inputs(torch, box):
    f64 = dict(dtype=torch.float64, device="cuda")
    d = {
        "x": [torch.tensor(np.ascontiguousarray(box.xyz[:, k]), **f64) for k in range(3)],
        "v": [torch.tensor(np.ascontiguousarray(box.vel[:, k]), **f64) for k in range(3)],
        "m": torch.tensor(box.mass, **f64),
        "lst": torch.tensor(box.listttm2(), dtype=torch.int32, device="cuda"),
    }
    return d


def _noalloc(lib, torch, box, d, precision):
    n = box.natms
    f = torch.zeros((3, n), dtype=torch.float64, device="cuda")
    ae = torch.zeros(n, dtype=torch.float64, device="cuda")
    sc = np.zeros(capi.NSCALARS)
    cell = np.ascontiguousarray(box.cell, dtype=np.float64)
    rc = lib.mbx_mbpol_forces_noalloc(precision, box.imcon, cell.ctypes.data_as(C.POINTER(C.c_double)),
                                      3 * box.nw, d["lst"].data_ptr(), n,
                                      *[t.data_ptr() for t in d["x"]], *[f[k].data_ptr() for k in range(3)],
                                      *[t.data_ptr() for t in d["v"]], d["m"].data_ptr(), ae.data_ptr(),
                                      sc.ctypes.data_as(C.POINTER(C.c_double)), None)
    assert rc == 0
    torch.cuda.synchronize()
    return f.cpu().numpy(), ae.cpu().numpy(), sc


def _with_context(torch, box, d, precision):
    n = box.natms
    ctx = capi.Context(0)
    try:
        f = torch.zeros((3, n), dtype=torch.float64, device="cuda")
        ae = torch.zeros(n, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()   # the context works on its own stream
        sc = ctx.mbpol_forces_device(precision, box.imcon, box.cell, 3 * box.nw, d["lst"].data_ptr(), n,
                                     [t.data_ptr() for t in d["x"]], [f[k].data_ptr() for k in range(3)],
                                     [t.data_ptr() for t in d["v"]], d["m"].data_ptr(), ae.data_ptr())
        torch.cuda.synchronize()
        return f.cpu().numpy(), ae.cpu().numpy(), sc
    finally:
        ctx.close()


def _rel(a, b):
    return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))


@pytest.mark.parametrize("precision,tol", [(capi.FP64, TOL64), (capi.MIXED, TOL_MIXED)])
def test_noalloc_matches_device_entry_point_twice(precision, tol):
    torch = pytest.importorskip("torch")
    lib = capi.load()
    box = systems.config0(seed=31)
    d = _device_inputs(torch, box)
    f_ref, ae_ref, sc_ref = _with_context(torch, box, d, precision)
    for _ in range(2):   # the static array keeps the previous call's contents
        f, ae, sc = _noalloc(lib, torch, box, d, precision)
        assert _rel(f, f_ref) <= tol
        assert _rel(ae, ae_ref) <= tol
        for q in (capi.S_ENG2, capi.S_ENG3, capi.S_VIR):
            assert abs(sc[q] - sc_ref[q]) <= tol * abs(sc_ref[q])
        assert _rel(sc[capi.S_JPOT:capi.S_JPOT + 3], sc_ref[capi.S_JPOT:capi.S_JPOT + 3]) <= tol
        assert _rel(sc[capi.S_JKIN:capi.S_JKIN + 3], sc_ref[capi.S_JKIN:capi.S_JKIN + 3]) <= tol


def test_noalloc_rejects_oversized_systems():
    torch = pytest.importorskip("torch")
    lib = capi.load()
    box = systems.box_for(520, seed=3)
    d = _device_inputs(torch, box)
    n = box.natms
    f = torch.zeros((3, n), dtype=torch.float64, device="cuda")
    cell = np.ascontiguousarray(box.cell, dtype=np.float64)
    rc = lib.mbx_mbpol_forces_noalloc(capi.FP64, 1, cell.ctypes.data_as(C.POINTER(C.c_double)), 3 * box.nw,
                                      d["lst"].data_ptr(), n, *[t.data_ptr() for t in d["x"]],
                                      *[f[k].data_ptr() for k in range(3)], None, None, None, None, None, None, None)
    assert rc == 1   # MBX_ERR_ARG, nothing computed
    assert float(f.abs().max()) == 0.0
