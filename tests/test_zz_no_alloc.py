"""mbx_mbpol_forces_noalloc against the allocating device entry point.

Callers that cannot allocate device memory where they need forces (under a foreign
memory pool, in a driver that forbids allocation after start-up) use
mbx_mbpol_forces_noalloc, which keeps its intermediates in one static device array.
This file runs last; it checks the no-allocation entry point through the C ABI against
mbx_mbpol_forces_device on the same device inputs, on two calls in a row (the shared
array keeps the previous call's contents): a cubic and a parallelepiped box, a single
water, and a box too dense for the fixed lists (refused, forces untouched, the next
call correct).
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


def _noalloc(lib, torch, box, d, precision, expect=0):
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
    assert rc == expect
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


def _triclinic(nw, seed):
    box = systems.box_for(nw, seed=seed)
    L = box.L
    # a sheared cell (imcon 3) of the same volume: the waters imaged into it
    box.cell = np.array([L, 0, 0, 0.2 * L, L, 0, 0.1 * L, -0.15 * L, L], dtype=np.float64)
    box.imcon = 3
    return box


@pytest.mark.parametrize("which", ["cubic", "parallelepiped"])
@pytest.mark.parametrize("precision,tol", [(capi.FP64, TOL64), (capi.MIXED, TOL_MIXED)])
def test_noalloc_matches_device_entry_point_twice(precision, tol, which):
    torch = pytest.importorskip("torch")
    lib = capi.load()
    box = systems.config0(seed=31) if which == "cubic" else _triclinic(128, 7)
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


def test_noalloc_single_water():
    """One water: no dimers or trimers; the heat current's kinetic part as the context's."""
    torch = pytest.importorskip("torch")
    lib = capi.load()
    box = systems.box_for(1, seed=2)
    d = _device_inputs(torch, box)
    f_ref, ae_ref, sc_ref = _with_context(torch, box, d, capi.FP64)
    for _ in range(2):
        f, ae, sc = _noalloc(lib, torch, box, d, capi.FP64)
        assert float(np.abs(f).max()) == 0.0 and float(np.abs(ae).max()) == 0.0
        np.testing.assert_allclose(sc, sc_ref, rtol=1e-14, atol=0)


def test_noalloc_capacity_refused_then_recovers():
    """A box far denser than liquid water (216 waters in a 12 A cell: ~140 partners within
    6.5 A against the fixed 64) is refused with MBX_ERR_CAPACITY and leaves the forces and
    energies untouched; the next call on a normal box is correct."""
    torch = pytest.importorskip("torch")
    lib = capi.load()
    dense = systems.water_box(216, 12.0, 5, lattice=6)
    dd = _device_inputs(torch, dense)
    f, ae, _ = _noalloc(lib, torch, dense, dd, capi.FP64, expect=3)   # MBX_ERR_CAPACITY
    assert float(np.abs(f).max()) == 0.0 and float(np.abs(ae).max()) == 0.0
    box = systems.config0(seed=31)
    d = _device_inputs(torch, box)
    f_ref, ae_ref, sc_ref = _with_context(torch, box, d, capi.FP64)
    f, ae, sc = _noalloc(lib, torch, box, d, capi.FP64)
    assert _rel(f, f_ref) <= TOL64
    assert _rel(ae, ae_ref) <= TOL64
    assert abs(sc[capi.S_ENG3] - sc_ref[capi.S_ENG3]) <= TOL64 * abs(sc_ref[capi.S_ENG3])
