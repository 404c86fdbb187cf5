"""Path-integral bead coupling on the device (mbx_pimd.cu) against the host restatement
of the reference's centroid_matrix.f / centroid_spring_force.f (mbx/pimd.py): the
normal-mode transforms and the spring forces, energies and centroid-virial term, for a
water box's beads (the layout of mbx_water_step_multi: bead after bead)."""
import ctypes as C

import numpy as np
import pytest

from mbx import capi, pimd, systems

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("P,langevin,add", [(8, False, True), (32, False, True), (16, True, True),
                                            (16, True, False)])
def test_spring_forces_and_transforms_on_device(mbx_ctx, P, langevin, add):
    torch = pytest.importorskip("torch")
    box = systems.box_for(64, seed=8)
    n = box.natms
    rng = np.random.default_rng(P)
    x = box.xyz[None] + rng.normal(0.0, 0.05, size=(P, n, 3))       # bead positions
    f = rng.normal(0.0, 100.0, size=(P, n, 3))                      # physical forces
    mass = np.array(box.mass, np.float64)
    hbar, beta, fs = 6.350780668, 1.0 / (0.8314462618 * 298.0), 0.5   # DL_POLY units, 298 K
    want, e_spring, e_deriv = pimd.spring_forces(x, f, mass, hbar, beta, force_scale=fs, langevin=langevin,
                                                 add_spring_to_forces=add)
    dev = dict(dtype=torch.float64, device="cuda")
    X = [torch.tensor(np.ascontiguousarray(x[:, :, k].reshape(-1)), **dev) for k in range(3)]
    F = [torch.tensor(np.ascontiguousarray(f[:, :, k].reshape(-1)), **dev) for k in range(3)]
    M = torch.tensor(mass, **dev)
    en = np.zeros(2)
    torch.cuda.synchronize()
    rc = mbx_ctx.lib.mbx_pimd_spring_forces_device(mbx_ctx.h, P, int(langevin), int(add), hbar, beta, fs, n,
                                                   *[t.data_ptr() for t in X], *[t.data_ptr() for t in F],
                                                   M.data_ptr(), en.ctypes.data_as(C.POINTER(C.c_double)))
    assert rc == 0
    got = np.stack([t.cpu().numpy().reshape(P, n) for t in F], -1)
    assert np.abs(got - want).max() <= 1e-12 * np.abs(want).max()
    assert abs(en[0] - e_spring) <= 1e-12 * abs(e_spring)
    assert abs(en[1] - e_deriv) <= 1e-11 * max(abs(e_deriv), 1e-300)
    # normal-mode transforms of the bead positions (x block), both ways
    c, c2n, _ = pimd.transformation_matrix(P, langevin)
    Q = torch.empty_like(X[0])
    R = torch.empty_like(X[0])
    assert mbx_ctx.lib.mbx_pimd_transform_device(mbx_ctx.h, P, int(langevin), 1, n, X[0].data_ptr(),
                                                 Q.data_ptr()) == 0
    assert mbx_ctx.lib.mbx_pimd_transform_device(mbx_ctx.h, P, int(langevin), 0, n, Q.data_ptr(),
                                                 R.data_ptr()) == 0
    q_ref = pimd.to_nmode(x[:, :, 0], c2n)
    assert np.abs(Q.cpu().numpy().reshape(P, n) - q_ref).max() <= 1e-12 * np.abs(q_ref).max()
    assert np.abs(R.cpu().numpy().reshape(P, n) - x[:, :, 0]).max() <= 1e-11 * np.abs(x).max()


def test_odd_bead_count_refused(mbx_ctx):
    assert mbx_ctx.lib.mbx_pimd_transform_device(mbx_ctx.h, 5, 0, 1, 4, None, None) == capi.ERR_ARG
