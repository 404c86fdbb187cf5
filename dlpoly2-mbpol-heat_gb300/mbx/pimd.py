"""Path-integral bead coupling of the reference's PIMD/CMD mode, on the host: the
normal-mode transformation matrices and the ring-polymer spring forces, for a caller that
evaluates the beads' physical forces with mbx_water_step_multi and propagates them itself.
The reference's i-PI build instead leaves this coupling to the i-PI server (mbx_ipi_run).

Restated from SOURCE/centroid_matrix.f (transformation_matrix, the cart <-> normal-mode
transforms) and SOURCE/centroid_spring_force.f (the spring forces, the spring energy and
the centroid-virial estimator), with the beads as a leading array axis instead of MPI ring
ranks.  The number of beads is even, as there.
"""
import math

import numpy as np


def transformation_matrix(nbead, langevin=False):
    """(nmode_to_cart[bead, mode], cart_to_nmode[mode, bead], lambda_nmode[mode]) of
    SOURCE/centroid_matrix.f:3-135 (0-based here).  Without Langevin: columns 1, the
    alternating mode, sqrt(2) cos / -sqrt(2) sin pairs; cart_to_nmode = nmode_to_cart^T / P;
    lambda = P * 2 (1 - cos(2 pi n / P)) per pair, 4 P for the alternating mode.  With
    Langevin: the orthonormal ordering (centroid, cos modes, alternating, sin modes),
    lambda = 1."""
    P = int(nbead)
    if P < 2 or P % 2:
        raise ValueError("the number of beads must be even")
    c = np.zeros((P, P))
    if not langevin:
        c[:, 0] = 1.0
        for n1 in range(1, P // 2 + 1):
            c[2 * n1 - 1, P - 1] = -1.0
            c[2 * n1 - 2, P - 1] = 1.0
        for n1 in range(1, P + 1):
            t = 2.0 * math.pi * (n1 - 1) / P
            for n2 in range(1, P // 2):
                c[n1 - 1, 2 * n2 - 1] = math.sqrt(2.0) * math.cos(t * n2)
                c[n1 - 1, 2 * n2] = -math.sqrt(2.0) * math.sin(t * n2)
        c2n = c.T / P
        lam = np.zeros(P)
        for n in range(1, P // 2):
            v = 2.0 * (1.0 - math.cos(2.0 * math.pi * n / P)) * P
            lam[2 * n - 1] = v
            lam[2 * n] = v
        lam[P - 1] = 4.0 * P
    else:
        for n1 in range(1, P + 1):
            a = math.sqrt(1.0 / P)
            c[n1 - 1, 0] = a
            c[n1 - 1, P // 2] = a * (-1.0) ** n1
            b = math.sqrt(2.0 / P)
            t = 2.0 * math.pi * n1 / P
            for n2 in range(2, P // 2 + 1):
                c[n1 - 1, n2 - 1] = b * math.cos(t * (n2 - 1))
                c[n1 - 1, n2 + P // 2 - 1] = b * math.sin(t * (n2 + P / 2.0 - 1.0))
        c2n = c.T.copy()
        lam = np.ones(P)
    return c, c2n, lam


def to_nmode(x, cart_to_nmode):
    """normal-mode coordinates of bead coordinates x[P, ...] (SOURCE/centroid_matrix.f:140-203)"""
    return np.tensordot(cart_to_nmode, x, axes=(1, 0))


def to_cart(q, nmode_to_cart):
    """bead coordinates of normal-mode coordinates q[P, ...]
    (SOURCE/centroid_matrix.f:208-270)"""
    return np.tensordot(nmode_to_cart, q, axes=(1, 0))


def spring_forces(x, f, mass, hbar, beta, force_scale=1.0, langevin=False, add_spring_to_forces=True):
    """SOURCE/centroid_spring_force.f: x[P, N, 3] bead positions, f[P, N, 3] their physical
    forces, mass[N] physical masses.  Returns (forces with the springs added, spring energy
    0.5 coeff sum_k sum_i m_i |r_i^k - r_i^(k-1)|^2, centroid-virial term
    0.5 sum_k sum_i -(r_i^k - c_i) . f_i^k / force_scale) with coeff = P / (hbar beta)^2 and
    c the centroid (the first normal mode, scaled to a position)."""
    x = np.asarray(x, np.float64)
    f = np.asarray(f, np.float64)
    m = np.asarray(mass, np.float64)[None, :, None]
    P = x.shape[0]
    coeff = P / (hbar * beta) ** 2
    _, c2n, _ = transformation_matrix(P, langevin)
    fac1 = 1.0 / math.sqrt(P) if langevin else 1.0
    fac3 = 0.0 if (langevin and not add_spring_to_forces) else force_scale
    centroid = to_nmode(x, c2n)[0] * fac1
    prev = np.roll(x, 1, axis=0)     # bead k - 1 (ring)
    nxt = np.roll(x, -1, axis=0)     # bead k + 1
    d1 = x - centroid[None]
    d2 = x - prev
    d3 = x - nxt
    e_deriv = 0.5 * float(-(d1 * f).sum()) / force_scale
    e_spring = 0.5 * coeff * float((m * d2 ** 2).sum())
    out = f - coeff * m * (d2 + d3) * fac3
    return out, e_spring, e_deriv
