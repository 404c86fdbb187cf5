"""Host-side path-integral bead coupling (mbx/pimd.py): the reference's normal-mode
matrices (SOURCE/centroid_matrix.f) and spring forces (SOURCE/centroid_spring_force.f),
pinned by self-consistency: the transforms invert each other, the ring-polymer Laplacian
is diagonal in the modes with the restated lambda, the spring forces are minus the
gradient of the spring energy, and the centroid is the first mode."""
import numpy as np
import pytest

from mbx import pimd


@pytest.mark.parametrize("P", [2, 4, 8, 32])
@pytest.mark.parametrize("langevin", [False, True])
def test_transforms_invert(P, langevin):
    c, c2n, lam = pimd.transformation_matrix(P, langevin)
    np.testing.assert_allclose(c2n @ c, np.eye(P), atol=1e-13)
    x = np.random.default_rng(P).normal(size=(P, 5, 3))
    np.testing.assert_allclose(pimd.to_cart(pimd.to_nmode(x, c2n), c), x, atol=1e-12)
    if langevin:
        np.testing.assert_allclose(c.T @ c, np.eye(P), atol=1e-13)   # orthonormal
        assert (lam == 1.0).all()


@pytest.mark.parametrize("P", [4, 8, 16])
def test_ring_laplacian_is_diagonal_in_the_modes(P):
    c, c2n, lam = pimd.transformation_matrix(P, False)
    L = 2 * np.eye(P) - np.roll(np.eye(P), 1, axis=0) - np.roll(np.eye(P), -1, axis=0)
    np.testing.assert_allclose(c.T @ L @ c, np.diag(lam), atol=1e-10)
    assert lam[0] == 0.0


@pytest.mark.parametrize("langevin", [False, True])
def test_spring_forces_are_minus_the_gradient(langevin):
    rng = np.random.default_rng(3)
    P, N = 8, 6
    x = rng.normal(size=(P, N, 3))
    mass = rng.uniform(1.0, 16.0, N)
    hbar, beta, fs = 0.7, 1.3, 1.0
    f0 = np.zeros_like(x)
    f, e, _ = pimd.spring_forces(x, f0, mass, hbar, beta, force_scale=fs, langevin=langevin)
    h = 1e-6
    for idx in [(0, 0, 0), (3, 2, 1), (7, 5, 2)]:
        xp, xm = x.copy(), x.copy()
        xp[idx] += h
        xm[idx] -= h
        ep = pimd.spring_forces(xp, f0, mass, hbar, beta, force_scale=fs, langevin=langevin)[1]
        em = pimd.spring_forces(xm, f0, mass, hbar, beta, force_scale=fs, langevin=langevin)[1]
        assert abs(-(ep - em) / (2 * h) - f[idx]) <= 1e-6 * max(1.0, abs(f[idx]))
    # the springs alone exert no net force
    np.testing.assert_allclose(f.sum(axis=(0, 1)), 0.0, atol=1e-9)


def test_centroid_virial_uses_the_first_mode():
    rng = np.random.default_rng(4)
    P, N = 4, 3
    x = rng.normal(size=(P, N, 3))
    f = rng.normal(size=(P, N, 3))
    for langevin in (False, True):
        _, _, ed = pimd.spring_forces(x, f, np.ones(N), 1.0, 1.0, langevin=langevin)
        want = 0.5 * float(-((x - x.mean(axis=0)) * f).sum())
        assert abs(ed - want) <= 1e-12 * abs(want)


def test_odd_bead_counts_are_refused():
    with pytest.raises(ValueError):
        pimd.transformation_matrix(3)


@pytest.mark.parametrize("P", [2, 8, 32])
@pytest.mark.parametrize("langevin", [False, True])
def test_library_matrices_match_the_restatement(P, langevin):
    """mbx_pimd_matrices (host code of the library) = mbx/pimd.py's restatement."""
    import ctypes as C
    from mbx import capi
    lib = capi.load()
    D = C.POINTER(C.c_double)
    n2c, c2n, lam = np.zeros((P, P)), np.zeros((P, P)), np.zeros(P)
    assert lib.mbx_pimd_matrices(P, int(langevin), n2c.ctypes.data_as(D), c2n.ctypes.data_as(D),
                                 lam.ctypes.data_as(D)) == 0
    c, c2, l = pimd.transformation_matrix(P, langevin)
    np.testing.assert_allclose(n2c, c, rtol=0, atol=1e-15)
    np.testing.assert_allclose(c2n, c2, rtol=0, atol=1e-15)
    np.testing.assert_allclose(lam, l, rtol=1e-15, atol=0)
    assert lib.mbx_pimd_matrices(3, 0, None, None, None) == capi.ERR_ARG
