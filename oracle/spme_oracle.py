"""SPME and Ewald k-space oracles in numpy (test infrastructure only).

Only tests/ and bench.py's CPU-baseline leg use this module; nothing on the product path
imports it.

Three restatements:

* ``ewald_spme_charges``: the reference's charge-only smooth particle-mesh Ewald,
  following SOURCE/ewald_spme.f:1-362 step by step (fractional coordinates
  K (s + 1/2) with Fortran ``int`` truncation, SOURCE/bspgen.f's spline recursion,
  SOURCE/bspcoe.f's Euler-spline moduli, the spherical k cut at 1.05 x half the grid
  with the Nyquist index counted as -K/2, the convolution, energy and stress, and
  SOURCE/spme_for.f's forces with the mean force removed).  The FFT is numpy's.

* ``spme_kspace``: the SPME of the GB300 path for charges AND induced point dipoles (the
  reference has no SPME for dipoles: its polar branch runs the explicit Ewald sum of
  SOURCE/ewald1p.f).  Dipoles are spread as mu . grad of the B-splines; energies, forces
  (second spline derivatives), fields, potentials, the stress with the dipoles' strain
  term and ewald1p's heat-current term from SPME structure factors.  Its charge part is
  the reference's (above) except that the Nyquist frequencies carry no weight.

* ``ewald_kspace``: the explicit Ewald k-space sum of SOURCE/ewald1p.f for given charges
  and dipoles over the reference's half-space k vectors (cut at 1.05 x min(kmax_a w_a)),
  the quantities of ``spme_kspace`` without the particle-mesh approximation.

Units: Angstrom, e, DL_POLY internal energy; R4PIE0 = 138935.4835 (SOURCE/dl_params.inc:60).
"""
import math

import numpy as np

R4PIE0 = 138935.4835
TWOPI = 2.0 * math.pi
_OA = (0, 1, 2, 0, 0, 1)
_OB = (0, 1, 2, 1, 2, 2)


def invert(cell):
    """rcell of SOURCE/invert.f for the DL_POLY cell (cell[0:3] the first vector)."""
    a = np.asarray(cell, np.float64)
    b = np.empty(9)
    b[0] = a[4] * a[8] - a[5] * a[7]
    b[1] = a[2] * a[7] - a[1] * a[8]
    b[2] = a[1] * a[5] - a[2] * a[4]
    b[3] = a[5] * a[6] - a[3] * a[8]
    b[4] = a[0] * a[8] - a[2] * a[6]
    b[5] = a[2] * a[3] - a[0] * a[5]
    b[6] = a[3] * a[7] - a[4] * a[6]
    b[7] = a[1] * a[6] - a[0] * a[7]
    b[8] = a[0] * a[4] - a[1] * a[3]
    d = a[0] * b[0] + a[3] * b[1] + a[6] * b[2]
    return b / d, abs(d)


def widths(a):
    """Perpendicular widths of the cell given by the 9-vector a (dcell's celprp(7..9))."""
    a = np.asarray(a, np.float64)
    axb = np.array([a[1] * a[5] - a[2] * a[4], a[2] * a[3] - a[0] * a[5], a[0] * a[4] - a[1] * a[3]])
    bxc = np.array([a[4] * a[8] - a[5] * a[7], a[5] * a[6] - a[3] * a[8], a[3] * a[7] - a[4] * a[6]])
    cxa = np.array([a[7] * a[2] - a[1] * a[8], a[0] * a[8] - a[2] * a[6], a[1] * a[6] - a[0] * a[7]])
    v = abs(a[0] * bxc[0] + a[1] * bxc[1] + a[2] * bxc[2])
    return np.array([v / np.linalg.norm(bxc), v / np.linalg.norm(cxa), v / np.linalg.norm(axb)])


def kvec(m1, m2, m3, rc):
    """k = 2 pi sum_a m_a (rc[a], rc[a+3], rc[a+6]) (the reference's rkx3, rky3, rkz3)."""
    return np.stack([TWOPI * (m1 * rc[0] + m2 * rc[1] + m3 * rc[2]),
                     TWOPI * (m1 * rc[3] + m2 * rc[4] + m3 * rc[5]),
                     TWOPI * (m1 * rc[6] + m2 * rc[7] + m3 * rc[8])], -1)


# --------------------------------------------------------------------------------------
# the reference's charge SPME
def _bspgen(t, nospl):
    """SOURCE/bspgen.f for one coordinate array t: bsp[:, j-1], bsd[:, j-1], j = 1..nospl."""
    n = t.shape[0]
    it = np.trunc(t)                       # Fortran int()
    bsp = np.zeros((n, nospl))
    bsd = np.zeros((n, nospl))
    bsd[:, 0] = 1.0
    bsd[:, 1] = -1.0
    bsp[:, 0] = t - it
    bsp[:, 1] = 1.0 - t + it
    for k in range(3, nospl + 1):
        bsp[:, k - 1] = 0.0
        for j in range(k, 1, -1):
            if k == nospl:
                bsd[:, j - 1] = bsp[:, j - 1] - bsp[:, j - 2]
            aaa = t + float(j - 1) - it
            bsp[:, j - 1] = (aaa * bsp[:, j - 1] + (float(k) - aaa) * bsp[:, j - 2]) / float(k - 1)
        if k == nospl:
            bsd[:, 0] = bsp[:, 0]
        bsp[:, 0] = (t - it) * bsp[:, 0] / float(k - 1)
    return bsp, bsd


def _bspcoe(nospl, K):
    """|bsc(i)|^2 of SOURCE/bspcoe.f along one axis, i = 0..K-1."""
    csp = np.zeros(nospl + 1)
    csp[1] = 0.0
    csp[2] = 1.0
    for k in range(3, nospl + 1):
        csp[k] = 0.0
        for j in range(k, 1, -1):
            csp[j] = (float(j - 1) * csp[j] + float(k - j + 1) * csp[j - 1]) / float(k - 1)
    i = np.arange(K)
    ww = np.exp(1j * TWOPI * np.arange(K) / K)
    ccc = np.zeros(K, np.complex128)
    for k in range(0, nospl - 1):
        ccc += csp[k + 2] * ww[(i * k) % K]
    bsc = ww[(i * (nospl - 1)) % K] / ccc
    return np.abs(bsc) ** 2


def ewald_spme_charges(xyz, chge, cell, alpha, K, nospl, epsq=1.0):
    """SOURCE/ewald_spme.f (imcon 1-3, one node) with SOURCE/spme_for.f.

    Returns (engcpe including the self term, stress[9], forces n x 3)."""
    xyz = np.asarray(xyz, np.float64)
    q = np.asarray(chge, np.float64)
    n = xyz.shape[0]
    K1, K2, K3 = K
    rcell, volm = invert(cell)
    engsic = -R4PIE0 / epsq * alpha * np.sum(q ** 2) / math.sqrt(math.pi)
    rvolm = TWOPI / volm
    ralph = -0.25 / alpha ** 2
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    txx = K1 * (rcell[0] * x + rcell[3] * y + rcell[6] * z + 0.5)
    tyy = K2 * (rcell[1] * x + rcell[4] * y + rcell[7] * z + 0.5)
    tzz = K3 * (rcell[2] * x + rcell[5] * y + rcell[8] * z + 0.5)
    bspx, bsdx = _bspgen(txx, nospl)
    bspy, bsdy = _bspgen(tyy, nospl)
    bspz, bsdz = _bspgen(tzz, nospl)
    # 1-based grid indices as the reference computes them (0-based below)
    def idx(t, Kd):
        ll = np.trunc(t).astype(np.int64)[:, None] - np.arange(1, nospl + 1)[None, :] + 2
        ll = np.where(ll > Kd, 1, ll)
        ll = np.where(ll < 1, ll + Kd, ll)
        return ll - 1
    jx, jy, jz = idx(txx, K1), idx(tyy, K2), idx(tzz, K3)
    qqc = np.zeros((K3, K2, K1))   # [l][k][j]
    w = q[:, None, None, None] * bspz[:, :, None, None] * bspy[:, None, :, None] * bspx[:, None, None, :]
    np.add.at(qqc, (jz[:, :, None, None], jy[:, None, :, None], jx[:, None, None, :]), w)
    # dlpfft3(0, 1, ...): the transform with exp(+i ...); numpy's ifftn times the size
    qqq = np.fft.ifftn(qqc) * qqc.size
    rcpcut = 0.5 * min(K1 * widths(rcell)[0], K2 * widths(rcell)[1], K3 * widths(rcell)[2])
    rcpcut = rcpcut * 1.05 * TWOPI
    rcpct2 = rcpcut ** 2
    def freq(Kd):
        j = np.arange(1, Kd + 1)
        return np.where(j > Kd // 2, j - Kd - 1, j - 1).astype(np.float64)
    ll, kk, jj = np.meshgrid(freq(K3), freq(K2), freq(K1), indexing="ij")
    kv = kvec(jj, kk, ll, rcell)
    rksq = np.sum(kv ** 2, -1)
    bb1 = (_bspcoe(nospl, K3)[:, None, None] * _bspcoe(nospl, K2)[None, :, None] *
           _bspcoe(nospl, K1)[None, None, :])
    inside = (rksq > 1e-6) & (rksq <= rcpct2)
    rs = np.where(inside, rksq, 1.0)
    vterm = np.where(inside, bb1 * np.exp(ralph * rs) / rs * qqq, 0.0)
    akv = np.where(inside, 2.0 * (1.0 / rs - ralph) * np.real(vterm * np.conj(qqq)), 0.0)
    omg = np.zeros(9)
    omg[0] = -np.sum(kv[..., 0] ** 2 * akv)
    omg[4] = -np.sum(kv[..., 1] ** 2 * akv)
    omg[8] = -np.sum(kv[..., 2] ** 2 * akv)
    omg[1] = -np.sum(kv[..., 0] * kv[..., 1] * akv)
    omg[2] = -np.sum(kv[..., 0] * kv[..., 2] * akv)
    omg[5] = -np.sum(kv[..., 1] * kv[..., 2] * akv)
    eng1 = np.real(np.sum(vterm * np.conj(qqq)))
    # dlpfft3(0, -1, ...): exp(-i ...), unnormalised
    qpot = np.fft.fftn(vterm)
    # spme_for
    fac = -2.0 * rvolm * R4PIE0 / epsq
    qs = np.real(qpot)[jz[:, :, None, None], jy[:, None, :, None], jx[:, None, None, :]]
    bdx = np.sum(qs * bsdx[:, None, None, :] * bspy[:, None, :, None] * bspz[:, :, None, None], (1, 2, 3)) * K1
    bdy = np.sum(qs * bspx[:, None, None, :] * bsdy[:, None, :, None] * bspz[:, :, None, None], (1, 2, 3)) * K2
    bdz = np.sum(qs * bspx[:, None, None, :] * bspy[:, None, :, None] * bsdz[:, :, None, None], (1, 2, 3)) * K3
    f = np.empty((n, 3))
    f[:, 0] = fac * q * (bdx * rcell[0] + bdy * rcell[1] + bdz * rcell[2])
    f[:, 1] = fac * q * (bdx * rcell[3] + bdy * rcell[4] + bdz * rcell[5])
    f[:, 2] = fac * q * (bdx * rcell[6] + bdy * rcell[7] + bdz * rcell[8])
    f -= f.mean(0)
    engcpe = rvolm * R4PIE0 * eng1 / epsq + engsic
    scal1 = rvolm * R4PIE0 / epsq
    st = np.array([omg[0] + eng1, omg[1], omg[2], omg[1], omg[4] + eng1, omg[5], omg[2], omg[5], omg[8] + eng1])
    return engcpe, scal1 * st, f


# --------------------------------------------------------------------------------------
# SPME for charges and dipoles (the GB300 path's method)
def bspline(w, p):
    """M_p(w + j), j = 0..p-1, and its first and second derivatives (n x p each)."""
    n = w.shape[0]
    a = np.zeros((n, p))
    a[:, 0] = w
    a[:, 1] = 1.0 - w
    d1 = d2 = None
    for m in range(2, p):
        if m == p - 2:
            d2 = a.copy()
            d2[:, 1:] -= 2.0 * a[:, :-1]
            d2[:, 2:] += a[:, :-2]
        if m == p - 1:
            d1 = a.copy()
            d1[:, 1:] -= a[:, :-1]
        new = a.copy()
        for j in range(m, -1, -1):
            lo = a[:, j - 1] if j >= 1 else 0.0
            new[:, j] = ((w + j) * a[:, j] + (m + 1 - w - j) * lo) / m
        a = new
    return a, d1, d2


def moduli(p, K):
    """|b(m)|^2 along one axis (bspcoe's moduli), 0 where the denominator vanishes."""
    a, _, _ = bspline(np.zeros(1), p)     # a[0, j] = M_p(j)
    i = np.arange(K)
    den = np.zeros(K, np.complex128)
    for k in range(p - 1):
        den += a[0, k + 1] * np.exp(1j * TWOPI * ((i * k) % K) / K)
    d2 = np.abs(den) ** 2
    return np.where(d2 > 1e-30, 1.0 / np.where(d2 > 1e-30, d2, 1.0), 0.0)


def influence(cell, alpha, K, p):
    """G[iz, iy, ix] = |b|^2 exp(-k^2 / 4 alpha^2) / k^2 inside the reference's sphere, 0 at
    m = 0, beyond the sphere and at the Nyquist frequencies; and the k vectors."""
    rc, _ = invert(cell)
    K1, K2, K3 = K
    def freq(Kd):
        i = np.arange(Kd)
        return np.where(i < Kd // 2, i, i - Kd).astype(np.float64)
    m3, m2, m1 = np.meshgrid(freq(K3), freq(K2), freq(K1), indexing="ij")
    kv = kvec(m1, m2, m3, rc)
    rksq = np.sum(kv ** 2, -1)
    wr = widths(rc)
    rcpcut = 0.5 * min(K1 * wr[0], K2 * wr[1], K3 * wr[2]) * 1.05 * TWOPI
    nyq = np.zeros(rksq.shape, bool)
    for ax, Kd in ((2, K1), (1, K2), (0, K3)):
        if Kd % 2 == 0:
            sl = [slice(None)] * 3
            sl[ax] = Kd // 2
            nyq[tuple(sl)] = True
    inside = (rksq > 1e-6) & (rksq <= rcpcut ** 2) & ~nyq
    bsq = moduli(p, K3)[:, None, None] * moduli(p, K2)[None, :, None] * moduli(p, K1)[None, None, :]
    rs = np.where(inside, rksq, 1.0)
    G = np.where(inside, bsq * np.exp(-0.25 / alpha ** 2 * rs) / rs, 0.0)
    return G, kv, rksq


def _splines(xyz, cell, K, p):
    rc, _ = invert(cell)
    out = []
    for a in range(3):
        t = K[a] * (rc[a] * xyz[:, 0] + rc[a + 3] * xyz[:, 1] + rc[a + 6] * xyz[:, 2] + 0.5)
        fl = np.floor(t)
        th, d1, d2 = bspline(t - fl, p)
        gi = (fl.astype(np.int64)[:, None] - np.arange(p)[None, :]) % K[a]
        out.append((gi, th, d1, d2))
    jac = np.array([[K[a] * rc[a + 3 * c] for c in range(3)] for a in range(3)])
    return out, jac, rc


def heat_kterm(kx, s1, s2, Mc, Ms, V1, V2, W1, W2, f, akv2):
    """ewald1p's heat-current term of each k vector (vectorised over k; arrays (..., 3) and
    (..., 3, 3) with W[c][b]); the same regrouping as the GPU path."""
    kW1 = np.einsum("...c,...cb->...b", kx, W1)
    kW2 = np.einsum("...c,...cb->...b", kx, W2)
    P = s1[..., None] * V1 + s2[..., None] * kW1 + s2[..., None] * V2 - s1[..., None] * kW2
    kp = np.sum(kx * P, -1)
    Q = (-Ms[..., :, None] * V1[..., None, :] + s2[..., None, None] * W1 + Mc[..., :, None] * kW1[..., None, :] +
         Mc[..., :, None] * V2[..., None, :] - s1[..., None, None] * W2 + Ms[..., :, None] * kW2[..., None, :])
    out = np.zeros(kx.shape)
    for aa in range(3):
        y = 0.0
        for b in range(3):
            lo, hi = min(aa, b), max(aa, b)
            y = y + kx[..., lo] * Q[..., hi, b]
        out[..., aa] = f * (P[..., aa] - akv2 * kx[..., aa] * kp + y)
    return out


def _stress(sfac, omg6, eng1):
    o = omg6
    return sfac * np.array([o[0] + eng1, o[3], o[4], o[3], o[1] + eng1, o[5], o[4], o[5], o[2] + eng1])


def spme_kspace(xyz, chge, cell, alpha, K, p, dip=None, vel=None, epsq=1.0):
    """SPME k space of charges and point dipoles (the quantities of mbx_spme_kspace):
    dict(engc, eng, stress, jpot, forces, field, pot)."""
    xyz = np.asarray(xyz, np.float64)
    q = np.asarray(chge, np.float64)
    n = xyz.shape[0]
    mu = np.zeros((n, 3)) if dip is None else np.asarray(dip, np.float64)
    sp, jac, rc = _splines(xyz, cell, K, p)
    (gx, tx, dx, ddx), (gy, ty, dy, ddy), (gz, tz, dz, ddz) = sp
    _, volm = invert(cell)
    sfac = 2.0 * (TWOPI / volm) * R4PIE0 / epsq
    mt = mu @ jac.T                                     # mu_t[a] = sum_c jac[a][c] mu_c
    K1, K2, K3 = K
    ix = (gz[:, :, None, None], gy[:, None, :, None], gx[:, None, None, :])
    th = tz[:, :, None, None] * ty[:, None, :, None] * tx[:, None, None, :]
    gth = [tz[:, :, None, None] * ty[:, None, :, None] * dx[:, None, None, :],
           tz[:, :, None, None] * dy[:, None, :, None] * tx[:, None, None, :],
           dz[:, :, None, None] * ty[:, None, :, None] * tx[:, None, None, :]]
    wdip = sum(mt[:, a, None, None, None] * gth[a] for a in range(3))
    Qtot = np.zeros((K3, K2, K1))
    Qq = np.zeros((K3, K2, K1))
    np.add.at(Qtot, ix, q[:, None, None, None] * th + wdip)
    np.add.at(Qq, ix, q[:, None, None, None] * th)
    N = Qtot.size
    G, kv, rksq = influence(cell, alpha, K, p)
    Ftot = np.fft.ifftn(Qtot) * N        # sum_g Q(g) exp(+2 pi i m.g / K)
    Fq = np.fft.ifftn(Qq) * N
    rs = np.where(G > 0, rksq, 1.0)
    akv2 = np.where(G > 0, 2.0 * (1.0 / rs + 0.25 / alpha ** 2), 0.0)
    engc = 0.5 * np.sum(G * np.abs(Fq) ** 2)
    eng1 = 0.5 * np.sum(G * np.abs(Ftot) ** 2)
    omg = np.array([-0.5 * np.sum(G * akv2 * np.abs(Ftot) ** 2 * kv[..., _OA[i]] * kv[..., _OB[i]]) for i in range(6)])
    phi_tot = np.real(np.fft.fftn(G * Ftot))
    phi_q = np.real(np.fft.fftn(G * Fq))
    pt = phi_tot[ix]
    D = np.stack([np.sum(pt * gth[a], (1, 2, 3)) for a in range(3)], -1) @ jac      # D_r[c] = sum_a jac[a][c] D_t[a]
    # second derivatives of M in t space
    hth = {(0, 0): tz[:, :, None, None] * ty[:, None, :, None] * ddx[:, None, None, :],
           (1, 1): tz[:, :, None, None] * ddy[:, None, :, None] * tx[:, None, None, :],
           (2, 2): ddz[:, :, None, None] * ty[:, None, :, None] * tx[:, None, None, :],
           (0, 1): tz[:, :, None, None] * dy[:, None, :, None] * dx[:, None, None, :],
           (0, 2): dz[:, :, None, None] * ty[:, None, :, None] * dx[:, None, None, :],
           (1, 2): dz[:, :, None, None] * dy[:, None, :, None] * tx[:, None, None, :]}
    W = np.zeros((n, 3))
    for a in range(3):
        for b in range(3):
            h = hth[(min(a, b), max(a, b))]
            W[:, a] += mt[:, b] * np.sum(pt * h, (1, 2, 3))
    W = W @ jac
    forces = -sfac * (q[:, None] * D + W)
    forces -= forces.mean(0)
    field = -sfac * D
    pot = sfac * np.sum(pt * th, (1, 2, 3))
    for i in range(6):
        omg[i] += np.sum(mu[:, _OB[i]] * D[:, _OA[i]])
    jpot = np.zeros(3)
    if vel is not None:
        v = np.asarray(vel, np.float64)
        def sf(wgt):
            Qw = np.zeros((K3, K2, K1))
            np.add.at(Qw, ix, wgt[:, None, None, None] * th)
            return np.fft.ifftn(Qw) * N
        Smu = np.stack([sf(mu[:, c]) for c in range(3)], -1)
        Sqv = np.stack([sf(q * v[:, b]) for b in range(3)], -1)
        Smv = np.stack([np.stack([sf(mu[:, c] * v[:, b]) for b in range(3)], -1) for c in range(3)], -2)
        t = heat_kterm(kv, np.real(Ftot), np.imag(Ftot), np.real(Smu), np.imag(Smu), np.real(Sqv), np.imag(Sqv),
                       np.real(Smv), np.imag(Smv), sfac * G, akv2)
        jpot = 0.5 * np.sum(np.where(G[..., None] > 0, t, 0.0), (0, 1, 2))
    return dict(engc=sfac * engc, eng=sfac * eng1, stress=_stress(sfac, omg, eng1), jpot=jpot, forces=forces,
                field=field, pot=pot)


# --------------------------------------------------------------------------------------
# explicit Ewald k-space sum (SOURCE/ewald1p.f)
def ewald_kvectors(cell, alpha, kmax):
    """The half-space k vectors of ewald1p (SOURCE/ewald1p.f:159-172, :279-348) in its order."""
    rc, volm = invert(cell)
    wr = widths(rc)
    rcpcut = min(kmax[0] * wr[0], kmax[1] * wr[1], kmax[2] * wr[2]) * 1.05 * TWOPI
    ks = []
    mmin, nmin = 0, 1
    for ll in range(0, kmax[0] + 1):
        for mm in range(mmin, kmax[1] + 1):
            for nn in range(nmin, kmax[2] + 1):
                ks.append((ll, mm, nn))
            nmin = -kmax[2]
        mmin = -kmax[1]
    ks = np.array(ks, np.float64)
    kv = kvec(ks[:, 0], ks[:, 1], ks[:, 2], rc)
    rksq = np.sum(kv ** 2, -1)
    keep = rksq <= rcpcut ** 2
    return kv[keep], rksq[keep], volm


def ewald_kspace(xyz, chge, cell, alpha, kmax, dip=None, vel=None, epsq=1.0):
    """The explicit Ewald k-space sum of charges and point dipoles: the quantities of
    spme_kspace (dict) without the mesh."""
    xyz = np.asarray(xyz, np.float64)
    q = np.asarray(chge, np.float64)
    n = xyz.shape[0]
    mu = np.zeros((n, 3)) if dip is None else np.asarray(dip, np.float64)
    kv, rksq, volm = ewald_kvectors(cell, alpha, kmax)
    sfac = 2.0 * (TWOPI / volm) * R4PIE0 / epsq
    ralph = -0.25 / alpha ** 2
    akk = np.exp(ralph * rksq) / rksq
    akv2 = 2.0 * (1.0 / rksq - ralph)
    ph = kv @ xyz.T                                   # K x n
    c, s = np.cos(ph), np.sin(ph)
    ckcs, ckss = c @ q, s @ q
    Mc, Ms = c @ mu, s @ mu                           # K x 3
    skc, sks = np.sum(kv * Mc, -1), np.sum(kv * Ms, -1)
    s1, s2 = ckcs - sks, ckss + skc
    s12 = s1 ** 2 + s2 ** 2
    engc = np.sum(akk * (ckcs ** 2 + ckss ** 2))
    eng1 = np.sum(akk * s12)
    omg = np.array([np.sum(-akk * akv2 * s12 * kv[:, _OA[i]] * kv[:, _OB[i]] -
                           2.0 * akk * kv[:, _OA[i]] * Ms[:, _OB[i]] * s1 +
                           2.0 * akk * kv[:, _OA[i]] * Mc[:, _OB[i]] * s2) for i in range(6)])
    scale = 2.0 * sfac
    kmu = mu @ kv.T                                   # n x K
    fv = q[:, None] * (c.T * (akk * s2) - s.T * (akk * s1)) - kmu * (c.T * (akk * s1) + s.T * (akk * s2))
    forces = -scale * (fv @ kv)
    forces -= forces.mean(0)
    field = -scale * ((c.T * (akk * s2) - s.T * (akk * s1)) @ kv)
    pot = scale * ((c.T * (akk * s1) + s.T * (akk * s2)).sum(1))
    jpot = np.zeros(3)
    if vel is not None:
        v = np.asarray(vel, np.float64)
        V1, V2 = c @ (q[:, None] * v), s @ (q[:, None] * v)
        mv = mu[:, :, None] * v[:, None, :]
        W1 = np.einsum("kj,jcb->kcb", c, mv)
        W2 = np.einsum("kj,jcb->kcb", s, mv)
        jpot = np.sum(heat_kterm(kv, s1, s2, Mc, Ms, V1, V2, W1, W2, sfac * akk, akv2), 0)
    return dict(engc=sfac * engc, eng=sfac * eng1, stress=_stress(sfac, omg, eng1), jpot=jpot, forces=forces,
                field=field, pot=pot)
