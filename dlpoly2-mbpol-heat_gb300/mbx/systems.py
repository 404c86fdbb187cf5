"""Seeded synthetic water boxes (the benchmark workloads).

A box is built the way the benchmark configurations describe it: O atoms on a
jittered cubic lattice (the first ``nw`` sites of an ``m**3`` lattice filling the
box), each molecule at the rigid MB-pol-like geometry (OH 0.9572 A, HOH 104.52 deg)
with a uniformly random orientation, then Gaussian noise (sigma 0.02 A) on every
atom, and Maxwell-Boltzmann velocities.  The site layout is DL_POLY's for pure
TTM/MB-pol water: atoms 0..3nw-1 are (O, H1, H2) per molecule, then the nw M
sites (SOURCE/ttm2list.f:20-77); M sites start at the O position.

Units are DL_POLY's: Angstrom, ps, amu, 10 J/mol.
"""
import math

import numpy as np

BOLTZ = 0.831451115          # SOURCE/dl_params.inc:64, 10 J/mol/K
MASS_O = 15.9994
MASS_H = 1.00794
R_OH = 0.9572
THETA_HOH = math.radians(104.52)
LATTICE_JITTER = 0.10         # A, uniform half-width of the lattice jitter


def _random_rotations(rng, n):
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    return np.stack([
        np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)], -1),
        np.stack([2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)], -1),
        np.stack([2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)], -1),
    ], 1)


class WaterBox:
    """Positions/velocities of one periodic water box in DL_POLY site order."""

    def __init__(self, nw, L, xyz, vel, seed):
        self.nw = nw
        self.L = float(L)
        self.cell = np.array([L, 0, 0, 0, L, 0, 0, 0, L], dtype=np.float64)
        self.imcon = 1
        self.xyz = xyz          # (4*nw, 3)
        self.vel = vel          # (4*nw, 3)
        self.seed = seed

    @property
    def natms(self):
        return 4 * self.nw

    @property
    def mass(self):
        m = np.zeros(self.natms)
        m[0:3 * self.nw:3] = MASS_O
        m[1:3 * self.nw:3] = MASS_H
        m[2:3 * self.nw:3] = MASS_H
        return m

    def listttm2(self):
        """1-based atom indices of the water atoms (O,H1,H2 per molecule)."""
        return np.arange(1, 3 * self.nw + 1, dtype=np.int32)

    def listang(self):
        """1-based H-O-H angle triples (H1, O, H2), O the central atom (angfrc's ib)."""
        o = 3 * np.arange(self.nw, dtype=np.int32) + 1
        return np.stack([o + 1, o, o + 2], 1).astype(np.int32)

    def monomers(self):
        return np.ascontiguousarray(self.xyz[:3 * self.nw].reshape(self.nw, 9))


def water_box(nw, L, seed, lattice=None, sigma=0.02, temperature=298.0, jitter=LATTICE_JITTER):
    rng = np.random.default_rng(seed)
    if lattice is None:
        lattice = int(math.ceil(nw ** (1.0 / 3.0) - 1e-9))
    a = L / lattice
    g = np.arange(lattice)
    sites = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)[:nw]
    O = (sites + 0.5) * a + rng.uniform(-jitter, jitter, size=(nw, 3))
    half = 0.5 * THETA_HOH
    body = np.array([[0.0, 0.0, 0.0],
                     [R_OH * math.sin(half), 0.0, R_OH * math.cos(half)],
                     [-R_OH * math.sin(half), 0.0, R_OH * math.cos(half)]])
    R = _random_rotations(rng, nw)
    mol = O[:, None, :] + np.einsum("nij,aj->nai", R, body)
    mol += rng.normal(scale=sigma, size=mol.shape)
    xyz = np.zeros((4 * nw, 3))
    xyz[:3 * nw] = mol.reshape(-1, 3)
    xyz[3 * nw:] = mol[:, 0, :]
    mass = np.zeros(4 * nw)
    mass[0:3 * nw:3] = MASS_O
    mass[1:3 * nw:3] = MASS_H
    mass[2:3 * nw:3] = MASS_H
    vel = np.zeros((4 * nw, 3))
    s = np.sqrt(BOLTZ * temperature / mass[:3 * nw])
    vel[:3 * nw] = rng.normal(size=(3 * nw, 3)) * s[:, None]
    vel[:3 * nw] -= (mass[:3 * nw, None] * vel[:3 * nw]).sum(0) / mass[:3 * nw].sum()
    return WaterBox(nw, L, xyz, vel, seed)


def config0(seed=20240):
    """256 H2O, L = 19.73 A (0.997 g/cm^3), jittered 7^3 lattice."""
    return water_box(256, 19.73, seed, lattice=7)


def config1(seed=20241):
    """4096 H2O, L = 49.70 A, jittered 16^3 lattice."""
    return water_box(4096, 49.70, seed, lattice=16)


def box_for(nw, seed, density=0.997):
    """A box of nw waters at the given density (g/cm^3), lattice as small as fits."""
    mw = 18.01528
    L = (nw * mw / (density * 0.6022140857)) ** (1.0 / 3.0)
    return water_box(nw, L, seed)


def beads_from(box, nbeads, sigma, seed):
    """Path-integral-like replicas: copies of ``box`` with independent Gaussian noise."""
    rng = np.random.default_rng(seed)
    out = []
    for b in range(nbeads):
        xyz = box.xyz.copy()
        xyz[:3 * box.nw] += rng.normal(scale=sigma, size=(3 * box.nw, 3))
        out.append(WaterBox(box.nw, box.L, xyz, box.vel.copy(), (box.seed, b)))
    return out


def config2(seed=20242):
    """32 path-integral beads of the 256-water box, each with sigma 0.05 A noise."""
    return beads_from(config0(), 32, 0.05, seed)


def config3(seed=20243, nbox=64, sizes=(64, 128, 256, 512, 1024)):
    """Uneven independent boxes: sizes drawn uniformly from ``sizes``, each box seeded
    like the 256-water box at 0.997 g/cm^3 and 298 K."""
    rng = np.random.default_rng(seed)
    nws = rng.choice(np.asarray(sizes), size=nbox)
    return [box_for(int(n), (seed, b)) for b, n in enumerate(nws)]


class BoxSet:
    """Several boxes packed in the multi-box layout: box b's 4*nw_b sites (waters then
    M sites) follow the sites of boxes 0..b-1."""

    def __init__(self, boxes):
        self.boxes = list(boxes)
        self.nw_box = np.array([b.nw for b in self.boxes], dtype=np.int32)
        self.cells = np.ascontiguousarray(np.concatenate([b.cell for b in self.boxes]), dtype=np.float64)
        self.imcon = 1
        self.offsets = np.concatenate([[0], np.cumsum(4 * self.nw_box)]).astype(np.int64)
        self.xyz = np.concatenate([b.xyz for b in self.boxes])
        self.vel = np.concatenate([b.vel for b in self.boxes])
        self.mass = np.concatenate([b.mass for b in self.boxes])

    @property
    def nbox(self):
        return len(self.boxes)

    @property
    def natms(self):
        return int(self.offsets[-1])

    @property
    def nw(self):
        return int(self.nw_box.sum())

    def split(self, a):
        """Per-box views of a per-atom array."""
        return [a[self.offsets[b]:self.offsets[b + 1]] for b in range(self.nbox)]


# Dispersion inputs of a water box: types O = 1, H = 2, M site = 3 (no dispersion) and
# one molecule per water (its M site included).
def water_types(box):
    nw = box.nw
    ltype = np.zeros(box.natms, dtype=np.int32)
    ltype[0:3 * nw:3] = 1
    ltype[1:3 * nw:3] = 2
    ltype[2:3 * nw:3] = 2
    ltype[3 * nw:4 * nw] = 3
    mol = np.concatenate([np.repeat(np.arange(nw), 3), np.arange(nw)]).astype(np.int32)
    return ltype, mol


# Tang-Toennies C6 parameters {C6, a6, C8, a8} per pair type (O-O, H-O, H-H, then the
# M-site pairs, which do not interact), in DL_POLY internal units (10 J/mol, Angstrom).
# The reference reads MB-pol's values from its FIELD file, which it does not ship; these
# are values of the same form and magnitude chosen for the synthetic benchmark and tests.
DISP_PARAMS_SYNTHETIC = np.array([
    [600.0 * 418.4, 3.2, 0.0, 0.0],    # O-O
    [200.0 * 418.4, 3.6, 0.0, 0.0],    # H-O
    [60.0 * 418.4, 3.9, 0.0, 0.0],     # H-H
    [0.0, 0.0, 0.0, 0.0],              # M-O
    [0.0, 0.0, 0.0, 0.0],              # M-H
    [0.0, 0.0, 0.0, 0.0],              # M-M
])


# TTM4-F electrostatics settings of the reference's `vmbpol` keyword
# (SOURCE/simdef_cmd.f:1040-1060): Thole exp-4 damping with athole 0.055 (intermolecular
# and H-H), 0.626 (O-H); charge-charge and charge-dipole smearing 0.4; M-site gamma.
EATD = 4.803239   # Debye per e*Angstrom (SOURCE/module.f90:38)
POLAR_NPRM = 15


def polar_params(alpha=0.3, kmax=(8, 8, 8), rcut=9.0, toler_debye=1e-8, omega=0.3, maxit=22581,
                 athole=0.055, athole12=0.626, athole13=0.055, ascc=0.4, ascd=0.4, gamma=0.426706882, epsq=1.0):
    """Parameter vector of the polar Ewald path: {alpha, rcut, epsq, toler (e A), sor_omega,
    athole, athole12, athole13, ascc, ascd, gamma, kmax1, kmax2, kmax3, maxit}.  toler is the
    CONTROL `iter` value in Debye (SOURCE/simdef_cmd.f:728-740, default 1e-8); omega the SOR
    weight of the old dipole (SOURCE/iter.f:50-51, default 0.3)."""
    k = tuple(int(v) for v in kmax)
    return np.array([alpha, rcut, epsq, toler_debye / EATD, omega, athole, athole12, athole13, ascc, ascd, gamma,
                     k[0], k[1], k[2], maxit], dtype=np.float64)


def kmax_scaled(L, kmax0=8, L0=19.73):
    """kmax that keeps the k-space cutoff 2*pi*kmax/L of the 256-water box (kmax 8 at 19.73 A)."""
    return int(math.ceil(kmax0 * L / L0 - 1e-9))


def polarizabilities(nw):
    """Per-site (polr, polr2): Thole widths and polarizabilities in A^3.  The reference reads
    both from FIELD (`polar`, `polar2` per site, SOURCE/sysdef_cmd.f:466-469), which it does
    not ship; these are MB-pol's published values (O 1.310, H 0.294).  The M site carries no
    dipole (polr2 0) and O's width for the Thole smearing of its charge."""
    polr = np.empty(4 * nw)
    polr2 = np.empty(4 * nw)
    polr[0:3 * nw:3] = 1.310
    polr[1:3 * nw:3] = 0.294
    polr[2:3 * nw:3] = 0.294
    polr[3 * nw:] = 1.310
    polr2[:3 * nw] = polr[:3 * nw]
    polr2[3 * nw:] = 0.0
    return polr, polr2


def polar_params_for(cell, maxit=22581):
    """The server's Ewald settings for a cell (mbx_server_submit_step): rcut = min(9, 0.49 x
    the narrowest width), alpha = 2.7 / rcut, kmax per axis ceil(8 alpha w / (0.3 x 19.73))."""
    a = np.asarray(cell, dtype=np.float64)
    bxc = np.array([a[4] * a[8] - a[5] * a[7], a[5] * a[6] - a[3] * a[8], a[3] * a[7] - a[4] * a[6]])
    cxa = np.array([a[7] * a[2] - a[1] * a[8], a[0] * a[8] - a[2] * a[6], a[1] * a[6] - a[0] * a[7]])
    axb = np.array([a[1] * a[5] - a[2] * a[4], a[2] * a[3] - a[0] * a[5], a[0] * a[4] - a[1] * a[3]])
    v = abs(a[0] * bxc[0] + a[1] * bxc[1] + a[2] * bxc[2])
    w = [v / np.sqrt(bxc @ bxc), v / np.sqrt(cxa @ cxa), v / np.sqrt(axb @ axb)]
    rcut = min(9.0, 0.49 * min(w))
    alpha = 2.7 / rcut
    km = tuple(max(1, int(math.ceil(8.0 * alpha * wi / (0.3 * 19.73) - 1e-9))) for wi in w)
    return polar_params(alpha=alpha, kmax=km, rcut=rcut, toler_debye=1e-8, maxit=maxit)
