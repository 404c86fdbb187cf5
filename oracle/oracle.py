"""ctypes binding of the CPU oracle (test infrastructure; see oracle.h).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
TABLES = os.path.join(REPO, "dlpoly2-mbpol-heat_gb300", "tables")

_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_L = C.POINTER(C.c_long)


def _p(a, t=_D):
    return None if a is None else a.ctypes.data_as(t)


class Oracle:
    def __init__(self, path=None):
        path = path or os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            raise FileNotFoundError("oracle library missing: %s (run make -C oracle)" % path)
        self.lib = C.CDLL(path)
        L = self.lib
        L.orc_load_tables.argtypes = [C.c_char_p, C.c_char_p]
        for f in ("orc_poly2b", "orc_poly3b", "orc_poly2b_naive", "orc_poly3b_naive"):
            getattr(L, f).argtypes = [_D, _D]
            getattr(L, f).restype = C.c_double
        L.orc_2b.argtypes = [_D, _D, _D, _D]
        L.orc_2b.restype = C.c_double
        L.orc_3b.argtypes = [_D, _D, _D, _D, _D, _D]
        L.orc_3b.restype = C.c_double
        L.orc_2b_vars.argtypes = [_D, _D, _D]
        L.orc_3b_vars.argtypes = [_D, _D, _D, _D]
        L.orc_image_monomers.argtypes = [C.c_int, _D, C.c_int, _D]
        L.orc_mbpol_forces.argtypes = [C.c_int, _D, C.c_int, _I] + [_D] * 15 + [C.c_int, C.c_int, _I, C.c_long, _L, _I, C.c_long, _L,
                                       C.c_int]
        L.orc_mbpol_forces.restype = C.c_int
        for f in ("orc_trimer_sample", "orc_dimer_sample"):
            getattr(L, f).argtypes = [C.c_int, _D, C.c_int, _D, _I, C.c_long, C.c_int]
            getattr(L, f).restype = C.c_double
        L.orc_mbpol_ranks.argtypes = [C.c_int, _D, C.c_int, _I, _D, _D, _D, C.c_int, C.c_int, C.c_int, C.c_int,
                                      C.c_int]
        L.orc_mbpol_ranks.restype = C.c_double
        L.orc_pes_load.argtypes = [C.c_char_p]
        L.orc_ps_couple.argtypes = [C.c_double] * 9 + [_D, _D, _D]
        L.orc_angfrc_ps.argtypes = [C.c_int, _D, C.c_int, _I] + [_D] * 14
        L.orc_dms_load.argtypes = [C.c_char_p]
        L.orc_msites.argtypes = [C.c_int, _D, C.c_int, _I, _D, _D, _D, C.c_double]
        L.orc_qdetermine.argtypes = [C.c_int, _D, C.c_int, _I, _D, _D, _D, C.c_double, _D, _D]
        L.orc_qdetermine.restype = C.c_double
        L.orc_tang_toennies.argtypes = [C.c_int, C.c_double]
        L.orc_tang_toennies.restype = C.c_double
        L.orc_tang_toennies_lr.argtypes = [C.c_int, C.c_double]
        L.orc_tang_toennies_lr.restype = C.c_double
        L.orc_disp_tables.argtypes = [C.c_int, _D, C.c_int, C.c_double, _D, _D]
        L.orc_dispersion.argtypes = [C.c_int, _D, C.c_int, _I, _I, C.c_int, _D, C.c_double, C.c_int] + [_D] * 14
        L.orc_dispersion.restype = C.c_long
        L.orc_disp_lrc.argtypes = [C.c_int, _D, _I, C.c_double, C.c_double, _D, _D]
        L.orc_polar.argtypes = [_D, C.c_int, _D, C.c_int] + [_D] * 20 + [C.c_int]
        L.orc_induced_error.argtypes = [_D, C.c_int, _D, C.c_int] + [_D] * 11
        L.orc_induced_error.restype = None
        for f in ("orc_erfcc", "orc_gammln"):
            getattr(L, f).argtypes = [C.c_double]
            getattr(L, f).restype = C.c_double
        L.orc_gammq.argtypes = [C.c_double, C.c_double]
        L.orc_gammq.restype = C.c_double
        if L.orc_dms_load(os.path.join(TABLES, "ps_dms.tbl").encode()):
            raise RuntimeError("orc_dms_load failed")
        if L.orc_pes_load(os.path.join(TABLES, "ps_pes.tbl").encode()):
            raise RuntimeError("orc_pes_load failed")
        rc = L.orc_load_tables(os.path.join(TABLES, "poly2b.tbl").encode(),
                               os.path.join(TABLES, "poly3b.tbl").encode())
        if rc:
            raise RuntimeError("orc_load_tables failed: %d" % rc)

    # -- polynomials / models -------------------------------------------------
    def poly(self, body, x, naive=False):
        x = np.ascontiguousarray(x, dtype=np.float64)
        g = np.zeros_like(x)
        f = getattr(self.lib, "orc_poly%s%s" % (body, "_naive" if naive else ""))
        return f(_p(x), _p(g)), g

    def model2b(self, w1, w2):
        w1 = np.ascontiguousarray(w1, np.float64)
        w2 = np.ascontiguousarray(w2, np.float64)
        g1 = np.zeros(9)
        g2 = np.zeros(9)
        e = self.lib.orc_2b(_p(w1), _p(w2), _p(g1), _p(g2))
        return e, g1, g2

    def model3b(self, w1, w2, w3):
        w = [np.ascontiguousarray(v, np.float64) for v in (w1, w2, w3)]
        g = [np.zeros(9) for _ in range(3)]
        e = self.lib.orc_3b(_p(w[0]), _p(w[1]), _p(w[2]), _p(g[0]), _p(g[1]), _p(g[2]))
        return e, g[0], g[1], g[2]

    def vars2b(self, w1, w2):
        v = np.zeros(31)
        self.lib.orc_2b_vars(_p(np.ascontiguousarray(w1, np.float64)), _p(np.ascontiguousarray(w2, np.float64)),
                             _p(v))
        return v

    def vars3b(self, w1, w2, w3):
        v = np.zeros(36)
        w = [np.ascontiguousarray(u, np.float64) for u in (w1, w2, w3)]
        self.lib.orc_3b_vars(_p(w[0]), _p(w[1]), _p(w[2]), _p(v))
        return v

    # -- driver ---------------------------------------------------------------
    def mbpol_forces(self, box, dense=False, velocities=True, lists=False, nthreads=1):
        """mbpol_forces + heat bookkeeping on a WaterBox; returns a dict."""
        n = box.natms
        x = np.ascontiguousarray(box.xyz[:, 0])
        y = np.ascontiguousarray(box.xyz[:, 1])
        z = np.ascontiguousarray(box.xyz[:, 2])
        f = np.zeros((3, n))
        ae = np.zeros(n)
        e2 = C.c_double(0)
        e3 = C.c_double(0)
        vir = C.c_double(0)
        stress = np.zeros(9)
        jpot = np.zeros(3)
        v = [np.ascontiguousarray(box.vel[:, k]) for k in range(3)] if velocities else [None] * 3
        lst = box.listttm2()
        nw = box.nw
        cap_p = nw * 80 if lists else 0
        cap_t = nw * 400 if lists else 0
        pairs = np.zeros(2 * max(cap_p, 1), np.int32) if lists else None
        trip = np.zeros(3 * max(cap_t, 1), np.int32) if lists else None
        npairs = C.c_long(0)
        ntrip = C.c_long(0)
        rc = self.lib.orc_mbpol_forces(box.imcon, _p(box.cell), nw, _p(lst, _I), _p(x), _p(y), _p(z),
                                       _p(f[0]), _p(f[1]), _p(f[2]), C.byref(e2), C.byref(e3), C.byref(vir),
                                       _p(stress), _p(ae), _p(v[0]), _p(v[1]), _p(v[2]), _p(jpot),
                                       1 if dense else 0, n, _p(pairs, _I), cap_p, C.byref(npairs),
                                       _p(trip, _I), cap_t, C.byref(ntrip), nthreads)
        if rc:
            raise RuntimeError("orc_mbpol_forces: list capacity exceeded")
        out = dict(eng2=e2.value, eng3=e3.value, vir=vir.value, stress=stress, forces=f.T.copy(),
                   atomic_energy=ae, jpot=jpot, npairs=npairs.value, ntrip=ntrip.value)
        if lists:
            out["pairs"] = pairs[:2 * npairs.value].reshape(-1, 2).copy()
            out["trimers"] = trip[:3 * ntrip.value].reshape(-1, 3).copy()
        if velocities:
            m = box.mass
            vel = box.vel
            kin = 0.5 * m * (vel * vel).sum(1)
            eng = kin[:3 * nw] + ae[:3 * nw]
            out["jkin"] = (eng[:, None] * vel[:3 * nw]).sum(0)
        return out

    def sample(self, body, box, monomers, lst, nthreads):
        lst = np.ascontiguousarray(lst, dtype=np.int32)
        f = self.lib.orc_trimer_sample if body == 3 else self.lib.orc_dimer_sample
        n = lst.shape[0]
        return f(box.imcon, _p(box.cell), box.nw, _p(np.ascontiguousarray(monomers, np.float64)),
                 _p(lst, _I), n, nthreads)

    def ranks(self, box, rank_begin, rank_end, size, nthreads):
        """Energy of ranks [rank_begin, rank_end) of a `size`-rank split (CPU baseline work)."""
        x, y, z = (np.ascontiguousarray(box.xyz[:, k]) for k in range(3))
        lst = np.ascontiguousarray(box.listttm2(), dtype=np.int32)
        return self.lib.orc_mbpol_ranks(box.imcon, _p(box.cell), box.nw, _p(lst, _I), _p(x), _p(y), _p(z),
                                        box.natms, rank_begin, rank_end, size, nthreads)

    def angfrc_ps(self, box, velocities=True):
        """angfrc (keya 9) over the box's H-O-H angles with the heat hooks."""
        n = box.natms
        x, y, z = (np.ascontiguousarray(box.xyz[:, k]) for k in range(3))
        f = np.zeros((3, n))
        eng = C.c_double(0)
        vir = C.c_double(0)
        stress = np.zeros(9)
        ae = np.zeros(n)
        jpot = np.zeros(3)
        v = [np.ascontiguousarray(box.vel[:, k]) for k in range(3)] if velocities else [None] * 3
        lst = np.ascontiguousarray(box.listang(), dtype=np.int32)
        self.lib.orc_angfrc_ps(box.imcon, _p(box.cell), box.nw, _p(lst, _I), _p(x), _p(y), _p(z), _p(f[0]),
                               _p(f[1]), _p(f[2]), C.byref(eng), C.byref(vir), _p(stress), _p(ae), _p(v[0]),
                               _p(v[1]), _p(v[2]), _p(jpot))
        return dict(engang=eng.value, virang=vir.value, stress=stress, forces=f.T.copy(), atomic_energy=ae,
                    jpot=jpot)

    def msites_dms(self, box, gamma=0.426706882):
        """M-site positions and DMS charges; returns (xyz with M sites, chge, dp[nw,6], worst |sum q|)."""
        x, y, z = (np.ascontiguousarray(box.xyz[:, k]).copy() for k in range(3))
        lst = np.ascontiguousarray(box.listttm2(), dtype=np.int32)
        self.lib.orc_msites(box.imcon, _p(box.cell), box.nw, _p(lst, _I), _p(x), _p(y), _p(z), gamma)
        chge = np.zeros(box.natms)
        dp = np.zeros((box.nw, 6))
        worst = self.lib.orc_qdetermine(box.imcon, _p(box.cell), box.nw, _p(lst, _I), _p(x), _p(y), _p(z), gamma,
                                        _p(chge), _p(dp))
        return np.stack([x, y, z], 1), chge, dp, worst

    def dispersion(self, box, ltype, mol, prm, rcut=9.0, mxgrid=0, velocities=True):
        """srfrce2 with type-12 tables over every intermolecular pair within rcut."""
        n = box.natms
        x, y, z = (np.ascontiguousarray(box.xyz[:, k]) for k in range(3))
        f = np.zeros((3, n))
        eng = C.c_double(0)
        vir = C.c_double(0)
        stress = np.zeros(9)
        ae = np.zeros(n)
        jpot = np.zeros(3)
        v = [np.ascontiguousarray(box.vel[:, k]) for k in range(3)] if velocities else [None] * 3
        prm = np.ascontiguousarray(prm, dtype=np.float64).reshape(-1, 4)
        nt = int(round((np.sqrt(8 * prm.shape[0] + 1) - 1) / 2))
        mxgrid = mxgrid or max(1000, int(rcut / 0.0001 + 0.5) + 4)
        lt = np.ascontiguousarray(ltype, dtype=np.int32)
        mo = np.ascontiguousarray(mol, dtype=np.int32)
        npairs = self.lib.orc_dispersion(box.imcon, _p(box.cell), n, _p(lt, _I), _p(mo, _I), nt, _p(prm.ravel().copy()),
                                         rcut, mxgrid, _p(x), _p(y), _p(z), _p(f[0]), _p(f[1]), _p(f[2]),
                                         C.byref(eng), C.byref(vir), _p(stress), _p(ae), _p(v[0]), _p(v[1]),
                                         _p(v[2]), _p(jpot))
        return dict(eng=eng.value, vir=vir.value, stress=stress, forces=f.T.copy(), atomic_energy=ae, jpot=jpot,
                    npairs=npairs)

    def disp_lrc(self, prm, numtyp, rcut, volm):
        prm = np.ascontiguousarray(prm, dtype=np.float64).reshape(-1, 4)
        nt = int(round((np.sqrt(8 * prm.shape[0] + 1) - 1) / 2))
        e = C.c_double(0)
        v = C.c_double(0)
        self.lib.orc_disp_lrc(nt, _p(prm.ravel().copy()), _p(np.ascontiguousarray(numtyp, dtype=np.int32), _I), rcut,
                              volm, C.byref(e), C.byref(v))
        return e.value, v.value

    def polar(self, sites, cell, imcon, nw, chge, dp, polr, polr2, prm, dip0=None, vel=None, dense=False):
        """TTM4-F electrostatics (orc_polar) on 4*nw sites.  Returns a dict with site forces,
        energies, virial, stress, dipoles, per-site energies, jpot/jkin and the iteration count."""
        n = 4 * nw
        x, y, z = (np.ascontiguousarray(sites[:, k], dtype=np.float64) for k in range(3))
        dip = np.zeros((3, n)) if dip0 is None else np.ascontiguousarray(np.asarray(dip0, np.float64).T).copy()
        f = np.zeros((3, n))
        out = np.zeros(16)
        ae = np.zeros(n)
        jpot = np.zeros(3)
        jkin = np.zeros(3)
        v = [np.ascontiguousarray(vel[:, k], dtype=np.float64) for k in range(3)] if vel is not None else [None] * 3
        rc = self.lib.orc_polar(_p(np.ascontiguousarray(prm, np.float64)), imcon, _p(np.ascontiguousarray(cell, np.float64)),
                                nw, _p(x), _p(y), _p(z), _p(np.ascontiguousarray(chge, np.float64)),
                                _p(np.ascontiguousarray(dp, np.float64)), _p(np.ascontiguousarray(polr, np.float64)),
                                _p(np.ascontiguousarray(polr2, np.float64)), _p(dip[0]), _p(dip[1]), _p(dip[2]),
                                _p(f[0]), _p(f[1]), _p(f[2]), _p(out), _p(ae), _p(v[0]), _p(v[1]), _p(v[2]),
                                _p(jpot), _p(jkin), int(dense))
        return dict(status=rc, forces=f.T.copy(), engcpe=out[0], vircpe=out[1], stress=out[2:11].copy(),
                    iterations=int(out[11]), deltadip=out[12], eng_polar=out[13], eng_kspace=out[14],
                    eng_real=out[15], dipoles=dip.T.copy(), atomic_energy=ae, jpot=jpot, jkin=jkin)

    def induced_error(self, sites, cell, imcon, nw, chge, dp, polr, polr2, prm, dipoles):
        """induced_error (SOURCE/induced_error.f90) of the given dipoles (sites x 3) under the
        oracle's fields: (L2 norm, largest component) of mu - polr2 E(mu) / r4pie0."""
        x, y, z = (np.ascontiguousarray(sites[:, k], dtype=np.float64) for k in range(3))
        d = [np.ascontiguousarray(np.asarray(dipoles, np.float64)[:, k]) for k in range(3)]
        r = np.zeros(2)
        self.lib.orc_induced_error(_p(np.ascontiguousarray(prm, np.float64)), imcon,
                                   _p(np.ascontiguousarray(cell, np.float64)), nw, _p(x), _p(y), _p(z),
                                   _p(np.ascontiguousarray(chge, np.float64)), _p(np.ascontiguousarray(dp, np.float64)),
                                   _p(np.ascontiguousarray(polr, np.float64)), _p(np.ascontiguousarray(polr2, np.float64)),
                                   _p(d[0]), _p(d[1]), _p(d[2]), _p(r))
        return float(r[0]), float(r[1])

    def image_monomers(self, box):
        m = box.monomers().copy()
        self.lib.orc_image_monomers(box.imcon, _p(box.cell), box.nw, _p(m))
        return m


def aspc_coefficients(k):
    """Kolafa's ASPC predictor coefficients B_1..B_{k+2}, built as aspc_init builds them
    (SOURCE/aspc.f90:106-114): B_j = (-1)^(j+1) j (4k+6)/(k+3) prod_{m<j} (k+2-m)/(k+3+m)."""
    rk = float(k)
    t = 1.0 / (rk + 3.0)
    out = []
    for j in range(1, k + 3):
        out.append((1.0 if j % 2 else -1.0) * j * (4.0 * rk + 6.0) * t)
        t = t * (rk + 2.0 - j) / (rk + 3.0 + j)
    return out


class AspcDriver:
    """The reference's ASPC step sequence around the dipole solve: aspc_predict before
    forces and aspc_set after it (SOURCE/dlpoly_cmd.f:2273-2320, SOURCE/aspc.f90:118-251),
    with the loop branch of SOURCE/forces.f:334-366 (SOR weight 0.3 for steps below 5; one
    iteration, marked converged, after iter_nstep steps)."""

    def __init__(self, k, iter_nstep):
        self.k, self.niter = int(k), int(iter_nstep)
        self.B = aspc_coefficients(self.k)
        self.hist = None     # k+2 dipole arrays, newest first (zeros after aspc_init)
        self.step_count = 0  # nstep_for_guess

    def step(self, orc, sites, cell, imcon, nw, chge, dp, polr, polr2, prm, dip0=None, vel=None):
        n = 4 * nw
        if self.hist is None:
            self.hist = [np.zeros((n, 3)) for _ in range(self.k + 2)]
        self.step_count += 1
        dip = np.zeros((n, 3)) if dip0 is None else np.array(dip0, np.float64)
        if self.step_count > self.niter:
            dip = self.B[0] * self.hist[0]
            for b, h in zip(self.B[1:], self.hist[1:]):
                dip = dip + b * h
        p = np.array(prm, np.float64).copy()
        if self.step_count < 5:
            p[4] = 0.3
        if self.step_count > self.niter:
            p[14] = 0            # one iteration; the oracle then reports status 1
        res = orc.polar(sites, cell, imcon, nw, chge, dp, polr, polr2, p, dip0=dip, vel=vel)
        self.hist.insert(0, res["dipoles"].copy())
        del self.hist[self.k + 2:]
        return res


def load(path=None):
    return Oracle(path)
