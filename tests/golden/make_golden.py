"""Generate golden vectors for the MB-pol 2B/3B models from the REFERENCE's own C++.

The reference's polynomial sources (SOURCE/mbpol-2b-poly.cpp, poly-2b-v6x.cpp,
mbpol-3b-poly.cpp, poly-3b-v2x.cpp) are compiled from the reference tree by
``make -C oracle ref REFSRC=<the reference SOURCE directory>`` (the build recipe
``__graft_entry__.build()`` does this when the reference tree is mounted) into
oracle/_ref/libmbpol_ref.so; this script calls their
exported C entry points ``mbpol_2b_poly_`` / ``mbpol_3b_poly_``
(SOURCE/mbpol-2b-poly.cpp:1888, SOURCE/mbpol-3b-poly.cpp:1526) on seeded water
dimers and trimers and stores inputs and outputs in ``mbpol_models.npz``.

Geometries come from seeded synthetic water boxes: every dimer/trimer sample is a
pair/triple of molecules imaged next to each other, spanning the 2B switching
region (4.5-6.5 A), beyond the 2B cutoff, and all 3B switching regimes.

Run here (the reference tree is present):  python tests/golden/make_golden.py
"""
import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "dlpoly2-mbpol-heat_gb300"))
from mbx import systems  # noqa: E402

_D = C.POINTER(C.c_double)


def _img(d, L):
    return d - L * np.round(d / L)


def _clusters(seed, n2, n3):
    rng = np.random.default_rng(seed)
    dimers, trimers = [], []
    boxes = [systems.config0(seed=seed + k) for k in range(4)] + [systems.box_for(64, seed + 11)]
    for box in boxes:
        m = box.monomers().copy()
        # H next to O
        for h in (3, 6):
            m[:, h:h + 3] = m[:, 0:3] + _img(m[:, h:h + 3] - m[:, 0:3], box.L)
        nw = box.nw
        d = _img(m[:, None, 0:3] - m[None, :, 0:3], box.L)
        r = np.sqrt((d * d).sum(-1))
        iu = np.argwhere(np.triu(r < 7.2, 1))
        pick = rng.choice(len(iu), size=min(n2 // len(boxes), len(iu)), replace=False)
        for i, j in iu[pick]:
            w1 = m[i].copy()
            w2 = m[j].copy()
            sh = (w2[0:3] + _img(w1[0:3] - w2[0:3], box.L)) - w1[0:3]
            w1 += np.tile(sh, 3)
            dimers.append((w1, w2))
        count = 0
        tries = 0
        while count < n3 // len(boxes) and tries < 100000:
            tries += 1
            c = rng.integers(nw)
            nb = np.where((r[c] < 5.0) & (np.arange(nw) != c))[0]
            if len(nb) < 2:
                continue
            a, b = rng.choice(nb, 2, replace=False)
            ws = []
            for k in (a, c, b):
                w = m[k].copy()
                sh = (m[c][0:3] + _img(w[0:3] - m[c][0:3], box.L)) - w[0:3]
                ws.append(w + np.tile(sh, 3))
            trimers.append(tuple(ws))
            count += 1
    return dimers, trimers


def main():
    lib = C.CDLL(os.path.join(REPO, "oracle", "_ref", "libmbpol_ref.so"))
    lib.mbpol_2b_poly_.argtypes = [_D] * 6
    lib.mbpol_3b_poly_.argtypes = [_D] * 8
    dimers, trimers = _clusters(20240, 240, 240)
    W2 = np.array([np.stack(d) for d in dimers])          # (n, 2, 9)
    W3 = np.array([np.stack(t) for t in trimers])         # (n, 3, 9)
    E2 = np.zeros(len(W2))
    G2 = np.zeros((len(W2), 2, 9))
    F2 = np.zeros((len(W2), 108))
    for k in range(len(W2)):
        w1 = np.ascontiguousarray(W2[k, 0])
        w2 = np.ascontiguousarray(W2[k, 1])
        e = C.c_double(0)
        g1 = np.full(9, np.nan)
        g2 = np.full(9, np.nan)
        fm = np.zeros(108)
        lib.mbpol_2b_poly_(w1.ctypes.data_as(_D), w2.ctypes.data_as(_D), C.byref(e), g1.ctypes.data_as(_D),
                           g2.ctypes.data_as(_D), fm.ctypes.data_as(_D))
        E2[k] = e.value
        # the reference leaves g untouched beyond the cutoff: record zeros there.  Its 2B
        # force matrix takes the 6 diagonal entries from an uninitialised local array
        # (SOURCE/mbpol-2b-poly.cpp:454, :627-634); its HEAT_STRESS reader skips them
        # (SOURCE/mbpol.f90:551-553), and so do the tests
        G2[k, 0] = np.nan_to_num(g1)
        G2[k, 1] = np.nan_to_num(g2)
        F2[k] = fm
    E3 = np.zeros(len(W3))
    G3 = np.zeros((len(W3), 3, 9))
    F3 = np.zeros((len(W3), 243))
    for k in range(len(W3)):
        w = [np.ascontiguousarray(W3[k, q]) for q in range(3)]
        e = C.c_double(0)
        g = [np.zeros(9) for _ in range(3)]
        fm = np.zeros(243)
        lib.mbpol_3b_poly_(*(v.ctypes.data_as(_D) for v in w), C.byref(e), *(v.ctypes.data_as(_D) for v in g),
                           fm.ctypes.data_as(_D))
        E3[k] = e.value
        G3[k] = np.stack(g)
        F3[k] = fm
    # raw polynomial probes: variables drawn in the physical range (0, 1.5]
    rng = np.random.default_rng(7)
    X2 = rng.uniform(0.01, 1.5, size=(16, 31))
    X3 = rng.uniform(0.01, 1.5, size=(16, 36))
    # the generated evaluators themselves (x2o::poly_2b_v6x::eval, x2o::poly_3b_v2x::eval)
    # with the model's coefficient arrays, read from the tables' C lines
    P = {}
    for body, X, sym, nv in (("2b", X2, "_ZN3x2o11poly_2b_v6x4evalEPKdS2_Pd", 31),
                             ("3b", X3, "_ZN3x2o11poly_3b_v2x4evalEPKdS2_Pd", 36)):
        f = getattr(lib, sym)
        f.argtypes = [_D, _D, _D]
        f.restype = C.c_double
        coef = []
        with open(os.path.join(REPO, "dlpoly2-mbpol-heat_gb300", "tables", "poly%s.tbl" % body)) as fh:
            for line in fh:
                if line[0] == "C":
                    coef.append(float(line.split()[2]))
        a = np.array(coef)
        PE = np.zeros(len(X))
        PG = np.zeros((len(X), nv))
        for k in range(len(X)):
            x = np.ascontiguousarray(X[k])
            g = np.zeros(nv)
            PE[k] = f(a.ctypes.data_as(_D), x.ctypes.data_as(_D), g.ctypes.data_as(_D))
            PG[k] = g
        P["PE" + body] = PE
        P["PG" + body] = PG
    np.savez_compressed(os.path.join(HERE, "mbpol_models.npz"), W2=W2, E2=E2, G2=G2, FM2=F2, W3=W3, E3=E3, G3=G3, FM3=F3,
                        X2=X2, X3=X3, **P)
    print("dimers %d (nonzero %d), trimers %d (nonzero %d)" % (len(W2), (E2 != 0).sum(), len(W3), (E3 != 0).sum()))


if __name__ == "__main__":
    main()
