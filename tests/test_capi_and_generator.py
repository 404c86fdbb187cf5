"""libmbx.so loads and exports every declared symbol; the PTX generator covers the tables."""
import os
import sys

import numpy as np
import pytest

from conftest import PKG


def test_library_exports_every_header_symbol():
    from mbx import capi
    lib = capi.load()
    names = capi.header_functions()
    assert "mbx_mbpol_forces" in names and "mbpol_2b_poly_" in names
    for n in names:
        assert getattr(lib, n) is not None


def test_no_cpu_fallback_without_library(tmp_path):
    from mbx import capi
    with pytest.raises(capi.MbxError):
        capi.load(str(tmp_path / "missing.so"))


def _interpret(root, x):
    """Run the depth-first trie scheme of the generated kernels in Python."""
    g = np.zeros(len(x))

    def walk(node, pi):
        S = 0.0 if node.k is None else A[node.k]
        for j in sorted(node.ch):
            ch = node.ch[j]
            if not ch.ch:
                S += x[j] * A[ch.k]
                g[j] += pi * A[ch.k]
            else:
                Sc = walk(ch, pi * x[j])
                S += x[j] * Sc
                g[j] += pi * Sc
        return S

    return walk(root, 1.0), g


def test_trie_scheme_matches_reference_polynomial(golden):
    sys.path.insert(0, os.path.join(PKG, "gen"))
    import gen_poly_ptx
    global A
    for body in ("2b", "3b"):
        nv, coef, monos = gen_poly_ptx.read_table(os.path.join(PKG, "tables", "poly%s.tbl" % body))
        A = coef
        root = gen_poly_ptx.build_trie(monos)
        x = golden["X" + body[0]][0]
        e, g = _interpret(root, x)
        assert abs(e - golden["PE" + body][0]) <= 1e-12 * abs(e)
        assert np.max(np.abs(g - golden["PG" + body][0])) <= 1e-12 * np.max(np.abs(g))
        # the chunks partition the root's children
        for n in (2, 6, 12):
            chunks = gen_poly_ptx.split_root(root, n)
            flat = sorted(v for c in chunks for v in c)
            assert flat == sorted(root.ch)


def test_generated_ptx_declares_all_chunks(tmp_path):
    sys.path.insert(0, os.path.join(PKG, "gen"))
    import gen_poly_ptx
    paths = gen_poly_ptx.generate(os.path.join(PKG, "tables"), str(tmp_path))
    hdr = open(tmp_path / "mbx_poly_gen.cuh").read()
    for p in paths:
        name = os.path.basename(p)[:-4]
        if name != "mbx_poly_coef":
            assert name in hdr
            assert ".visible .func %s(" % name in open(p).read()


def test_group_form_of_3b_polynomial_matches_reference(golden):
    """The looped FP32 3B function evaluates E(x) = sum over the 48 trimer relabellings
    of a representative polynomial f.  In exact arithmetic (FP64 here) the sum equals
    the reference polynomial and its gradient at the golden points and at shifted
    variables (the kernels evaluate the shifted re-expansion)."""
    sys.path.insert(0, os.path.join(PKG, "gen"))
    import gen_poly_ptx as g
    global A
    nv, coef, monos = g.read_table(os.path.join(PKG, "tables", "poly3b.tbl"))
    G = g.group_3b()
    assert len(G) == 48 and G[0] == list(range(nv)) and len({tuple(p) for p in G}) == 48
    full = {tuple(sorted(m)): coef[k] for k, m in monos}
    reps = g.group_reduce(full, G)
    assert len(reps) == len(coef)          # one representative per coefficient class
    A = [c for _, c in reps]
    root = g.build_trie([(i, m) for i, (m, _) in enumerate(reps)])
    x = golden["X3"][0]
    e, grad = 0.0, np.zeros(nv)
    for p in G:
        ep, gp = _interpret(root, x[p])
        e += ep
        np.add.at(grad, p, gp)
    assert abs(e - golden["PE3b"][0]) <= 1e-10 * abs(e)
    assert np.max(np.abs(grad - golden["PG3b"][0])) <= 1e-10 * np.max(np.abs(grad))
    # the shifted re-expansion is invariant too (class-wise centres)
    sp = g.shifted_polynomial(monos, coef, g.shift_centres("3b"))
    sp.pop((), None)
    assert len(g.group_reduce({tuple(sorted(m)): c for m, c in sp.items()}, G)) > 0
