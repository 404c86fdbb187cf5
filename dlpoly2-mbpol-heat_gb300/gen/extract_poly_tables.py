"""Extract the MB-pol 2B/3B permutationally invariant polynomials as monomial tables.

The reference ships each polynomial only as machine-generated straight-line code
(``poly_2b_v6x::eval`` in SOURCE/poly-2b-v6x.cpp:5 and ``poly_3b_v2x::eval`` in
SOURCE/poly-3b-v2x.cpp:5).  That code is a nested (Horner-like) factorisation of

    E(x) = sum_k a[k] * P_k(x),      P_k = sum of monomials of one symmetry orbit,

built from three operations only: ``+``, ``*`` and the literal ``2.0``.  This
script expands the returned energy expression symbolically into its monomials,
checks that every monomial has multiplier 1 and belongs to exactly one
coefficient, and writes a plain-text table:

    C <k> <a[k] as repr(float)>          one line per coefficient
    M <k> <v1> [<v2> ...]                one line per monomial (sorted variable indices)

The coefficient values come from ``the_poly[]`` in SOURCE/mbpol-2b-poly.cpp:685
and SOURCE/mbpol-3b-poly.cpp:316.  The tables are the model's parameters (data),
committed so that builds need nothing from the reference tree.

Usage: python extract_poly_tables.py <reference SOURCE dir> <output dir>
"""
import os
import re
import sys
from collections import defaultdict

_TOKEN = re.compile(r"t\d+|a\[\d+\]|x\[\d+\]|\d+\.\d*|[+*()]")


def _expand(src_text):
    """Expand the returned expression of a generated ``eval`` into {(k, monomial): mult}."""
    body = src_text[src_text.index("{", src_text.index("::eval")) + 1:]
    defs = {n: e.replace("\n", "").replace(" ", "")
            for n, e in re.findall(r"const double (t\d+) = ([^;]*);", body, re.S)}
    ret = re.search(r"return ([^;]*);", body).group(1).replace("\n", "").replace(" ", "")
    memo = {}

    def mul(p, q):
        r = defaultdict(float)
        for (ka, ma), ca in p.items():
            for (kb, mb), cb in q.items():
                if ka >= 0 and kb >= 0:
                    raise ValueError("expression is not linear in the coefficients")
                r[(max(ka, kb), tuple(sorted(ma + mb)))] += ca * cb
        return dict(r)

    def add(p, q):
        r = dict(p)
        for key, c in q.items():
            r[key] = r.get(key, 0.0) + c
        return r

    def parse(s):
        toks = _TOKEN.findall(s)
        pos = [0]

        def expr():
            v = term()
            while pos[0] < len(toks) and toks[pos[0]] == "+":
                pos[0] += 1
                v = add(v, term())
            return v

        def term():
            v = atom()
            while pos[0] < len(toks) and toks[pos[0]] == "*":
                pos[0] += 1
                v = mul(v, atom())
            return v

        def atom():
            t = toks[pos[0]]
            pos[0] += 1
            if t == "(":
                v = expr()
                if toks[pos[0]] != ")":
                    raise ValueError("unbalanced parentheses")
                pos[0] += 1
                return v
            if t[0] == "t":
                if t not in memo:
                    memo[t] = parse(defs[t])
                return memo[t]
            if t[0] == "a":
                return {(int(t[2:-1]), ()): 1.0}
            if t[0] == "x":
                return {(-1, (int(t[2:-1]),)): 1.0}
            return {(-1, ()): float(t)}

        v = expr()
        if pos[0] != len(toks):
            raise ValueError("trailing tokens")
        return v

    sys.setrecursionlimit(100000)
    return parse(ret)


def _coefficients(model_text):
    block = re.search(r"the_poly\[\]\s*=\s*\{(.*?)\};", model_text, re.S).group(1)
    vals = []
    for line in block.split("\n"):
        line = line.split("//")[0].strip().rstrip(",")
        if line:
            vals.append(float(line))
    return vals


def extract(poly_cpp, model_cpp, n_vars, n_coef, out_path, title):
    with open(poly_cpp) as f:
        expanded = _expand(f.read())
    with open(model_cpp) as f:
        coef = _coefficients(f.read())
    if len(coef) != n_coef:
        raise ValueError("coefficient count %d != %d" % (len(coef), n_coef))
    seen = set()
    monos = []
    for (k, m), mult in expanded.items():
        if k < 0 or mult != 1.0 or not m:
            raise ValueError("unexpected term %r" % ((k, m, mult),))
        if any(v >= n_vars for v in m) or m in seen:
            raise ValueError("bad or duplicated monomial %r" % (m,))
        seen.add(m)
        monos.append((k, m))
    if set(k for k, _ in monos) != set(range(n_coef)):
        raise ValueError("some coefficient has no monomial")
    monos.sort()
    with open(out_path, "w") as f:
        f.write("# %s\n# n_vars %d n_coef %d n_mono %d\n" % (title, n_vars, n_coef, len(monos)))
        for k, c in enumerate(coef):
            f.write("C %d %r\n" % (k, c))
        for k, m in monos:
            f.write("M %d %s\n" % (k, " ".join(str(v) for v in m)))
    return len(monos)


def fortran_arrays(module_f90, module_name, names):
    """Values of the initialised arrays `names` inside `module <module_name>` of a
    Fortran source (array constructors (/ ... /), D exponents)."""
    with open(module_f90) as f:
        text = f.read()
    start = text.index("module %s" % module_name)
    end = text.index("end module %s" % module_name, start)
    body = text[start:end]
    out = {}
    for name in names:
        m = re.search(r"::\s*%s\s*\(\s*1\s*:\s*(\d+)\s*\)\s*=\s*\(/(.*?)/\)" % name, body, re.S)
        if not m:
            m = re.search(r"::\s*%s\s*\(\s*(\d+)\s*\)\s*=\s*\(/(.*?)/\)" % name, body, re.S)
        n = int(m.group(1))
        raw = m.group(2).replace("&", " ").replace("\n", " ")
        vals = [v.strip() for v in raw.split(",") if v.strip()]
        if len(vals) != n:
            raise ValueError("%s: %d values, expected %d" % (name, len(vals), n))
        out[name] = [v.replace("D", "E").replace("d", "e") for v in vals]
    return out


def write_arrays(path, title, arrays):
    with open(path, "w") as f:
        f.write("# %s\n" % title)
        for name, vals in arrays.items():
            f.write("%s %d %s\n" % (name, len(vals), " ".join(vals)))


def main():
    src, out = sys.argv[1], sys.argv[2]
    os.makedirs(out, exist_ok=True)
    n2 = extract(os.path.join(src, "poly-2b-v6x.cpp"), os.path.join(src, "mbpol-2b-poly.cpp"),
                 31, 1153, os.path.join(out, "poly2b.tbl"),
                 "MB-pol 2B polynomial x2b_v6x (SOURCE/poly-2b-v6x.cpp, SOURCE/mbpol-2b-poly.cpp)")
    n3 = extract(os.path.join(src, "poly-3b-v2x.cpp"), os.path.join(src, "mbpol-3b-poly.cpp"),
                 36, 1163, os.path.join(out, "poly3b.tbl"),
                 "MB-pol 3B polynomial x3b_v2x (SOURCE/poly-3b-v2x.cpp, SOURCE/mbpol-3b-poly.cpp)")
    print("2B monomials %d, 3B monomials %d" % (n2, n3))
    # 1-body Partridge-Schwenke PES (module ps_type_pes, SOURCE/module.f90:49-604)
    pes = fortran_arrays(os.path.join(src, "module.f90"), "ps_type_pes",
                         ["idx1", "idx2", "idx3", "c5z", "cbasis", "ccore", "crest", "cmass0",
                          "idxm1", "idxm2", "idxm3"])
    write_arrays(os.path.join(out, "ps_pes.tbl"),
                 "Partridge-Schwenke 1-body PES expansion (module ps_type_pes, SOURCE/module.f90:49-604)", pes)
    # Partridge-Schwenke dipole-moment surface (module ps_type_dms, SOURCE/module.f90:745-918)
    dms = fortran_arrays(os.path.join(src, "module.f90"), "ps_type_dms", ["idx1", "idx2", "idx3", "coef"])
    write_arrays(os.path.join(out, "ps_dms.tbl"),
                 "Partridge-Schwenke dipole-moment surface (module ps_type_dms, SOURCE/module.f90:745-918)", dms)


if __name__ == "__main__":
    main()
