"""Generate the MB-pol polynomial kernels as PTX (value + gradient).

Input: a monomial table written by extract_poly_tables.py (E(x) = sum over
monomials of a[k] * prod x[v]).  Output: one PTX module per chunk, each with one
relocatable device function  f(const T* x, T* acc)  that adds its share of
[E, dE/dx_0 .. dE/dx_{nv-1}] into acc, plus a module holding the coefficient
arrays and a C++ header declaring the functions.  The functions are linked into
the fused per-cluster kernels (relocatable device code), so a whole cluster
evaluation -- variables, polynomial, chain rule, accumulation -- is one launch.

Evaluation scheme.  The monomials (sorted variable-index tuples) form a prefix
tree.  Walking it depth first, a node p carries the product pi_p of the variables
on its path (its adjoint) and returns S_p, the sum of its subtree divided by pi_p:

    S_p   = a_p + sum_{child j} x_j * S_{p+j}
    dE/dx_j += pi_p * S_{p+j}               for every edge p -> p+j

so the value costs one FMA per edge and the gradient one more; leaves (S = a) need
no product at all.  Everything lives in registers: x[], the gradient
accumulators, and one (pi, S) pair per tree level (degree <= 4).  The root's
children are split into chunks of similar cost so that ptxas compiles them in
parallel and each kernel stays small.

FP64 coefficients sit in a .const array (ptxas folds them into DFMA operands).
The FP32 kernels evaluate the polynomial re-expanded around per-class shift
centres (see SHIFT_CLASSES), with the coefficients as FFMA immediates.
"""
import itertools
import os
import struct
import sys
from collections import defaultdict
from fractions import Fraction

# Shift centres of the mixed-precision (FP32) polynomials, one per variable class:
# medians of each class over seeded synthetic water boxes (the benchmark's
# generator), rounded to float.  E(x) is re-expanded EXACTLY (rational arithmetic)
# in d = x - centre, which removes the large cancelling terms that the raw
# polynomial has in FP32 (e.g. the 3B O-O variables sit near 0.86 and the intra
# O-H ones near 2.76).  Class boundaries follow the variable order of
# SOURCE/mbpol-2b-poly.cpp:415-445 and SOURCE/mbpol-3b-poly.cpp:170-206.
SHIFT_CLASSES = {
    "2b": [(0, 2, 1.39557), (2, 6, 1.07224), (6, 10, 0.0393031), (10, 14, 0.0334345), (14, 15, 0.0207425),
           (15, 23, 0.353591), (23, 27, 0.292828), (27, 31, 0.297902)],
    "3b": [(0, 3, 0.672721), (3, 9, 2.76008), (9, 21, 0.739614), (21, 33, 1.80399), (33, 36, 0.860788)],
}


def shift_centres(body):
    out = []
    for a, b, c in SHIFT_CLASSES[body]:
        out += [float(struct.unpack("<f", struct.pack("<f", c))[0])] * (b - a)
    return out


def shifted_polynomial(monos, coef, centres):
    """Exact re-expansion of sum_k a_k prod_v x_v in d_v = x_v - centre_v.

    Returns {monomial tuple: coefficient (float64)}; () is the constant term."""
    out = defaultdict(Fraction)
    cen = [Fraction(c) for c in centres]
    for k, m in monos:
        a = Fraction(coef[k])
        for pick in itertools.product((0, 1), repeat=len(m)):
            f = a
            for v, keep in zip(m, pick):
                if not keep:
                    f *= cen[v]
            out[tuple(v for v, keep in zip(m, pick) if keep)] += f
    return {m: float(c) for m, c in out.items() if c != 0}


def read_table(path):
    coef, monos = [], []
    n_vars = None
    with open(path) as f:
        for line in f:
            if line.startswith("# n_vars"):
                n_vars = int(line.split()[2])
            elif line[0] == "C":
                _, k, a = line.split()
                assert int(k) == len(coef)
                coef.append(float(a))
            elif line[0] == "M":
                parts = line.split()
                monos.append((int(parts[1]), tuple(int(v) for v in parts[2:])))
    return n_vars, coef, monos


class Node:
    __slots__ = ("ch", "k")

    def __init__(self):
        self.ch = {}
        self.k = None     # coefficient index of the monomial ending here


def build_trie(monos):
    root = Node()
    for k, m in monos:
        n = root
        for v in m:
            n = n.ch.setdefault(v, Node())
        n.k = k
    return root


def cost(node):
    c = 0
    for ch in node.ch.values():
        c += 2 if not ch.ch else 3 + cost(ch)
    return c


def split_root(root, nchunks):
    """Greedy balance of the root's children by op count."""
    items = sorted(((cost_child(root.ch[v]), v) for v in root.ch), reverse=True)
    bins = [[0, []] for _ in range(nchunks)]
    for c, v in items:
        b = min(bins, key=lambda x: x[0])
        b[0] += c
        b[1].append(v)
    return [sorted(b[1]) for b in bins if b[1]]


def cost_child(ch):
    return 2 if not ch.ch else 3 + cost(ch)


def _hex(val, f64):
    if f64:
        return "0x%016X" % struct.unpack("<Q", struct.pack("<d", val))[0]
    return "0x%08X" % struct.unpack("<I", struct.pack("<f", val))[0]


def coef_symbol(body, prec):
    return "MBX_COEF_%s_%s" % (body.upper(), prec.upper())


def emit_coef_module(tables, pair_tables=()):
    """One module holding every coefficient array (the .const bank is shared)."""
    out = ["// generated by gen_poly_ptx.py -- do not edit",
           ".version 8.8\n.target sm_103a\n.address_size 64\n"]
    for body, coef in tables:
        vals = ",".join(_hex(c, True) for c in coef)
        out.append(".visible .const .align 8 .b64 %s[%d] = {%s};" % (coef_symbol(body, "f64"), len(coef), vals))
    for sym, distinct in pair_tables:
        vals = ",".join("0x%016X" % _pair_hex(c) for c in distinct)
        out.append(".visible .const .align 8 .b64 %s[%d] = {%s};" % (sym, len(distinct), vals))
    return "\n".join(out) + "\n"


def _trie_body(root, top_vars, ty, zero, operand):
    """PTX of the prefix-tree walk over the root's children `top_vars`: %S0 += the
    chunk's value, %g<j> += its derivatives.  Returns (lines, variables used)."""
    body = []
    used = set()

    def walk(node, pi, d):
        S = "%%S%d" % d
        if node.k is not None:
            body.append("mov.%s %s, %s;" % (ty, S, operand(node.k, body)))
        else:
            body.append("mov.%s %s, %s;" % (ty, S, zero))
        for j in sorted(node.ch):
            ch = node.ch[j]
            used.add(j)
            if not ch.ch:
                c = operand(ch.k, body)
                body.append("fma.rn.%s %s, %%x%d, %s, %s;" % (ty, S, j, c, S))
                body.append("fma.rn.%s %%g%d, %s, %s, %%g%d;" % (ty, j, pi, c, j))
            else:
                pic = "%%P%d" % (d + 1)
                body.append("mul.rn.%s %s, %s, %%x%d;" % (ty, pic, pi, j))
                walk(ch, pic, d + 1)
                body.append("fma.rn.%s %s, %%x%d, %%S%d, %s;" % (ty, S, j, d + 1, S))
                body.append("fma.rn.%s %%g%d, %s, %%S%d, %%g%d;" % (ty, j, pi, d + 1, j))

    for j in top_vars:
        ch = root.ch[j]
        used.add(j)
        if not ch.ch:
            c = operand(ch.k, body)
            body.append("fma.rn.%s %%S0, %%x%d, %s, %%S0;" % (ty, j, c))
            body.append("add.rn.%s %%g%d, %%g%d, %s;" % (ty, j, j, c))
        else:
            walk(ch, "%%x%d" % j, 1)
            body.append("fma.rn.%s %%S0, %%x%d, %%S1, %%S0;" % (ty, j))
            body.append("add.rn.%s %%g%d, %%g%d, %%S1;" % (ty, j, j))
    return body, used


def _f32imm(v):
    return "0f%08X" % struct.unpack("<I", struct.pack("<f", v))[0]


# Symmetry of the 3B polynomial.  Its 36 variables are functions of atom pairs of the
# trimer (SOURCE/mbpol-3b-poly.cpp:170-206; atoms 0..8 = Oa Ha1 Ha2 Ob Hb1 Hb2 Oc Hc1
# Hc2), and E is invariant under the 48 relabellings G of the trimer: the 6
# permutations of the waters times the 8 swaps of the two H atoms within each water
# (the polynomial's 1163 coefficient classes are exactly the orbits of G on its 33525
# monomials).  So E(x) = sum_{g in G} f(g x) for the polynomial f holding one
# representative monomial per orbit, with coefficient a * |orbit| / |G|.  Evaluated
# as a loop over g, f is ~1.75x the operations of E but 1/27 of the code (~43 KB of
# FP32 instructions instead of ~1.2 MB): the straight-line form left the FP32 pipe
# ~23 % busy waiting for instruction fetch, the loop keeps it ~52 % busy and runs the
# 3B kernel in 2.7 ms instead of 3.2 ms on the 4096-water box.
VARS_3B = [(1, 2), (4, 5), (7, 8), (0, 1), (0, 2), (3, 4), (3, 5), (6, 7), (6, 8),
           (1, 4), (1, 5), (1, 7), (1, 8), (2, 4), (2, 5), (2, 7), (2, 8),
           (4, 7), (4, 8), (5, 7), (5, 8),
           (0, 4), (0, 5), (0, 7), (0, 8), (3, 1), (3, 2), (3, 7), (3, 8), (6, 1), (6, 2), (6, 4), (6, 5),
           (0, 3), (0, 6), (3, 6)]


def group_3b():
    """The 48 relabellings of a trimer as permutations of the 3B variables (identity first)."""
    index = {frozenset(p): i for i, p in enumerate(VARS_3B)}
    out = []
    for perm in itertools.permutations(range(3)):
        for sw in itertools.product((0, 1), repeat=3):
            amap = {}
            for m in range(3):
                h1, h2 = 3 * perm[m] + 1, 3 * perm[m] + 2
                if sw[m]:
                    h1, h2 = h2, h1
                amap[3 * m] = 3 * perm[m]
                amap[3 * m + 1] = h1
                amap[3 * m + 2] = h2
            out.append([index[frozenset((amap[a], amap[b]))] for a, b in VARS_3B])
    return out


def group_reduce(poly, perms):
    """poly {sorted monomial tuple: coefficient} invariant under `perms` -> the
    representative polynomial f as a sorted list of (monomial, coefficient)."""
    seen = set()
    reps = []
    for m in sorted(poly):
        if m in seen:
            continue
        orb = set(tuple(sorted(p[v] for v in m)) for p in perms)
        for o in orb:
            if abs(poly.get(o, 0.0) - poly[m]) > 1e-12 * max(1.0, abs(poly[m])):
                raise ValueError("polynomial is not invariant under the group")
        seen |= orb
        r = min(orb)
        reps.append((r, poly[m] * len(orb) / len(perms)))
    return sorted(reps)


def emit_group_chunk(name, n_vars, reps, perms, const_term):
    """FP32 device function  name(const float* x, float* acc)  adding E = const +
    sum_g f(g x) and its gradient, looping over the group: each pass loads the permuted
    variables, walks f's prefix tree and scatters the gradient back."""
    coef = [c for _, c in reps]
    root = build_trie([(i, m) for i, (m, _) in enumerate(reps)])
    body, used = _trie_body(root, sorted(root.ch), "f32", "0f00000000", lambda k, b: _f32imm(coef[k]))
    table = "%s_perm" % name
    offs = ",".join(str(4 * p[j]) for p in perms for j in range(n_vars))
    out = ["// generated by gen_poly_ptx.py -- do not edit",
           ".version 8.8\n.target sm_103a\n.address_size 64\n",
           ".const .align 4 .u32 %s[%d] = {%s};" % (table, len(perms) * n_vars, offs),
           ".visible .func %s(.param .b64 px, .param .b64 pacc)\n{" % name,
           " .reg .f32 %%x<%d>, %%g<%d>, %%S<6>, %%P<6>, %%t, %%E;" % (n_vars, n_vars),
           " .reg .b64 %rd<8>;",
           " .reg .b32 %r<4>;",
           " .reg .pred %p;",
           " ld.param.u64 %rd1, [px];",
           " ld.param.u64 %rd2, [pacc];",
           " mov.u64 %%rd3, %s;" % table,
           " mov.f32 %E, 0f00000000;",
           " mov.u32 %r1, 0;",
           "$L_group:",
           " mul.wide.u32 %%rd5, %%r1, %d;" % (4 * n_vars),
           " add.u64 %rd4, %rd3, %rd5;"]
    for j in sorted(used):
        out.append(" ld.const.u32 %%r2, [%%rd4+%d]; cvt.u64.u32 %%rd6, %%r2; add.u64 %%rd7, %%rd1, %%rd6;"
                   " ld.f32 %%x%d, [%%rd7];" % (4 * j, j))
        out.append(" mov.f32 %%g%d, 0f00000000;" % j)
    out.append(" mov.f32 %S0, 0f00000000;")
    out.extend(" " + l for l in body)
    out.append(" add.rn.f32 %E, %E, %S0;")
    for j in sorted(used):
        out.append(" ld.const.u32 %%r2, [%%rd4+%d]; cvt.u64.u32 %%rd6, %%r2; add.u64 %%rd7, %%rd2, %%rd6;"
                   " ld.f32 %%t, [%%rd7+4]; add.rn.f32 %%t, %%t, %%g%d; st.f32 [%%rd7+4], %%t;" % (4 * j, j))
    out += [" add.u32 %r1, %r1, 1;",
            " setp.lt.u32 %%p, %%r1, %d;" % len(perms),
            " @%p bra $L_group;",
            " add.rn.f32 %%E, %%E, %s;" % _f32imm(const_term),
            " ld.f32 %t, [%rd2+0]; add.rn.f32 %t, %t, %E; st.f32 [%rd2+0], %t;",
            " ret;\n}"]
    return "\n".join(out) + "\n"


def emit_chunk(name, body_name, n_vars, coef, root, top_vars, f64, const_term=0.0):
    """A device function  name(const T* x, T* acc):  acc[0] += E_chunk, acc[1+j] += dE_chunk/dx_j.

    FP64 chunks read their coefficients from the shared .const array (orbit
    coefficients, the reference's own polynomial).  FP32 chunks evaluate the shifted
    polynomial, whose per-monomial coefficients are FFMA immediates."""
    prec = "f64" if f64 else "f32"
    ty = prec
    sz = 8 if f64 else 4
    zero = "0d0000000000000000" if f64 else "0f00000000"
    sym = coef_symbol(body_name, prec)
    body = []
    used = set()

    def operand(k):
        if f64:
            body.append("ld.const.f64 %%c, [%s+%d];" % (sym, 8 * k))
            return "%c"
        return "0f%08X" % struct.unpack("<I", struct.pack("<f", coef[k]))[0]

    def walk(node, pi, d):
        S = "%%S%d" % d
        if node.k is not None:
            body.append("mov.%s %s, %s;" % (ty, S, operand(node.k)))
        else:
            body.append("mov.%s %s, %s;" % (ty, S, zero))
        for j in sorted(node.ch):
            ch = node.ch[j]
            used.add(j)
            if not ch.ch:
                c = operand(ch.k)
                body.append("fma.rn.%s %s, %%x%d, %s, %s;" % (ty, S, j, c, S))
                body.append("fma.rn.%s %%g%d, %s, %s, %%g%d;" % (ty, j, pi, c, j))
            else:
                pic = "%%P%d" % (d + 1)
                body.append("mul.rn.%s %s, %s, %%x%d;" % (ty, pic, pi, j))
                walk(ch, pic, d + 1)
                body.append("fma.rn.%s %s, %%x%d, %%S%d, %s;" % (ty, S, j, d + 1, S))
                body.append("fma.rn.%s %%g%d, %s, %%S%d, %%g%d;" % (ty, j, pi, d + 1, j))

    if f64:
        body.append("mov.f64 %%S0, 0d%016X;" % struct.unpack("<Q", struct.pack("<d", const_term))[0])
    else:
        body.append("mov.f32 %%S0, 0f%08X;" % struct.unpack("<I", struct.pack("<f", const_term))[0])
    for j in top_vars:
        ch = root.ch[j]
        used.add(j)
        if not ch.ch:
            c = operand(ch.k)
            body.append("fma.rn.%s %%S0, %%x%d, %s, %%S0;" % (ty, j, c))
            body.append("add.rn.%s %%g%d, %%g%d, %s;" % (ty, j, j, c))
        else:
            walk(ch, "%%x%d" % j, 1)
            body.append("fma.rn.%s %%S0, %%x%d, %%S1, %%S0;" % (ty, j))
            body.append("add.rn.%s %%g%d, %%g%d, %%S1;" % (ty, j, j))

    out = ["// generated by gen_poly_ptx.py -- do not edit",
           ".version 8.8\n.target sm_103a\n.address_size 64\n"]
    if f64:
        out.append(".extern .const .align 8 .b64 %s[%d];" % (sym, len(coef)))
    out += [".visible .func %s(.param .b64 px, .param .b64 pacc)\n{" % name,
            " .reg .%s %%x<%d>, %%g<%d>, %%S<6>, %%P<6>, %%c, %%t;" % (ty, n_vars, n_vars),
            " .reg .b64 %rd<3>;",
            " ld.param.u64 %rd1, [px];",
            " ld.param.u64 %rd2, [pacc];"]
    for j in sorted(used):
        out.append(" ld.%s %%x%d, [%%rd1+%d];" % (ty, j, sz * j))
        out.append(" mov.%s %%g%d, %s;" % (ty, j, zero))
    out.extend(" " + l for l in body)
    out.append(" ld.%s %%t, [%%rd2+0]; add.rn.%s %%t, %%t, %%S0; st.%s [%%rd2+0], %%t;" % (ty, ty, ty))
    for j in sorted(used):
        off = sz * (j + 1)
        out.append(" ld.%s %%t, [%%rd2+%d]; add.rn.%s %%t, %%t, %%g%d; st.%s [%%rd2+%d], %%t;"
                   % (ty, off, ty, j, ty, off))
    out.append(" ret;\n}")
    return "\n".join(out) + "\n"


# chunk counts: enough to keep every ptxas job short (they run in parallel)
CHUNKS = {"2b": {"f64": 2, "f32": 4}, "3b": {"f64": 6}}


def _write_if_changed(path, text):
    if os.path.exists(path):
        with open(path) as f:
            if f.read() == text:
                return
    with open(path, "w") as f:
        f.write(text)


def generate(table_dir, out_dir):
    """Write the PTX modules and the C++ header that declares/dispatches them.

    Returns the list of PTX paths to compile."""
    os.makedirs(out_dir, exist_ok=True)
    made = []
    tables = []
    pair_tables = []
    decls = ["// generated by gen_poly_ptx.py -- do not edit", "#pragma once", ""]
    disp = []
    for body in ("2b", "3b"):
        n_vars, coef, monos = read_table(os.path.join(table_dir, "poly%s.tbl" % body))
        tables.append((body, coef))
        centres = shift_centres(body)
        sp = shifted_polynomial(monos, coef, centres)
        items = sorted(sp.items())
        coef32 = [c for _, c in items]
        root32 = build_trie([(i, m) for i, (m, _) in enumerate(items) if m])
        const32 = sp.get((), 0.0)
        root64 = build_trie(monos)
        for prec in ("f64", "f32"):
            ctype = "double" if prec == "f64" else "float"
            root = root64 if prec == "f64" else root32
            cf = coef if prec == "f64" else coef32
            if body == "3b" and prec == "f32":
                # one looped function over the water relabellings (see group_3b)
                name = "mbx_poly3b_f32_grp"
                poly = {tuple(sorted(m)): c for m, c in sp.items() if m}
                text = emit_group_chunk(name, n_vars, group_reduce(poly, group_3b()), group_3b(), const32)
                path = os.path.join(out_dir, name + ".ptx")
                _write_if_changed(path, text)
                made.append(path)
                decls.append('extern "C" __device__ void %s(const float* x, float* acc);' % name)
                disp.append("template <> __device__ __forceinline__ void poly3b<float>(const float* x, float* acc) {")
                disp.append("    %s(x, acc);" % name)
                disp.append("}")
                continue
            chunks = split_root(root, CHUNKS[body][prec])
            names = []
            for c, top in enumerate(chunks):
                name = "mbx_poly%s_%s_c%d" % (body, prec, c)
                text = emit_chunk(name, body, n_vars, cf, root, top, prec == "f64",
                                  const_term=(const32 if (prec != "f64" and c == 0) else 0.0))
                path = os.path.join(out_dir, name + ".ptx")
                _write_if_changed(path, text)
                made.append(path)
                names.append(name)
                decls.append('extern "C" __device__ void %s(const %s* x, %s* acc);' % (name, ctype, ctype))
            disp.append("template <> __device__ __forceinline__ void poly%s<%s>(const %s* x, %s* acc) {"
                        % (body, ctype, ctype, ctype))
            disp.extend("    %s(x, acc);" % n for n in names)
            disp.append("}")
            # one chunk at a time (the chunks' contributions add up to the whole polynomial)
            disp.append("constexpr int kPoly%s%sParts = %d;" % (body.upper(), prec.upper(), len(names)))
            disp.append("__device__ __forceinline__ void poly%s_%s_part(int p, const %s* x, %s* acc) {"
                        % (body, prec, ctype, ctype))
            disp.append("    switch (p) {")
            disp.extend("    case %d: %s(x, acc); break;" % (c, n) for c, n in enumerate(names))
            disp.append("    default: break;")
            disp.append("    }")
            disp.append("}")
        decls.append("constexpr int kPoly%sVars = %d;" % (body.upper(), n_vars))
        decls.append("// FP32 polynomial variables are x - kShift%s[v]" % body.upper())
        decls.append("__device__ constexpr float kShift%s[%d] = {%s};"
                     % (body.upper(), n_vars, ", ".join("%.9gf" % c for c in centres)))
    path = os.path.join(out_dir, "mbx_poly_coef.ptx")
    _write_if_changed(path, emit_coef_module(tables, pair_tables))
    made.append(path)
    hdr = decls + ["", "template <typename T> __device__ void poly2b(const T* x, T* acc);",
                   "template <typename T> __device__ void poly3b(const T* x, T* acc);"] + disp
    _write_if_changed(os.path.join(out_dir, "mbx_poly_gen.cuh"), "\n".join(hdr) + "\n")
    return made


def chunk_counts():
    return {b: dict(v) for b, v in CHUNKS.items()}


if __name__ == "__main__":
    for path in generate(sys.argv[1], sys.argv[2]):
        print(path)
