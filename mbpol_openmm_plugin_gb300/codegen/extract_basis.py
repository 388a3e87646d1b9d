"""Extract the permutationally-invariant polynomial bases of MB-pol's two- and
three-body terms, and the model's coefficient tables, from the reference
sources, and write them as data files under ``mbpol_openmm_plugin_gb300/data``.

The reference evaluates each polynomial with Maple-generated straight-line
code (platforms/reference/src/poly-2b-v6x.cpp:3-13841,
platforms/reference/src/poly-3b-v2x.cpp:3-28378).  Its energy is linear in the
fit coefficients ``a[k]``::

    E(x) = sum_k a[k] * p_k(x),   p_k(x) = sum over the k-th orbit of monomials

This script expands the generated energy expression symbolically (the
gradient part of the generated code is ignored) and records, for every
monomial ``x[v1]*x[v2]*...`` (degree <= 4), the coefficient index ``k`` and
the integer multiplicity.  The evaluators that this project ships are then
generated from that basis by ``gen_poly.py``; no generated reference code is
reused.  The coefficient values (the fitted model parameters) are read from
mbpol_2body_constants.h:52-1210, mbpol_3body_constants.h:22-1188, and the
one-body tables from mbpol_interaction_constants.h:24-426.

Run once, in a checkout that has the reference next to it::

    python -m mbpol_openmm_plugin_gb300.codegen.extract_basis /path/to/reference
"""
import os
import re
import sys
from collections import defaultdict

HERE = os.path.dirname(os.path.abspath(__file__))
DATA = os.path.join(os.path.dirname(HERE), "data")

TOKEN = re.compile(r"\s*(?:(t\d+)|a\[(\d+)\]|x\[(\d+)\]|df\[(\d+)\]|(\d+\.\d*(?:[eE][-+]?\d+)?|\d+)|(.))")


class Poly:
    """Sparse polynomial in x whose coefficients are linear forms in a.

    terms: {monomial (sorted tuple of var indices): {a_index or -1: float}}
    (-1 is the constant, i.e. no a-dependence)."""

    __slots__ = ("terms",)

    def __init__(self, terms=None):
        self.terms = terms if terms is not None else {}

    @staticmethod
    def const(c):
        return Poly({(): {-1: float(c)}})

    @staticmethod
    def coef(k):
        return Poly({(): {k: 1.0}})

    @staticmethod
    def var(v):
        return Poly({(v,): {-1: 1.0}})

    def add(self, o, sign=1.0):
        out = {m: dict(c) for m, c in self.terms.items()}
        for m, c in o.terms.items():
            d = out.setdefault(m, {})
            for k, v in c.items():
                d[k] = d.get(k, 0.0) + sign * v
        return Poly(out)

    def mul(self, o):
        out = {}
        for m1, c1 in self.terms.items():
            for m2, c2 in o.terms.items():
                m = tuple(sorted(m1 + m2))
                d = out.setdefault(m, {})
                for k1, v1 in c1.items():
                    for k2, v2 in c2.items():
                        if k1 >= 0 and k2 >= 0:
                            raise ValueError("expression is not linear in a")
                        k = k1 if k1 >= 0 else k2
                        d[k] = d.get(k, 0.0) + v1 * v2
        return Poly(out)


def parse_statements(path):
    src = open(path).read()
    body = src[src.index("{", src.index("eval(")) + 1:]
    stmts = {}
    ret = None
    for raw in body.split(";"):
        st = " ".join(raw.split())
        if not st or st.startswith("double df[") or st == "}":
            continue
        if st.startswith("return "):
            ret = st[len("return "):]
            continue
        m = re.match(r"const double (t\d+) = (.*)$", st)
        if m:
            stmts[m.group(1)] = m.group(2)
            continue
        m = re.match(r"(df\[\d+\]) = (.*)$", st)
        if m:
            stmts[m.group(1)] = m.group(2)
            continue
        m = re.match(r"(g\[\d+\]) = (.*)$", st)
        if m:
            continue
    return stmts, ret


def tokenize(expr):
    toks = []
    pos = 0
    while pos < len(expr):
        m = TOKEN.match(expr, pos)
        if not m:
            break
        pos = m.end()
        t, a, x, df, num, op = m.groups()
        if t:
            toks.append(("ref", t))
        elif a is not None:
            toks.append(("a", int(a)))
        elif x is not None:
            toks.append(("x", int(x)))
        elif df is not None:
            toks.append(("ref", "df[%s]" % df))
        elif num is not None:
            toks.append(("num", float(num)))
        elif op and op.strip():
            toks.append(("op", op))
    return toks


class Evaluator:
    def __init__(self, stmts):
        self.stmts = stmts
        self.memo = {}

    def value(self, name):
        if name in self.memo:
            return self.memo[name]
        v = self.expr(self.stmts[name])
        self.memo[name] = v
        return v

    def expr(self, text):
        toks = tokenize(text)
        pos = [0]

        def peek():
            return toks[pos[0]] if pos[0] < len(toks) else ("end", None)

        def take():
            t = toks[pos[0]]
            pos[0] += 1
            return t

        def atom():
            kind, val = take()
            if kind == "op" and val == "(":
                v = sum_()
                assert take() == ("op", ")")
                return v
            if kind == "op" and val == "-":
                return atom().mul(Poly.const(-1.0))
            if kind == "op" and val == "+":
                return atom()
            if kind == "ref":
                return self.value(val)
            if kind == "a":
                return Poly.coef(val)
            if kind == "x":
                return Poly.var(val)
            if kind == "num":
                return Poly.const(val)
            raise ValueError("unexpected token %r in %s" % ((kind, val), text[:80]))

        def prod():
            v = atom()
            while peek() == ("op", "*"):
                take()
                v = v.mul(atom())
            return v

        def sum_():
            if peek() in (("op", "-"), ("op", "+")):
                sign = -1.0 if take()[1] == "-" else 1.0
                v = prod().mul(Poly.const(sign))
            else:
                v = prod()
            while peek() in (("op", "+"), ("op", "-")):
                sign = 1.0 if take()[1] == "+" else -1.0
                v = v.add(prod(), sign)
            return v

        sys.setrecursionlimit(100000)
        out = sum_()
        assert pos[0] == len(toks), "trailing tokens in %s" % text[:80]
        return out


def extract(path, ncoef):
    stmts, ret = parse_statements(path)
    ev = Evaluator(stmts)
    poly = ev.expr(ret)
    rows = []
    for mono, coefs in poly.terms.items():
        for k, c in coefs.items():
            if abs(c) < 1e-12:
                continue
            if k < 0:
                raise ValueError("constant term without coefficient: %r %r" % (mono, c))
            if abs(c - round(c)) > 1e-9:
                raise ValueError("non-integer multiplicity %r for a[%d] %r" % (c, k, mono))
            rows.append((k, int(round(c)), mono))
    rows.sort(key=lambda r: (r[0], len(r[2]), r[2]))
    used = {r[0] for r in rows}
    assert used <= set(range(ncoef)), "coefficient index out of range"
    return rows


def read_table(path, start_marker, n):
    """Read n floating-point numbers following start_marker."""
    src = open(path).read()
    i = src.index(start_marker)
    nums = re.findall(r"[-+]?\d+\.\d+(?:[eE][-+]?\d+)?", src[i + len(start_marker):])
    return [float(v) for v in nums[:n]]


def read_int_table(path, start_marker, n):
    src = open(path).read()
    i = src.index(start_marker)
    j = src.index("};", i)
    nums = re.findall(r"\d+", src[i + len(start_marker):j])
    vals = [int(v) for v in nums]
    assert len(vals) == n, (start_marker, len(vals))
    return vals


def write_basis(name, rows, nvars, ncoef, source):
    path = os.path.join(DATA, name)
    with open(path, "w") as f:
        f.write("# MB-pol polynomial basis: E(x) = sum_rows a[k] * mult * prod x[v]\n")
        f.write("# extracted from %s (energy expression only)\n" % source)
        f.write("# columns: k mult v1 [v2 [v3 [v4]]]\n")
        f.write("nvars %d ncoef %d nrows %d\n" % (nvars, ncoef, len(rows)))
        for k, mult, mono in rows:
            f.write("%d %d %s\n" % (k, mult, " ".join(str(v) for v in mono)))
    return path


def write_coeffs(name, vals, source):
    path = os.path.join(DATA, name)
    with open(path, "w") as f:
        f.write("# MB-pol fitted coefficients, from %s\n" % source)
        f.write("n %d\n" % len(vals))
        for v in vals:
            f.write("%.16e\n" % v)
    return path


def main(ref):
    src = os.path.join(ref, "platforms", "reference", "src")
    os.makedirs(DATA, exist_ok=True)
    rows2 = extract(os.path.join(src, "poly-2b-v6x.cpp"), 1153)
    print("2B: %d monomials" % len(rows2))
    write_basis("poly2b_basis.txt", rows2, 31, 1153, "platforms/reference/src/poly-2b-v6x.cpp:3-13841")
    c2 = read_table(os.path.join(src, "mbpol_2body_constants.h"), "const double thefit[] = {", 1153)
    write_coeffs("poly2b_coeffs.txt", c2, "platforms/reference/src/mbpol_2body_constants.h:52-1210")
    rows3 = extract(os.path.join(src, "poly-3b-v2x.cpp"), 1163)
    print("3B: %d monomials" % len(rows3))
    write_basis("poly3b_basis.txt", rows3, 36, 1163, "platforms/reference/src/poly-3b-v2x.cpp:3-28378")
    c3 = read_table(os.path.join(src, "mbpol_3body_constants.h"), "const double thefit[] = {", 1163)
    write_coeffs("poly3b_coeffs.txt", c3, "platforms/reference/src/mbpol_3body_constants.h:22-1188")
    # one-body tables (mbpol_interaction_constants.h:24-426)
    ic = os.path.join(src, "mbpol_interaction_constants.h")
    tabs = {t: read_table(ic, "const double %s[245] = {" % t, 245) for t in ("c5zA", "cbasis", "ccore", "crest")}
    idx = {t: read_int_table(ic, "const size_t %s[245] = {" % t, 245) for t in ("idx1", "idx2", "idx3")}
    with open(os.path.join(DATA, "onebody_tables.txt"), "w") as f:
        f.write("# MB-pol one-body (PES) tables, from platforms/reference/src/mbpol_interaction_constants.h:24-426\n")
        f.write("# columns: c5zA cbasis ccore crest idx1 idx2 idx3\n")
        f.write("n 245\n")
        for i in range(245):
            f.write("%.16e %.16e %.16e %.16e %d %d %d\n" % (
                tabs["c5zA"][i], tabs["cbasis"][i], tabs["ccore"][i], tabs["crest"][i],
                idx["idx1"][i], idx["idx2"][i], idx["idx3"][i]))


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MBPOL_REFERENCE_DIR")
    if not ref:
        sys.exit("usage: extract_basis.py REFERENCE_CHECKOUT (or set MBPOL_REFERENCE_DIR)")
    main(ref)
