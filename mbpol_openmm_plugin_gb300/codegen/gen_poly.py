"""Generate this project's evaluators for the MB-pol 2-body and 3-body
permutationally-invariant polynomials from the extracted basis
(``data/poly{2b,3b}_basis.txt``) and the fitted coefficients
(``data/poly{2b,3b}_coeffs.txt``).

Evaluation scheme (this project's own; not the reference's Maple code):
every monomial x[v1]*x[v2]*x[v3]*x[v4] (v1<=v2<=v3<=v4 after a variable
relabelling chosen to maximise prefix sharing) is a root-to-node path in a
trie of depth <= 4 whose node carries the merged coefficient
c = sum of a[k]*mult over basis rows with that monomial.  A depth-first walk
computes value and gradient in one pass with O(1) live state per level::

    P_d = P_{d-1} * x[v_d]               (prefix product, only if children)
    V_d = c_d + sum_children x[v_child] * V_child
    g[v_d] += V_d * P_{d-1}               (reverse-mode contribution)
    E = V_root

Outputs:

* ``csrc/gen/poly2b_tables.inc`` / ``poly3b_tables.inc`` — the trie as
  level arrays of nodes {coefficient as an FP32 (hi, lo) pair, variable,
  end of children}, walked by the data-driven double-float kernel
  (csrc/poly_df.cu).  Plain FP32 is not enough: the monomial sum cancels by
  a factor of ~1e4-1e5, so the walk runs Dot2-style in double-float (Ogita,
  Rump, Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput. 26,
  2005).  A straight-line generated kernel was measured too: nvcc did not
  finish one seventh of the three-body trie in 30 minutes;
* ``oracle/gen/poly2b_prog.h`` / ``poly3b_prog.h`` — the same walk as a
  table (level, variable, coefficient) interpreted in FP64 by the oracle port.
"""
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
DATA = os.path.join(PKG, "data")


def load_basis(name):
    rows = []
    nvars = None
    for line in open(os.path.join(DATA, name)):
        if line.startswith("#"):
            continue
        if line.startswith("nvars"):
            nvars = int(line.split()[1])
            continue
        t = [int(v) for v in line.split()]
        rows.append((t[0], t[1], tuple(t[2:])))
    return nvars, rows


def load_coeffs(name):
    vals = []
    for line in open(os.path.join(DATA, name)):
        if line.startswith("#") or line.startswith("n "):
            continue
        vals.append(float(line))
    return vals


def merged_monomials(rows, coeffs, perm):
    """{sorted relabelled monomial: coefficient}; perm maps original var -> label."""
    mono = {}
    for k, mult, m in rows:
        key = tuple(sorted(perm[v] for v in m))
        mono[key] = mono.get(key, 0.0) + coeffs[k] * mult
    return mono


def build_trie(mono):
    """Nested dict trie: node = {'c': coef, 'ch': {label: node}}."""
    root = {"c": 0.0, "ch": {}}
    for m, c in mono.items():
        node = root
        for v in m:
            node = node["ch"].setdefault(v, {"c": 0.0, "ch": {}})
        node["c"] += c
    return root


def trie_cost(mono):
    prefixes = set()
    for m in mono:
        for d in range(1, len(m)):
            prefixes.add(m[:d])
    return 2 * len(mono) + 3 * len(prefixes)


def choose_perm(nvars, rows):
    """Relabel variables to reduce the number of trie prefixes: try the
    identity, its reverse, and orders by occurrence count."""
    count = [0] * nvars
    for _, _, m in rows:
        for v in m:
            count[v] += 1
    cands = [list(range(nvars)), list(range(nvars))[::-1]]
    by_freq = sorted(range(nvars), key=lambda v: count[v])
    cands.append(by_freq)
    cands.append(by_freq[::-1])
    best = None
    for order in cands:
        perm = [0] * nvars
        for label, v in enumerate(order):
            perm[v] = label
        cost = trie_cost(merged_monomials(rows, [1.0] * 2000, perm))
        if best is None or cost < best[0]:
            best = (cost, perm)
    return best[1]


def split_df(c):
    """c (FP64) -> (hi, lo) FP32 pair with hi + lo ~= c to ~48 bits."""
    import struct
    hi = struct.unpack(">f", struct.pack(">f", c))[0]
    lo = struct.unpack(">f", struct.pack(">f", c - hi))[0]
    return hi, lo


def emit_tables(name, nvars, root, perm, out_path, nmono):
    """Trie as four arrays for the data-driven kernel (csrc/poly_df.cu):
    level-1, level-2, level-3 nodes {hi, lo, var, end} where `end` is one
    past the node's last child in the next level, and leaves {hi, lo, var}.
    Coefficients are split into FP32 (hi, lo) pairs."""
    inv = [0] * nvars
    for v, label in enumerate(perm):
        inv[label] = v
    L1, L2, L3, LV = [], [], [], []
    for l1 in sorted(root["ch"]):
        n1 = root["ch"][l1]
        for l2 in sorted(n1["ch"]):
            n2 = n1["ch"][l2]
            for l3 in sorted(n2["ch"]):
                n3 = n2["ch"][l3]
                for l4 in sorted(n3["ch"]):
                    LV.append((n3["ch"][l4]["c"], inv[l4]))
                L3.append((n3["c"], inv[l3], len(LV)))
            L2.append((n2["c"], inv[l2], len(L3)))
        L1.append((n1["c"], inv[l1], len(L2)))
    lines = ["// Generated by mbpol_openmm_plugin_gb300/codegen/gen_poly.py from data/%s_basis.txt" % name,
             "// and data/%s_coeffs.txt.  Do not edit.  %d monomials as a depth-first trie:" % (name, nmono),
             "// nodes {coef hi, coef lo, variable, end of children}, leaves {coef hi, coef lo, variable, 0}.",
             "#define %s_NVARS %d" % (name.upper(), nvars),
             "#define %s_N1 %d" % (name.upper(), len(L1)),
             "#define %s_N2 %d" % (name.upper(), len(L2)),
             "#define %s_N3 %d" % (name.upper(), len(L3)),
             "#define %s_NL %d" % (name.upper(), len(LV))]

    def node_rows(arr, sym):
        lines.append("static const PolyNode %s[%d] = {" % (sym, len(arr)))
        for c, v, end in arr:
            hi, lo = split_df(c)
            lines.append("{%sf, %sf, %d, %d}," % (float.hex(hi), float.hex(lo), v, end))
        lines.append("};")

    node_rows(L1, name + "_l1")
    node_rows(L2, name + "_l2")
    node_rows(L3, name + "_l3")
    lines.append("static const PolyNode %s_leaf[%d] = {" % (name, len(LV)))
    for c, v in LV:
        hi, lo = split_df(c)
        lines.append("{%sf, %sf, %d, 0}," % (float.hex(hi), float.hex(lo), v))
    lines.append("};")
    with open(out_path, "w") as f:
        f.write("\n".join(lines) + "\n")


def emit_prog(name, nvars, root, perm, out_path, nmono):
    """Pre-order table: one entry per trie node (level 1..4, original var, coef)."""
    entries = []

    def walk(node, level):
        for label in sorted(node["ch"]):
            ch = node["ch"][label]
            entries.append((level, perm.index(label), ch["c"]))
            walk(ch, level + 1)

    walk(root, 1)
    with open(out_path, "w") as f:
        f.write("/* Generated by mbpol_openmm_plugin_gb300/codegen/gen_poly.py from data/%s_basis.txt\n" % name)
        f.write(" * and data/%s_coeffs.txt.  Do not edit.  Pre-order trie of %d monomials:\n" % (name, nmono))
        f.write(" * {level, variable, coefficient}; interpreted by oracle/mbpol_oracle.c. */\n")
        f.write("#define %s_NVARS %d\n" % (name.upper(), nvars))
        f.write("#define %s_NPROG %d\n" % (name.upper(), len(entries)))
        f.write("static const mbpol_prog_entry %s_prog[%d] = {\n" % (name, len(entries)))
        for lev, v, c in entries:
            f.write("{%d,%d,%.17e},\n" % (lev, v, c))
        f.write("};\n")


def generate(name):
    nvars, rows = load_basis("%s_basis.txt" % name)
    coeffs = load_coeffs("%s_coeffs.txt" % name)
    perm = choose_perm(nvars, rows)
    mono = merged_monomials(rows, coeffs, perm)
    root = build_trie(mono)
    cuda_dir = os.path.join(PKG, "csrc", "gen")
    prog_dir = os.path.join(ROOT, "oracle", "gen")
    os.makedirs(cuda_dir, exist_ok=True)
    os.makedirs(prog_dir, exist_ok=True)
    emit_tables(name, nvars, root, perm, os.path.join(cuda_dir, "%s_tables.inc" % name), len(mono))
    emit_prog(name, nvars, root, perm, os.path.join(prog_dir, "%s_prog.h" % name), len(mono))
    print("%s: %d monomials, cost %d ops" % (name, len(mono), trie_cost(mono)))


if __name__ == "__main__":
    for n in sys.argv[1:] or ["poly2b", "poly3b"]:
        generate(n)
