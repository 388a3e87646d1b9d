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

so a leaf costs 2 FMAs and an internal node 3 operations.  Outputs:

* ``csrc/gen/poly2b.ptx`` / ``poly3b.ptx`` — straight-line PTX kernels
  evaluating the walk in double-float (FP32-pair) arithmetic on the FP32
  pipe (coefficients are FFMA immediates, no coefficient memory traffic),
  assembled by ptxas alone: nvcc's front end takes tens of minutes on a
  function this long.  Plain FP32 is not enough: the monomial sum cancels by
  a factor of ~1e4-1e5 (terms of 1e2-1e5 kcal/mol summing to ~1), so FP32
  rounding leaves ~1e-3 relative error; the Dot2-style double-float walk
  (Ogita, Rump, Oishi, "Accurate sum and dot product", SIAM J. Sci. Comput.
  26, 2005) brings it to the FP64 level at ~11x the FP32 operation count;
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


def fmt(c):
    s = "%.9e" % c
    return s + "f"


def f32hex(c):
    import struct
    return "0f%08X" % struct.unpack(">I", struct.pack(">f", c))[0]


def split_df(c):
    """c (FP64) -> (hi, lo) FP32 pair with hi + lo ~= c to ~48 bits."""
    import struct
    hi = struct.unpack(">f", struct.pack(">f", c))[0]
    lo = struct.unpack(">f", struct.pack(">f", c - hi))[0]
    return hi, lo


def df_program(nvars, root, perm):
    """The depth-first walk as a list of double-float operations.

    Every value that accumulates (V per level, E, g) is a pair (s, c) of
    FP32 numbers updated Dot2-style: s <- s + p with the exact rounding
    error of the sum (TwoSum) and of the product (TwoProd by FMA) added into
    c.  Products x*x are exact pairs; coefficients are (hi, lo) FP32 pairs.
    Ops (operands are original variable indices):
      ('p2', i, j)         P2 = x_i * x_j                  (exact pair)
      ('p3', k)            P3 = P2 * x_k
      ('set', lev, c)      V_lev = c
      ('leaf', l, c)       V3 += c x_l ;  g_l += c P3
      ('close3', k)        V2 += V3 x_k ; g_k += V3 P2
      ('close2', j, i)     V1 += V2 x_j ; g_j += V2 x_i
      ('close1', i)        E  += V1 x_i ; g_i += V1
    """
    inv = [0] * nvars
    for v, label in enumerate(perm):
        inv[label] = v
    ops = []
    for l1 in sorted(root["ch"]):
        n1 = root["ch"][l1]
        i = inv[l1]
        ops.append(("set", 1, n1["c"]))
        for l2 in sorted(n1["ch"]):
            n2 = n1["ch"][l2]
            j = inv[l2]
            ops.append(("set", 2, n2["c"]))
            if n2["ch"]:
                ops.append(("p2", i, j))
            for l3 in sorted(n2["ch"]):
                n3 = n2["ch"][l3]
                k = inv[l3]
                ops.append(("set", 3, n3["c"]))
                if n3["ch"]:
                    ops.append(("p3", k))
                for l4 in sorted(n3["ch"]):
                    assert not n3["ch"][l4]["ch"]
                    ops.append(("leaf", inv[l4], n3["ch"][l4]["c"]))
                ops.append(("close3", k))
            ops.append(("close2", j, i))
        ops.append(("close1", i))
    return ops


def f32hex(c):
    import struct
    return "0f%08X" % struct.unpack(">I", struct.pack(">f", c))[0]


def emit_ptx(name, nvars, ops, out_path, nmono):
    """Write a standalone PTX kernel ``<name>_batch`` evaluating the walk in
    double-float arithmetic on the FP32 pipe.

    Layout: X and G are variable-major float arrays ([nvars][stride]),
    E is [stride]; thread t of the grid-stride loop handles units t, t+grid, ...
    Explicit .rn rounding keeps ptxas from fusing or reassociating the
    error-free transformations."""
    body = []
    w = body.append

    def two_sum_acc(sh, sl, p, q):
        # (sh, sl) += p + q   with p the main term, q its low-order part
        w("    add.rn.f32 %%ts, %s, %s;" % (sh, p))
        w("    sub.rn.f32 %%tb, %%ts, %s;" % sh)
        w("    sub.rn.f32 %t1, %ts, %tb;")
        w("    sub.rn.f32 %%t1, %s, %%t1;" % sh)
        w("    sub.rn.f32 %%t2, %s, %%tb;" % p)
        w("    add.rn.f32 %t1, %t1, %t2;")
        w("    mov.f32 %s, %%ts;" % sh)
        w("    add.rn.f32 %s, %s, %%t1;" % (sl, sl))
        w("    add.rn.f32 %s, %s, %s;" % (sl, sl, q))

    def prod_df_f(ah, al, x):
        # (p, q) = (ah + al) * x
        w("    mul.rn.f32 %%p, %s, %s;" % (ah, x))
        w("    neg.f32 %np, %p;")
        w("    fma.rn.f32 %%q, %s, %s, %%np;" % (ah, x))
        w("    fma.rn.f32 %%q, %s, %s, %%q;" % (al, x))

    def prod_df_df(ah, al, bh, bl):
        w("    mul.rn.f32 %%p, %s, %s;" % (ah, bh))
        w("    neg.f32 %np, %p;")
        w("    fma.rn.f32 %%q, %s, %s, %%np;" % (ah, bh))
        w("    fma.rn.f32 %%q, %s, %s, %%q;" % (ah, bl))
        w("    fma.rn.f32 %%q, %s, %s, %%q;" % (al, bh))

    X = lambda v: "%%x%d" % v
    for v in range(nvars):
        w("    mov.f32 %%gh%d, 0f00000000;" % v)
        w("    mov.f32 %%gl%d, 0f00000000;" % v)
    w("    mov.f32 %Eh, 0f00000000;")
    w("    mov.f32 %El, 0f00000000;")
    for op in ops:
        kind = op[0]
        if kind == "set":
            hi, lo = split_df(op[2])
            w("    mov.f32 %%V%dh, %s;" % (op[1], f32hex(hi)))
            w("    mov.f32 %%V%dl, %s;" % (op[1], f32hex(lo)))
        elif kind == "p2":
            w("    mul.rn.f32 %%P2h, %s, %s;" % (X(op[1]), X(op[2])))
            w("    neg.f32 %np, %P2h;")
            w("    fma.rn.f32 %%P2l, %s, %s, %%np;" % (X(op[1]), X(op[2])))
        elif kind == "p3":
            prod_df_f("%P2h", "%P2l", X(op[1]))
            w("    mov.f32 %P3h, %p;")
            w("    mov.f32 %P3l, %q;")
        elif kind == "leaf":
            l = op[1]
            hi, lo = split_df(op[2])
            H, L = f32hex(hi), f32hex(lo)
            # V3 += c x_l
            w("    mul.rn.f32 %%p, %s, %s;" % (X(l), H))
            w("    neg.f32 %np, %p;")
            w("    fma.rn.f32 %%q, %s, %s, %%np;" % (X(l), H))
            w("    fma.rn.f32 %%q, %s, %s, %%q;" % (X(l), L))
            two_sum_acc("%V3h", "%V3l", "%p", "%q")
            # g_l += c P3
            w("    mul.rn.f32 %%p, %%P3h, %s;" % H)
            w("    neg.f32 %np, %p;")
            w("    fma.rn.f32 %%q, %%P3h, %s, %%np;" % H)
            w("    fma.rn.f32 %%q, %%P3l, %s, %%q;" % H)
            w("    fma.rn.f32 %%q, %%P3h, %s, %%q;" % L)
            two_sum_acc("%%gh%d" % l, "%%gl%d" % l, "%p", "%q")
        elif kind == "close3":
            k = op[1]
            prod_df_f("%V3h", "%V3l", X(k))
            two_sum_acc("%V2h", "%V2l", "%p", "%q")
            prod_df_df("%V3h", "%V3l", "%P2h", "%P2l")
            two_sum_acc("%%gh%d" % k, "%%gl%d" % k, "%p", "%q")
        elif kind == "close2":
            j, i = op[1], op[2]
            prod_df_f("%V2h", "%V2l", X(j))
            two_sum_acc("%V1h", "%V1l", "%p", "%q")
            prod_df_f("%V2h", "%V2l", X(i))
            two_sum_acc("%%gh%d" % j, "%%gl%d" % j, "%p", "%q")
        elif kind == "close1":
            i = op[1]
            prod_df_f("%V1h", "%V1l", X(i))
            two_sum_acc("%Eh", "%El", "%p", "%q")
            two_sum_acc("%%gh%d" % i, "%%gl%d" % i, "%V1h", "%V1l")
    head = """// Generated by mbpol_openmm_plugin_gb300/codegen/gen_poly.py from data/{name}_basis.txt
// and data/{name}_coeffs.txt.  Do not edit.  {nmono} monomials; depth-first
// trie walk computing value and gradient in double-float (FP32-pair)
// arithmetic (scheme in gen_poly.py).
// X, G: [{nvars}][stride] floats (variable-major); E: [stride] floats.
.version 8.8
.target sm_103a
.address_size 64

.visible .entry {name}_batch(
    .param .u64 pX, .param .u64 pG, .param .u64 pE,
    .param .u32 pN, .param .u32 pStride)
.maxntid 128, 1, 1
{{
    .reg .f32 %x<{nvars}>;
    .reg .f32 %gh<{nvars}>;
    .reg .f32 %gl<{nvars}>;
    .reg .f32 %Eh, %El, %P2h, %P2l, %P3h, %P3l, %V1h, %V1l, %V2h, %V2l, %V3h, %V3l;
    .reg .f32 %p, %q, %np, %ts, %tb, %t1, %t2;
    .reg .u32 %i, %n, %stride, %step, %t0, %tn;
    .reg .u64 %X, %G, %Eb, %off, %rowb, %a;
    .reg .pred %pr;
    ld.param.u64 %X, [pX];
    ld.param.u64 %G, [pG];
    ld.param.u64 %Eb, [pE];
    ld.param.u32 %n, [pN];
    ld.param.u32 %stride, [pStride];
    cvta.to.global.u64 %X, %X;
    cvta.to.global.u64 %G, %G;
    cvta.to.global.u64 %Eb, %Eb;
    mov.u32 %t0, %ctaid.x;
    mov.u32 %tn, %ntid.x;
    mov.u32 %i, %tid.x;
    mad.lo.u32 %i, %t0, %tn, %i;
    mov.u32 %t0, %nctaid.x;
    mul.lo.u32 %step, %t0, %tn;
    mul.wide.u32 %rowb, %stride, 4;
LOOP:
    setp.ge.u32 %pr, %i, %n;
    @%pr bra DONE;
    mul.wide.u32 %off, %i, 4;
""".format(name=name, nmono=nmono, nvars=nvars)
    loads = []
    for v in range(nvars):
        loads.append("    add.u64 %a, %X, %off;" if v == 0 else "    add.u64 %a, %a, %rowb;")
        loads.append("    ld.global.nc.f32 %%x%d, [%%a];" % v)
    stores = []
    for v in range(nvars):
        stores.append("    add.u64 %a, %G, %off;" if v == 0 else "    add.u64 %a, %a, %rowb;")
        stores.append("    add.rn.f32 %%gh%d, %%gh%d, %%gl%d;" % (v, v, v))
        stores.append("    st.global.f32 [%%a], %%gh%d;" % v)
    stores.append("    add.rn.f32 %Eh, %Eh, %El;")
    stores.append("    add.u64 %a, %Eb, %off;")
    stores.append("    st.global.f32 [%a], %Eh;")
    tail = """    add.u32 %i, %i, %step;
    bra.uni LOOP;
DONE:
    ret;
}
"""
    with open(out_path, "w") as f:
        f.write(head + "\n".join(loads) + "\n" + "\n".join(body) + "\n" + "\n".join(stores) + "\n" + tail)


def emulate_df(ops, X):
    """Numpy emulation (FP32 values, FMA as one rounding of an exact FP64
    product-sum) of the emitted walk; X: (nvars, n).  Returns E, G (float64)."""
    import numpy as np
    f = np.float32

    def fma(a, b, c):
        return (a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64)).astype(f)

    n = X.shape[1]
    x = X.astype(f)
    z = lambda: np.zeros(n, f)
    gh = [z() for _ in range(X.shape[0])]
    gl = [z() for _ in range(X.shape[0])]
    st = {k: z() for k in ("Eh", "El", "P2h", "P2l", "P3h", "P3l", "V1h", "V1l", "V2h", "V2l", "V3h", "V3l")}

    def acc(hk, lk, p, q, store=None):
        sh = st[hk] if store is None else store[0][store[1]]
        ts = (sh + p).astype(f)
        tb = (ts - sh).astype(f)
        t1 = (sh - (ts - tb).astype(f)).astype(f)
        t2 = (p - tb).astype(f)
        e = (t1 + t2).astype(f)
        if store is None:
            st[hk] = ts
            st[lk] = ((st[lk] + e).astype(f) + q).astype(f)
        else:
            store[0][store[1]] = ts
            store[2][store[1]] = ((store[2][store[1]] + e).astype(f) + q).astype(f)

    def pdf(ah, al, xv):
        p = (ah * xv).astype(f)
        q = fma(ah, xv, -p)
        return p, fma(al, xv, q)

    for op in ops:
        kind = op[0]
        if kind == "set":
            hi, lo = split_df(op[2])
            st["V%dh" % op[1]] = np.full(n, hi, f)
            st["V%dl" % op[1]] = np.full(n, lo, f)
        elif kind == "p2":
            p = (x[op[1]] * x[op[2]]).astype(f)
            st["P2h"], st["P2l"] = p, fma(x[op[1]], x[op[2]], -p)
        elif kind == "p3":
            st["P3h"], st["P3l"] = pdf(st["P2h"], st["P2l"], x[op[1]])
        elif kind == "leaf":
            l = op[1]
            hi, lo = (np.full(n, v, f) for v in split_df(op[2]))
            p = (x[l] * hi).astype(f)
            q = fma(x[l], lo, fma(x[l], hi, -p))
            acc("V3h", "V3l", p, q)
            p = (st["P3h"] * hi).astype(f)
            q = fma(st["P3h"], lo, fma(st["P3l"], hi, fma(st["P3h"], hi, -p)))
            acc(None, None, p, q, store=(gh, l, gl))
        elif kind == "close3":
            k = op[1]
            p, q = pdf(st["V3h"], st["V3l"], x[k])
            acc("V2h", "V2l", p, q)
            p = (st["V3h"] * st["P2h"]).astype(f)
            q = fma(st["V3l"], st["P2h"], fma(st["V3h"], st["P2l"], fma(st["V3h"], st["P2h"], -p)))
            acc(None, None, p, q, store=(gh, k, gl))
        elif kind == "close2":
            j, i = op[1], op[2]
            p, q = pdf(st["V2h"], st["V2l"], x[j])
            acc("V1h", "V1l", p, q)
            p, q = pdf(st["V2h"], st["V2l"], x[i])
            acc(None, None, p, q, store=(gh, j, gl))
        elif kind == "close1":
            i = op[1]
            p, q = pdf(st["V1h"], st["V1l"], x[i])
            acc("Eh", "El", p, q)
            acc(None, None, st["V1h"], st["V1l"], store=(gh, i, gl))
    E = (st["Eh"] + st["El"]).astype(f).astype(np.float64)
    G = np.stack([(gh[v] + gl[v]).astype(f).astype(np.float64) for v in range(X.shape[0])])
    return E, G


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
