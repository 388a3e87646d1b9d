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

* ``csrc/gen/poly2b.ptx`` / ``poly3b.ptx`` — straight-line FP32 PTX
  kernels (coefficients become FFMA immediates, no coefficient memory
  traffic), assembled by ptxas alone: nvcc's front end takes tens of minutes
  on a function this long, ptxas about twenty seconds;
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


def emit_ptx(name, nvars, root, perm, out_path, nmono):
    """Write a standalone PTX kernel ``<name>_batch``.

    Layout: X and G are variable-major float arrays ([nvars][stride]),
    E is [stride]; thread t of the grid-stride loop handles units t, t+grid, ...
    The depth-first walk is written instruction by instruction so that at
    most ~nvars*2+8 values are live."""
    inv = [0] * nvars
    for v, label in enumerate(perm):
        inv[label] = v
    body = []
    w = body.append

    def X(label):
        return "%%x%d" % inv[label]

    def G(label):
        return "%%g%d" % inv[label]

    for v in range(nvars):
        w("    mov.f32 %%g%d, 0f00000000;" % v)
    w("    mov.f32 %E, 0f00000000;")
    for l1 in sorted(root["ch"]):
        n1 = root["ch"][l1]
        w("    mov.f32 %%V1, %s;" % f32hex(n1["c"]))
        if n1["ch"]:
            w("    mov.f32 %%P1, %s;" % X(l1))
        for l2 in sorted(n1["ch"]):
            n2 = n1["ch"][l2]
            w("    mov.f32 %%V2, %s;" % f32hex(n2["c"]))
            if n2["ch"]:
                w("    mul.rn.f32 %%P2, %%P1, %s;" % X(l2))
            for l3 in sorted(n2["ch"]):
                n3 = n2["ch"][l3]
                w("    mov.f32 %%V3, %s;" % f32hex(n3["c"]))
                if n3["ch"]:
                    w("    mul.rn.f32 %%P3, %%P2, %s;" % X(l3))
                for l4 in sorted(n3["ch"]):
                    c4 = f32hex(n3["ch"][l4]["c"])
                    assert not n3["ch"][l4]["ch"]
                    w("    fma.rn.f32 %%V3, %s, %s, %%V3;" % (X(l4), c4))
                    w("    fma.rn.f32 %s, %%P3, %s, %s;" % (G(l4), c4, G(l4)))
                w("    fma.rn.f32 %%V2, %%V3, %s, %%V2;" % X(l3))
                w("    fma.rn.f32 %s, %%V3, %%P2, %s;" % (G(l3), G(l3)))
            w("    fma.rn.f32 %%V1, %%V2, %s, %%V1;" % X(l2))
            w("    fma.rn.f32 %s, %%V2, %%P1, %s;" % (G(l2), G(l2)))
        w("    fma.rn.f32 %%E, %%V1, %s, %%E;" % X(l1))
        w("    add.rn.f32 %s, %s, %%V1;" % (G(l1), G(l1)))
    head = """// Generated by mbpol_openmm_plugin_gb300/codegen/gen_poly.py from data/{name}_basis.txt
// and data/{name}_coeffs.txt.  Do not edit.  {nmono} monomials; depth-first
// trie walk computing value and gradient in FP32 (scheme in gen_poly.py).
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
    .reg .f32 %g<{nvars}>;
    .reg .f32 %E, %P1, %P2, %P3, %V1, %V2, %V3;
    .reg .u32 %i, %n, %stride, %step, %t0, %t1;
    .reg .u64 %X, %G, %Eb, %off, %rowb, %a;
    .reg .pred %p;
    ld.param.u64 %X, [pX];
    ld.param.u64 %G, [pG];
    ld.param.u64 %Eb, [pE];
    ld.param.u32 %n, [pN];
    ld.param.u32 %stride, [pStride];
    cvta.to.global.u64 %X, %X;
    cvta.to.global.u64 %G, %G;
    cvta.to.global.u64 %Eb, %Eb;
    mov.u32 %t0, %ctaid.x;
    mov.u32 %t1, %ntid.x;
    mad.lo.u32 %i, %t0, %t1, %tid.x;
    mov.u32 %t0, %nctaid.x;
    mul.lo.u32 %step, %t0, %t1;
    mul.wide.u32 %rowb, %stride, 4;
LOOP:
    setp.ge.u32 %p, %i, %n;
    @%p bra DONE;
    mul.wide.u32 %off, %i, 4;
""".format(name=name, nmono=nmono, nvars=nvars)
    loads = []
    for v in range(nvars):
        if v == 0:
            loads.append("    add.u64 %a, %X, %off;")
        else:
            loads.append("    add.u64 %a, %a, %rowb;")
        loads.append("    ld.global.nc.f32 %%x%d, [%%a];" % v)
    stores = []
    for v in range(nvars):
        if v == 0:
            stores.append("    add.u64 %a, %G, %off;")
        else:
            stores.append("    add.u64 %a, %a, %rowb;")
        stores.append("    st.global.f32 [%%a], %%g%d;" % v)
    stores.append("    add.u64 %a, %Eb, %off;")
    stores.append("    st.global.f32 [%a], %E;")
    tail = """    add.u32 %i, %i, %step;
    bra.uni LOOP;
DONE:
    ret;
}
"""
    with open(out_path, "w") as f:
        f.write(head + "\n".join(loads) + "\n" + "\n".join(body) + "\n" + "\n".join(stores) + "\n" + tail)


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
    emit_ptx(name, nvars, root, perm, os.path.join(cuda_dir, "%s.ptx" % name), len(mono))
    emit_prog(name, nvars, root, perm, os.path.join(prog_dir, "%s_prog.h" % name), len(mono))
    print("%s: %d monomials, cost %d ops" % (name, len(mono), trie_cost(mono)))


if __name__ == "__main__":
    for n in sys.argv[1:] or ["poly2b", "poly3b"]:
        generate(n)
