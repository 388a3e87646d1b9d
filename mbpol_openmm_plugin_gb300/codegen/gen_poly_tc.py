"""Tables for the tensor-core evaluation of the MB-pol three-body polynomial
(csrc/poly_tc.cu).  This project's own formulation; the reference evaluates
the generated straight-line code of platforms/reference/src/poly-3b-v2x.cpp
in FP64.

1. Shift.  With d = x - x0 (x0 from data/poly*_shift.txt, chosen by
   codegen/choose_shift.py), the polynomial E(x) = sum_m c_m x^m of degree
   <= 4 is re-expanded exactly (FP64) as E = sum_m c'_m d^m.  Its terms
   cancel ~250x less than the original ones.
2. Quadratic form.  With y the degree <= 2 monomials of d
   (y = [1, d_0..d_{n-1}, d_i d_j (i <= j)], NY = 1 + n + n(n+1)/2 rows),
   every monomial of degree <= 4 is a product y_p y_q; placing each once
   gives a matrix C with E = y^T C y, and with S = (C + C^T)/2
       z = S y,   E = y . z,   dE/dd_i = 2 sum_m z_m dy_m/dd_i.
   z for a tile of units is one matrix product S[NY x NY] . Y[NY x units]:
   the tensor-core part.
3. Operands in fp16.  Row k of Y is scaled by 2^s_k (s_k from the sampled
   bound of |y_k|, so that |y'_k| <= 2^12 there); the columns of S are
   scaled back and each row of the result by 2^r_m (|row| <= 2^14).  The
   scaled S is split into three fp16 pieces (S = S0 + S1 + S2 to ~33 bits)
   and Y' into two (22 bits) by the kernel; the products S0Y0 + S0Y1 + S1Y0
   + S2Y0 are accumulated per 16-wide k-tile and added to FP32 sums.
4. Sparsity.  S is stored as 16x16 tiles in the register layout of the
   A operand of mma.m16n8k16 (PTX ISA, "Matrix fragments for
   mma.m16n8k16": lane l = 4g + q holds rows g, g+8 and columns 2q, 2q+1,
   2q+8, 2q+9); all-zero tiles are left out.  Row tiles are dealt to the
   kernel's eight warps by their tile counts (longest first).

The two-body polynomial stays on the double-float walk (csrc/poly_df.cu):
its coulomb-like variables range over [0.001, 46] and its long-range pairs
are ~0.03 kcal/mol sums of 1e3 terms, so the shift leaves a cancellation of
~3e5, and FP32-accumulated products measured (in an FP32 emulation of this
scheme) 5e-5 relative error of the summed two-body energy.  `build` works
for either; `generate` emits the three-body tables.

Output: a C++ source with the tables, written next to the build objects by
build.py.  `evaluate` computes value and gradient from the tables in FP64
and `trie_eval` from the unshifted monomials; the CPU tests compare them.
"""
import itertools
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
DATA = os.path.join(PKG, "data")
sys.path.insert(0, os.path.dirname(PKG))
from mbpol_openmm_plugin_gb300.codegen import gen_poly  # noqa: E402

NWARPS = 8
TC5_PARTS = 3     # tcgen05 kernel: K split, rows of S per chunk
TC5_ROWS = 64
Y_LOG2_MAX = 12   # |y'_k| <= 2^12 over the sampled inputs
S_LOG2_MAX = 14   # max |scaled row of S| = 2^14


def load_shift(name):
    x0, bnd = [], []
    for line in open(os.path.join(DATA, "%s_shift.txt" % name)):
        if line.startswith("#"):
            continue
        t = line.split()
        x0.append(float(t[1]))
        bnd.append(float(t[2]))
    return np.array(x0), np.array(bnd)


def shifted_monomials(mono, x0):
    """{sorted monomial of d: coefficient} of sum_m c_m prod (x0_v + d_v)."""
    out = {}
    for m, c in mono.items():
        for keep in itertools.product((0, 1), repeat=len(m)):
            coef = c
            key = []
            for v, k in zip(m, keep):
                if k:
                    key.append(v)
                else:
                    coef *= x0[v]
            key = tuple(key)
            out[key] = out.get(key, 0.0) + coef
    return out


def ylist(nv):
    return [()] + [(i,) for i in range(nv)] + [(i, j) for i in range(nv) for j in range(i, nv)]


def quad_matrix(smono, nv):
    ys = ylist(nv)
    idx = {m: k for k, m in enumerate(ys)}
    ny = len(ys)
    C = np.zeros((ny, ny))
    for m, c in smono.items():
        d = len(m)
        if d <= 2:
            p, q = (), m
        elif d == 3:
            p, q = m[:1], m[1:]
        else:
            p, q = m[:2], m[2:]
        C[idx[p], idx[q]] += c
    return 0.5 * (C + C.T), ys


def pow2_exp(v):
    """e with 2^(e-1) < v <= 2^e (v > 0)."""
    return int(np.ceil(np.log2(v)))


def f16_split(a, npieces):
    parts = []
    r = a.astype(np.float64)
    for _ in range(npieces):
        h = r.astype(np.float16)
        parts.append(h)
        r = r - h.astype(np.float64)
    return parts


class TCTables:
    pass


def build(name):
    nv, rows = gen_poly.load_basis("%s_basis.txt" % name)
    coeffs = gen_poly.load_coeffs("%s_coeffs.txt" % name)
    mono = gen_poly.merged_monomials(rows, coeffs, list(range(nv)))
    x0, bnd = load_shift(name)
    smono = shifted_monomials(mono, x0)
    S, ys = quad_matrix(smono, nv)
    ny = len(ys)
    npad = (ny + 15) // 16 * 16
    # row scale of Y': |y'_k| <= 2^Y_LOG2_MAX at the sampled bounds
    ybound = np.array([np.prod([bnd[v] for v in m]) if m else 1.0 for m in ys])
    s_exp = np.array([Y_LOG2_MAX - pow2_exp(b) for b in ybound], dtype=np.int64)
    Sc = S * np.ldexp(1.0, -s_exp)[None, :]
    rmax = np.abs(Sc).max(axis=1)
    r_exp = np.array([S_LOG2_MAX - pow2_exp(v) if v > 0 else 0 for v in rmax], dtype=np.int64)
    A = np.zeros((npad, npad))
    A[:ny, :ny] = Sc * np.ldexp(1.0, r_exp)[:, None]
    pieces = f16_split(A, 3)
    assert all(np.isfinite(p.astype(np.float64)).all() for p in pieces)
    nt = npad // 16
    occ = np.zeros((nt, nt), bool)
    for p in pieces:
        occ |= (p.astype(np.float64) != 0).reshape(nt, 16, nt, 16).any(axis=(1, 3))
    # deal row tiles to warps, longest first (each row tile is one warp's)
    counts = occ.sum(axis=1)
    load = [0] * NWARPS
    owned = [[] for _ in range(NWARPS)]
    for rt in sorted(range(nt), key=lambda r: (-counts[r], r)):
        w = min(range(NWARPS), key=lambda i: (load[i], i))
        owned[w].append(rt)
        load[w] += int(counts[rt]) + 2   # +2: the row tile's write-out
    warp_begin, rt_id, rt_entry, ent_kt = [0], [], [0], []
    frag = []
    lanes = np.arange(32)
    g, q = lanes >> 2, lanes & 3
    for w in range(NWARPS):
        for rt in sorted(owned[w]):
            rt_id.append(rt)
            for kt in np.nonzero(occ[rt])[0]:
                ent_kt.append(int(kt))
                for p in pieces:
                    bits = p.view(np.uint16)
                    r0, c0 = rt * 16, kt * 16

                    def pk(rr, cc):
                        return bits[r0 + rr, c0 + cc].astype(np.uint32) | (
                            bits[r0 + rr, c0 + cc + 1].astype(np.uint32) << 16)
                    frag.append(np.stack([pk(g, 2 * q), pk(g + 8, 2 * q), pk(g, 2 * q + 8), pk(g + 8, 2 * q + 8)],
                                         axis=1))   # [32 lanes][4 regs]
            rt_entry.append(len(ent_kt))
        warp_begin.append(len(rt_id))
    t = TCTables()
    t.name, t.nv, t.ny, t.npad = name, nv, ny, npad
    t.x0, t.bnd, t.ys, t.S = x0, bnd, ys, S
    t.s_exp, t.r_exp = s_exp, r_exp
    t.pieces = pieces
    t.occ = occ
    t.warp_begin = np.array(warp_begin, np.int32)
    t.rt_id = np.array(rt_id, np.int32)
    t.rt_entry = np.array(rt_entry, np.int32)
    t.ent_kt = np.array(ent_kt, np.int32)
    t.frag = np.array(frag, np.uint32).reshape(-1)   # [entry][piece][lane][reg]
    t.nmono = len(smono)
    tc5_stream(t)
    return t


def tc5_stream(t):
    """The S blocks of the tcgen05 kernel (csrc/poly_tc5.cu), in the order
    it consumes them: K in TC5_PARTS parts (Y' of one part is held in tensor
    memory), then chunks of TC5_ROWS rows of S (the N of the MMA), then the
    part's 16-wide k-tiles with a nonzero entry in the chunk.  A block holds
    the three fp16 pieces, each TC5_ROWS x 16 in the no-swizzle K-major
    layout of a shared-memory operand: 8-row x 16-byte core matrices,
    [k half][row group][row][8 k] (PTX ISA, "Shared memory descriptor",
    canonical K-major layout without swizzling)."""
    nkt = t.npad // 16
    nch = t.npad // TC5_ROWS
    bounds = tc5_part_bounds(nkt)
    assert t.npad % TC5_ROWS == 0
    occ = np.zeros((nch, nkt), bool)
    for p in t.pieces:
        occ |= (p.astype(np.float64) != 0).reshape(nch, TC5_ROWS, nkt, 16).any(axis=(1, 3))
    blocks, kt_local, begin = [], [], [0]
    for part in range(TC5_PARTS):
        for c in range(nch):
            for kt in range(bounds[part], bounds[part + 1]):
                if not occ[c, kt]:
                    continue
                kt_local.append(kt - bounds[part])
                for p in t.pieces:
                    sub = p.view(np.uint16)[c * TC5_ROWS:(c + 1) * TC5_ROWS, kt * 16:(kt + 1) * 16]
                    # [row group][row][k half][8 k] -> [k half][row group][row][8 k]
                    blocks.append(sub.reshape(TC5_ROWS // 8, 8, 2, 8).transpose(2, 0, 1, 3).reshape(-1))
            begin.append(len(kt_local))
    t.tc5_sblk = np.concatenate(blocks).astype(np.uint16)
    t.tc5_kt = np.array(kt_local, np.uint8)
    t.tc5_begin = np.array(begin, np.int32)      # [parts * chunks + 1]


def tc5_part_bounds(nkt):
    """First k-tile of each K part (the kernel computes the same)."""
    return [(p * nkt + TC5_PARTS - 1) // TC5_PARTS for p in range(TC5_PARTS + 1)]


def tc5_dense(t):
    """The scaled S (sum of the pieces, FP64) rebuilt from the tcgen05 block
    stream: the CPU tests compare it with the pieces."""
    nch = t.npad // TC5_ROWS
    bounds = tc5_part_bounds(t.npad // 16)
    A = np.zeros((t.npad, t.npad))
    per = 3 * TC5_ROWS * 16
    for part in range(TC5_PARTS):
        for c in range(nch):
            i = part * nch + c
            for b in range(t.tc5_begin[i], t.tc5_begin[i + 1]):
                kt = bounds[part] + int(t.tc5_kt[b])
                for q in range(3):
                    raw = t.tc5_sblk[b * per + q * TC5_ROWS * 16:b * per + (q + 1) * TC5_ROWS * 16]
                    sub = raw.reshape(2, TC5_ROWS // 8, 8, 8).transpose(1, 2, 0, 3).reshape(TC5_ROWS, 16)
                    A[c * TC5_ROWS:(c + 1) * TC5_ROWS, kt * 16:(kt + 1) * 16] += sub.view(np.float16).astype(np.float64)
    return A


def ymeta(t):
    """Per Y row k (padded): a, b (variable indices; nv stands for the
    factor 1, nv + 1 for 0 in padding rows), s_exp."""
    a = np.full(t.npad, t.nv + 1, np.int32)
    b = np.full(t.npad, t.nv, np.int32)
    s = np.zeros(t.npad, np.int32)
    for k, m in enumerate(t.ys):
        a[k] = m[0] if len(m) >= 1 else t.nv
        if len(m) == 2:
            b[k] = m[1]
        s[k] = t.s_exp[k]
    return a, b, s


def emit(tables, path):
    lines = ["// Generated by mbpol_openmm_plugin_gb300/codegen/gen_poly_tc.py from data/poly*_basis.txt,",
             "// data/poly*_coeffs.txt and data/poly*_shift.txt.  Do not edit.",
             '#include "poly_tc.h"', "namespace mbpol {"]

    def arr(ctype, sym, vals, fmt="%d", per=16):
        lines.append("static const %s %s[%d] = {" % (ctype, sym, len(vals)))
        for i in range(0, len(vals), per):
            lines.append(",".join(fmt % v for v in vals[i:i + per]) + ",")
        lines.append("};")

    for t in tables:
        n = t.name
        a, b, s = ymeta(t)
        x0h = t.x0.astype(np.float32)
        x0l = (t.x0 - x0h.astype(np.float64)).astype(np.float32)
        arr("float", n + "_x0h", [float.hex(float(v)) + "f" for v in x0h], "%s", 8)
        arr("float", n + "_x0l", [float.hex(float(v)) + "f" for v in x0l], "%s", 8)
        arr("float", n + "_inv_bound", [float.hex(float(np.float32(1.0 / v))) + "f" for v in t.bnd], "%s", 8)
        meta = (a.astype(np.uint32) | (b.astype(np.uint32) << 8) | ((s + 128).astype(np.uint32) << 16))
        arr("unsigned int", n + "_ymeta", meta.tolist())
        rs = np.zeros(t.npad)
        rs[:t.ny] = np.ldexp(1.0, -t.r_exp)
        arr("float", n + "_rowscale", [float.hex(float(v)) + "f" for v in rs], "%s", 8)
        arr("int", n + "_warp_begin", t.warp_begin.tolist())
        arr("int", n + "_rt_id", t.rt_id.tolist())
        arr("int", n + "_rt_entry", t.rt_entry.tolist())
        arr("unsigned short", n + "_ent_kt", t.ent_kt.tolist())
        arr("unsigned int", n + "_frag", ["0x%08x" % v for v in t.frag.tolist()], "%s", 12)
        arr("unsigned short", n + "_sblk", ["0x%04x" % v for v in t.tc5_sblk.tolist()], "%s", 16)
        arr("unsigned char", n + "_blk_kt", t.tc5_kt.tolist())
        arr("int", n + "_blk_begin", t.tc5_begin.tolist())
        lines.append("extern const PolyTCTables k_%s = {%d, %d, %d, %d, %d, %s_x0h, %s_x0l, %s_inv_bound, %s_ymeta,"
                     " %s_rowscale, %s_warp_begin, %s_rt_id, %s_rt_entry, %s_ent_kt, %s_frag, %d, %d, %d,"
                     " %s_sblk, %s_blk_kt, %s_blk_begin};" % (
                         n, t.nv, t.ny, t.npad, len(t.rt_id), len(t.ent_kt), n, n, n, n, n, n, n, n, n, n,
                         TC5_PARTS, TC5_ROWS, len(t.tc5_kt), n, n, n))
    lines.append("}  // namespace mbpol")
    text = "\n".join(lines) + "\n"
    if not os.path.exists(path) or open(path).read() != text:
        with open(path, "w") as f:
            f.write(text)


def evaluate(t, X):
    """FP64 evaluation of the tables (sum of the three S pieces, unscaled):
    value and gradient for inputs X [units][nv]."""
    D = X - t.x0
    ny = t.ny
    Y = np.ones((len(X), ny))
    for k, m in enumerate(t.ys):
        for v in m:
            Y[:, k] *= D[:, v]
    A = sum(p.astype(np.float64) for p in t.pieces)[:ny, :ny]
    S = A * np.ldexp(1.0, -t.r_exp)[:, None] * np.ldexp(1.0, t.s_exp)[None, :]
    Z = Y @ S.T
    E = (Y * Z).sum(axis=1)
    G = np.zeros_like(X)
    for k, m in enumerate(t.ys):
        if len(m) == 1:
            G[:, m[0]] += 2 * Z[:, k]
        elif len(m) == 2:
            i, j = m
            if i == j:
                G[:, i] += 4 * Z[:, k] * D[:, i]
            else:
                G[:, i] += 2 * Z[:, k] * D[:, j]
                G[:, j] += 2 * Z[:, k] * D[:, i]
    return E, G


def trie_eval(name, X):
    """FP64 value and gradient of the unshifted polynomial (the trie walk of
    gen_poly, vectorised over units)."""
    nv, rows = gen_poly.load_basis("%s_basis.txt" % name)
    coeffs = gen_poly.load_coeffs("%s_coeffs.txt" % name)
    mono = gen_poly.merged_monomials(rows, coeffs, list(range(nv)))
    E = np.zeros(len(X))
    G = np.zeros_like(X)
    for m, c in mono.items():
        t = c * np.prod(X[:, list(m)], axis=1)
        E += t
        for pos, v in enumerate(m):
            rest = list(m[:pos]) + list(m[pos + 1:])
            G[:, v] += c * np.prod(X[:, rest], axis=1) if rest else c
    return E, G


def generate(out_path):
    tabs = [build("poly3b")]
    emit(tabs, out_path)
    for t in tabs:
        print("%s: %d shifted monomials, NY %d (padded %d), %d of %d tiles kept, per-warp tiles %s; "
              "tcgen05 stream: %d blocks of %d rows" % (
                  t.name, t.nmono, t.ny, t.npad, len(t.ent_kt), (t.npad // 16) ** 2,
                  [int(t.rt_entry[t.warp_begin[w + 1]] - t.rt_entry[t.warp_begin[w]]) for w in range(NWARPS)],
                  len(t.tc5_kt), TC5_ROWS))
    return tabs


if __name__ == "__main__":
    generate(sys.argv[1] if len(sys.argv) > 1 else os.path.join(PKG, "_build", "poly_tc_tables.cpp"))
