// Data-driven double-float evaluation of the MB-pol 2-body and 3-body
// permutationally-invariant polynomials (value and gradient).
//
// The polynomial E(x) = sum_m c_m x^m (degree <= 4; 12,725 monomials for the
// two-body term, 33,525 for the three-body term; basis extracted from
// platforms/reference/src/poly-2b-v6x.cpp and poly-3b-v2x.cpp) is stored as a
// trie (codegen/gen_poly.py).  A depth-first walk computes E and dE/dx with
// O(1) live state per level:
//     P_d = P_{d-1} x_{v_d};  V_d = c_d + sum_children x_child V_child;
//     g_{v_d} += V_d P_{d-1};  E = V_root.
// Plain FP32 is not accurate enough: the monomial terms cancel by a factor of
// 1e4-1e5, leaving ~1e-3 relative error.  Every accumulation is therefore a
// pair (s, c) of FP32 values updated Dot2-style (error-free TwoProd by FMA
// and TwoSum, errors collected in c; Ogita, Rump & Oishi, SIAM J. Sci.
// Comput. 26 (2005)), which gives FP64-level results on the FP32 pipe.
//
// kParts threads per unit (dimer or trimer), each walking a part of the trie.
// The variables x ([variable][unit]) and the gradient ([variable][thread])
// live in shared memory as (hi, lo) float2 pairs, so every access of a warp
// is one conflict-free 8-byte load or store; the trie tables are read with
// warp-uniform addresses.  X: [2][nvars][stride] floats (FP64 variables as
// hi and lo planes); G: [nvars][stride]; E: [stride].
#include <memory>
#include <mutex>
#include <vector>

#include "mbpol_internal.cuh"
#include "poly_tables.h"

namespace mbpol {

#include "gen/poly2b_tables.inc"
#include "gen/poly3b_tables.inc"

namespace {

// Each unit (dimer or trimer) is walked by kParts threads, each taking a
// contiguous part of the trie; a block holds kUnits units.
#ifndef MBPOL_WALK_PARTS
#define MBPOL_WALK_PARTS 3
#endif
constexpr int kParts = MBPOL_WALK_PARTS;
constexpr int kUnits = 64;
constexpr int kBlock = kParts * kUnits;
// resident blocks per SM (shared memory: three-body block of
// 36 * (kUnits + kBlock) * 8 bytes plus static data)
constexpr int kBlocksPerSm = kParts == 2 ? 4 : (kParts == 3 ? 3 : 1);
// Blocks left out of the walk's persistent grid, so that the electrostatics
// stream finds room beside it: with three parts the walk alone is fastest
// on every SM, but the electrostatics then end the learned-guess MD step.
// Measured on box4096 (ms per step over 1000 steps): 0 blocks 12.48, 12
// blocks 12.14, 24 blocks 12.02, 36 blocks 12.19; two parts 12.32.
#ifndef MBPOL_WALK_RESERVE_BLOCKS
#define MBPOL_WALK_RESERVE_BLOCKS 24
#endif

struct DF {
    float h, l;
};

// (a.h + a.l) += p + q, p the leading part (TwoSum of a.h and p)
__device__ __forceinline__ void acc(DF& a, float p, float q) {
    const float s = __fadd_rn(a.h, p);
    const float bb = __fsub_rn(s, a.h);
    const float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    a.h = s;
    a.l = __fadd_rn(a.l, __fadd_rn(e, q));
}

// (p, q) = (a.h + a.l) * x
__device__ __forceinline__ void mul_df_f(const DF a, float x, float& p, float& q) {
    p = __fmul_rn(a.h, x);
    q = __fmaf_rn(a.h, x, -p);
    q = __fmaf_rn(a.l, x, q);
}

// (p, q) = (a.h + a.l) * (b.h + b.l), dropping a.l * b.l
__device__ __forceinline__ void mul_df_df(const DF a, const DF b, float& p, float& q) {
    p = __fmul_rn(a.h, b.h);
    q = __fmaf_rn(a.h, b.h, -p);
    q = __fmaf_rn(a.h, b.l, q);
    q = __fmaf_rn(a.l, b.h, q);
}

// One leaf L (coefficient c, variable l) under a level-3 node with prefix
// product P3: V3 += c x_l and g_l += c P3.
__device__ __forceinline__ void leaf_update(const PolyNode& L, float xl, float xll, const DF& P3, DF& V3, DF& g) {
    float p, q;
    p = __fmul_rn(xl, L.hi);
    q = __fmaf_rn(xl, L.hi, -p);
    q = __fmaf_rn(xl, L.lo, q);
    q = __fmaf_rn(xll, L.hi, q);
    acc(V3, p, q);
    p = __fmul_rn(P3.h, L.hi);
    q = __fmaf_rn(P3.h, L.hi, -p);
    q = __fmaf_rn(P3.l, L.hi, q);
    q = __fmaf_rn(P3.h, L.lo, q);
    acc(g, p, q);
}

// Shared-memory strides: the variables are shared by the two threads of a
// unit ([variable][unit]), each thread has its own gradient pairs
// ([variable][thread]).
constexpr int kXS = kUnits;         // variable plane stride
constexpr int kGS = kBlock;         // gradient plane stride

// U sibling nodes without children (leaves, or level-3 nodes without
// leaves) under a parent with prefix product P: V += c x and g += c P for
// each, with all loads first, then the updates in order (V's summation order
// is unchanged), then the stores.  Siblings have distinct variables.  xv
// points at this thread's unit, gv at this thread's gradient column; both
// hold (hi, lo) pairs, one 8-byte access each.
template <int U>
__device__ __forceinline__ void childless_batch(const PolyNode (&L)[U], const float2* xv, float2* gv, const DF& P,
                                                DF& V) {
    float2 x[U], g[U];
    #pragma unroll
    for (int u = 0; u < U; ++u) {
        x[u] = xv[L[u].var * kXS];
        g[u] = gv[L[u].var * kGS];
    }
    #pragma unroll
    for (int u = 0; u < U; ++u) {
        DF gu = {g[u].x, g[u].y};
        leaf_update(L[u], x[u].x, x[u].y, P, V, gu);
        g[u] = make_float2(gu.h, gu.l);
    }
    #pragma unroll
    for (int u = 0; u < U; ++u) gv[L[u].var * kGS] = g[u];
}

template <int U>
__device__ __forceinline__ void leaf_batch(const PolyNode* __restrict__ lv, const float2* xv, float2* gv,
                                           const DF& P3, DF& V3) {
    PolyNode L[U];
    #pragma unroll
    for (int u = 0; u < U; ++u) L[u] = lv[u];
    childless_batch<U>(L, xv, gv, P3, V3);
}

// One part of the trie: level-1 nodes [a0, a1), level-2 nodes [c2_0, c2_1)
// and the level-3 nodes and leaves under them, which start at c3_0 and
// cl_0.  When a cut falls inside the children of a level-1 node, the parts
// on both sides visit that node and all but the first leave out its
// coefficient (skip_coef): E = sum_i x_i V_i and g_i += V_i are linear in
// V_i.
struct WalkPart {
    int a0, a1, c2_0, c2_1, c3_0, cl_0, skip_coef;
};
struct WalkSplit {
    WalkPart part[kParts];
};

// kParts threads per unit (dimer or trimer), each walking a part of the
// trie: the unit's variables are stored once for all of them, so a thread
// needs NV * (8 + 8 / kParts) bytes of shared memory (its gradient pairs
// and its share of the variables).  With three parts an SM holds three
// 192-thread blocks (18 warps; two parts held 16, one part 12).  The parts'
// energy and gradient pairs are added at the end (double-float, fixed
// order).  The registers are capped at 80 per thread, so that a quarter of
// the register file stays free for the electrostatics kernels of the other
// stream, which then run beside the walk (a cap of 72 made the walk slower
// than the overlap gains).
template <int NV>
__global__ void __launch_bounds__(kBlock, 768 / kBlock) poly_df_kernel(const PolyNode* __restrict__ l1,
                                                          const PolyNode* __restrict__ l2,
                                                          const PolyNode* __restrict__ l3, int n3,
                                                          const PolyNode* __restrict__ lv, const WalkSplit split,
                                                          const float* __restrict__ X, float* __restrict__ G,
                                                          float* __restrict__ E, int n, int stride) {
    extern __shared__ float2 smem2[];
    float2* xv_all = smem2;                  // [NV][kUnits]  variables (hi, lo)
    float2* gv_all = xv_all + NV * kUnits;   // [NV][kBlock]  gradient pairs
    __shared__ float e_other[kParts - 1][2][kUnits];  // the other parts' energy pairs
    const int t = threadIdx.x;
    const int part = t / kUnits;             // warp-uniform
    const int tu = t % kUnits;
    // this thread's part, selected field by field (no dynamic indexing of
    // the parameter array)
    WalkPart W = split.part[0];
    #pragma unroll
    for (int k = 1; k < kParts; ++k)
        if (part == k) {
            W.a0 = split.part[k].a0;
            W.a1 = split.part[k].a1;
            W.c2_0 = split.part[k].c2_0;
            W.c2_1 = split.part[k].c2_1;
            W.c3_0 = split.part[k].c3_0;
            W.cl_0 = split.part[k].cl_0;
            W.skip_coef = split.part[k].skip_coef;
        }
    const float2* xv = xv_all + tu;
    float2* gv = gv_all + t;
    for (int base = blockIdx.x * kUnits; base < n; base += gridDim.x * kUnits) {
        const int u = base + tu;
        const bool live = u < n;
        for (int v = part; v < NV; v += kParts)
            xv_all[v * kXS + tu] = live ? make_float2(X[(size_t)v * stride + u], X[(size_t)(NV + v) * stride + u])
                                        : make_float2(0.f, 0.f);
        #pragma unroll
        for (int v = 0; v < NV; ++v) gv[v * kGS] = make_float2(0.f, 0.f);
        __syncthreads();
        DF Ev = {0.f, 0.f};
        int c2 = W.c2_0, c3 = W.c3_0, cl = W.cl_0;
        // The next level-3 node is read one step ahead.  Children of a node
        // have distinct variables, so several leaves' gradient pairs can be
        // read before any of them is written back; a parent's own pair is
        // read only after its children's writes (a child may share its
        // variable).
        PolyNode Cn = c3 < n3 ? l3[c3] : PolyNode{0.f, 0.f, 0, 0};
        for (int a = W.a0; a < W.a1; ++a) {
            const PolyNode A = l1[a];
            const float2 xa = xv[A.var * kXS];
            const float xi = xa.x, xil = xa.y;
            DF V1 = {A.hi, A.lo};
            if (a == W.a0 && W.skip_coef) V1 = DF{0.f, 0.f};
            const int e2 = min(A.end, W.c2_1);
            for (; c2 < e2; ++c2) {
                const PolyNode B = l2[c2];
                const float2 xb = xv[B.var * kXS];
                const float xj = xb.x, xjl = xb.y;
                DF V2 = {B.hi, B.lo};
                DF P2;
                P2.h = __fmul_rn(xi, xj);
                P2.l = __fmaf_rn(xi, xj, -P2.h);
                P2.l = __fmaf_rn(xi, xjl, P2.l);
                P2.l = __fmaf_rn(xil, xj, P2.l);
                for (; c3 < B.end; ++c3) {
                    const PolyNode C = Cn;
                    if (NV == 31 && C.end == cl && c3 + 4 <= B.end) {
                        // four level-3 nodes without leaves act as four leaves
                        // of B (prefix product P2); taken for the two-body trie,
                        // where 90% of the level-3 nodes have no leaves (in the
                        // three-body trie the look-ahead loads measured slower)
                        const PolyNode C4[4] = {C, l3[c3 + 1], l3[c3 + 2], l3[c3 + 3]};
                        if (C4[1].end == cl && C4[2].end == cl && C4[3].end == cl) {
                            childless_batch<4>(C4, xv, gv, P2, V2);
                            c3 += 3;
                            if (c3 + 1 < n3) Cn = l3[c3 + 1];
                            continue;
                        }
                    }
                    if (c3 + 1 < n3) Cn = l3[c3 + 1];
                    const float2 xc = xv[C.var * kXS];
                    const float xk = xc.x, xkl = xc.y;
                    DF V3 = {C.hi, C.lo};
                    const int cend = C.end;
                    if (cl < cend) {
                        DF P3;
                        mul_df_f(P2, xk, P3.h, P3.l);
                        P3.l = __fmaf_rn(P2.h, xkl, P3.l);
                        // leaves in batches of four: their nodes and operands are
                        // loaded together, so the L2 latency of the node reads
                        // overlaps (leaf variables of one node are distinct;
                        // batches of eight measured slower)
                        if (NV == 31 && cl + 4 <= cend) {
                            // two-body trie: the next batch's nodes are read
                            // while this batch computes (in the three-body
                            // trie this look-ahead measured slower)
                            PolyNode Lc[4];
                            #pragma unroll
                            for (int w = 0; w < 4; ++w) Lc[w] = lv[cl + w];
                            for (;;) {
                                const bool more = cl + 8 <= cend;
                                PolyNode Ln[4];
                                if (more) {
                                    #pragma unroll
                                    for (int w = 0; w < 4; ++w) Ln[w] = lv[cl + 4 + w];
                                }
                                childless_batch<4>(Lc, xv, gv, P3, V3);
                                cl += 4;
                                if (!more) break;
                                #pragma unroll
                                for (int w = 0; w < 4; ++w) Lc[w] = Ln[w];
                            }
                        }
                        for (; cl + 4 <= cend; cl += 4) leaf_batch<4>(lv + cl, xv, gv, P3, V3);
                        for (; cl < cend; ++cl) {
                            const PolyNode L = lv[cl];
                            const float2 xl = xv[L.var * kXS], g0 = gv[L.var * kGS];
                            DF g = {g0.x, g0.y};
                            leaf_update(L, xl.x, xl.y, P3, V3, g);
                            gv[L.var * kGS] = make_float2(g.h, g.l);
                        }
                    }
                    float p, q;
                    mul_df_f(V3, xk, p, q);
                    q = __fmaf_rn(V3.h, xkl, q);
                    acc(V2, p, q);
                    mul_df_df(V3, P2, p, q);
                    const float2 g0 = gv[C.var * kGS];
                    DF g = {g0.x, g0.y};
                    acc(g, p, q);
                    gv[C.var * kGS] = make_float2(g.h, g.l);
                }
                float p, q;
                mul_df_f(V2, xj, p, q);
                q = __fmaf_rn(V2.h, xjl, q);
                acc(V1, p, q);
                mul_df_f(V2, xi, p, q);
                q = __fmaf_rn(V2.h, xil, q);
                const float2 g0 = gv[B.var * kGS];
                DF g = {g0.x, g0.y};
                acc(g, p, q);
                gv[B.var * kGS] = make_float2(g.h, g.l);
            }
            float p, q;
            mul_df_f(V1, xi, p, q);
            q = __fmaf_rn(V1.h, xil, q);
            acc(Ev, p, q);
            const float2 g0 = gv[A.var * kGS];
            DF g = {g0.x, g0.y};
            acc(g, V1.h, V1.l);
            gv[A.var * kGS] = make_float2(g.h, g.l);
        }
        if (part) {
            e_other[part - 1][0][tu] = Ev.h;
            e_other[part - 1][1][tu] = Ev.l;
        }
        __syncthreads();
        if (live) {
            // the parts' pairs added in order, the variables divided among
            // the unit's threads
            for (int v = part; v < NV; v += kParts) {
                const float2 g0 = gv_all[v * kGS + tu];
                DF g = {g0.x, g0.y};
                #pragma unroll
                for (int k = 1; k < kParts; ++k) {
                    const float2 gk = gv_all[v * kGS + k * kUnits + tu];
                    acc(g, gk.x, gk.y);
                }
                G[(size_t)v * stride + u] = __fadd_rn(g.h, g.l);
            }
            if (!part) {
                #pragma unroll
                for (int k = 0; k < kParts - 1; ++k) acc(Ev, e_other[k][0][tu], e_other[k][1][tu]);
                E[u] = __fadd_rn(Ev.h, Ev.l);
            }
        }
        __syncthreads();
    }
}

// Split of a trie into kParts parts at level-2 nodes: part k ends where the
// modelled work (level-3 nodes and leaves weighted by their instruction
// counts) reaches cut[k] of the total.  The model undercounts the per-node
// overhead of the later parts, so the fastest cuts measured on GB300
// (box4096, sweeps) give the earlier parts more than an equal share.
WalkSplit make_split(const PolyNode* l1, int n1, const PolyNode* l2, int n2, const PolyNode* l3,
                     const double (&cut)[kParts - 1]) {
    std::vector<double> w(n2);
    double total = 0.0;
    int c3 = 0, cl = 0;
    for (int j = 0; j < n2; ++j) {
        double wj = 0.0;
        for (; c3 < l2[j].end; ++c3) {
            const int nl = l3[c3].end - cl;
            wj += nl > 0 ? 12.0 + 7.0 * nl : 8.0;
            cl = l3[c3].end;
        }
        w[j] = wj;
        total += wj;
    }
    // m[k]: first level-2 node of part k; every part gets at least one
    // (n2 >= kParts for both tries)
    int m[kParts + 1];
    m[0] = 0;
    m[kParts] = n2;
    int j = 0;
    double pre = 0.0;
    for (int k = 1; k < kParts; ++k) {
        while (j < n2 && pre + w[j] <= cut[k - 1] * total) pre += w[j++];
        if (j <= m[k - 1]) pre += w[j++];
        if (j > n2 - (kParts - k)) j = n2 - (kParts - k);
        m[k] = j;
    }
    // a_start[k]: the level-1 node holding level-2 node m[k]; inside[k]:
    // m[k] is not that node's first child (the node is shared with part k-1)
    int a_start[kParts + 1], inside[kParts + 1];
    for (int k = 1; k < kParts; ++k) {
        int a = 0;
        while (a < n1 && l1[a].end <= m[k]) ++a;
        a_start[k] = a;
        inside[k] = (a == 0 ? 0 : l1[a - 1].end) != m[k];
    }
    WalkSplit s;
    for (int k = 0; k < kParts; ++k) {
        const int a0 = k == 0 ? 0 : a_start[k];
        const int a1 = k == kParts - 1 ? n1 : a_start[k + 1] + (inside[k + 1] ? 1 : 0);
        const int c30 = m[k] == 0 ? 0 : l2[m[k] - 1].end;
        const int cl0 = c30 == 0 ? 0 : l3[c30 - 1].end;
        s.part[k] = WalkPart{a0, a1, m[k], m[k + 1], c30, cl0, k > 0 && inside[k] ? 1 : 0};
    }
    return s;
}

// Cuts.  Sweeps of the walks alone on box4096 (ms per launch): three-body
// (0.36, 0.69) 10.15, (0.37, 0.72) 9.81, (0.36, 0.76) 9.61, (0.37, 0.76)
// 9.53, (0.37, 0.80) 10.54; two-body (0.38, 0.71) 1.73, (0.40, 0.75) 1.56,
// (0.42, 0.75) 1.63.  In the MD step, where the electrostatics stream runs
// beside the walks and ends the step, the less balanced cuts are faster
// (ms per step over 1000 steps, same GPU: 12.10 and 12.01 against 12.39 and
// 12.40): a block's parts that finish early wait at the barrier and leave
// issue slots to the electrostatics.
#ifndef MBPOL_WALK_CUTS_2B
#define MBPOL_WALK_CUTS_2B {0.38, 0.71}
#endif
#ifndef MBPOL_WALK_CUTS_3B
#define MBPOL_WALK_CUTS_3B {0.36, 0.69}
#endif

const WalkSplit& split2() {
    static const double cut[kParts - 1] = MBPOL_WALK_CUTS_2B;
    static const WalkSplit s = make_split(poly2b_l1, POLY2B_N1, poly2b_l2, POLY2B_N2, poly2b_l3, cut);
    return s;
}
const WalkSplit& split3() {
    static const double cut[kParts - 1] = MBPOL_WALK_CUTS_3B;
    static const WalkSplit s = make_split(poly3b_l1, POLY3B_N1, poly3b_l2, POLY3B_N2, poly3b_l3, cut);
    return s;
}

template <int NV>
constexpr int walk_smem() {
    return NV * (2 * kUnits + 2 * kBlock) * (int)sizeof(float);
}

template <int NV>
int walk_blocks(int n, int num_sms, int reserve_blocks) {
    int blocks = (n + kUnits - 1) / kUnits;
    const int cap = num_sms * kBlocksPerSm - (reserve_blocks < 0 ? MBPOL_WALK_RESERVE_BLOCKS : reserve_blocks);
    if (blocks > cap) blocks = cap > num_sms ? cap : num_sms;
    return blocks;
}

template <int NV>
struct PolyTables {
    PolyNode *l1 = nullptr, *l2 = nullptr, *l3 = nullptr, *lv = nullptr;
    int n1 = 0;
};

cudaError_t upload(const PolyNode* src, size_t n, PolyNode** dst) {
    cudaError_t e = cudaMalloc(dst, n * sizeof(PolyNode));
    if (e != cudaSuccess) return e;
    return cudaMemcpy(*dst, src, n * sizeof(PolyNode), cudaMemcpyHostToDevice);
}

}  // namespace

// The trie tables of one device (uploaded once per device and process).
struct PolyWalkTables {
    bool ready = false;
    PolyTables<31> t2;
    PolyTables<36> t3;
};

namespace {
std::mutex g_walk_mu;
std::vector<std::unique_ptr<PolyWalkTables>> g_walk;  // by device ordinal
}  // namespace

cudaError_t poly2b_kernel_setup() {
    return cudaFuncSetAttribute(poly_df_kernel<31>, cudaFuncAttributeMaxDynamicSharedMemorySize, walk_smem<31>());
}

cudaError_t poly_tables_upload(int device, const PolyWalkTables** out) {
    std::lock_guard<std::mutex> lock(g_walk_mu);
    if (device < 0) return cudaErrorInvalidDevice;
    if ((size_t)device >= g_walk.size()) g_walk.resize((size_t)device + 1);
    if (!g_walk[(size_t)device]) g_walk[(size_t)device].reset(new PolyWalkTables());
    PolyWalkTables& w = *g_walk[(size_t)device];
    if (!w.ready) {
        cudaError_t e;
        if ((e = upload(poly2b_l1, POLY2B_N1, &w.t2.l1)) || (e = upload(poly2b_l2, POLY2B_N2, &w.t2.l2)) ||
            (e = upload(poly2b_l3, POLY2B_N3, &w.t2.l3)) || (e = upload(poly2b_leaf, POLY2B_NL, &w.t2.lv)) ||
            (e = upload(poly3b_l1, POLY3B_N1, &w.t3.l1)) || (e = upload(poly3b_l2, POLY3B_N2, &w.t3.l2)) ||
            (e = upload(poly3b_l3, POLY3B_N3, &w.t3.l3)) || (e = upload(poly3b_leaf, POLY3B_NL, &w.t3.lv)))
            return e;
        w.t2.n1 = POLY2B_N1;
        w.t3.n1 = POLY3B_N1;
        if ((e = poly2b_kernel_setup())) return e;
        if ((e = cudaFuncSetAttribute(poly_df_kernel<36>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      walk_smem<36>())))
            return e;
        w.ready = true;
    }
    *out = &w;
    return cudaSuccess;
}

int walk_default_reserve() { return MBPOL_WALK_RESERVE_BLOCKS; }

void launch_poly2b_with(cudaStream_t st, const PolyNode* l1, const PolyNode* l2, const PolyNode* l3,
                        const PolyNode* lv, const float* X, float* G, float* E, int n, int stride, int num_sms,
                        int reserve_blocks) {
    if (n <= 0) return;
    count_launch();
    poly_df_kernel<31><<<walk_blocks<31>(n, num_sms, reserve_blocks), kBlock, walk_smem<31>(), st>>>(
        l1, l2, l3, POLY2B_N3, lv, split2(), X, G, E, n, stride);
}

void launch_poly2b(cudaStream_t st, const PolyWalkTables* t, const float* X, float* G, float* E, int n, int stride,
                   int num_sms, int reserve_blocks) {
    launch_poly2b_with(st, t->t2.l1, t->t2.l2, t->t2.l3, t->t2.lv, X, G, E, n, stride, num_sms, reserve_blocks);
}

void launch_poly3b(cudaStream_t st, const PolyWalkTables* t, const float* X, float* G, float* E, int n, int stride,
                   int num_sms, int reserve_blocks) {
    if (n <= 0) return;
    count_launch();
    poly_df_kernel<36><<<walk_blocks<36>(n, num_sms, reserve_blocks), kBlock, walk_smem<36>(), st>>>(
        t->t3.l1, t->t3.l2, t->t3.l3, POLY3B_N3, t->t3.lv, split3(), X, G, E, n, stride);
}

}  // namespace mbpol
