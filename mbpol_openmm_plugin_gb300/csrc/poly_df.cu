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
// One thread per unit (dimer or trimer).  The variables x and the gradient
// pairs (gh, gl) live in shared memory, [variable][thread], so every access
// of a warp is one conflict-free wavefront; the trie tables are read with
// warp-uniform addresses.  X: [2][nvars][stride] floats (FP64 variables as
// hi and lo planes); G: [nvars][stride]; E: [stride].
#include "mbpol_internal.cuh"
#include "poly_tables.h"

namespace mbpol {

#include "gen/poly2b_tables.inc"
#include "gen/poly3b_tables.inc"

namespace {

constexpr int kBlock = 128;

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

// U leaves of one level-3 node: all loads first, then the updates in leaf
// order (V3's summation order is unchanged), then the stores.
template <int U>
__device__ __forceinline__ void leaf_batch(const PolyNode* __restrict__ lv, const float* xs, const float* xq,
                                           float* gh, float* gl, int t, const DF& P3, DF& V3) {
    PolyNode L[U];
    int o[U];
    float x[U], xl[U];
    DF g[U];
    #pragma unroll
    for (int u = 0; u < U; ++u) L[u] = lv[u];
    #pragma unroll
    for (int u = 0; u < U; ++u) {
        o[u] = L[u].var * kBlock + t;
        x[u] = xs[o[u]];
        xl[u] = xq[o[u]];
        g[u].h = gh[o[u]];
        g[u].l = gl[o[u]];
    }
    #pragma unroll
    for (int u = 0; u < U; ++u) leaf_update(L[u], x[u], xl[u], P3, V3, g[u]);
    #pragma unroll
    for (int u = 0; u < U; ++u) {
        gh[o[u]] = g[u].h;
        gl[o[u]] = g[u].l;
    }
}

template <int NV>
__global__ void __launch_bounds__(kBlock) poly_df_kernel(const PolyNode* __restrict__ l1, int n1,
                                                          const PolyNode* __restrict__ l2,
                                                          const PolyNode* __restrict__ l3, int n3,
                                                          const PolyNode* __restrict__ lv,
                                                          const float* __restrict__ X, float* __restrict__ G,
                                                          float* __restrict__ E, int n, int stride) {
    extern __shared__ float smem[];
    float* xs = smem;                  // [NV][kBlock]   variables, high part
    float* xq = smem + NV * kBlock;    // [NV][kBlock]   variables, low part
    float* gh = xq + NV * kBlock;      // [NV][kBlock]
    float* gl = gh + NV * kBlock;      // [NV][kBlock]
    const int t = threadIdx.x;
    for (int base = blockIdx.x * kBlock; base < n; base += gridDim.x * kBlock) {
        const int u = base + t;
        const bool live = u < n;
        #pragma unroll
        for (int v = 0; v < NV; ++v) {
            xs[v * kBlock + t] = live ? X[(size_t)v * stride + u] : 0.f;
            xq[v * kBlock + t] = live ? X[(size_t)(NV + v) * stride + u] : 0.f;
            gh[v * kBlock + t] = 0.f;
            gl[v * kBlock + t] = 0.f;
        }
        DF Ev = {0.f, 0.f};
        int c2 = 0, c3 = 0, cl = 0;
        // The next level-3 node is read one step ahead.  Children of a node
        // have distinct variables, so several leaves' gradient pairs can be
        // read before any of them is written back; a parent's own pair is
        // read only after its children's writes (a child may share its
        // variable).
        PolyNode Cn = n3 > 0 ? l3[0] : PolyNode{0.f, 0.f, 0, 0};
        for (int a = 0; a < n1; ++a) {
            const PolyNode A = l1[a];
            const float xi = xs[A.var * kBlock + t], xil = xq[A.var * kBlock + t];
            DF V1 = {A.hi, A.lo};
            for (; c2 < A.end; ++c2) {
                const PolyNode B = l2[c2];
                const float xj = xs[B.var * kBlock + t], xjl = xq[B.var * kBlock + t];
                DF V2 = {B.hi, B.lo};
                DF P2;
                P2.h = __fmul_rn(xi, xj);
                P2.l = __fmaf_rn(xi, xj, -P2.h);
                P2.l = __fmaf_rn(xi, xjl, P2.l);
                P2.l = __fmaf_rn(xil, xj, P2.l);
                for (; c3 < B.end; ++c3) {
                    const PolyNode C = Cn;
                    if (c3 + 1 < n3) Cn = l3[c3 + 1];
                    const float xk = xs[C.var * kBlock + t], xkl = xq[C.var * kBlock + t];
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
                        for (; cl + 4 <= cend; cl += 4) leaf_batch<4>(lv + cl, xs, xq, gh, gl, t, P3, V3);
                        for (; cl < cend; ++cl) {
                            const PolyNode L = lv[cl];
                            const int o = L.var * kBlock + t;
                            DF g = {gh[o], gl[o]};
                            leaf_update(L, xs[o], xq[o], P3, V3, g);
                            gh[o] = g.h;
                            gl[o] = g.l;
                        }
                    }
                    float p, q;
                    mul_df_f(V3, xk, p, q);
                    q = __fmaf_rn(V3.h, xkl, q);
                    acc(V2, p, q);
                    mul_df_df(V3, P2, p, q);
                    const int o = C.var * kBlock + t;
                    DF g = {gh[o], gl[o]};
                    acc(g, p, q);
                    gh[o] = g.h;
                    gl[o] = g.l;
                }
                float p, q;
                mul_df_f(V2, xj, p, q);
                q = __fmaf_rn(V2.h, xjl, q);
                acc(V1, p, q);
                mul_df_f(V2, xi, p, q);
                q = __fmaf_rn(V2.h, xil, q);
                const int o = B.var * kBlock + t;
                DF g = {gh[o], gl[o]};
                acc(g, p, q);
                gh[o] = g.h;
                gl[o] = g.l;
            }
            float p, q;
            mul_df_f(V1, xi, p, q);
            q = __fmaf_rn(V1.h, xil, q);
            acc(Ev, p, q);
            const int o = A.var * kBlock + t;
            DF g = {gh[o], gl[o]};
            acc(g, V1.h, V1.l);
            gh[o] = g.h;
            gl[o] = g.l;
        }
        if (live) {
            #pragma unroll
            for (int v = 0; v < NV; ++v) G[(size_t)v * stride + u] = __fadd_rn(gh[v * kBlock + t], gl[v * kBlock + t]);
            E[u] = __fadd_rn(Ev.h, Ev.l);
        }
    }
}

template <int NV>
struct PolyTables {
    PolyNode *l1 = nullptr, *l2 = nullptr, *l3 = nullptr, *lv = nullptr;
    int n1 = 0;
};

PolyTables<31> g_t2;
PolyTables<36> g_t3;
int g_dev_uploaded = -1;

template <class T>
cudaError_t upload(const PolyNode* src, size_t n, PolyNode** dst) {
    cudaError_t e = cudaMalloc(dst, n * sizeof(PolyNode));
    if (e != cudaSuccess) return e;
    return cudaMemcpy(*dst, src, n * sizeof(PolyNode), cudaMemcpyHostToDevice);
}

}  // namespace

cudaError_t poly_tables_upload(int device) {
    if (g_dev_uploaded == device) return cudaSuccess;
    cudaError_t e;
    if ((e = upload<int>(poly2b_l1, POLY2B_N1, &g_t2.l1)) || (e = upload<int>(poly2b_l2, POLY2B_N2, &g_t2.l2)) ||
        (e = upload<int>(poly2b_l3, POLY2B_N3, &g_t2.l3)) || (e = upload<int>(poly2b_leaf, POLY2B_NL, &g_t2.lv)) ||
        (e = upload<int>(poly3b_l1, POLY3B_N1, &g_t3.l1)) || (e = upload<int>(poly3b_l2, POLY3B_N2, &g_t3.l2)) ||
        (e = upload<int>(poly3b_l3, POLY3B_N3, &g_t3.l3)) || (e = upload<int>(poly3b_leaf, POLY3B_NL, &g_t3.lv)))
        return e;
    g_t2.n1 = POLY2B_N1;
    g_t3.n1 = POLY3B_N1;
    const int sm2 = 4 * 31 * kBlock * (int)sizeof(float), sm3 = 4 * 36 * kBlock * (int)sizeof(float);
    if ((e = cudaFuncSetAttribute(poly_df_kernel<31>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm2))) return e;
    if ((e = cudaFuncSetAttribute(poly_df_kernel<36>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm3))) return e;
    g_dev_uploaded = device;
    return cudaSuccess;
}

void launch_poly2b(cudaStream_t st, const float* X, float* G, float* E, int n, int stride, int num_sms) {
    if (n <= 0) return;
    int blocks = (n + kBlock - 1) / kBlock;
    if (blocks > num_sms * 4) blocks = num_sms * 4;
    count_launch();
    poly_df_kernel<31><<<blocks, kBlock, 4 * 31 * kBlock * sizeof(float), st>>>(g_t2.l1, g_t2.n1, g_t2.l2, g_t2.l3,
                                                                                POLY2B_N3, g_t2.lv, X, G, E, n, stride);
}

cudaError_t poly2b_kernel_setup() {
    return cudaFuncSetAttribute(poly_df_kernel<31>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                4 * 31 * kBlock * (int)sizeof(float));
}

void launch_poly2b_with(cudaStream_t st, const PolyNode* l1, int n1, const PolyNode* l2, const PolyNode* l3,
                        const PolyNode* lv, const float* X, float* G, float* E, int n, int stride, int num_sms) {
    if (n <= 0) return;
    int blocks = (n + kBlock - 1) / kBlock;
    if (blocks > num_sms * 4) blocks = num_sms * 4;
    count_launch();
    poly_df_kernel<31><<<blocks, kBlock, 4 * 31 * kBlock * sizeof(float), st>>>(l1, n1, l2, l3, POLY2B_N3, lv, X, G, E, n,
                                                                                stride);
}

void launch_poly3b(cudaStream_t st, const float* X, float* G, float* E, int n, int stride, int num_sms) {
    if (n <= 0) return;
    int blocks = (n + kBlock - 1) / kBlock;
    if (blocks > num_sms * 4) blocks = num_sms * 4;
    count_launch();
    poly_df_kernel<36><<<blocks, kBlock, 4 * 36 * kBlock * sizeof(float), st>>>(g_t3.l1, g_t3.n1, g_t3.l2, g_t3.l3,
                                                                                POLY3B_N3, g_t3.lv, X, G, E, n, stride);
}

}  // namespace mbpol
