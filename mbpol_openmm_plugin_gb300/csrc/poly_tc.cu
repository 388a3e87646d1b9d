// Three-body MB-pol polynomial (value and gradient) on the tensor cores.
//
// The reference evaluates E(x) = sum_m c_m x^m (36 variables, degree 4,
// 33,525 monomials; platforms/reference/src/poly-3b-v2x.cpp:3-28378) as
// straight-line FP64 code.  Here (tables from codegen/gen_poly_tc.py):
//   d = x - x0 (x0 a fixed expansion point; the re-expanded polynomial's
//   terms cancel ~250x less than the original's),
//   y = [1, d_i, d_i d_j (i <= j)] (703 rows), E = y^T S y with S symmetric,
//   z = S y, E = y . z, dE/dd_i = 2 sum_m z_m dy_m/dd_i.
// z for a tile of 64 trimers is the product S[703 x 703] . Y[703 x 64],
// computed with mma.sync.m16n8k16 (fp16 operands, FP32 accumulation): S as
// three fp16 pieces (tables, in the A-fragment register layout), Y' (Y with
// per-row power-of-two scales) as two pieces split here; per 16-wide k-tile
// the products S0Y0 + S0Y1 + S1Y0 + S2Y0 start from zero and are then added
// to FP32 sums, so the tensor cores' own accumulation rounding stays
// relative to one k-tile.  All-zero 16x16 tiles of S (57%) are skipped.
// The epilogue (E and the gradient, double-float sums in a fixed order)
// reads z back from a per-block scratch slice, so results do not depend on
// scheduling.
//
// Block: 512 threads (16 warps: each of the tables' 8 row-tile groups taken
// by two warps, each for 32 of the tile's trimers) and 196 KB of shared
// memory; one block per SM, persistent over tiles of 64 trimers.  Inputs X [2][36][stride] (the
// variables as FP32 hi and lo planes), outputs G [36][stride], E [stride].
#include <cuda_fp16.h>

#include <mutex>
#include <vector>

#include "mbpol_internal.cuh"
#include "poly_tc.h"
#include "poly_tc_common.cuh"
#include "poly_tc_dev.h"

namespace mbpol {

namespace {

constexpr int kTU = 64;        // units (trimers) per tile
constexpr int kGroups = 8;     // row-tile groups of the tables (codegen/gen_poly_tc.py NWARPS)
constexpr int kTWarps = 16;    // two warps per group, each for half of the tile's trimers
constexpr int kTThreads = 32 * kTWarps;
constexpr int kQ = kTThreads / kTU;  // threads per trimer in the epilogue

template <int NV, int NPAD>
struct TCShape {
    static constexpr int NY = 1 + NV + NV * (NV + 1) / 2;
    static constexpr int KS = NPAD + 8;                   // Y row stride (halves): conflict-free ldmatrix
    static constexpr int DS = NV + 2;                     // d row stride: d_nv = 1, d_{nv+1} = 0
    static constexpr size_t Y_BYTES = (size_t)2 * kTU * KS * sizeof(__half);
    static constexpr size_t D_BYTES = (size_t)kTU * DS * sizeof(float);
    static constexpr size_t SMEM = Y_BYTES + D_BYTES + kTU * sizeof(unsigned) + kQ * kTU * sizeof(float2);
    static_assert(NY <= NPAD && NPAD % 16 == 0, "padding");
};

__device__ __forceinline__ unsigned smem_u32(const void* p) {
    return (unsigned)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void ldsm_x4(unsigned addr, unsigned& r0, unsigned& r1, unsigned& r2, unsigned& r3) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3)
                 : "r"(addr));
}

// d += A . B (m16n8k16, fp16 operands, FP32 accumulators)
__device__ __forceinline__ void mma16816(float (&d)[4], const uint4& a, unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a.x), "r"(a.y), "r"(a.z), "r"(a.w), "r"(b0), "r"(b1));
}

template <int NV, int NPAD>
__global__ void __launch_bounds__(kTThreads, 1)
    poly_tc_kernel(const PolyTCDev tab, const float* __restrict__ X, float* __restrict__ G, float* __restrict__ E,
                   int n, int stride, float* __restrict__ zscratch) {
    using Sh = TCShape<NV, NPAD>;
    constexpr int KS = Sh::KS, DS = Sh::DS, NY = Sh::NY;
    extern __shared__ __align__(16) unsigned char smem[];
    __half* ysm = reinterpret_cast<__half*>(smem);                           // [2][kTU][KS]
    float* dsm = reinterpret_cast<float*>(smem + Sh::Y_BYTES);               // [kTU][DS]
    unsigned* umax = reinterpret_cast<unsigned*>(smem + Sh::Y_BYTES + Sh::D_BYTES);  // [kTU]
    float2* epart = reinterpret_cast<float2*>(umax + kTU);                   // [kQ][kTU]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    float* zs = zscratch + (size_t)blockIdx.x * NPAD * kTU;                  // [NPAD][kTU]
    const int ntiles = (n + kTU - 1) / kTU;

    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const int base = tile * kTU;
        // ---- d = x - x0 and the per-unit bound ratio max_v |d_v| / bound_v
        if (tid < kTU) umax[tid] = 0u;
        __syncthreads();
        for (int i = tid; i < kTU * NV; i += kTThreads) {
            const int t = i % kTU, v = i / kTU, u = base + t;
            float d = 0.f;
            if (u < n) d = __fadd_rn(__fsub_rn(X[(size_t)v * stride + u], tab.x0h[v]),
                                     __fsub_rn(X[(size_t)(NV + v) * stride + u], tab.x0l[v]));
            dsm[t * DS + v] = d;
            atomicMax(&umax[t], __float_as_uint(fabsf(d) * tab.inv_bound[v]));
        }
        if (tid < kTU) {
            dsm[tid * DS + NV] = 1.f;
            dsm[tid * DS + NV + 1] = 0.f;
        }
        __syncthreads();
        // ---- Y' = Y 2^(s_k - e_t) as two fp16 pieces, [piece][unit][k].
        // |d_v| <= m bound_v gives |y'_k| <= 2^12 max(1, m)^2; e_t keeps
        // |y'| <= 2^15 (fp16 range) for units beyond the sampled bounds.
        for (int i = tid; i < kTU * (NPAD / 2); i += kTThreads) {
            const int t = i / (NPAD / 2), k = 2 * (i % (NPAD / 2));
            const int e = unit_exp(__uint_as_float(umax[t]));
            const float* dt = dsm + t * DS;
            float y[2];
            #pragma unroll
            for (int h = 0; h < 2; ++h) {
                const unsigned meta = tab.ymeta[k + h];
                const int a = meta & 255, b = (meta >> 8) & 255, s = (int)((meta >> 16) & 255) - 128;
                y[h] = __fmul_rn(__fmul_rn(dt[a], dt[b]), exp2i(s - e));
            }
            const __half h0 = __float2half_rn(y[0]), h1 = __float2half_rn(y[1]);
            const __half l0 = __float2half_rn(__fsub_rn(y[0], __half2float(h0)));
            const __half l1 = __float2half_rn(__fsub_rn(y[1], __half2float(h1)));
            *reinterpret_cast<__half2*>(ysm + (size_t)t * KS + k) = __halves2half2(h0, h1);
            *reinterpret_cast<__half2*>(ysm + (size_t)(kTU + t) * KS + k) = __halves2half2(l0, l1);
        }
        __syncthreads();
        // ---- z = S Y' on the tensor cores: each pair of warps owns whole row
        // tiles (a group of the tables), each warp half of the trimers
        {
            const int g = lane >> 2, q = lane & 3;
            const int grp = warp >> 1, nh = warp & 1;
            // ldmatrix.x4 row addresses: matrices (units 0-7, k 0-7),
            // (units 0-7, k 8-15), (units 8-15, k 0-7), (units 8-15, k 8-15)
            // of this warp's 32 trimers
            const int mi = lane >> 3, r = lane & 7;
            const unsigned yb_hi =
                smem_u32(ysm) + (unsigned)(((nh * 32 + (mi >> 1) * 8 + r) * KS + (mi & 1) * 8) * 2);
            const unsigned yb_lo = yb_hi + (unsigned)(kTU * KS * 2);
            const int i0 = tab.warp_begin[grp], i1 = tab.warp_begin[grp + 1];
            const int e_end = tab.rt_entry[i1];
            int e = tab.rt_entry[i0];
            const uint4* fr = reinterpret_cast<const uint4*>(tab.frag);
            uint4 fa0, fa1, fa2;
            int kt = 0;
            if (e < e_end) {
                fa0 = fr[(size_t)(e * 3 + 0) * 32 + lane];
                fa1 = fr[(size_t)(e * 3 + 1) * 32 + lane];
                fa2 = fr[(size_t)(e * 3 + 2) * 32 + lane];
                kt = tab.ent_kt[e];
            }
            for (int i = i0; i < i1; ++i) {
                const int rt = tab.rt_id[i];
                const int ee = tab.rt_entry[i + 1];
                float acc[4][4];
                #pragma unroll
                for (int j = 0; j < 4; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
                for (; e < ee; ++e) {
                    // next tile's fragments while this one computes
                    uint4 fn0 = fa0, fn1 = fa1, fn2 = fa2;
                    int ktn = kt;
                    if (e + 1 < e_end) {
                        fn0 = fr[(size_t)((e + 1) * 3 + 0) * 32 + lane];
                        fn1 = fr[(size_t)((e + 1) * 3 + 1) * 32 + lane];
                        fn2 = fr[(size_t)((e + 1) * 3 + 2) * 32 + lane];
                        ktn = tab.ent_kt[e + 1];
                    }
                    const unsigned koff = (unsigned)(kt * 32);   // 16 halves
                    #pragma unroll
                    for (int jp = 0; jp < 2; ++jp) {
                        const unsigned uoff = (unsigned)(jp * 16 * KS * 2);
                        unsigned bh[4], bl[4];
                        ldsm_x4(yb_hi + uoff + koff, bh[0], bh[1], bh[2], bh[3]);
                        ldsm_x4(yb_lo + uoff + koff, bl[0], bl[1], bl[2], bl[3]);
                        #pragma unroll
                        for (int jj = 0; jj < 2; ++jj) {
                            // two chains of two products each (S0 Y0 + S1 Y0, S0 Y1 + S2 Y0),
                            // both started from zero in this k-tile
                            float d[4] = {0.f, 0.f, 0.f, 0.f}, c[4] = {0.f, 0.f, 0.f, 0.f};
                            mma16816(d, fa0, bh[2 * jj], bh[2 * jj + 1]);
                            mma16816(c, fa0, bl[2 * jj], bl[2 * jj + 1]);
                            mma16816(d, fa1, bh[2 * jj], bh[2 * jj + 1]);
                            mma16816(c, fa2, bh[2 * jj], bh[2 * jj + 1]);
                            float* a = acc[2 * jp + jj];
                            #pragma unroll
                            for (int k = 0; k < 4; ++k) a[k] = __fadd_rn(__fadd_rn(a[k], d[k]), c[k]);
                        }
                    }
                    fa0 = fn0;
                    fa1 = fn1;
                    fa2 = fn2;
                    kt = ktn;
                }
                // rows rt*16 + g and + 8, units 32 nh + 8j + 2q, + 1
                const int m0 = rt * 16 + g, m1 = m0 + 8;
                const float s0 = tab.rowscale[m0], s1 = tab.rowscale[m1];
                #pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int u = 32 * nh + 8 * j + 2 * q;
                    *reinterpret_cast<float2*>(zs + (size_t)m0 * kTU + u) =
                        make_float2(acc[j][0] * s0, acc[j][1] * s0);
                    *reinterpret_cast<float2*>(zs + (size_t)m1 * kTU + u) =
                        make_float2(acc[j][2] * s1, acc[j][3] * s1);
                }
            }
        }
        __syncthreads();
        // ---- E = y . z and dE/dd_i = 2 sum_m z_m dy_m/dd_i; kQ threads per
        // unit, fixed summation order
        {
            const int t = tid % kTU, qd = tid / kTU, u = base + t;
            const float ze = exp2i(unit_exp(__uint_as_float(umax[t])));
            const float* dt = dsm + t * DS;
            float2 es = make_float2(0.f, 0.f);
            for (int r = qd; r < NY; r += kQ) {
                const unsigned meta = tab.ymeta[r];
                const float y = __fmul_rn(dt[meta & 255], dt[(meta >> 8) & 255]);
                df_fma(es, y, __fmul_rn(zs[(size_t)r * kTU + t], ze));
            }
            epart[qd * kTU + t] = es;
            for (int v = qd; v < NV; v += kQ) {
                // rows (v) and (min(v,j), max(v,j))
                float2 gs = make_float2(0.f, 0.f);
                df_fma(gs, 2.f, zs[(size_t)(1 + v) * kTU + t]);
                #pragma unroll 4
                for (int j = 0; j < NV; ++j) {
                    const int a = min(v, j), b = max(v, j);
                    const int row = 1 + NV + a * NV - (a * (a - 1)) / 2 + (b - a);
                    df_fma(gs, (j == v ? 4.f : 2.f) * dt[j], zs[(size_t)row * kTU + t]);
                }
                if (u < n) G[(size_t)v * stride + u] = __fmul_rn(__fadd_rn(gs.x, gs.y), ze);
            }
        }
        __syncthreads();
        if (tid < kTU && base + tid < n) {
            float2 es = epart[tid];
            #pragma unroll
            for (int k = 1; k < kQ; ++k) df_add(es, epart[k * kTU + tid]);
            E[base + tid] = __fadd_rn(es.x, es.y);
        }
        __syncthreads();
    }
}

using Shape3 = TCShape<36, 704>;

struct DevCopy {
    bool ready = false;
    PolyTCDev d3;
};
std::mutex g_mu;
std::vector<DevCopy> g_dev;

template <class T>
cudaError_t upload_array(const T* src, size_t n, const T** dst, std::vector<void*>& owned) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, n * sizeof(T));
    if (e != cudaSuccess) return e;
    owned.push_back(p);
    *dst = static_cast<const T*>(p);
    return cudaMemcpy(p, src, n * sizeof(T), cudaMemcpyHostToDevice);
}

cudaError_t upload_tc(const PolyTCTables& h, PolyTCDev* d) {
    std::vector<void*> owned;
    cudaError_t e;
    d->nv = h.nv;
    d->ny = h.ny;
    d->npad = h.npad;
    d->parts5 = h.parts5;
    d->rows5 = h.rows5;
    d->nblk5 = h.nblk5;
    if ((e = upload_array(h.x0h, (size_t)h.nv, &d->x0h, owned)) ||
        (e = upload_array(h.x0l, (size_t)h.nv, &d->x0l, owned)) ||
        (e = upload_array(h.inv_bound, (size_t)h.nv, &d->inv_bound, owned)) ||
        (e = upload_array(h.ymeta, (size_t)h.npad, &d->ymeta, owned)) ||
        (e = upload_array(h.rowscale, (size_t)h.npad, &d->rowscale, owned)) ||
        (e = upload_array(h.warp_begin, (size_t)kGroups + 1, &d->warp_begin, owned)) ||
        (e = upload_array(h.rt_id, (size_t)h.nrt, &d->rt_id, owned)) ||
        (e = upload_array(h.rt_entry, (size_t)h.nrt + 1, &d->rt_entry, owned)) ||
        (e = upload_array(h.ent_kt, (size_t)h.nent, &d->ent_kt, owned)) ||
        (e = upload_array(h.frag, (size_t)h.nent * 3 * 32 * 4, &d->frag, owned)) ||
        (e = upload_array(h.sblk, (size_t)h.nblk5 * 3 * h.rows5 * 16, &d->sblk, owned)) ||
        (e = upload_array(h.blk_kt, (size_t)h.nblk5, &d->blk_kt, owned)) ||
        (e = upload_array(h.blk_begin, (size_t)h.parts5 * (h.npad / h.rows5) + 1, &d->blk_begin, owned))) {
        for (void* p : owned) cudaFree(p);
        return e;
    }
    return cudaSuccess;
}

}  // namespace

cudaError_t poly_tc_setup(int device, const PolyTCDev** out) {
    std::lock_guard<std::mutex> lock(g_mu);
    if (device < 0) return cudaErrorInvalidDevice;
    if ((size_t)device >= g_dev.size()) g_dev.resize((size_t)device + 1);
    DevCopy& c = g_dev[(size_t)device];
    if (!c.ready) {
        cudaError_t e = cudaFuncSetAttribute(poly_tc_kernel<36, 704>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)Shape3::SMEM);
        if (e != cudaSuccess) return e;
        if (k_poly3b.nv != 36 || k_poly3b.npad != 704 || k_poly3b.parts5 != 3 || k_poly3b.rows5 != 64)
            return cudaErrorInvalidValue;
        if ((e = poly_tc5_prepare())) return e;
        if ((e = upload_tc(k_poly3b, &c.d3))) return e;
        c.ready = true;
    }
    *out = &c.d3;
    return cudaSuccess;
}

// SMs left out of the persistent grid, so that the electrostatics stream
// finds room beside the three-body kernel (a block takes a whole SM's
// registers).  Measured on box4096 (learned arm, ms per step over 300
// steps): 0 SMs 6.121, 24 6.041, 52 6.015, 76 5.980; the plain arm 9.151
// (0) and 9.050 (52).  52 keeps the kernel alone at ~2.5 ms.
#ifndef MBPOL_TC_RESERVE_SMS
#define MBPOL_TC_RESERVE_SMS 52
#endif

size_t poly3b_tc_scratch_floats(int num_sms) { return (size_t)num_sms * 704 * kTU; }

void launch_poly3b_tc(cudaStream_t st, const PolyTCDev* tab, const float* X, float* G, float* E, int n, int stride,
                      int num_sms, float* zscratch, int reserve_sms) {
    if (n <= 0) return;
    count_launch();
    const int ntiles = (n + kTU - 1) / kTU;
    int blocks = num_sms - (reserve_sms < 0 ? MBPOL_TC_RESERVE_SMS : reserve_sms);
    if (blocks < num_sms / 2) blocks = num_sms / 2;
    if (blocks > ntiles) blocks = ntiles;
    poly_tc_kernel<36, 704><<<blocks, kTThreads, Shape3::SMEM, st>>>(*tab, X, G, E, n, stride, zscratch);
}

}  // namespace mbpol
