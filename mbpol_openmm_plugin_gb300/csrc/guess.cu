// Learned initial guess for the induced dipoles (no reference counterpart:
// the reference's solver always starts from alpha * E_fixed,
// platforms/reference/src/MBPolReferenceElectrostaticsForce.cpp:557-616).
//
// Descriptors (per water, 48 numbers, in the water's own frame e1 = O-H
// bisector, e2 = in plane toward H1, e3 = e1 x e2): for every O and H atom of
// another water within 0.6 nm of O, six Gaussian radial functions
// exp(-((r - R_k)/0.09)^2) fc(r), R_k = 0.15 + 0.09 k nm,
// fc = (cos(pi r/0.6) + 1)/2, summed as scalars and times the unit vector's
// three frame components (s*24 + k*4 + c, s = 0 for O atoms, 1 for H).
//
// Network input (64): the 48 descriptors, the permanent field at O, H1, H2 in
// the same frame (9; the field the solver starts from, which carries the
// long-range electrostatics a 0.6 nm descriptor cannot see), 7 zeros.
// Network: x = bf16((in - mean)/std), h1 = SiLU(W1 x + b1), h2 = SiLU(W2 h1 +
// b2), y = W3 h2 + b3 (64-64-64-9), the O, H1, H2 dipoles in the frame in
// units of 1e-3 e nm.  Prediction (every solve that uses a network) runs on
// the fifth-generation tensor cores, tcgen05.mma with the activations in
// tensor memory (mlp_tc5_kernel).  Training runs every product as
// mma.sync.m16n8k16 with BF16 operands and FP32 accumulation, one warp per
// 16 samples; each layer's accumulator fragments are re-packed in registers
// as the next layer's A fragments; it recomputes the forward pass,
// back-propagates with the same instruction (the transposed operands of the
// weight gradients go through per-warp shared-memory tiles), sums the
// gradients in shared memory per block and updates with Adam.
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "guess.h"
#include "mbpol_internal.cuh"
#include "umma.cuh"

namespace mbpol {

using namespace guess;

struct GuessBuffers {
    float* params = nullptr;  // kBlockFloats (FP32 masters + mean + 1/std)
    float* adam_m = nullptr;
    float* adam_v = nullptr;
    float* grad = nullptr;    // kParams
    double* loss = nullptr;   // [0] tail accumulator, [1] scratch
    double* stats = nullptr;  // 2 * kIn (column sums, sums of squares)
    float* desc = nullptr;    // [cap_mol][64]
    float* frames = nullptr;  // [cap_mol][9]
    float* ybuf = nullptr;    // [cap_mol][9]
    int cap_mol = 0;
    float* X = nullptr;       // dataset [cap_s][64]
    float* T = nullptr;       // dataset [cap_s][9]
    long cap_s = 0;
    float* hx = nullptr;      // staging for loss_grad [cap_h][64], [cap_h][9], [cap_h][9]
    float* ht = nullptr;
    float* hy = nullptr;
    int cap_h = 0;
    int* status = nullptr;    // set by the tcgen05 inference kernel when a wait gives up
    __half* wpack = nullptr;  // fp16 operand image of the weights (pack_weights_kernel)
    int adam_t = 0;
    bool stats_set = false;
};

namespace {

constexpr float kRC = 0.6f, kR0 = 0.15f, kDR = 0.09f, kSigma = 0.09f;
constexpr float kPiF = 3.14159265358979f;
constexpr int kWarps = 4;  // warps per block in the network kernels

struct GBox {
    float L[3], inv[3];
    int periodic;
};

__global__ void descriptor_kernel(int nmol, int K, const float* __restrict__ off, const int* __restrict__ nb,
                                  const float* __restrict__ nbd, const int* __restrict__ nnb, int cap, GBox box,
                                  const float* __restrict__ E0, float* __restrict__ D, float* __restrict__ F,
                                  int mode) {
    const int A = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (A >= nmol) return;
    const float* oA = off + 3 * (size_t)K * A;
    float a[3] = {oA[3], oA[4], oA[5]}, b[3] = {oA[6], oA[7], oA[8]};
    const float ia = rsqrtf(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    const float ib = rsqrtf(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
    float e1[3], e2[3], e3[3];
    #pragma unroll
    for (int k = 0; k < 3; ++k) {
        a[k] *= ia;
        b[k] *= ib;
        e1[k] = a[k] + b[k];
    }
    float nn = rsqrtf(e1[0] * e1[0] + e1[1] * e1[1] + e1[2] * e1[2]);
    #pragma unroll
    for (int k = 0; k < 3; ++k) e1[k] *= nn;
    float pe = 0.f;
    #pragma unroll
    for (int k = 0; k < 3; ++k) {
        e2[k] = a[k] - b[k];
        pe += e2[k] * e1[k];
    }
    #pragma unroll
    for (int k = 0; k < 3; ++k) e2[k] -= pe * e1[k];
    nn = rsqrtf(e2[0] * e2[0] + e2[1] * e2[1] + e2[2] * e2[2]);
    #pragma unroll
    for (int k = 0; k < 3; ++k) e2[k] *= nn;
    e3[0] = e1[1] * e2[2] - e1[2] * e2[1];
    e3[1] = e1[2] * e2[0] - e1[0] * e2[2];
    e3[2] = e1[0] * e2[1] - e1[1] * e2[0];

    float acc[kFeat];
    float nf[kNbField];  // mode 1: neighbours' field changes (lab frame)
    #pragma unroll
    for (int c = 0; c < kFeat; ++c) acc[c] = 0.f;
    #pragma unroll
    for (int c = 0; c < kNbField; ++c) nf[c] = 0.f;
    const int n = min(nnb[A], cap);
    for (int t = lane; t < n; t += 32) {
        const int B = nb[(size_t)A * cap + t];
        const float* dd = nbd + 3 * ((size_t)A * cap + t);
        const float* oB = off + 3 * (size_t)K * B;
        if (mode == 1) {
            // O-O vector: the list's FP32 minimum-image vector plus B's O offset
            float d[3] = {dd[0] + oB[0], dd[1] + oB[1], dd[2] + oB[2]};
            if (box.periodic) {
                #pragma unroll
                for (int k = 0; k < 3; ++k) d[k] -= box.L[k] * rintf(d[k] * box.inv[k]);
            }
            const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (r2 < kRC * kRC) {
                const float fc = 0.5f * (cosf(kPiF * sqrtf(r2) / kRC) + 1.f);
                const float* fB = E0 + 3 * (size_t)K * B;
                #pragma unroll
                for (int k = 0; k < 3; ++k) {
                    nf[k] += fc * fB[k];
                    nf[3 + k] += fc * (fB[3 + k] + fB[6 + k]);
                }
            }
        }
        #pragma unroll
        for (int s = 0; s < 3; ++s) {
            float d[3] = {dd[0] + oB[3 * s], dd[1] + oB[3 * s + 1], dd[2] + oB[3 * s + 2]};
            if (box.periodic) {
                #pragma unroll
                for (int k = 0; k < 3; ++k) d[k] -= box.L[k] * rintf(d[k] * box.inv[k]);
            }
            const float r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (r2 >= kRC * kRC) continue;
            const float r = sqrtf(r2), ir = 1.f / r;
            const float fc = 0.5f * (cosf(kPiF * r / kRC) + 1.f);
            const float p1 = (d[0] * e1[0] + d[1] * e1[1] + d[2] * e1[2]) * ir;
            const float p2 = (d[0] * e2[0] + d[1] * e2[1] + d[2] * e2[2]) * ir;
            const float p3 = (d[0] * e3[0] + d[1] * e3[1] + d[2] * e3[2]) * ir;
            const int base = s == 0 ? 0 : 24;
            #pragma unroll
            for (int k = 0; k < 6; ++k) {
                const float x = (r - (kR0 + kDR * k)) / kSigma;
                const float g = expf(-x * x) * fc;
                acc[base + 4 * k] += g;
                acc[base + 4 * k + 1] += g * p1;
                acc[base + 4 * k + 2] += g * p2;
                acc[base + 4 * k + 3] += g * p3;
            }
        }
    }
    #pragma unroll
    for (int c = 0; c < kFeat; ++c) {
        float v = acc[c];
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) D[(size_t)A * kIn + c] = v;
    }
    if (lane == 0) {
        #pragma unroll
        for (int s = 0; s < 3; ++s) {
            const float* e = E0 + 3 * ((size_t)K * A + s);
            D[(size_t)A * kIn + kFeat + 3 * s] = e[0] * e1[0] + e[1] * e1[1] + e[2] * e1[2];
            D[(size_t)A * kIn + kFeat + 3 * s + 1] = e[0] * e2[0] + e[1] * e2[1] + e[2] * e2[2];
            D[(size_t)A * kIn + kFeat + 3 * s + 2] = e[0] * e3[0] + e[1] * e3[1] + e[2] * e3[2];
        }
        for (int c = kFeat + kField; c < kIn; ++c) D[(size_t)A * kIn + c] = 0.f;
    }
    if (mode == 1) {
        // neighbour sums in the water's frame (fixed-order warp reduction)
        #pragma unroll
        for (int c = 0; c < kNbField; ++c) {
            #pragma unroll
            for (int o = 16; o > 0; o >>= 1) nf[c] += __shfl_xor_sync(0xffffffffu, nf[c], o);
        }
        if (lane == 0) {
            #pragma unroll
            for (int g = 0; g < 2; ++g) {
                const float* e = nf + 3 * g;
                float* out = D + (size_t)A * kIn + kFeat + kField + 3 * g;
                out[0] = e[0] * e1[0] + e[1] * e1[1] + e[2] * e1[2];
                out[1] = e[0] * e2[0] + e[1] * e2[1] + e[2] * e2[2];
                out[2] = e[0] * e3[0] + e[1] * e3[1] + e[2] * e3[2];
            }
        }
    }
    if (lane == 0) {
        #pragma unroll
        for (int k = 0; k < 3; ++k) {
            F[(size_t)A * 9 + k] = e1[k];
            F[(size_t)A * 9 + 3 + k] = e2[k];
            F[(size_t)A * 9 + 6 + k] = e3[k];
        }
    }
}

// --------------------------------------------------------------- network
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}
__device__ __forceinline__ uint32_t lds2(const __nv_bfloat16* p) { return *reinterpret_cast<const uint32_t*>(p); }

// D += A B, m16n8k16, BF16 operands, FP32 accumulators
__device__ __forceinline__ void mma16816(float (&c)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float silu(float z) { return z / (1.f + expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
    const float s = 1.f / (1.f + expf(-z));
    return s * (1.f + z * (1.f - s));
}

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Shared memory of the network kernels (BF16 element offsets, then floats).
struct SmemPlan {
    static constexpr int W1 = 0;                       // [64][64]
    static constexpr int W2 = W1 + kHidden * kIn;      // [64][64]
    static constexpr int W2T = W2 + kHidden * kHidden;  // [64][64] (W2 transposed)
    static constexpr int W3 = W2T + kHidden * kHidden;  // [16][64] (rows >= 9 zero)
    static constexpr int W3T = W3 + 16 * kHidden;       // [64][16]
    static constexpr int BF16_END = W3T + kHidden * 16;
    // per-warp transposed tiles (BF16), [feature or neuron][16 samples]
    static constexpr int XT = 0, A1T = XT + kIn * 16, A2T = A1T + kHidden * 16, Z1T = A2T + kHidden * 16,
                         Z2T = Z1T + kHidden * 16, DYT = Z2T + kHidden * 16, WARP = DYT + 16 * 16;
    // floats after the BF16 area: b1[64], b2[64], b3[16], mean[64], inv[64]
    static constexpr int FB1 = 0, FB2 = 64, FB3 = 128, FMEAN = 144, FINV = 208, F_END = 272;
    static size_t bytes(bool train) {
        size_t b = sizeof(__nv_bfloat16) * (size_t)BF16_END + sizeof(float) * F_END;
        if (train) b += sizeof(float) * (size_t)kParams + sizeof(__nv_bfloat16) * (size_t)WARP * kWarps;
        return b;
    }
};

// One kernel for inference (TRAIN = false: Y = network(X)) and training
// (TRAIN = true: loss and gradient of a batch added to loss[0], grad).
// Row r of the batch is sample rows[r] (identity when random_seed == 0,
// else a hashed uniform draw from nsrc samples).
template <bool TRAIN>
__global__ void __launch_bounds__(32 * kWarps) mlp_kernel(int n, const float* __restrict__ params,
                                                           const float* __restrict__ X, const float* __restrict__ T,
                                                           long nsrc, unsigned long long random_seed, float inv_n,
                                                           float* __restrict__ Y, float* __restrict__ grad,
                                                           double* __restrict__ loss) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    using P = SmemPlan;
    __nv_bfloat16* sb = reinterpret_cast<__nv_bfloat16*>(smem_raw);
    float* sf = reinterpret_cast<float*>(sb + P::BF16_END);
    float* sG = sf + P::F_END;
    __nv_bfloat16* sWarpAll = reinterpret_cast<__nv_bfloat16*>(sG + kParams);
    const int tid = threadIdx.x;
    // stage the weights (BF16, with the transposes the backward pass reads)
    for (int i = tid; i < kHidden * kIn; i += blockDim.x) sb[P::W1 + i] = __float2bfloat16_rn(params[kW1 + i]);
    for (int i = tid; i < kHidden * kHidden; i += blockDim.x) {
        const int o = i / kHidden, k = i % kHidden;
        const __nv_bfloat16 w = __float2bfloat16_rn(params[kW2 + i]);
        sb[P::W2 + i] = w;
        sb[P::W2T + k * kHidden + o] = w;
    }
    for (int i = tid; i < 16 * kHidden; i += blockDim.x) {
        const int o = i / kHidden, h = i % kHidden;
        const __nv_bfloat16 w = __float2bfloat16_rn(o < kOut ? params[kW3 + i] : 0.f);
        sb[P::W3 + i] = w;
        sb[P::W3T + h * 16 + o] = w;
    }
    for (int i = tid; i < kHidden; i += blockDim.x) {
        sf[P::FB1 + i] = params[kB1 + i];
        sf[P::FB2 + i] = params[kB2 + i];
    }
    for (int i = tid; i < 16; i += blockDim.x) sf[P::FB3 + i] = i < kOut ? params[kB3 + i] : 0.f;
    for (int i = tid; i < kIn; i += blockDim.x) {
        sf[P::FMEAN + i] = params[kParams + i];
        sf[P::FINV + i] = params[kParams + kIn + i];
    }
    if (TRAIN)
        for (int i = tid; i < kParams; i += blockDim.x) sG[i] = 0.f;
    __syncthreads();

    const int warp = tid >> 5, lane = tid & 31, g = lane >> 2, t = lane & 3;
    __nv_bfloat16* sw = sWarpAll + (size_t)warp * P::WARP;
    const __nv_bfloat16* W1 = sb + P::W1;
    const __nv_bfloat16* W2 = sb + P::W2;
    const __nv_bfloat16* W2T = sb + P::W2T;
    const __nv_bfloat16* W3 = sb + P::W3;
    const __nv_bfloat16* W3T = sb + P::W3T;
    double lsum = 0.0;
    const int ntiles = (n + 15) / 16;
    for (int tile = blockIdx.x * kWarps + warp; tile < ntiles; tile += gridDim.x * kWarps) {
        const int rA = tile * 16 + g, rB = rA + 8;
        const bool vA = rA < n, vB = rB < n;
        long sA = rA, sBr = rB;
        if (random_seed) {
            sA = (long)(mix64(random_seed ^ (0xD1B54A32D192ED03ull * (unsigned long long)(rA + 1))) %
                        (unsigned long long)nsrc);
            sBr = (long)(mix64(random_seed ^ (0xD1B54A32D192ED03ull * (unsigned long long)(rB + 1))) %
                         (unsigned long long)nsrc);
        }
        // ---- layer 1 inputs: standardised inputs as A fragments
        float xv[4][8];
        uint32_t ax[4][4];
        #pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            const int c0 = 16 * kk + 2 * t;
            const int cols[4] = {c0, c0 + 1, c0 + 8, c0 + 9};
            #pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int c = cols[q];
                xv[kk][q] = vA ? (X[sA * kIn + c] - sf[P::FMEAN + c]) * sf[P::FINV + c] : 0.f;
                xv[kk][4 + q] = vB ? (X[sBr * kIn + c] - sf[P::FMEAN + c]) * sf[P::FINV + c] : 0.f;
            }
            ax[kk][0] = pack_bf16(xv[kk][0], xv[kk][1]);
            ax[kk][1] = pack_bf16(xv[kk][4], xv[kk][5]);
            ax[kk][2] = pack_bf16(xv[kk][2], xv[kk][3]);
            ax[kk][3] = pack_bf16(xv[kk][6], xv[kk][7]);
        }
        auto put = [&](int base, int col, int row, float v) { sw[base + col * 16 + row] = __float2bfloat16_rn(v); };
        if (TRAIN) {
            #pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
                const int c0 = 16 * kk + 2 * t;
                const int cols[4] = {c0, c0 + 1, c0 + 8, c0 + 9};
                #pragma unroll
                for (int q = 0; q < 4; ++q) {
                    put(P::XT, cols[q], g, xv[kk][q]);
                    put(P::XT, cols[q], g + 8, xv[kk][4 + q]);
                }
            }
        }
        // ---- layer 1
        float z1[8][4];
        #pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int col = 8 * j + 2 * t;
            z1[j][0] = z1[j][2] = sf[P::FB1 + col];
            z1[j][1] = z1[j][3] = sf[P::FB1 + col + 1];
            const __nv_bfloat16* wr = W1 + (8 * j + g) * kIn + 2 * t;
            #pragma unroll
            for (int kk = 0; kk < 4; ++kk) mma16816(z1[j], ax[kk], lds2(wr + 16 * kk), lds2(wr + 16 * kk + 8));
        }
        uint32_t a1[4][4];
        #pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            float h[2][4];
            #pragma unroll
            for (int e = 0; e < 4; ++e) {
                h[0][e] = silu(z1[2 * kk][e]);
                h[1][e] = silu(z1[2 * kk + 1][e]);
            }
            a1[kk][0] = pack_bf16(h[0][0], h[0][1]);
            a1[kk][1] = pack_bf16(h[0][2], h[0][3]);
            a1[kk][2] = pack_bf16(h[1][0], h[1][1]);
            a1[kk][3] = pack_bf16(h[1][2], h[1][3]);
            if (TRAIN) {
                #pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int c = 8 * (2 * kk + u) + 2 * t;
                    put(P::A1T, c, g, h[u][0]);
                    put(P::A1T, c + 1, g, h[u][1]);
                    put(P::A1T, c, g + 8, h[u][2]);
                    put(P::A1T, c + 1, g + 8, h[u][3]);
                }
            }
        }
        // ---- layer 2
        float z2[8][4];
        #pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int col = 8 * j + 2 * t;
            z2[j][0] = z2[j][2] = sf[P::FB2 + col];
            z2[j][1] = z2[j][3] = sf[P::FB2 + col + 1];
            const __nv_bfloat16* wr = W2 + (8 * j + g) * kHidden + 2 * t;
            #pragma unroll
            for (int kk = 0; kk < 4; ++kk) mma16816(z2[j], a1[kk], lds2(wr + 16 * kk), lds2(wr + 16 * kk + 8));
        }
        uint32_t a2[4][4];
        #pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            float h[2][4];
            #pragma unroll
            for (int e = 0; e < 4; ++e) {
                h[0][e] = silu(z2[2 * kk][e]);
                h[1][e] = silu(z2[2 * kk + 1][e]);
            }
            a2[kk][0] = pack_bf16(h[0][0], h[0][1]);
            a2[kk][1] = pack_bf16(h[0][2], h[0][3]);
            a2[kk][2] = pack_bf16(h[1][0], h[1][1]);
            a2[kk][3] = pack_bf16(h[1][2], h[1][3]);
            if (TRAIN) {
                #pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int c = 8 * (2 * kk + u) + 2 * t;
                    put(P::A2T, c, g, h[u][0]);
                    put(P::A2T, c + 1, g, h[u][1]);
                    put(P::A2T, c, g + 8, h[u][2]);
                    put(P::A2T, c + 1, g + 8, h[u][3]);
                }
            }
        }
        // ---- layer 3 (outputs padded to 16)
        float y[2][4];
        #pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int col = 8 * j + 2 * t;
            y[j][0] = y[j][2] = sf[P::FB3 + col];
            y[j][1] = y[j][3] = sf[P::FB3 + col + 1];
            const __nv_bfloat16* wr = W3 + (8 * j + g) * kHidden + 2 * t;
            #pragma unroll
            for (int kk = 0; kk < 4; ++kk) mma16816(y[j], a2[kk], lds2(wr + 16 * kk), lds2(wr + 16 * kk + 8));
        }
        if (!TRAIN) {
            #pragma unroll
            for (int j = 0; j < 2; ++j)
                #pragma unroll
                for (int e = 0; e < 4; ++e) {
                    const int col = 8 * j + 2 * t + (e & 1);
                    const int row = e < 2 ? rA : rB;
                    if (row < n && col < kOut) Y[(size_t)row * kOut + col] = y[j][e];
                }
            continue;
        }
        // ---- backward: residuals and output gradient
        float dy[2][4];
        #pragma unroll
        for (int j = 0; j < 2; ++j)
            #pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int col = 8 * j + 2 * t + (e & 1);
                const bool v = (e < 2 ? vA : vB) && col < kOut;
                const long srow = e < 2 ? sA : sBr;
                const float r = v ? y[j][e] - T[srow * kOut + col] : 0.f;
                lsum += (double)r * r;
                dy[j][e] = r * inv_n;
                if (Y && v) Y[(size_t)(e < 2 ? rA : rB) * kOut + col] = y[j][e];
            }
        // column sums over the tile's 16 rows: lanes with equal t share columns
        auto colsum = [&](float v) {
            v += __shfl_xor_sync(0xffffffffu, v, 4);
            v += __shfl_xor_sync(0xffffffffu, v, 8);
            v += __shfl_xor_sync(0xffffffffu, v, 16);
            return v;
        };
        #pragma unroll
        for (int j = 0; j < 2; ++j) {
            const float s0 = colsum(dy[j][0] + dy[j][2]), s1 = colsum(dy[j][1] + dy[j][3]);
            const int col = 8 * j + 2 * t;
            if (g == 0) {
                if (col < kOut) atomicAdd(&sG[kB3 + col], s0);
                if (col + 1 < kOut) atomicAdd(&sG[kB3 + col + 1], s1);
            }
        }
        uint32_t ady[4] = {pack_bf16(dy[0][0], dy[0][1]), pack_bf16(dy[0][2], dy[0][3]),
                           pack_bf16(dy[1][0], dy[1][1]), pack_bf16(dy[1][2], dy[1][3])};
        // da2 = dy W3 ; dz2 = da2 * SiLU'(z2)
        float dz2[8][4];
        #pragma unroll
        for (int j = 0; j < 8; ++j) {
            dz2[j][0] = dz2[j][1] = dz2[j][2] = dz2[j][3] = 0.f;
            const __nv_bfloat16* wr = W3T + (8 * j + g) * 16 + 2 * t;
            mma16816(dz2[j], ady, lds2(wr), lds2(wr + 8));
            #pragma unroll
            for (int e = 0; e < 4; ++e) dz2[j][e] *= dsilu(z2[j][e]);
            const float s0 = colsum(dz2[j][0] + dz2[j][2]), s1 = colsum(dz2[j][1] + dz2[j][3]);
            if (g == 0) {
                atomicAdd(&sG[kB2 + 8 * j + 2 * t], s0);
                atomicAdd(&sG[kB2 + 8 * j + 2 * t + 1], s1);
            }
        }
        uint32_t adz2[4][4];
        #pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            adz2[kk][0] = pack_bf16(dz2[2 * kk][0], dz2[2 * kk][1]);
            adz2[kk][1] = pack_bf16(dz2[2 * kk][2], dz2[2 * kk][3]);
            adz2[kk][2] = pack_bf16(dz2[2 * kk + 1][0], dz2[2 * kk + 1][1]);
            adz2[kk][3] = pack_bf16(dz2[2 * kk + 1][2], dz2[2 * kk + 1][3]);
        }
        // da1 = dz2 W2 ; dz1 = da1 * SiLU'(z1)
        float dz1[8][4];
        #pragma unroll
        for (int j = 0; j < 8; ++j) {
            dz1[j][0] = dz1[j][1] = dz1[j][2] = dz1[j][3] = 0.f;
            const __nv_bfloat16* wr = W2T + (8 * j + g) * kHidden + 2 * t;
            #pragma unroll
            for (int kk = 0; kk < 4; ++kk) mma16816(dz1[j], adz2[kk], lds2(wr + 16 * kk), lds2(wr + 16 * kk + 8));
            #pragma unroll
            for (int e = 0; e < 4; ++e) dz1[j][e] *= dsilu(z1[j][e]);
            const float s0 = colsum(dz1[j][0] + dz1[j][2]), s1 = colsum(dz1[j][1] + dz1[j][3]);
            if (g == 0) {
                atomicAdd(&sG[kB1 + 8 * j + 2 * t], s0);
                atomicAdd(&sG[kB1 + 8 * j + 2 * t + 1], s1);
            }
        }
        // ---- transposed BF16 tiles [column][sample] of the hidden
        // gradients (inputs and activations were written in the forward pass)
        #pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int c = 8 * j + 2 * t;
            put(P::Z1T, c, g, dz1[j][0]);
            put(P::Z1T, c + 1, g, dz1[j][1]);
            put(P::Z1T, c, g + 8, dz1[j][2]);
            put(P::Z1T, c + 1, g + 8, dz1[j][3]);
            put(P::Z2T, c, g, dz2[j][0]);
            put(P::Z2T, c + 1, g, dz2[j][1]);
            put(P::Z2T, c, g + 8, dz2[j][2]);
            put(P::Z2T, c + 1, g + 8, dz2[j][3]);
        }
        #pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int c = 8 * j + 2 * t;
            put(P::DYT, c, g, dy[j][0]);
            put(P::DYT, c + 1, g, dy[j][1]);
            put(P::DYT, c, g + 8, dy[j][2]);
            put(P::DYT, c + 1, g + 8, dy[j][3]);
        }
        __syncwarp();
        // weight gradients: dW[o][i] = sum_s dZ[s][o] A[s][i] as
        // (16-row tiles of dZ^T) x (A over the 16 samples)
        auto wgrad = [&](int zt, int mtiles, int at, int ntiles, int out_off, int ncols, int nrows_valid) {
            for (int mi = 0; mi < mtiles; ++mi) {
                uint32_t af[4];
                const __nv_bfloat16* ar = sw + zt + (16 * mi + g) * 16 + 2 * t;
                af[0] = lds2(ar);
                af[1] = lds2(ar + 8 * 16);
                af[2] = lds2(ar + 8);
                af[3] = lds2(ar + 8 * 16 + 8);
                for (int j = 0; j < ntiles; ++j) {
                    float c[4] = {0.f, 0.f, 0.f, 0.f};
                    const __nv_bfloat16* br = sw + at + (8 * j + g) * 16 + 2 * t;
                    mma16816(c, af, lds2(br), lds2(br + 8));
                    const int o0 = 16 * mi + g, i0 = 8 * j + 2 * t;
                    if (o0 < nrows_valid) {
                        atomicAdd(&sG[out_off + o0 * ncols + i0], c[0]);
                        atomicAdd(&sG[out_off + o0 * ncols + i0 + 1], c[1]);
                    }
                    if (o0 + 8 < nrows_valid) {
                        atomicAdd(&sG[out_off + (o0 + 8) * ncols + i0], c[2]);
                        atomicAdd(&sG[out_off + (o0 + 8) * ncols + i0 + 1], c[3]);
                    }
                }
            }
        };
        wgrad(P::DYT, 1, P::A2T, 8, kW3, kHidden, kOut);
        wgrad(P::Z2T, 4, P::A1T, 8, kW2, kHidden, kHidden);
        wgrad(P::Z1T, 4, P::XT, 8, kW1, kIn, kHidden);
        __syncwarp();
    }
    if (TRAIN) {
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
        if (lane == 0 && lsum != 0.0) atomicAdd(loss, 0.5 * lsum * (double)inv_n);
        __syncthreads();
        for (int i = tid; i < kParams; i += blockDim.x) atomicAdd(&grad[i], sG[i]);
    }
}

// ------------------------------------------------ inference on tcgen05
// The forward pass for prediction (not training) on the fifth-generation
// tensor cores: a block of 128 threads takes tiles of 128 samples (M = 128,
// thread t owns sample row t, which is tensor-memory lane t).  Each layer is
// four tcgen05.mma.kind::f16 (K = 16 each) issued by one thread: A, the
// layer's input activations, in tensor memory (two fp16 per 32-bit column,
// column 8 j + c of k-tile j holding inputs 16 j + 2c and 16 j + 2c + 1); B,
// the layer's weights [out][in], in shared memory as no-swizzle K-major core
// matrices (per k-tile [k half][row group][row][8 k]); D, FP32 in tensor
// memory (lane = sample, column = output).  Between layers each thread reads
// its row of D, adds the bias, applies SiLU and writes the fp16 activations
// back as the next layer's A.  fp16 operands (the products are rounded less
// than by the training kernel's bf16; the weights and activations of this
// network are far inside fp16's range), FP32 accumulation.
//
// Tensor memory: 128 columns (X, later H2, at 0-31; H1 at 32-63; D at
// 64-127).  The block's ~19.5 KB of shared memory keeps it off the SMs that
// run the three-body tensor kernel (which holds all 512 columns and ~218 KB
// of shared memory), so its allocation never waits on that kernel.  Every
// wait is bounded; a block that gives up writes NaN outputs for its tiles
// and records the failure in *status.
constexpr int kTcRows = 128;   // samples per tile
constexpr int kTcCols = 128;   // tensor-memory columns
constexpr int kColA0 = 0, kColA1 = 32, kColD = 64;
constexpr int kW3Rows = 16;    // layer 3's N (outputs padded to 16)

// element index of weight (n, k) in the shared-memory B operand of N rows
__host__ __device__ constexpr int bmat_index(int n, int k, int N) {
    return (k >> 4) * (N * 16) + ((k & 15) >> 3) * (N * 8) + (n >> 3) * 64 + (n & 7) * 8 + (k & 7);
}

__device__ __forceinline__ uint32_t pack_f16(float lo, float hi) {
    const __half2 h = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&h);
}

__device__ __forceinline__ bool mlp_wait(uint32_t bar, uint32_t parity, volatile int* abort_flag, int* status) {
    return umma::mbar_wait(bar, parity, abort_flag, status, 1);
}

// The fp16 operand image of W1, W2, W3 (W3 padded to 16 rows) in the
// shared-memory B layout, made once per parameter change.
constexpr int kPackW1 = 0, kPackW2 = kHidden * kIn, kPackW3 = kPackW2 + kHidden * kHidden;
constexpr int kPackHalves = kPackW3 + kW3Rows * kHidden;
__global__ void pack_weights_kernel(const float* __restrict__ params, __half* __restrict__ wpack) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kPackW2) {
        wpack[kPackW1 + bmat_index(i / kIn, i % kIn, kHidden)] = __float2half_rn(params[kW1 + i]);
    } else if (i < kPackW3) {
        const int j = i - kPackW2;
        wpack[kPackW2 + bmat_index(j / kHidden, j % kHidden, kHidden)] = __float2half_rn(params[kW2 + j]);
    } else if (i < kPackHalves) {
        const int j = i - kPackW3, o = j / kHidden;
        wpack[kPackW3 + bmat_index(o, j % kHidden, kW3Rows)] = __float2half_rn(o < kOut ? params[kW3 + j] : 0.f);
    }
}

__global__ void __launch_bounds__(kTcRows) mlp_tc5_kernel(int n, const float* __restrict__ params,
                                                         const __half* __restrict__ wpack,
                                                         const float* __restrict__ X, float* __restrict__ Y,
                                                         int* __restrict__ status) {
    using namespace umma;
    __shared__ __align__(128) __half sW1[kHidden * kIn];
    __shared__ __align__(128) __half sW2[kHidden * kHidden];
    __shared__ __align__(128) __half sW3[kW3Rows * kHidden];
    __shared__ float sB1[kHidden], sB2[kHidden], sB3[kW3Rows], sMean[kIn], sInv[kIn];
    __shared__ __align__(8) uint64_t s_bar;
    __shared__ uint32_t s_tmem;
    __shared__ int s_abort;
    const int tid = threadIdx.x, warp = tid >> 5;
    {
        // the packed weights, 16 bytes per thread and copy
        const uint4* src = reinterpret_cast<const uint4*>(wpack);
        for (int i = tid; i < kPackW2 / 8; i += kTcRows) reinterpret_cast<uint4*>(sW1)[i] = src[kPackW1 / 8 + i];
        for (int i = tid; i < (kPackW3 - kPackW2) / 8; i += kTcRows)
            reinterpret_cast<uint4*>(sW2)[i] = src[kPackW2 / 8 + i];
        for (int i = tid; i < (kPackHalves - kPackW3) / 8; i += kTcRows)
            reinterpret_cast<uint4*>(sW3)[i] = src[kPackW3 / 8 + i];
    }
    if (tid < kHidden) {
        sB1[tid] = params[kB1 + tid];
        sB2[tid] = params[kB2 + tid];
        sMean[tid] = params[kParams + tid];
        sInv[tid] = params[kParams + kIn + tid];
    }
    if (tid < kW3Rows) sB3[tid] = tid < kOut ? params[kB3 + tid] : 0.f;
    const uint32_t bar = smem_addr(&s_bar);
    if (warp == 0) {
        tmem_alloc(smem_addr(&s_tmem), kTcCols);
        tmem_relinquish();
    }
    if (tid == 0) {
        s_abort = 0;
        mbar_init(bar, 1);
        fence_barrier_init();
    }
    fence_proxy_async();  // the weights, written by generic stores, are read by the tensor cores
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tb = s_tmem;
    const uint32_t lb = tb + ((uint32_t)(32 * warp) << 16);  // this warp's lane quadrant
    const uint32_t w1 = smem_addr(sW1), w2 = smem_addr(sW2), w3 = smem_addr(sW3);
    const int ntiles = (n + kTcRows - 1) / kTcRows;
    uint32_t phase = 0;
    bool ok = true;
    int tile = blockIdx.x;
    for (; tile < ntiles && ok; tile += gridDim.x) {
        const int row = tile * kTcRows + tid;
        const bool valid = row < n;
        // standardised inputs -> A (columns 0-31)
        #pragma unroll
        for (int kt = 0; kt < kIn / 16; ++kt) {
            float x[16];
            #pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float4 f = valid ? reinterpret_cast<const float4*>(X + (size_t)row * kIn)[4 * kt + q]
                                       : make_float4(0.f, 0.f, 0.f, 0.f);
                x[4 * q] = f.x;
                x[4 * q + 1] = f.y;
                x[4 * q + 2] = f.z;
                x[4 * q + 3] = f.w;
            }
            uint32_t v[8];
            #pragma unroll
            for (int c = 0; c < 8; ++c) {
                const int k = 16 * kt + 2 * c;
                const float x0 = valid ? (x[2 * c] - sMean[k]) * sInv[k] : 0.f;
                const float x1 = valid ? (x[2 * c + 1] - sMean[k + 1]) * sInv[k + 1] : 0.f;
                v[c] = pack_f16(x0, x1);
            }
            tmem_st8(lb + kColA0 + 8 * kt, v);
        }
        tmem_wait_st();
        tc_fence_before();
        __syncthreads();
        float out[kW3Rows];
        #pragma unroll 1
        for (int layer = 0; layer < 3 && ok; ++layer) {
            if (tid == 0) {
                tc_fence_after();
                const uint32_t a_col = layer == 1 ? kColA1 : kColA0;
                const uint32_t wb = layer == 0 ? w1 : (layer == 1 ? w2 : w3);
                const int N = layer == 2 ? kW3Rows : kHidden;
                const uint32_t idesc = idesc_f16(kTcRows, N);
                #pragma unroll
                for (int kt = 0; kt < kHidden / 16; ++kt)
                    mma_ts(tb + kColD, tb + a_col + 8 * kt,
                           sdesc(wb + (uint32_t)(kt * N * 16 * 2), (uint32_t)(N * 16), 128u), idesc, kt > 0);
                mma_commit(bar);
            }
            ok = mlp_wait(bar, phase, reinterpret_cast<volatile int*>(&s_abort), status);
            phase ^= 1;
            ok = __syncthreads_and(ok);
            if (!ok) break;
            tc_fence_after();
            if (layer < 2) {
                // bias + SiLU -> fp16 -> the next layer's A (H1 at 32-63, H2 at 0-31)
                const float* bias = layer == 0 ? sB1 : sB2;
                const uint32_t dst = layer == 0 ? kColA1 : kColA0;
                #pragma unroll
                for (int half = 0; half < 2; ++half) {
                    float z[32];
                    tmem_ld32(lb + kColD + 32 * half, z);
                    tmem_wait_ld();
                    #pragma unroll
                    for (int q = 0; q < 2; ++q) {
                        uint32_t v[8];
                        #pragma unroll
                        for (int c = 0; c < 8; ++c) {
                            const int o = 32 * half + 16 * q + 2 * c;
                            v[c] = pack_f16(silu(z[16 * q + 2 * c] + bias[o]), silu(z[16 * q + 2 * c + 1] + bias[o + 1]));
                        }
                        tmem_st8(lb + dst + 8 * (2 * half + q), v);
                    }
                }
                tmem_wait_st();
                tc_fence_before();
                __syncthreads();
            } else {
                float z[16];
                tmem_ld16(lb + kColD, z);
                tmem_wait_ld();
                #pragma unroll
                for (int o = 0; o < kW3Rows; ++o) out[o] = z[o] + sB3[o];
            }
        }
        if (!ok) break;
        if (valid)
            #pragma unroll
            for (int o = 0; o < kOut; ++o) Y[(size_t)row * kOut + o] = out[o];
        // D and A are rewritten by the next tile only after every thread's loads
        tc_fence_before();
        __syncthreads();
        tc_fence_after();
    }
    if (!ok) {
        // a wait gave up: NaN outputs for this block's remaining tiles (the
        // solver then fails loudly), and one more bounded wait for the
        // outstanding commit before the tensor memory is freed
        for (int t = tile; t < ntiles; t += gridDim.x) {
            const int row = t * kTcRows + tid;
            if (row < n)
                for (int o = 0; o < kOut; ++o) Y[(size_t)row * kOut + o] = __int_as_float(0x7fc00000);
        }
        const long long t0 = clock64();
        while (!mbar_try_wait(bar, phase ^ 1) && clock64() - t0 < kWaitCycles) {
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) tmem_dealloc(tb, kTcCols);
}

__global__ void adam_kernel(int np, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, float lr, float b1, float b2, float c1, float c2, float eps) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi * c1) / (sqrtf(vi * c2) + eps);
}

// network outputs (frame components, `scale` e nm) -> lab-frame dipoles per site
__global__ void to_lab_kernel(int nmol, int K, const float* __restrict__ Y, const float* __restrict__ F,
                              float* __restrict__ m, float scale) {
    const int A = blockIdx.x * blockDim.x + threadIdx.x;
    if (A >= nmol) return;
    for (int s = 0; s < K; ++s)
        for (int d = 0; d < 3; ++d) {
            float v = 0.f;
            if (s < 3)
                for (int c = 0; c < 3; ++c) v += Y[(size_t)A * kOut + 3 * s + c] * F[(size_t)A * 9 + 3 * c + d];
            m[3 * ((size_t)K * A + s) + d] = scale * v;
        }
}

// converged FP64 dipoles (minus mu_base if given) -> frame components in
// units of `scale` (targets) appended at row0
__global__ void targets_kernel(int nmol, int K, const double* __restrict__ mu, const double* __restrict__ mu_base,
                               const float* __restrict__ F, const float* __restrict__ D, float* __restrict__ X,
                               float* __restrict__ T, long row0, double scale) {
    const int A = blockIdx.x * blockDim.x + threadIdx.x;
    if (A >= nmol) return;
    for (int s = 0; s < 3; ++s)
        for (int c = 0; c < 3; ++c) {
            double v = 0.0;
            for (int d = 0; d < 3; ++d) {
                const size_t i = 3 * ((size_t)K * A + s) + d;
                v += (mu[i] - (mu_base ? mu_base[i] : 0.0)) * (double)F[(size_t)A * 9 + 3 * c + d];
            }
            T[(row0 + A) * kOut + 3 * s + c] = (float)(v / scale);
        }
    for (int c = 0; c < kIn; ++c) X[(row0 + A) * kIn + c] = D[(size_t)A * kIn + c];
}

// column sums and sums of squares of the dataset (FP64 atomics)
__global__ void stats_kernel(long nrows, const float* __restrict__ X, double* __restrict__ stats) {
    const int c = blockIdx.y;
    double s = 0.0, s2 = 0.0;
    for (long r = blockIdx.x * (long)blockDim.x + threadIdx.x; r < nrows; r += (long)gridDim.x * blockDim.x) {
        const double v = X[r * kIn + c];
        s += v;
        s2 += v * v;
    }
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        s2 += __shfl_xor_sync(0xffffffffu, s2, o);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&stats[c], s);
        atomicAdd(&stats[kIn + c], s2);
    }
}

template <class T>
cudaError_t grow(T** p, size_t have, size_t need, size_t keep) {
    if (need <= have) return cudaSuccess;
    T* q = nullptr;
    cudaError_t e = cudaMalloc(&q, sizeof(T) * need);
    if (e != cudaSuccess) return e;
    if (*p && keep) {
        e = cudaMemcpy(q, *p, sizeof(T) * keep, cudaMemcpyDeviceToDevice);
        if (e != cudaSuccess) {
            cudaFree(q);
            return e;
        }
    }
    if (*p) cudaFree(*p);
    *p = q;
    return cudaSuccess;
}

cudaError_t mlp_attributes() {
    static int done = -1;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || done == dev) return e;
    if ((e = cudaFuncSetAttribute(mlp_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)SmemPlan::bytes(true))))
        return e;
    done = dev;
    return cudaSuccess;
}

unsigned long long mix64_host(unsigned long long z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int mlp_tc5_blocks(int n) {
    const int tiles = (n + kTcRows - 1) / kTcRows;
    return tiles < 1 ? 1 : (tiles > 1024 ? 1024 : tiles);
}

int mlp_blocks(int n) {
    const int tiles = (n + 15) / 16;
    const int b = (tiles + kWarps - 1) / kWarps;
    return b < 1 ? 1 : (b > 1024 ? 1024 : b);
}

#define GUESS_OK(expr)                          \
    do {                                        \
        cudaError_t e_ = (expr);                \
        if (e_ != cudaSuccess) return e_;       \
    } while (0)

// the weights changed: make the fp16 operand image the prediction kernel copies
cudaError_t repack_weights(GuessBuffers* b, cudaStream_t st) {
    if (!b->wpack) GUESS_OK(cudaMalloc(&b->wpack, sizeof(__half) * kPackHalves));
    if (!b->status) {
        GUESS_OK(cudaMalloc(&b->status, sizeof(int)));
        GUESS_OK(cudaMemset(b->status, 0, sizeof(int)));
    }
    count_launch();
    pack_weights_kernel<<<(kPackHalves + 255) / 256, 256, 0, st>>>(b->params, b->wpack);
    return cudaGetLastError();
}


}  // namespace

GuessNet::GuessNet(int mode) : b_(new GuessBuffers), mode_(mode) {}

GuessNet::~GuessNet() {
    for (void* p : {(void*)b_->params, (void*)b_->adam_m, (void*)b_->adam_v, (void*)b_->grad, (void*)b_->loss,
                    (void*)b_->stats, (void*)b_->desc, (void*)b_->frames, (void*)b_->ybuf, (void*)b_->X,
                    (void*)b_->T, (void*)b_->hx, (void*)b_->ht, (void*)b_->hy, (void*)b_->status, (void*)b_->wpack})
        if (p) cudaFree(p);
    delete b_;
}

const float* GuessNet::d_desc() const { return b_->desc; }
const float* GuessNet::d_frames() const { return b_->frames; }

cudaError_t GuessNet::descriptors(cudaStream_t st, int nmol, int K, const float* off, const int* nb,
                                  const float* nbd, const int* nnb, int cap, const double* box, int periodic,
                                  const float* field) {
    if (nmol > b_->cap_mol) {
        GUESS_OK(grow(&b_->desc, 0, (size_t)nmol * kIn, 0));
        GUESS_OK(grow(&b_->frames, 0, (size_t)nmol * 9, 0));
        GUESS_OK(grow(&b_->ybuf, 0, (size_t)nmol * kOut, 0));
        b_->cap_mol = nmol;
    }
    GBox gb{};
    gb.periodic = periodic;
    for (int k = 0; k < 3; ++k) {
        gb.L[k] = periodic ? (float)box[k] : 0.f;
        gb.inv[k] = periodic ? (float)(1.0 / box[k]) : 0.f;
    }
    count_launch();
    descriptor_kernel<<<(nmol * 32 + 127) / 128, 128, 0, st>>>(nmol, K, off, nb, nbd, nnb, cap, gb, field,
                                                               b_->desc, b_->frames, mode_);
    return cudaGetLastError();
}

cudaError_t GuessNet::collect(cudaStream_t st, int nmol, int K, const double* mu_d, const double* mu_base) {
    const long need = nsamples_ + nmol;
    if (need > b_->cap_s) {
        const long cap = need + need / 2 + 1024;
        GUESS_OK(cudaStreamSynchronize(st));
        GUESS_OK(grow(&b_->X, (size_t)b_->cap_s * kIn, (size_t)cap * kIn, (size_t)nsamples_ * kIn));
        GUESS_OK(grow(&b_->T, (size_t)b_->cap_s * kOut, (size_t)cap * kOut, (size_t)nsamples_ * kOut));
        b_->cap_s = cap;
    }
    count_launch();
    targets_kernel<<<(nmol + 127) / 128, 128, 0, st>>>(nmol, K, mu_d, mode_ == 1 ? mu_base : nullptr, b_->frames,
                                                        b_->desc, b_->X, b_->T, nsamples_,
                                                        mode_ == 1 ? (double)kResScale : (double)kOutScale);
    nsamples_ = need;
    return cudaGetLastError();
}

cudaError_t GuessNet::predict(cudaStream_t st, int nmol, int K, float* m_out) {
    if (!b_->wpack) return cudaErrorInvalidValue;  // set_params or train make the image
    count_launch();
    mlp_tc5_kernel<<<mlp_tc5_blocks(nmol), kTcRows, 0, st>>>(nmol, b_->params, b_->wpack, b_->desc, b_->ybuf,
                                                             b_->status);
    count_launch();
    to_lab_kernel<<<(nmol + 127) / 128, 128, 0, st>>>(nmol, K, b_->ybuf, b_->frames, m_out,
                                                       mode_ == 1 ? kResScale : kOutScale);
    return cudaGetLastError();
}

static void init_host_params(std::vector<float>& h, unsigned long long seed) {
    // He-style normal initialisation (SplitMix64 + Box-Muller); biases zero;
    // standardisation identity until the dataset statistics are set
    unsigned long long s = seed ? seed : 0x2545F4914F6CDD1Dull;
    auto next = [&]() {
        s += 0x9E3779B97F4A7C15ull;
        unsigned long long z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return ((z >> 11) + 0.5) * (1.0 / 9007199254740992.0);
    };
    auto normal = [&]() { return std::sqrt(-2.0 * std::log(next())) * std::cos(6.283185307179586 * next()); };
    h.assign(kBlockFloats, 0.f);
    for (int i = 0; i < kHidden * kIn; ++i) h[kW1 + i] = (float)(normal() * std::sqrt(2.0 / kIn));
    for (int i = 0; i < kHidden * kHidden; ++i) h[kW2 + i] = (float)(normal() * std::sqrt(2.0 / kHidden));
    for (int i = 0; i < kOut * kHidden; ++i) h[kW3 + i] = (float)(normal() * std::sqrt(1.0 / kHidden));
    for (int c = 0; c < kIn; ++c) h[kParams + kIn + c] = 1.f;
}

cudaError_t GuessNet::set_params(const float* h_block) {
    if (!b_->params) GUESS_OK(cudaMalloc(&b_->params, sizeof(float) * kBlockFloats));
    GUESS_OK(cudaMemcpy(b_->params, h_block, sizeof(float) * kBlockFloats, cudaMemcpyHostToDevice));
    b_->stats_set = true;
    b_->adam_t = 0;
    if (b_->adam_m) {
        GUESS_OK(cudaMemset(b_->adam_m, 0, sizeof(float) * kParams));
        GUESS_OK(cudaMemset(b_->adam_v, 0, sizeof(float) * kParams));
    }
    GUESS_OK(repack_weights(b_, 0));
    GUESS_OK(cudaStreamSynchronize(0));
    ready_ = true;
    return cudaSuccess;
}

cudaError_t GuessNet::get_params(float* h_block) const {
    if (!b_->params) return cudaErrorInvalidValue;
    return cudaMemcpy(h_block, b_->params, sizeof(float) * kBlockFloats, cudaMemcpyDeviceToHost);
}

cudaError_t GuessNet::train(cudaStream_t st, int steps, int batch, double lr, unsigned long long seed,
                            double* loss_out) {
    if (nsamples_ <= 0 || steps <= 0 || batch <= 0) return cudaErrorInvalidValue;
    GUESS_OK(mlp_attributes());
    if (!b_->params) {
        std::vector<float> h;
        init_host_params(h, seed);
        GUESS_OK(cudaMalloc(&b_->params, sizeof(float) * kBlockFloats));
        GUESS_OK(cudaMemcpy(b_->params, h.data(), sizeof(float) * kBlockFloats, cudaMemcpyHostToDevice));
    }
    if (!b_->adam_m) {
        GUESS_OK(cudaMalloc(&b_->adam_m, sizeof(float) * kParams));
        GUESS_OK(cudaMalloc(&b_->adam_v, sizeof(float) * kParams));
        GUESS_OK(cudaMemset(b_->adam_m, 0, sizeof(float) * kParams));
        GUESS_OK(cudaMemset(b_->adam_v, 0, sizeof(float) * kParams));
    }
    if (!b_->grad) GUESS_OK(cudaMalloc(&b_->grad, sizeof(float) * kParams));
    if (!b_->loss) GUESS_OK(cudaMalloc(&b_->loss, sizeof(double) * 2));
    if (!b_->stats) GUESS_OK(cudaMalloc(&b_->stats, sizeof(double) * 2 * kIn));
    if (!b_->stats_set) {
        // standardisation from the dataset, fixed from then on
        GUESS_OK(cudaMemsetAsync(b_->stats, 0, sizeof(double) * 2 * kIn, st));
        count_launch();
        stats_kernel<<<dim3(64, kIn), 256, 0, st>>>(nsamples_, b_->X, b_->stats);
        std::vector<double> hs(2 * kIn);
        GUESS_OK(cudaMemcpyAsync(hs.data(), b_->stats, sizeof(double) * 2 * kIn, cudaMemcpyDeviceToHost, st));
        GUESS_OK(cudaStreamSynchronize(st));
        std::vector<float> ms(2 * kIn);
        for (int c = 0; c < kIn; ++c) {
            const double mean = hs[c] / nsamples_;
            const double var = hs[kIn + c] / nsamples_ - mean * mean;
            ms[c] = (float)mean;
            // constant columns (the zero padding) keep unit scale
            ms[kIn + c] = (float)(var > 1e-20 ? 1.0 / std::sqrt(var) : 1.0);
        }
        GUESS_OK(cudaMemcpy(b_->params + kParams, ms.data(), sizeof(float) * 2 * kIn, cudaMemcpyHostToDevice));
        b_->stats_set = true;
    }
    GUESS_OK(cudaMemsetAsync(b_->loss, 0, sizeof(double) * 2, st));
    const int tail = steps / 10 > 0 ? steps / 10 : 1;
    const float b1 = 0.9f, b2 = 0.999f;
    for (int s = 0; s < steps; ++s) {
        GUESS_OK(cudaMemsetAsync(b_->grad, 0, sizeof(float) * kParams, st));
        const unsigned long long rs = mix64_host(seed * 0x9E3779B97F4A7C15ull + (unsigned long long)s + 1) | 1ull;
        count_launch();
        mlp_kernel<true><<<mlp_blocks(batch), 32 * kWarps, SmemPlan::bytes(true), st>>>(
            batch, b_->params, b_->X, b_->T, nsamples_, rs, 1.f / (float)batch, nullptr, b_->grad,
            b_->loss + (s >= steps - tail ? 0 : 1));
        ++b_->adam_t;
        const float c1 = (float)(1.0 / (1.0 - std::pow((double)b1, b_->adam_t)));
        const float c2 = (float)(1.0 / (1.0 - std::pow((double)b2, b_->adam_t)));
        // cosine decay of the step size over the run
        const float lr_s = (float)(lr * 0.5 * (1.0 + std::cos(3.141592653589793 * s / steps)));
        count_launch();
        adam_kernel<<<(kParams + 255) / 256, 256, 0, st>>>(kParams, b_->params, b_->grad, b_->adam_m, b_->adam_v,
                                                            lr_s, b1, b2, c1, c2, 1e-8f);
    }
    GUESS_OK(repack_weights(b_, st));
    double hl[2] = {0, 0};
    GUESS_OK(cudaMemcpyAsync(hl, b_->loss, sizeof(double) * 2, cudaMemcpyDeviceToHost, st));
    GUESS_OK(cudaStreamSynchronize(st));
    if (loss_out) *loss_out = hl[0] / tail;
    ready_ = true;
    return cudaGetLastError();
}

cudaError_t GuessNet::loss_grad(cudaStream_t st, const float* h_X, const float* h_T, int n, double* loss,
                                float* h_grad, float* h_Y) {
    if (!b_->params || n <= 0) return cudaErrorInvalidValue;
    GUESS_OK(mlp_attributes());
    if (!b_->grad) GUESS_OK(cudaMalloc(&b_->grad, sizeof(float) * kParams));
    if (!b_->loss) GUESS_OK(cudaMalloc(&b_->loss, sizeof(double) * 2));
    if (n > b_->cap_h) {
        GUESS_OK(grow(&b_->hx, 0, (size_t)n * kIn, 0));
        GUESS_OK(grow(&b_->ht, 0, (size_t)n * kOut, 0));
        GUESS_OK(grow(&b_->hy, 0, (size_t)n * kOut, 0));
        b_->cap_h = n;
    }
    GUESS_OK(cudaMemcpyAsync(b_->hx, h_X, sizeof(float) * (size_t)n * kIn, cudaMemcpyHostToDevice, st));
    GUESS_OK(cudaMemcpyAsync(b_->ht, h_T, sizeof(float) * (size_t)n * kOut, cudaMemcpyHostToDevice, st));
    GUESS_OK(cudaMemsetAsync(b_->grad, 0, sizeof(float) * kParams, st));
    GUESS_OK(cudaMemsetAsync(b_->loss, 0, sizeof(double), st));
    if (!b_->wpack) GUESS_OK(repack_weights(b_, st));
    count_launch();
    mlp_kernel<true><<<mlp_blocks(n), 32 * kWarps, SmemPlan::bytes(true), st>>>(
        n, b_->params, b_->hx, b_->ht, n, 0ull, 1.f / (float)n, b_->hy, b_->grad, b_->loss);
    GUESS_OK(cudaGetLastError());
    // the outputs by the inference kernel (the one the solver's guess uses)
    count_launch();
    mlp_tc5_kernel<<<mlp_tc5_blocks(n), kTcRows, 0, st>>>(n, b_->params, b_->wpack, b_->hx, b_->hy, b_->status);
    GUESS_OK(cudaGetLastError());
    GUESS_OK(cudaMemcpyAsync(loss, b_->loss, sizeof(double), cudaMemcpyDeviceToHost, st));
    GUESS_OK(cudaMemcpyAsync(h_grad, b_->grad, sizeof(float) * kParams, cudaMemcpyDeviceToHost, st));
    GUESS_OK(cudaMemcpyAsync(h_Y, b_->hy, sizeof(float) * (size_t)n * kOut, cudaMemcpyDeviceToHost, st));
    int kst = 0;
    GUESS_OK(cudaMemcpyAsync(&kst, b_->status, sizeof(int), cudaMemcpyDeviceToHost, st));
    GUESS_OK(cudaStreamSynchronize(st));
    return kst ? cudaErrorTimeout : cudaSuccess;
}

}  // namespace mbpol
