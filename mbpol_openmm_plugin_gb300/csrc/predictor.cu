// Learned linear predictor of the induced dipoles from the history of
// converged solves (guess = 2 once the history is long enough).
//
// With X_0 the newest converged dipoles and X_k those k steps older, the
// starting dipoles of the next solve are
//     mu = X_0 + sum_{j=1..J} a_j nabla^j X_0,
//     nabla^j X_b = sum_{i=0..j} (-1)^i C(j, i) X_{b+i}   (backward differences),
// J = kPredOrder.  a_j = 1 for j <= 3 and 0 above is the 4-point polynomial
// extrapolation; here the a_j are refitted before every solve by least
// squares on the last kPredWindow steps of the trajectory: each of those
// solves X_w (w = 0 .. W-1) is predicted from the solves before it,
//     minimise sum_w || X_w - X_{w+1} - sum_j a_j nabla^j X_{w+1} ||^2,
// over (a subsample of) all dipole components.  The backward differences
// are nearly orthogonal with geometrically falling norms, so the normal
// equations, scaled by their diagonal, are well conditioned; they are
// formed in FP64 (the high differences cancel to ~1e-10 of mu) with a
// fixed-order reduction and solved by an FP32 Cholesky on the device.  Columns that
// vanish (a history that is exactly polynomial) are left out; a system that
// is not positive definite falls back to the polynomial coefficients.
#include "guess.h"
#include "mbpol_internal.cuh"

namespace mbpol {

namespace {

constexpr int kJ = guess::kPredOrder;
constexpr int kW = guess::kPredWindow;
constexpr int kStats = guess::kPredStats;  // upper triangle of G, then b
constexpr int kGramThreads = 128;

// backward differences nabla^1 .. nabla^J of the sequence x[0 .. J] (x[0]
// the newest) by repeated differencing
__device__ __forceinline__ void backward_differences(const double (&x)[kJ + 1], double (&d)[kJ]) {
    double t[kJ + 1];
    #pragma unroll
    for (int i = 0; i <= kJ; ++i) t[i] = x[i];
    #pragma unroll
    for (int j = 1; j <= kJ; ++j) {
        #pragma unroll
        for (int i = 0; i <= kJ - j; ++i) t[i] = t[i] - t[i + 1];
        d[j - 1] = t[0];
    }
}

__global__ void __launch_bounds__(kGramThreads) predictor_gram_kernel(int n3, int stride, const PredictorRing ring,
                                                                      double* __restrict__ partials) {
    double S[kStats];
    #pragma unroll
    for (int k = 0; k < kStats; ++k) S[k] = 0.0;
    for (long e = ((long)blockIdx.x * blockDim.x + threadIdx.x) * stride; e < n3;
         e += (long)gridDim.x * blockDim.x * stride) {
        double x[guess::kPredHistory];
        #pragma unroll
        for (int k = 0; k < guess::kPredHistory; ++k) x[k] = ring.r[k][e];
        #pragma unroll
        for (int w = 0; w < kW; ++w) {
            double base[kJ + 1], d[kJ];
            #pragma unroll
            for (int i = 0; i <= kJ; ++i) base[i] = x[w + 1 + i];
            backward_differences(base, d);
            const double y = x[w] - x[w + 1];
            int k = 0;
            #pragma unroll
            for (int i = 0; i < kJ; ++i)
                #pragma unroll
                for (int j = i; j < kJ; ++j) S[k++] += d[i] * d[j];
            #pragma unroll
            for (int i = 0; i < kJ; ++i) S[k++] += d[i] * y;
        }
    }
    // block sum in a fixed order: warps by shuffles, then warp 0 over warps
    __shared__ double red[kGramThreads / 32][kStats];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    #pragma unroll
    for (int k = 0; k < kStats; ++k) {
        double v = S[k];
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < kStats) {
        double v = 0.0;
        for (int w = 0; w < kGramThreads / 32; ++w) v += red[w][threadIdx.x];
        partials[(size_t)blockIdx.x * kStats + threadIdx.x] = v;
    }
}

// The 7x7 system is solved in FP32 (FP64 division and square root are long
// instruction sequences on this part; one thread would spend tens of
// microseconds in them): the partial sums are added in FP64, the diagonal
// scaling makes the system well conditioned (condition number ~1e3), and
// the FP32 solution is good to ~1e-4 relative, ample for a starting guess.
__global__ void predictor_solve_kernel(int nblocks, const double* __restrict__ partials, double* __restrict__ coef) {
    __shared__ double S[kStats];
    if (threadIdx.x < kStats) {
        double v = 0.0;
        for (int b = 0; b < nblocks; ++b) v += partials[(size_t)b * kStats + threadIdx.x];
        S[threadIdx.x] = v;
    }
    __syncthreads();
    if (threadIdx.x != 0) return;
    float G[kJ][kJ], b[kJ], sc[kJ];
    bool keep[kJ];
    double gmax = 0.0;
    #pragma unroll
    for (int i = 0; i < kJ; ++i) {
        const int d = i * kJ - i * (i - 1) / 2;  // G[i][i] in the packed upper triangle
        gmax = fmax(gmax, S[d]);
    }
    // diagonal scaling; a column whose norm vanishes against the largest is
    // left out (its coefficient 0)
    #pragma unroll
    for (int i = 0; i < kJ; ++i) {
        const double gii = S[i * kJ - i * (i - 1) / 2];
        keep[i] = gii > 1e-24 * gmax && gii > 0.0;
        sc[i] = keep[i] ? rsqrtf((float)gii) : 0.f;
    }
    int k = 0;
    #pragma unroll
    for (int i = 0; i < kJ; ++i)
        #pragma unroll
        for (int j = i; j < kJ; ++j) {
            const float g = (keep[i] && keep[j]) ? (float)S[k] * sc[i] * sc[j] : (i == j ? 1.f : 0.f);
            G[i][j] = g;
            G[j][i] = g;
            ++k;
        }
    #pragma unroll
    for (int i = 0; i < kJ; ++i) {
        b[i] = keep[i] ? (float)S[k] * sc[i] : 0.f;
        ++k;
        G[i][i] += 1e-6f;
    }
    // Cholesky G = L L^T in place (lower triangle)
    bool ok = gmax > 0.0;
    #pragma unroll
    for (int j = 0; j < kJ; ++j) {
        float s = G[j][j];
        #pragma unroll
        for (int p = 0; p < j; ++p) s -= G[j][p] * G[j][p];
        ok = ok && s > 0.f;
        const float l = sqrtf(fmaxf(s, 1e-30f)), il = 1.f / l;
        G[j][j] = l;
        #pragma unroll
        for (int i = j + 1; i < kJ; ++i) {
            float t = G[i][j];
            #pragma unroll
            for (int p = 0; p < j; ++p) t -= G[i][p] * G[j][p];
            G[i][j] = t * il;
        }
    }
    float a[kJ], z[kJ];
    #pragma unroll
    for (int i = 0; i < kJ; ++i) {
        float t = b[i];
        #pragma unroll
        for (int p = 0; p < i; ++p) t -= G[i][p] * z[p];
        z[i] = t / G[i][i];
    }
    #pragma unroll
    for (int i = kJ - 1; i >= 0; --i) {
        float t = z[i];
        #pragma unroll
        for (int p = i + 1; p < kJ; ++p) t -= G[p][i] * a[p];
        a[i] = t / G[i][i];
    }
    #pragma unroll
    for (int i = 0; i < kJ; ++i) ok = ok && isfinite(a[i] * sc[i]);
    #pragma unroll
    for (int i = 0; i < kJ; ++i) coef[i] = ok ? (double)(a[i] * sc[i]) : (i < 3 ? 1.0 : 0.0);
}

__global__ void predictor_apply_kernel(int n3, const PredictorRing ring, const double* __restrict__ coef,
                                       double* __restrict__ mu_d, float* __restrict__ mu_f) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n3) return;
    double x[kJ + 1], d[kJ];
    #pragma unroll
    for (int i = 0; i <= kJ; ++i) x[i] = ring.r[i][e];
    backward_differences(x, d);
    double v = x[0];
    #pragma unroll
    for (int j = 0; j < kJ; ++j) v += coef[j] * d[j];
    mu_d[e] = v;
    mu_f[e] = (float)v;
}

}  // namespace

int predictor_partial_blocks() { return 76; }

cudaError_t predictor_fit(cudaStream_t st, int n3, const PredictorRing& ring, double* d_partials, double* d_coef) {
    const int blocks = predictor_partial_blocks();
    // about 8k components are ample for 7 coefficients
    const int stride = n3 > 8192 ? n3 / 8192 : 1;
    count_launch();
    predictor_gram_kernel<<<blocks, kGramThreads, 0, st>>>(n3, stride, ring, d_partials);
    count_launch();
    predictor_solve_kernel<<<1, 64, 0, st>>>(blocks, d_partials, d_coef);
    return cudaGetLastError();
}

cudaError_t predictor_apply(cudaStream_t st, int n3, const PredictorRing& ring, const double* d_coef, double* mu_d,
                            float* mu_f) {
    count_launch();
    predictor_apply_kernel<<<(n3 + 255) / 256, 256, 0, st>>>(n3, ring, d_coef, mu_d, mu_f);
    return cudaGetLastError();
}

}  // namespace mbpol
