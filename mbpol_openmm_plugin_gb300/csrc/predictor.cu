// Learned linear predictor of the induced dipoles from the history of
// converged solves (guess = 2 once the history is long enough).
//
// With X_0 the newest converged dipoles, X_k those k steps older, F_k =
// alpha E0 of the same steps (polarisability times permanent field) and
// F_new that of the geometry about to be solved, the starting dipoles are
//     mu = P(X) + g (F_new - P(F)),
//     P(Y) = Y_0 + sum_{j=1..J} a_j nabla^j Y_0,
//     nabla^j Y_b = sum_{i=0..j} (-1)^i C(j, i) Y_{b+i}   (backward differences),
// J = kPredOrder.  a = (1, 1, 1, 0, ...) is the 4-point polynomial
// extrapolation.  The a are refitted before every solve by least squares on
// the last kPredWindow steps of the dipoles: each of those solves X_w
// (w = 0 .. W-1) is predicted from the steps before it,
//     minimise sum_w || X_w - X_{w+1} - sum_j a_j nabla^j X_{w+1} ||^2,
// over (a subsample of) all dipole components.  The second term feeds in
// the part of the permanent field's change that the history does not
// predict (the field of the new geometry is known before the solve), with
// the weight g = kFieldGain, the mean response of the dipoles to it.  (A
// fitted weight came out smaller and worse: the FP32 field's rounding
// noise, amplified by the extrapolation, biases a least-squares weight
// towards zero.)
// The backward differences are nearly orthogonal with geometrically falling
// norms, so the normal equations, scaled by their diagonal, are well
// conditioned; they are formed in FP64 (the high differences cancel to
// ~1e-10 of mu) with a fixed-order reduction and solved by an FP32 Cholesky
// on the device.  Columns that vanish (a history that is exactly
// polynomial) are left out; a system that is not positive definite falls
// back to the polynomial coefficients.
#include "guess.h"
#include "mbpol_internal.cuh"

namespace mbpol {

namespace {

constexpr int kJ = guess::kPredOrder;
constexpr int kR = guess::kPredRegressors;
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
            double base[kJ + 1], d[kR];
            #pragma unroll
            for (int i = 0; i <= kJ; ++i) base[i] = x[w + 1 + i];
            backward_differences(base, d);
            const double y = x[w] - x[w + 1];
            int k = 0;
            #pragma unroll
            for (int i = 0; i < kR; ++i)
                #pragma unroll
                for (int j = i; j < kR; ++j) S[k++] += d[i] * d[j];
            #pragma unroll
            for (int i = 0; i < kR; ++i) S[k++] += d[i] * y;
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
    float G[kR][kR], b[kR], sc[kR];
    bool keep[kR];
    double gmax = 0.0;
    #pragma unroll
    for (int i = 0; i < kR; ++i) {
        const int d = i * kR - i * (i - 1) / 2;  // G[i][i] in the packed upper triangle
        gmax = fmax(gmax, S[d]);
    }
    // diagonal scaling; a column whose norm vanishes against the largest is
    // left out (its coefficient 0)
    #pragma unroll
    for (int i = 0; i < kR; ++i) {
        const double gii = S[i * kR - i * (i - 1) / 2];
        keep[i] = gii > 1e-24 * gmax && gii > 0.0;
        sc[i] = keep[i] ? rsqrtf((float)gii) : 0.f;
    }
    int k = 0;
    #pragma unroll
    for (int i = 0; i < kR; ++i)
        #pragma unroll
        for (int j = i; j < kR; ++j) {
            const float g = (keep[i] && keep[j]) ? (float)S[k] * sc[i] * sc[j] : (i == j ? 1.f : 0.f);
            G[i][j] = g;
            G[j][i] = g;
            ++k;
        }
    #pragma unroll
    for (int i = 0; i < kR; ++i) {
        b[i] = keep[i] ? (float)S[k] * sc[i] : 0.f;
        ++k;
        G[i][i] += 1e-6f;
    }
    // Cholesky G = L L^T in place (lower triangle)
    bool ok = gmax > 0.0;
    #pragma unroll
    for (int j = 0; j < kR; ++j) {
        float s = G[j][j];
        #pragma unroll
        for (int p = 0; p < j; ++p) s -= G[j][p] * G[j][p];
        ok = ok && s > 0.f;
        const float l = sqrtf(fmaxf(s, 1e-30f)), il = 1.f / l;
        G[j][j] = l;
        #pragma unroll
        for (int i = j + 1; i < kR; ++i) {
            float t = G[i][j];
            #pragma unroll
            for (int p = 0; p < j; ++p) t -= G[i][p] * G[j][p];
            G[i][j] = t * il;
        }
    }
    float a[kR], z[kR];
    #pragma unroll
    for (int i = 0; i < kR; ++i) {
        float t = b[i];
        #pragma unroll
        for (int p = 0; p < i; ++p) t -= G[i][p] * z[p];
        z[i] = t / G[i][i];
    }
    #pragma unroll
    for (int i = kR - 1; i >= 0; --i) {
        float t = z[i];
        #pragma unroll
        for (int p = i + 1; p < kR; ++p) t -= G[p][i] * a[p];
        a[i] = t / G[i][i];
    }
    #pragma unroll
    for (int i = 0; i < kR; ++i) ok = ok && isfinite(a[i] * sc[i]);
    #pragma unroll
    for (int i = 0; i < kR; ++i) coef[i] = ok ? (double)(a[i] * sc[i]) : (i < 3 ? 1.0 : 0.0);  // fallback: 4-point
}

__global__ void predictor_apply_kernel(int n3, const PredictorRing ring, const double* __restrict__ f_now,
                                       const double* __restrict__ coef, double* __restrict__ mu_d,
                                       float* __restrict__ mu_f, float* __restrict__ dF) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n3) return;
    double x[kJ + 1], d[kJ], fx[kJ + 1], fd[kJ];
    #pragma unroll
    for (int i = 0; i <= kJ; ++i) {
        x[i] = ring.r[i][e];
        fx[i] = ring.f[i][e];
    }
    backward_differences(x, d);
    backward_differences(fx, fd);
    double v = x[0], pf = fx[0];
    #pragma unroll
    for (int j = 0; j < kJ; ++j) {
        v += coef[j] * d[j];
        pf += coef[j] * fd[j];
    }
    const double df = f_now[e] - pf;
    v += guess::kFieldGain * df;
    mu_d[e] = v;
    mu_f[e] = (float)v;
    if (dF) dF[e] = (float)df;
}

__global__ void scaled_field_kernel(int n3, const float* __restrict__ E0, const float* __restrict__ pol,
                                    double* __restrict__ out) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n3) out[e] = (double)pol[e / 3] * (double)E0[e];
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

cudaError_t predictor_apply(cudaStream_t st, int n3, const PredictorRing& ring, const double* f_now,
                            const double* d_coef, double* mu_d, float* mu_f, float* dF) {
    count_launch();
    predictor_apply_kernel<<<(n3 + 255) / 256, 256, 0, st>>>(n3, ring, f_now, d_coef, mu_d, mu_f, dF);
    return cudaGetLastError();
}

// mu_d += m (the correction network's output), mu_f = float(mu_d)
__global__ void add_correction_kernel(int n3, const float* __restrict__ m, double* __restrict__ mu_d,
                                      float* __restrict__ mu_f) {
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n3) return;
    const double v = mu_d[e] + (double)m[e];
    mu_d[e] = v;
    mu_f[e] = (float)v;
}

cudaError_t add_correction(cudaStream_t st, int n3, const float* m, double* mu_d, float* mu_f) {
    count_launch();
    add_correction_kernel<<<(n3 + 255) / 256, 256, 0, st>>>(n3, m, mu_d, mu_f);
    return cudaGetLastError();
}

cudaError_t scaled_field(cudaStream_t st, int n3, const float* E0, const float* pol, double* out) {
    count_launch();
    scaled_field_kernel<<<(n3 + 255) / 256, 256, 0, st>>>(n3, E0, pol, out);
    return cudaGetLastError();
}

}  // namespace mbpol
