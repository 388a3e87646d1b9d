// Three-particle average virtual sites (the MB-pol M site,
// python/mbpol.xml:14): placement before an evaluation and force spreading
// after it, as OpenMM's ThreeParticleAverageSite does for the reference.
#include "mbpol_kernels.h"

namespace mbpol {

__global__ void place_vsites_kernel(int n, const int4* __restrict__ idx, const double* __restrict__ w,
                                    double* __restrict__ pos) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int4 s = idx[v];  // x = site, y,z,w = parents
    #pragma unroll
    for (int k = 0; k < 3; ++k)
        pos[3 * s.x + k] = w[3 * v] * pos[3 * s.y + k] + w[3 * v + 1] * pos[3 * s.z + k] + w[3 * v + 2] * pos[3 * s.w + k];
}

// One thread per site; parents of different sites are distinct for waters,
// but atomics keep arbitrary topologies correct.
__global__ void spread_vsites_kernel(int n, const int4* __restrict__ idx, const double* __restrict__ w,
                                     double* __restrict__ force) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= n) return;
    const int4 s = idx[v];
    #pragma unroll
    for (int k = 0; k < 3; ++k) {
        const double f = force[3 * s.x + k];
        force[3 * s.x + k] = 0.0;
        atomicAdd(force + 3 * s.y + k, w[3 * v] * f);
        atomicAdd(force + 3 * s.z + k, w[3 * v + 1] * f);
        atomicAdd(force + 3 * s.w + k, w[3 * v + 2] * f);
    }
}

void launch_place_vsites(cudaStream_t st, int n, const int4* idx, const double* w, double* pos) {
    if (n <= 0) return;
    count_launch();
    place_vsites_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, idx, w, pos);
}

void launch_spread_vsites(cudaStream_t st, int n, const int4* idx, const double* w, double* force) {
    if (n <= 0) return;
    count_launch();
    spread_vsites_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, idx, w, force);
}

}  // namespace mbpol
