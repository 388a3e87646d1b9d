// Device-resident molecular dynamics around the MB-pol force evaluation:
// velocity Verlet (NVE) with an optional Andersen thermostat (NVT), the role
// OpenMM's integrators play for the reference plugin
// (python/example_nvt_nve.py).  Massless particles (M sites) are virtual and
// are placed from their parents before each force evaluation.
// Units: nm, ps, amu, kJ/mol (F/m in nm/ps^2).
#include "mbpol_kernels.h"

namespace mbpol {

__global__ void verlet_kick_drift_kernel(int n, const double* __restrict__ invm, double* __restrict__ vel,
                                         double* __restrict__ pos, const double* __restrict__ force, double dt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double im = invm[i];
    if (im == 0.0) return;
    #pragma unroll
    for (int k = 0; k < 3; ++k) {
        double v = vel[3 * i + k] + 0.5 * dt * force[3 * i + k] * im;
        vel[3 * i + k] = v;
        pos[3 * i + k] += dt * v;
    }
}

// Second half kick; with nu > 0, Andersen collisions resample a particle's
// velocity from Maxwell-Boltzmann at temperature kT with probability nu*dt.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
    // SplitMix64 finaliser (Steele, Lea & Flood, OOPSLA 2014)
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
__device__ __forceinline__ double u01(unsigned long long h) { return ((h >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

__global__ void verlet_kick_kernel(int n, const double* __restrict__ invm, double* __restrict__ vel,
                                   const double* __restrict__ force, double dt, double kT, double nu,
                                   unsigned long long seed, unsigned long long step, double* __restrict__ ekin) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double ek = 0.0;
    if (i < n) {
        const double im = invm[i];
        if (im != 0.0) {
            double v[3];
            for (int k = 0; k < 3; ++k) v[k] = vel[3 * i + k] + 0.5 * dt * force[3 * i + k] * im;
            if (nu > 0.0) {
                const unsigned long long base = mix64(seed ^ mix64(step * 0x100000001B3ull + (unsigned long long)i));
                if (u01(base) < nu * dt) {
                    const double sd = sqrt(kT * im);
                    for (int k = 0; k < 3; ++k) {
                        // Box-Muller from two hashed uniforms
                        const double a = u01(mix64(base + 2 * k + 1)), b = u01(mix64(base + 2 * k + 2));
                        v[k] = sd * sqrt(-2.0 * log(a)) * cos(6.283185307179586 * b);
                    }
                }
            }
            for (int k = 0; k < 3; ++k) {
                vel[3 * i + k] = v[k];
                ek += 0.5 * v[k] * v[k] / im;
            }
        }
    }
    block_sum_atomic<128>(ek, ekin);
}

void launch_kick_drift(cudaStream_t st, int n, const double* invm, double* vel, double* pos, const double* force,
                       double dt) {
    count_launch();
    verlet_kick_drift_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, invm, vel, pos, force, dt);
}

void launch_kick(cudaStream_t st, int n, const double* invm, double* vel, const double* force, double dt, double kT,
                 double nu, unsigned long long seed, unsigned long long step, double* ekin) {
    count_launch();
    verlet_kick_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, invm, vel, force, dt, kT, nu, seed, step, ekin);
}

}  // namespace mbpol
