// MB-pol dispersion: E = -C6 * tt6(d6 r) / r^6 over O/H site pairs of
// different waters, with the Tang-Toennies damping
//     tt6(x) = 1 - exp(-x) * sum_{n=0..6} x^n / n!.
// Parameters (C6, d6 per site-class pair) and exclusions (same water, any M
// site) follow python/mbpol.xml:37-108, where the reference builds this term
// as an OpenMM CustomNonbondedForce (truncated at the nonbonded cutoff under
// PME, no switching, no long-range correction).
//
// One thread per (water i, neighbour slot); only j > i is evaluated so each
// water pair is visited once.  Chloride ions: dispersion_ions_kernel.  FP32 pair arithmetic from FP64 minimum-image
// differences; FP64 force atomics and energy reduction.
#include "mbpol_internal.cuh"
#include "mbpol_kernels.h"

namespace mbpol {

__constant__ float c_disp_c6[16];  // [class_i * 4 + class_j], kJ/mol nm^6
__constant__ float c_disp_d6[16];  // nm^-1

__global__ void dispersion_kernel(int nw, const int4* __restrict__ waters, const double* __restrict__ pos, Box box,
                                  const int* __restrict__ full, const int* __restrict__ nfull, int cap_full,
                                  float rc2, double* __restrict__ force, double* __restrict__ energy,
                                  ClusterSink cs) {
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = gid / cap_full, slot = gid - i * cap_full;
    double e_out = 0.0;
    if (i < nw && slot < min(nfull[i], cap_full)) {
        const int j = full[(size_t)i * cap_full + slot];
        if (j > i) {
            const int4 wi = waters[i], wj = waters[j];
            const int ai[3] = {wi.x, wi.y, wi.z}, aj[3] = {wj.x, wj.y, wj.z};
            double3 pi[3], pj[3];
            #pragma unroll
            for (int a = 0; a < 3; ++a) {
                pi[a] = load_pos(pos, ai[a]);
                pj[a] = load_pos(pos, aj[a]);
            }
            f3 fi[3], fj[3];
            #pragma unroll
            for (int a = 0; a < 3; ++a) fi[a] = fj[a] = mk(0.f, 0.f, 0.f);
            float e = 0.f;
            #pragma unroll
            for (int a = 0; a < 3; ++a) {
                #pragma unroll
                for (int b = 0; b < 3; ++b) {
                    double dx = pj[b].x - pi[a].x, dy = pj[b].y - pi[a].y, dz = pj[b].z - pi[a].z;
                    if (box.periodic) {
                        dx = min_image(dx, box.L[0], box.inv[0]);
                        dy = min_image(dy, box.L[1], box.inv[1]);
                        dz = min_image(dz, box.L[2], box.inv[2]);
                    }
                    f3 d = mk((float)dx, (float)dy, (float)dz);
                    float r2 = dot(d, d);
                    if (r2 > rc2) continue;
                    const int cls = (a == 0 ? 0 : 1) * 4 + (b == 0 ? 0 : 1);
                    const float c6 = c_disp_c6[cls], d6 = c_disp_d6[cls];
                    float r = sqrtf(r2);
                    float x = d6 * r;
                    float ex = expf(-x);
                    // sum_{n<=6} x^n/n! by Horner
                    float s6 = 1.f + x * (1.f + x * (0.5f + x * (1.f / 6.f + x * (1.f / 24.f + x * (1.f / 120.f + x * (1.f / 720.f))))));
                    float tt = 1.f - ex * s6;
                    float x6 = x * x * x;
                    x6 *= x6;
                    float dtt = d6 * ex * x6 * (1.f / 720.f);  // d tt6 / dr
                    float ir2 = 1.f / r2, ir6 = ir2 * ir2 * ir2;
                    e += -c6 * tt * ir6;
                    // dE/dr = -c6 (dtt r^-6 - 6 tt r^-7); force on j = -dE/dr * d/r
                    float dEdr = -c6 * (dtt * ir6 - 6.f * tt * ir6 / r);
                    f3 f = d * (-dEdr / r);
                    fj[b] += f;
                    fi[a] -= f;
                }
            }
            #pragma unroll
            for (int a = 0; a < 3; ++a) {
                add_force(force, ai[a], fi[a].x, fi[a].y, fi[a].z);
                add_force(force, aj[a], fj[a].x, fj[a].y, fj[a].z);
            }
            e_out = e;
            cluster_energy(cs, i, e_out);
        }
    }
    block_sum_atomic<128>(e_out, energy);
}

// Chloride ions (class CL = 3 of the tables, python/mbpol.xml:52-83): one
// thread per (ion, partner) with the partners the O, H1, H2 sites of every
// water, then the other ions (j > i); the same damped -C6 tt6 / r^6 with
// site distances within the cutoff.  Few ions per system, so the partners
// are not listed.
__global__ void dispersion_ions_kernel(int nion, const int* __restrict__ ions, int nw, const int4* __restrict__ waters,
                                       const double* __restrict__ pos, Box box, float rc2, double* __restrict__ force,
                                       double* __restrict__ energy) {
    const int np = 3 * nw + nion;
    const long gid = (long)blockIdx.x * blockDim.x + threadIdx.x;
    double e_out = 0.0;
    if (gid < (long)nion * np) {
        const int i = (int)(gid / np), j = (int)(gid - (long)i * np);
        int pj = -1, cls = 0;
        if (j < 3 * nw) {
            const int4 w = waters[j / 3];
            const int a = j % 3;
            pj = a == 0 ? w.x : (a == 1 ? w.y : w.z);
            cls = a == 0 ? 0 : 1;
        } else if (j - 3 * nw > i) {
            pj = ions[j - 3 * nw];
            cls = 3;
        }
        const int pi = ions[i];
        const float c6 = pj >= 0 ? c_disp_c6[3 * 4 + cls] : 0.f;
        if (c6 != 0.f) {
            const double3 a = load_pos(pos, pi), b = load_pos(pos, pj);
            double dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
            if (box.periodic) {
                dx = min_image(dx, box.L[0], box.inv[0]);
                dy = min_image(dy, box.L[1], box.inv[1]);
                dz = min_image(dz, box.L[2], box.inv[2]);
            }
            const f3 d = mk((float)dx, (float)dy, (float)dz);
            const float r2 = dot(d, d);
            if (r2 <= rc2) {
                const float d6 = c_disp_d6[3 * 4 + cls];
                const float r = sqrtf(r2), x = d6 * r, ex = expf(-x);
                const float s6 = 1.f + x * (1.f + x * (0.5f + x * (1.f / 6.f + x * (1.f / 24.f + x * (1.f / 120.f + x * (1.f / 720.f))))));
                const float tt = 1.f - ex * s6;
                float x6 = x * x * x;
                x6 *= x6;
                const float dtt = d6 * ex * x6 * (1.f / 720.f);
                const float ir2 = 1.f / r2, ir6 = ir2 * ir2 * ir2;
                const float dEdr = -c6 * (dtt * ir6 - 6.f * tt * ir6 / r);
                const f3 f = d * (-dEdr / r);
                add_force(force, pj, f.x, f.y, f.z);
                add_force(force, pi, -f.x, -f.y, -f.z);
                e_out = -c6 * tt * ir6;
            }
        }
    }
    block_sum_atomic<128>(e_out, energy);
}

void launch_dispersion_ions(cudaStream_t st, int nion, const int* ions, int nw, const int4* waters,
                            const double* pos, Box box, double rc, double* force, double* energy) {
    if (nion <= 0) return;
    const long total = (long)nion * (3 * (long)nw + nion);
    const float rc2 = rc > 1e15 ? 3.0e38f : (float)(rc * rc);
    count_launch();
    dispersion_ions_kernel<<<(int)((total + 127) / 128), 128, 0, st>>>(nion, ions, nw, waters, pos, box, rc2, force,
                                                                        energy);
}

void upload_dispersion_tables(const double* c6_4x4, const double* d6_4x4) {
    float c6[16], d6[16];
    for (int k = 0; k < 16; ++k) {
        c6[k] = (float)c6_4x4[k];
        d6[k] = (float)d6_4x4[k];
    }
    cudaMemcpyToSymbol(c_disp_c6, c6, sizeof(c6));
    cudaMemcpyToSymbol(c_disp_d6, d6, sizeof(d6));
}

void launch_dispersion(cudaStream_t st, int nw, const int4* waters, const double* pos, Box box, const int* full,
                       const int* nfull, int cap_full, double rc, double* force, double* energy,
                       ClusterSink cs) {
    if (nw <= 0 || cap_full <= 0) return;
    const long total = (long)nw * cap_full;
    const float rc2 = rc > 1e15 ? 3.0e38f : (float)(rc * rc);
    count_launch();
    dispersion_kernel<<<(int)((total + 127) / 128), 128, 0, st>>>(nw, waters, pos, box, full, nfull, cap_full, rc2,
                                                                   force, energy, cs);
}

}  // namespace mbpol
