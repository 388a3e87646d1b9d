// MB-pol dispersion: E = -C6 * tt6(d6 r) / r^6 over O/H site pairs of
// different waters, with the Tang-Toennies damping
//     tt6(x) = 1 - exp(-x) * sum_{n=0..6} x^n / n!.
// Parameters (C6, d6 per site-class pair) and exclusions (same water, any M
// site) follow python/mbpol.xml:37-108, where the reference builds this term
// as an OpenMM CustomNonbondedForce (truncated at the nonbonded cutoff under
// PME, no switching, no long-range correction).
//
// One warp per water i: the lanes take i's listed neighbours j > i in turn
// (each water pair once), keep i's forces in registers, summed over the warp
// at the end, and add j's with atomics.  Site positions are taken relative to
// each water's O (each H imaged next to its O in FP64, the O-O difference
// minimum-imaged in FP64), so a site pair's difference is an FP32 sum of
// three small vectors; a final FP32 minimum image makes it the per-site
// minimum image of the force field's nonbonded force in any box of at least
// twice the cutoff.  FP32 pair arithmetic; FP64 force atomics and energy
// sums.  Chloride ions: dispersion_ions_kernel.
#include "mbpol_internal.cuh"
#include "mbpol_kernels.h"

namespace mbpol {

__constant__ float c_disp_c6[16];  // [class_i * 4 + class_j], kJ/mol nm^6
__constant__ float c_disp_d6[16];  // nm^-1

constexpr int kDispBlock = 128;

// r_h - r_o with h imaged next to o (FP64 difference, then FP32).
__device__ __forceinline__ f3 site_offset(const double3 o, const double3 h, const Box& box) {
    double dx = h.x - o.x, dy = h.y - o.y, dz = h.z - o.z;
    if (box.periodic) {
        dx = min_image(dx, box.L[0], box.inv[0]);
        dy = min_image(dy, box.L[1], box.inv[1]);
        dz = min_image(dz, box.L[2], box.inv[2]);
    }
    return mk((float)dx, (float)dy, (float)dz);
}

__device__ __forceinline__ float lane_sum(float v) {
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ float min_image_f(float d, float L, float invL) {
    return d - L * floorf(d * invL + 0.5f);
}

__global__ void __launch_bounds__(kDispBlock) dispersion_kernel(
    int nw, const int4* __restrict__ waters, const double* __restrict__ pos, Box box,
    const int* __restrict__ full, const int* __restrict__ nfull, int cap_full, float rc2,
    double* __restrict__ force, double* __restrict__ energy, ClusterSink cs) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    double e_out = 0.0;
    if (i < nw) {  // uniform over the warp
        const float Lf[3] = {(float)box.L[0], (float)box.L[1], (float)box.L[2]};
        const float iLf[3] = {(float)box.inv[0], (float)box.inv[1], (float)box.inv[2]};
        const int4 wi = waters[i];
        const int ai[3] = {wi.x, wi.y, wi.z};
        const double3 oi = load_pos(pos, wi.x);
        const f3 si[3] = {mk(0.f, 0.f, 0.f), site_offset(oi, load_pos(pos, wi.y), box),
                          site_offset(oi, load_pos(pos, wi.z), box)};
        f3 fi[3];
        #pragma unroll
        for (int a = 0; a < 3; ++a) fi[a] = mk(0.f, 0.f, 0.f);
        const int n = min(nfull[i], cap_full);
        for (int t = lane; t < n; t += 32) {
            const int j = full[(size_t)i * cap_full + t];
            if (j <= i) continue;
            const int4 wj = waters[j];
            const int aj[3] = {wj.x, wj.y, wj.z};
            const double3 oj = load_pos(pos, wj.x);
            const f3 dO = site_offset(oi, oj, box);
            const f3 sj[3] = {mk(0.f, 0.f, 0.f), site_offset(oj, load_pos(pos, wj.y), box),
                              site_offset(oj, load_pos(pos, wj.z), box)};
            f3 fj[3];
            #pragma unroll
            for (int b = 0; b < 3; ++b) fj[b] = mk(0.f, 0.f, 0.f);
            float e = 0.f;
            #pragma unroll
            for (int a = 0; a < 3; ++a) {
                #pragma unroll
                for (int b = 0; b < 3; ++b) {
                    f3 d = dO + sj[b] - si[a];  // r_jb - r_ia
                    if (box.periodic) {
                        d.x = min_image_f(d.x, Lf[0], iLf[0]);
                        d.y = min_image_f(d.y, Lf[1], iLf[1]);
                        d.z = min_image_f(d.z, Lf[2], iLf[2]);
                    }
                    const float r2 = dot(d, d);
                    if (r2 > rc2) continue;
                    const int cls = (a == 0 ? 0 : 1) * 4 + (b == 0 ? 0 : 1);
                    const float c6 = c_disp_c6[cls], d6 = c_disp_d6[cls];
                    const float r = sqrtf(r2);
                    const float x = d6 * r;
                    const float ex = expf(-x);
                    // sum_{n<=6} x^n/n! by Horner
                    const float s6 = 1.f + x * (1.f + x * (0.5f + x * (1.f / 6.f + x * (1.f / 24.f + x * (1.f / 120.f + x * (1.f / 720.f))))));
                    const float tt = 1.f - ex * s6;
                    float x6 = x * x * x;
                    x6 *= x6;
                    const float dtt = d6 * ex * x6 * (1.f / 720.f);  // d tt6 / dr
                    const float ir2 = 1.f / r2, ir6 = ir2 * ir2 * ir2;
                    e += -c6 * tt * ir6;
                    // dE/dr = -c6 (dtt r^-6 - 6 tt r^-7); force on j = -dE/dr * d/r
                    const float dEdr = -c6 * (dtt * ir6 - 6.f * tt * ir6 / r);
                    const f3 f = d * (-dEdr / r);
                    fj[b] += f;
                    fi[a] -= f;
                }
            }
            #pragma unroll
            for (int b = 0; b < 3; ++b) add_force(force, aj[b], fj[b].x, fj[b].y, fj[b].z);
            e_out += (double)e;
        }
        #pragma unroll
        for (int a = 0; a < 3; ++a) {
            fi[a].x = lane_sum(fi[a].x);
            fi[a].y = lane_sum(fi[a].y);
            fi[a].z = lane_sum(fi[a].z);
        }
        if (lane == 0)
            #pragma unroll
            for (int a = 0; a < 3; ++a) add_force(force, ai[a], fi[a].x, fi[a].y, fi[a].z);
        cluster_energy(cs, i, e_out);
    }
    block_sum_atomic<kDispBlock>(e_out, energy);
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
    const float rc2 = rc > 1e15 ? 3.0e38f : (float)(rc * rc);
    const int per_block = kDispBlock / 32;
    count_launch();
    dispersion_kernel<<<(nw + per_block - 1) / per_block, kDispBlock, 0, st>>>(nw, waters, pos, box, full, nfull,
                                                                               cap_full, rc2, force, energy, cs);
}

}  // namespace mbpol
