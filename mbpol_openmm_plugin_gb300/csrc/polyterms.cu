// MB-pol one-, two- and three-body terms.
//
//  * one-body: one thread per water, FP64 (the 245-term PES has
//    coefficients up to 4e4 cm^-1 whose constant parts cancel; the term is
//    ~1% of the work).  Restates
//    platforms/reference/src/MBPolReferenceOneBodyForce.cpp:69-201.
//  * two-body: per O-O pair, variables (31 exp/Coulomb-like functions of
//    site distances incl. two lone-pair X sites per water) in FP64 ->
//    double-float polynomial walk (poly_df.cu) -> chain rule + switch in
//    FP32, FP64 force atomics.  Restates
//    platforms/reference/src/MBPolReferenceTwoBodyForce.cpp:110-296 and
//    mbpol_2body_constants.cpp:10-111.
//  * three-body: per trimer, 36 exp variables (FP64) -> poly_df.cu -> chain
//    rule and the product switch in FP32.  Restates
//    platforms/reference/src/MBPolReferenceThreeBodyForce.cpp:67-293.
#include "dfmath.cuh"
#include "mbpol_internal.cuh"
#include "mbpol_kernels.h"

namespace mbpol {

// ---------------------------------------------------------------- one-body
__constant__ double c_1b_coef[245];
__constant__ unsigned char c_1b_idx[3][245];

struct OneBodyParams {
    double reoh, b1, roh, alphaoh, deoh, phh1, phh2, costhe, cm1_kcalmol;
};
__constant__ OneBodyParams c_1b;

__global__ void onebody_kernel(int nw, const int4* __restrict__ waters, const double* __restrict__ pos,
                               Box box, double* __restrict__ force, double* __restrict__ energy, ClusterSink cs) {
    int w = blockIdx.x * blockDim.x + threadIdx.x;
    double e_out = 0.0;
    if (w < nw) {
        const int4 wi = waters[w];
        double3 O = load_pos(pos, wi.x);
        double3 H1 = image_to(O, load_pos(pos, wi.y), box);
        double3 H2 = image_to(O, load_pos(pos, wi.z), box);
        double r1[3] = {(H1.x - O.x) * 10.0, (H1.y - O.y) * 10.0, (H1.z - O.z) * 10.0};
        double r2[3] = {(H2.x - O.x) * 10.0, (H2.y - O.y) * 10.0, (H2.z - O.z) * 10.0};
        double rh[3] = {(H1.x - H2.x) * 10.0, (H1.y - H2.y) * 10.0, (H1.z - H2.z) * 10.0};
        double d1 = sqrt(r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2]);
        double d2 = sqrt(r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2]);
        double dh = sqrt(rh[0] * rh[0] + rh[1] * rh[1] + rh[2] * rh[2]);
        double costh = (r1[0] * r2[0] + r1[1] * r2[1] + r1[2] * r2[2]) / (d1 * d2);
        const OneBodyParams& P = c_1b;
        double ex1 = exp(-P.alphaoh * (d1 - P.roh));
        double ex2 = exp(-P.alphaoh * (d2 - P.roh));
        double Va = P.deoh * (ex1 * (ex1 - 2.0) + ex2 * (ex2 - 2.0));
        double Vb = P.phh1 * exp(-P.phh2 * dh);
        double dVa1 = 2.0 * P.alphaoh * P.deoh * ex1 * (1.0 - ex1) / d1;
        double dVa2 = 2.0 * P.alphaoh * P.deoh * ex2 * (1.0 - ex2) / d2;
        double dVb = -P.phh2 * Vb / dh;
        double x1 = (d1 - P.reoh) / P.reoh, x2 = (d2 - P.reoh) / P.reoh, x3 = costh - P.costhe;
        // powers p[i][n] = x^n, n = 0..15 (index shifted by one w.r.t. the
        // reference's fmat table, whose column 0 is a zero pad)
        double p1[16], p2[16], p3[16];
        p1[0] = p2[0] = p3[0] = 1.0;
        #pragma unroll
        for (int n = 1; n < 16; ++n) {
            p1[n] = p1[n - 1] * x1;
            p2[n] = p2[n - 1] * x2;
            p3[n] = p3[n - 1] * x3;
        }
        double efac = exp(-P.b1 * ((d1 - P.reoh) * (d1 - P.reoh) + (d2 - P.reoh) * (d2 - P.reoh)));
        double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
        for (int j = 1; j < 245; ++j) {
            const int a = c_1b_idx[0][j] - 1, b = c_1b_idx[1][j] - 1, c = c_1b_idx[2][j] - 1;
            const double cj = c_1b_coef[j];
            const double sym = p1[a] * p2[b] + p1[b] * p2[a];
            s0 += cj * sym * p3[c];
            double t1 = (a > 0 ? a * p1[a - 1] * p2[b] : 0.0) + (b > 0 ? b * p1[b - 1] * p2[a] : 0.0);
            double t2 = (b > 0 ? b * p1[a] * p2[b - 1] : 0.0) + (a > 0 ? a * p1[b] * p2[a - 1] : 0.0);
            s1 += cj * t1 * p3[c];
            s2 += cj * t2 * p3[c];
            s3 += (c > 0 ? cj * sym * c * p3[c - 1] : 0.0);
        }
        double Vc = 2.0 * c_1b_coef[0] + efac * s0;
        double e1 = (Va + Vb + Vc + 0.44739574026257) * P.cm1_kcalmol;
        e_out = e1 * kCalToJ;
        double dVcdr1 = (-2.0 * P.b1 * efac * (d1 - P.reoh) * s0 + efac * s1 / P.reoh) / d1;
        double dVcdr2 = (-2.0 * P.b1 * efac * (d2 - P.reoh) * s0 + efac * s2 / P.reoh) / d2;
        double dVcdcth = efac * s3;
        const double sc = P.cm1_kcalmol * kCalToJ * 10.0;
        double fH1[3], fH2[3];
        for (int k = 0; k < 3; ++k) {
            fH1[k] = (dVa1 * r1[k] + dVb * rh[k] + dVcdr1 * r1[k] +
                      dVcdcth * (r2[k] / (d1 * d2) - costh * r1[k] / (d1 * d1))) * sc;
            fH2[k] = (dVa2 * r2[k] - dVb * rh[k] + dVcdr2 * r2[k] +
                      dVcdcth * (r1[k] / (d1 * d2) - costh * r2[k] / (d2 * d2))) * sc;
        }
        add_force(force, wi.y, -fH1[0], -fH1[1], -fH1[2]);
        add_force(force, wi.z, -fH2[0], -fH2[1], -fH2[2]);
        add_force(force, wi.x, fH1[0] + fH2[0], fH1[1] + fH2[1], fH1[2] + fH2[2]);
        cluster_energy(cs, w, e_out);
    }
    block_sum_atomic<128>(e_out, energy);
}

// ---------------------------------------------------------------- two-body
// Variable table: sites 0 Oa 1 Ha1 2 Ha2 3 Ob 4 Hb1 5 Hb2 6 Xa1 7 Xa2 8 Xb1 9 Xb2.
// kind 0: exp(k(r0-r)); kind 1: exp(k(r0-r))/r.
struct Var2 {
    unsigned char a, b, kind;
    float k, r0;
    double kd;       // k in FP64
    float kdh, kdl;  // k as a double-float, for the variable kernel
};
__constant__ Var2 c_v2[31];
struct TwoBodyParams {
    float gamma_in, gamma_out, r2i, r2f;
};
__constant__ TwoBodyParams c_2b;

__device__ __forceinline__ void twobody_sites(const int4 wa, const int4 wb, const double* __restrict__ pos,
                                              const Box& box, f3 s[10]) {
    double3 Oa = load_pos(pos, wa.x);
    double3 Ha1 = image_to(Oa, load_pos(pos, wa.y), box);
    double3 Ha2 = image_to(Oa, load_pos(pos, wa.z), box);
    double3 Ob = image_to(Oa, load_pos(pos, wb.x), box);
    double3 Hb1 = image_to(Ob, load_pos(pos, wb.y), box);
    double3 Hb2 = image_to(Ob, load_pos(pos, wb.z), box);
    s[0] = mk(0.f, 0.f, 0.f);
    s[1] = rel_A(Oa, Ha1);
    s[2] = rel_A(Oa, Ha2);
    s[3] = rel_A(Oa, Ob);
    s[4] = rel_A(Oa, Hb1);
    s[5] = rel_A(Oa, Hb2);
    const float gi = c_2b.gamma_in, go = c_2b.gamma_out;
    // lone-pair sites of each monomer (mbpol_2body_constants.cpp:62-77)
    {
        f3 oh1 = s[1] - s[0], oh2 = s[2] - s[0];
        f3 inp = s[0] + (oh1 + oh2) * (0.5f * gi);
        f3 out = cross(oh1, oh2) * go;
        s[6] = inp + out;
        s[7] = inp - out;
    }
    {
        f3 oh1 = s[4] - s[3], oh2 = s[5] - s[3];
        f3 inp = s[3] + (oh1 + oh2) * (0.5f * gi);
        f3 out = cross(oh1, oh2) * go;
        s[8] = inp + out;
        s[9] = inp - out;
    }
}

// The polynomial inputs are computed in FP64 and handed over as FP32
// (hi, lo) pairs: the monomial sum amplifies input rounding by its
// cancellation factor, so FP32-rounded variables would cost ~5e-6 relative.
__device__ __forceinline__ void store_hl(float* __restrict__ X, int idx, int plane, double v) {
    const float h = (float)v;
    X[idx] = h;
    X[idx + plane] = (float)(v - (double)h);
}

struct d3v {
    double x, y, z;
};
__device__ __forceinline__ d3v dsub(double3 a, double3 b) { return d3v{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ double dnorm(d3v a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }

__global__ void twobody_vars_kernel(int npairs, const int2* __restrict__ pairs, const int4* __restrict__ waters,
                                    const double* __restrict__ pos, Box box, float* __restrict__ X, int stride) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npairs) return;
    const int2 pr = pairs[p];
    const int4 wa = waters[pr.x], wb = waters[pr.y];
    double3 S[10];
    S[0] = load_pos(pos, wa.x);
    S[1] = image_to(S[0], load_pos(pos, wa.y), box);
    S[2] = image_to(S[0], load_pos(pos, wa.z), box);
    S[3] = image_to(S[0], load_pos(pos, wb.x), box);
    S[4] = image_to(S[3], load_pos(pos, wb.y), box);
    S[5] = image_to(S[3], load_pos(pos, wb.z), box);
    const double3 O0 = S[0];
    for (int i = 0; i < 6; ++i)  // Angstrom, relative to Oa
        S[i] = make_double3((S[i].x - O0.x) * kNmToA, (S[i].y - O0.y) * kNmToA, (S[i].z - O0.z) * kNmToA);
    const double gi = -9.721486914088159e-02, go = 9.859272078406150e-02;
    for (int m = 0; m < 2; ++m) {
        const double3 O = S[3 * m], H1 = S[3 * m + 1], H2 = S[3 * m + 2];
        const d3v a = dsub(H1, O), b = dsub(H2, O);
        const d3v c = {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
        const double3 inp = make_double3(O.x + (a.x + b.x) * 0.5 * gi, O.y + (a.y + b.y) * 0.5 * gi,
                                         O.z + (a.z + b.z) * 0.5 * gi);
        S[6 + 2 * m] = make_double3(inp.x + c.x * go, inp.y + c.y * go, inp.z + c.z * go);
        S[7 + 2 * m] = make_double3(inp.x - c.x * go, inp.y - c.y * go, inp.z - c.z * go);
    }
    // as double-floats from here (the X sites are built in FP64 above)
    dfm::df R[10][3];
    #pragma unroll
    for (int i = 0; i < 10; ++i) {
        R[i][0] = dfm::from_double(S[i].x);
        R[i][1] = dfm::from_double(S[i].y);
        R[i][2] = dfm::from_double(S[i].z);
    }
    const int plane = 31 * stride;
    #pragma unroll 1
    for (int n = 0; n < 31; ++n) {
        const Var2 v = c_v2[n];
        const dfm::df r = dfm::dist(R[v.a], R[v.b]);
        dfm::df e = dfm::exp_df(dfm::mul(dfm::df{v.kdh, v.kdl}, dfm::sub(dfm::df{v.r0, 0.f}, r)));
        if (v.kind) e = dfm::mul(e, dfm::recip(r));
        X[n * stride + p] = e.h;
        X[n * stride + p + plane] = e.l;
    }
}

__global__ void twobody_forces_kernel(int npairs, const int2* __restrict__ pairs, const int4* __restrict__ waters,
                                      const double* __restrict__ pos, Box box, const float* __restrict__ G,
                                      const float* __restrict__ E, int stride, double* __restrict__ force,
                                      double* __restrict__ energy, ClusterSink cs) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    double e_out = 0.0;
    if (p < npairs) {
        const int2 pr = pairs[p];
        const int4 wa = waters[pr.x], wb = waters[pr.y];
        f3 s[10];
        twobody_sites(wa, wb, pos, box, s);
        f3 dOO = s[0] - s[3];
        float rOO = sqrtf(dot(dOO, dOO));
        if (rOO <= c_2b.r2f && rOO >= 2.0f) {
            f3 gr[10];
            #pragma unroll
            for (int i = 0; i < 10; ++i) gr[i] = mk(0.f, 0.f, 0.f);
            #pragma unroll
            for (int n = 0; n < 31; ++n) {
                const Var2 v = c_v2[n];
                f3 d = s[v.a] - s[v.b];
                float r = sqrtf(dot(d, d));
                float e = expf(v.k * (v.r0 - r));
                float gg;
                if (v.kind) {
                    float ri = 1.0f / r;
                    gg = -(v.k + ri) * e * ri * ri;
                } else {
                    gg = -v.k * e / r;
                }
                f3 dd = d * (gg * G[n * stride + p]);
                gr[v.a] += dd;
                gr[v.b] -= dd;
            }
            // distribute X-site gradients to O, H1, H2 (mbpol_2body_constants.cpp:81-102)
            const float gi = c_2b.gamma_in, go = c_2b.gamma_out;
            #pragma unroll
            for (int m = 0; m < 2; ++m) {
                const int o = 3 * m, h1 = o + 1, h2 = o + 2, x1 = 6 + 2 * m, x2 = 7 + 2 * m;
                f3 oh1 = s[h1] - s[o], oh2 = s[h2] - s[o];
                f3 gm = gr[x1] - gr[x2];
                f3 t1 = cross(oh2, gm), t2 = cross(oh1, gm);
                f3 gsum = gr[x1] + gr[x2];
                f3 inp = gsum * (0.5f * gi);
                f3 gh1 = inp + t1 * go;
                f3 gh2 = inp - t2 * go;
                gr[o] += gsum - (gh1 + gh2);
                gr[h1] += gh1;
                gr[h2] += gh2;
            }
            // switch (mbpol_2body_constants.cpp:96-111)
            float sw = 1.0f, gsw = 0.0f;
            if (rOO > c_2b.r2i) {
                const float t1 = kPiF / (c_2b.r2f - c_2b.r2i);
                const float x = (rOO - c_2b.r2i) * t1;
                gsw = -sinf(x) * t1 * 0.5f;
                sw = (1.0f + cosf(x)) * 0.5f;
            }
            const float Ep = E[p];
            const float fs = sw * (float)(kCalToJ * -10.0);
            const float gs = gsw * Ep / rOO * (float)(kCalToJ * -10.0);
            const int idx[6] = {wa.x, wa.y, wa.z, wb.x, wb.y, wb.z};
            #pragma unroll
            for (int i = 0; i < 6; ++i) {
                f3 f = gr[i] * fs;
                if (i == 0) f += dOO * gs;
                if (i == 3) f -= dOO * gs;
                add_force(force, idx[i], f.x, f.y, f.z);
            }
            e_out = (double)sw * (double)Ep * kCalToJ;
            cluster_energy(cs, pr.x, e_out);
        }
    }
    block_sum_atomic<128>(e_out, energy);
}

// -------------------------------------------------------------- three-body
// Sites 0 Oa 1 Ha1 2 Ha2 3 Ob 4 Hb1 5 Hb2 6 Oc 7 Hc1 8 Hc2; x = exp(-k(d - d0)).
struct Var3 {
    unsigned char a, b;
    float k, d0;
    double kd, dd;                // FP64 copies
    float kdh, kdl, ddh, ddl;     // the same as double-floats, for the variable kernel
};
__constant__ Var3 c_v3[36];
__constant__ float c_3b_rf;  // switch outer radius (A)

__device__ __forceinline__ void threebody_sites(const int4 wa, const int4 wb, const int4 wc,
                                                const double* __restrict__ pos, const Box& box, f3 s[9]) {
    double3 Oa = load_pos(pos, wa.x);
    double3 Ha1 = image_to(Oa, load_pos(pos, wa.y), box);
    double3 Ha2 = image_to(Oa, load_pos(pos, wa.z), box);
    double3 Ob = image_to(Oa, load_pos(pos, wb.x), box);
    double3 Hb1 = image_to(Ob, load_pos(pos, wb.y), box);
    double3 Hb2 = image_to(Ob, load_pos(pos, wb.z), box);
    double3 Oc = image_to(Oa, load_pos(pos, wc.x), box);
    double3 Hc1 = image_to(Oc, load_pos(pos, wc.y), box);
    double3 Hc2 = image_to(Oc, load_pos(pos, wc.z), box);
    s[0] = mk(0.f, 0.f, 0.f);
    s[1] = rel_A(Oa, Ha1);
    s[2] = rel_A(Oa, Ha2);
    s[3] = rel_A(Oa, Ob);
    s[4] = rel_A(Oa, Hb1);
    s[5] = rel_A(Oa, Hb2);
    s[6] = rel_A(Oa, Oc);
    s[7] = rel_A(Oa, Hc1);
    s[8] = rel_A(Oa, Hc2);
}

__global__ void threebody_vars_kernel(int ntrip, const int4* __restrict__ trips, const int4* __restrict__ waters,
                                      const double* __restrict__ pos, Box box, float* __restrict__ X, int stride) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= ntrip) return;
    const int4 tr = trips[t];
    const int4 wa = waters[tr.x], wb = waters[tr.y], wc = waters[tr.z];
    double3 S[9];
    S[0] = load_pos(pos, wa.x);
    S[1] = image_to(S[0], load_pos(pos, wa.y), box);
    S[2] = image_to(S[0], load_pos(pos, wa.z), box);
    S[3] = image_to(S[0], load_pos(pos, wb.x), box);
    S[4] = image_to(S[3], load_pos(pos, wb.y), box);
    S[5] = image_to(S[3], load_pos(pos, wb.z), box);
    S[6] = image_to(S[0], load_pos(pos, wc.x), box);
    S[7] = image_to(S[6], load_pos(pos, wc.y), box);
    S[8] = image_to(S[6], load_pos(pos, wc.z), box);
    // sites relative to the first O (Angstrom) as double-floats: the 36
    // distances and exponentials then run on the FP32 pipe (FP64 is kept
    // for the imaging only)
    dfm::df R[9][3];
    #pragma unroll
    for (int i = 0; i < 9; ++i) {
        R[i][0] = dfm::from_double((S[i].x - S[0].x) * kNmToA);
        R[i][1] = dfm::from_double((S[i].y - S[0].y) * kNmToA);
        R[i][2] = dfm::from_double((S[i].z - S[0].z) * kNmToA);
    }
    const int plane = 36 * stride;
    #pragma unroll 1
    for (int n = 0; n < 36; ++n) {
        const Var3 v = c_v3[n];
        const dfm::df e = dfm::exp_df(
            dfm::mul(dfm::df{-v.kdh, -v.kdl}, dfm::sub(dfm::dist(R[v.a], R[v.b]), dfm::df{v.ddh, v.ddl})));
        X[n * stride + t] = e.h;
        X[n * stride + t + plane] = e.l;
    }
}

__device__ __forceinline__ float sw3(float r, float rf, float& g) {
    if (r > rf) {
        g = 0.f;
        return 0.f;
    }
    const float t1 = kPiF / rf;
    const float x = r * t1;
    g = -sinf(x) * t1 * 0.5f;
    return (1.0f + cosf(x)) * 0.5f;
}

__global__ void threebody_forces_kernel(int ntrip, const int4* __restrict__ trips, const int4* __restrict__ waters,
                                        const double* __restrict__ pos, Box box, const float* __restrict__ G,
                                        const float* __restrict__ E, int stride, double* __restrict__ force,
                                        double* __restrict__ energy, ClusterSink cs) {
    int t = blockIdx.x * blockDim.x + threadIdx.x;
    double e_out = 0.0;
    if (t < ntrip) {
        const int4 tr = trips[t];
        const int4 wa = waters[tr.x], wb = waters[tr.y], wc = waters[tr.z];
        f3 s[9];
        threebody_sites(wa, wb, wc, pos, box, s);
        f3 rab = s[0] - s[3], rac = s[0] - s[6], rbc = s[3] - s[6];
        float dab = sqrtf(dot(rab, rab)), dac = sqrtf(dot(rac, rac)), dbc = sqrtf(dot(rbc, rbc));
        if (!(dab < 2.f || dac < 2.f || dbc < 2.f)) {
            float gab, gac, gbc;
            const float rf = c_3b_rf;
            const float sab = sw3(dab, rf, gab), sac = sw3(dac, rf, gac), sbc = sw3(dbc, rf, gbc);
            const float sw = sab * sac + sab * sbc + sac * sbc;
            const float Ep = E[t];
            f3 fr[9];
            #pragma unroll
            for (int i = 0; i < 9; ++i) fr[i] = mk(0.f, 0.f, 0.f);
            const float cf = (float)(kCalToJ * 10.0 * -1.0);
            #pragma unroll
            for (int n = 0; n < 36; ++n) {
                const Var3 v = c_v3[n];
                f3 d = s[v.a] - s[v.b];
                float r = sqrtf(dot(d, d));
                float gg = -v.k * (G[n * stride + t] * sw) * expf(-v.k * (r - v.d0)) / r * cf;
                f3 dd = d * gg;
                fr[v.a] += dd;
                fr[v.b] -= dd;
            }
            gab *= (sac + sbc) * Ep / dab;
            gac *= (sab + sbc) * Ep / dac;
            gbc *= (sab + sac) * Ep / dbc;
            fr[0] += (rab * gab + rac * gac) * cf;
            fr[3] += (rbc * gbc - rab * gab) * cf;
            fr[6] -= (rac * gac + rbc * gbc) * cf;
            const int idx[9] = {wa.x, wa.y, wa.z, wb.x, wb.y, wb.z, wc.x, wc.y, wc.z};
            #pragma unroll
            for (int i = 0; i < 9; ++i) add_force(force, idx[i], fr[i].x, fr[i].y, fr[i].z);
            e_out = (double)Ep * (double)sw * kCalToJ;
            cluster_energy(cs, tr.x, e_out);
        }
    }
    block_sum_atomic<128>(e_out, energy);
}

// ----------------------------------------------------------- host set-up
void upload_polyterm_constants(const double* c5z, const unsigned char* idx3x245) {
    // One-body constants: platforms/reference/src/mbpol_interaction_constants.h:4-22,368-375
    // and MBPolReferenceOneBodyForce.cpp:79-104.
    const double Eh_J = 4.35974434e-18, Na = 6.02214129e+23, kcal_J = 4184.0;
    const double c0 = 299792458.0, h_Js = 6.62606957e-34;
    const double Eh_kcalmol = Eh_J * Na / kcal_J;
    const double Eh_cm1 = 1.0e-2 * Eh_J / (c0 * h_Js);
    const double f5z = 0.999677885;
    OneBodyParams p;
    p.reoh = 0.958649;
    p.b1 = 2.0;
    p.roh = 0.9519607159623009;
    p.alphaoh = 2.587949757553683;
    p.deoh = f5z * 42290.92019288289;
    p.phh2 = 12.66426998162947;
    p.phh1 = f5z * 16.94879431193463 * exp(p.phh2);
    p.costhe = -.24780227221366464506;
    p.cm1_kcalmol = Eh_kcalmol / Eh_cm1;
    cudaMemcpyToSymbol(c_1b, &p, sizeof(p));
    cudaMemcpyToSymbol(c_1b_coef, c5z, 245 * sizeof(double));
    cudaMemcpyToSymbol(c_1b_idx, idx3x245, 3 * 245);

    // Two-body parameters: platforms/reference/src/mbpol_2body_constants.h:33-48
    const float kHHi = -6.480884773303821e-01f, kOHi = 1.674518993682975e+00f;
    const float kHHc = 1.148231864355956e+00f, kOHc = 1.205989761123099e+00f, kOOc = 1.395357065790959e+00f;
    const float kXH = 7.347036852042255e-01f, kXO = 7.998249864422826e-01f, kXX = 7.960663960630585e-01f;
    const Var2 v2[31] = {
        {1, 2, 0, kHHi, 1.f, 0.0}, {4, 5, 0, kHHi, 1.f}, {0, 1, 0, kOHi, 1.f}, {0, 2, 0, kOHi, 1.f},
        {3, 4, 0, kOHi, 1.f}, {3, 5, 0, kOHi, 1.f}, {1, 4, 1, kHHc, 4.f}, {1, 5, 1, kHHc, 4.f},
        {2, 4, 1, kHHc, 4.f}, {2, 5, 1, kHHc, 4.f}, {0, 4, 1, kOHc, 4.f}, {0, 5, 1, kOHc, 4.f},
        {3, 1, 1, kOHc, 4.f}, {3, 2, 1, kOHc, 4.f}, {0, 3, 1, kOOc, 4.f}, {6, 4, 0, kXH, 4.f},
        {6, 5, 0, kXH, 4.f},  {7, 4, 0, kXH, 4.f},  {7, 5, 0, kXH, 4.f},  {8, 1, 0, kXH, 4.f},
        {8, 2, 0, kXH, 4.f},  {9, 1, 0, kXH, 4.f},  {9, 2, 0, kXH, 4.f},  {0, 8, 0, kXO, 4.f},
        {0, 9, 0, kXO, 4.f},  {3, 6, 0, kXO, 4.f},  {3, 7, 0, kXO, 4.f},  {6, 8, 0, kXX, 4.f},
        {6, 9, 0, kXX, 4.f},  {7, 8, 0, kXX, 4.f},  {7, 9, 0, kXX, 4.f}};
    Var2 v2d[31];
    const double kd2[8] = {-6.480884773303821e-01, 1.674518993682975e+00, 1.148231864355956e+00, 1.205989761123099e+00,
                           1.395357065790959e+00, 7.347036852042255e-01, 7.998249864422826e-01, 7.960663960630585e-01};
    const float kf2[8] = {kHHi, kOHi, kHHc, kOHc, kOOc, kXH, kXO, kXX};
    for (int n = 0; n < 31; ++n) {
        v2d[n] = v2[n];
        for (int q = 0; q < 8; ++q)
            if (v2[n].k == kf2[q]) v2d[n].kd = kd2[q];
    }
    for (int n = 0; n < 31; ++n) {
        v2d[n].kdh = (float)v2d[n].kd;
        v2d[n].kdl = (float)(v2d[n].kd - (double)v2d[n].kdh);
    }
    cudaMemcpyToSymbol(c_v2, v2d, sizeof(v2d));
    TwoBodyParams tp = {-9.721486914088159e-02f, 9.859272078406150e-02f, 4.5f, 6.5f};
    cudaMemcpyToSymbol(c_2b, &tp, sizeof(tp));

    // Three-body parameters: platforms/reference/src/mbpol_3body_constants.h:5-20
    const float kHHi3 = -2.254303257872797e+00f, kOHi3 = -2.564771901404151e-01f;
    const float kHH = 4.247920544074333e-01f, kOH = 8.128985941165371e-01f, kOO = 3.749457984616480e-02f;
    const float dHHi = 1.690594510379166e+00f, dOHi = -2.999999868517452e+00f;
    const float dHH = 3.499031358429095e+00f, dOH = 4.854042963514281e+00f, dOO = 4.816312044947604e-08f;
    const Var3 v3[36] = {
        {1, 2, kHHi3, dHHi}, {4, 5, kHHi3, dHHi}, {7, 8, kHHi3, dHHi}, {0, 1, kOHi3, dOHi}, {0, 2, kOHi3, dOHi},
        {3, 4, kOHi3, dOHi}, {3, 5, kOHi3, dOHi}, {6, 7, kOHi3, dOHi}, {6, 8, kOHi3, dOHi}, {1, 4, kHH, dHH},
        {1, 5, kHH, dHH},    {1, 7, kHH, dHH},    {1, 8, kHH, dHH},    {2, 4, kHH, dHH},    {2, 5, kHH, dHH},
        {2, 7, kHH, dHH},    {2, 8, kHH, dHH},    {4, 7, kHH, dHH},    {4, 8, kHH, dHH},    {5, 7, kHH, dHH},
        {5, 8, kHH, dHH},    {0, 4, kOH, dOH},    {0, 5, kOH, dOH},    {0, 7, kOH, dOH},    {0, 8, kOH, dOH},
        {3, 1, kOH, dOH},    {3, 2, kOH, dOH},    {3, 7, kOH, dOH},    {3, 8, kOH, dOH},    {6, 1, kOH, dOH},
        {6, 2, kOH, dOH},    {6, 4, kOH, dOH},    {6, 5, kOH, dOH},    {0, 3, kOO, dOO},    {0, 6, kOO, dOO},
        {3, 6, kOO, dOO}};
    Var3 v3d[36];
    const double kd3[5] = {-2.254303257872797e+00, -2.564771901404151e-01, 4.247920544074333e-01,
                           8.128985941165371e-01, 3.749457984616480e-02};
    const float kf3[5] = {kHHi3, kOHi3, kHH, kOH, kOO};
    const double dd3[5] = {1.690594510379166e+00, -2.999999868517452e+00, 3.499031358429095e+00,
                           4.854042963514281e+00, 4.816312044947604e-08};
    for (int n = 0; n < 36; ++n) {
        v3d[n] = v3[n];
        for (int q = 0; q < 5; ++q)
            if (v3[n].k == kf3[q]) {
                v3d[n].kd = kd3[q];
                v3d[n].dd = dd3[q];
            }
    }
    for (int n = 0; n < 36; ++n) {
        v3d[n].kdh = (float)v3d[n].kd;
        v3d[n].kdl = (float)(v3d[n].kd - (double)v3d[n].kdh);
        v3d[n].ddh = (float)v3d[n].dd;
        v3d[n].ddl = (float)(v3d[n].dd - (double)v3d[n].ddh);
    }
    cudaMemcpyToSymbol(c_v3, v3d, sizeof(v3d));
    const float rf = 4.5f;
    cudaMemcpyToSymbol(c_3b_rf, &rf, sizeof(rf));
}

void launch_onebody(cudaStream_t st, int nw, const int4* waters, const double* pos, Box box, double* force,
                    double* energy, ClusterSink cs) {
    if (nw <= 0) return;
    count_launch();
    onebody_kernel<<<(nw + 127) / 128, 128, 0, st>>>(nw, waters, pos, box, force, energy, cs);
}

void launch_twobody_vars(cudaStream_t st, int npairs, const int2* pairs, const int4* waters, const double* pos,
                         Box box, float* X, int stride) {
    if (npairs <= 0) return;
    count_launch();
    twobody_vars_kernel<<<(npairs + 127) / 128, 128, 0, st>>>(npairs, pairs, waters, pos, box, X, stride);
}

void launch_twobody_forces(cudaStream_t st, int npairs, const int2* pairs, const int4* waters, const double* pos,
                           Box box, const float* G, const float* E, int stride, double* force, double* energy,
                           ClusterSink cs) {
    if (npairs <= 0) return;
    count_launch();
    twobody_forces_kernel<<<(npairs + 127) / 128, 128, 0, st>>>(npairs, pairs, waters, pos, box, G, E, stride,
                                                                 force, energy, cs);
}

void launch_threebody_vars(cudaStream_t st, int ntrip, const int4* trips, const int4* waters, const double* pos,
                           Box box, float* X, int stride) {
    if (ntrip <= 0) return;
    count_launch();
    threebody_vars_kernel<<<(ntrip + 127) / 128, 128, 0, st>>>(ntrip, trips, waters, pos, box, X, stride);
}

void launch_threebody_forces(cudaStream_t st, int ntrip, const int4* trips, const int4* waters,
                             const double* pos, Box box, const float* G, const float* E, int stride,
                             double* force, double* energy, ClusterSink cs) {
    if (ntrip <= 0) return;
    count_launch();
    threebody_forces_kernel<<<(ntrip + 127) / 128, 128, 0, st>>>(ntrip, trips, waters, pos, box, G, E, stride,
                                                                  force, energy, cs);
}

}  // namespace mbpol
