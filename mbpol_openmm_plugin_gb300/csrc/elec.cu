// MB-pol electrostatics on the GPU: geometry-dependent charges, Thole-damped
// permanent and induced fields, the induced-dipole solver, smooth PME
// (order 5, hand-written spread/gather, cuFFT for the 3D FFT only) and the
// energy/forces including the charge-derivative terms.
//
// Restates platforms/reference/src/MBPolReferenceElectrostaticsForce.cpp:
//   charges + dq/dr         computeWaterCharge                 :2793-3096
//   Thole scale factors     getAndScaleInverseRs(13justScaleTCC) :261-359, gammq.cpp:133-178
//   fixed field             NoCutoff :361-420, PME :1342-1439
//   induced field / solver  :438-647 (NoCutoff), :2280-2470 (PME), update :516-531,
//                           convergence :557-616
//   energy / forces         NoCutoff :649-836, PME :2510-2777, recip :2113-2265, self :2472-2508
//   PME grids               B-spline moduli :1248-1340, splines :1446-1554, spread :1610-1674,1823-1908,
//                           convolution :1676-1713, potentials :1715-1821,1910-2111
// The reference keeps two identical dipole sets ("d" and "p"); one set is
// solved here and every formula is reduced accordingly (d = p).
//
// Layout: molecules of K consecutive sites (K = 4: O, H1, H2, M; or K = 3
// without M).  Per evaluation a full molecule neighbour list (j != i,
// O-O distance <= cutoff + 0.24 nm; all molecules for NoCutoff) stores j and
// the FP64 minimum-image O-O vector rounded to FP32; site-site vectors are
// that vector plus FP32 intramolecular offsets, so no FP64 arithmetic is
// needed in the pair loops.  Pair kernels run one warp per molecule over its
// full list, so each molecule's sites are written by exactly one warp.
#include <cufft.h>

#include <cmath>
#include <cstring>
#include <sstream>
#include <vector>

#include "elec.h"
#include "mbpol_kernels.h"
#include "guess.h"

namespace mbpol {

namespace {

constexpr int kMaxK = 4;
constexpr float kSqrtPiF = 1.77245385091f;  // reference SQRT_PI (MBPolReferenceElectrostaticsForce.cpp:1097)
constexpr double kSqrtPi = 1.77245385091;
constexpr double kElectric = 138.9354558456;  // reference _electric (:52)
constexpr double kDebye = 48.033324;          // reference _debye (:60)
constexpr double kSOR = 0.55;                 // reference _polarSOR (:59)

// largest distance of a molecule's sites from its first site that the cell
// grid of the electrostatics list allows for (water: O-H ~0.1 nm)
constexpr float kCellReach = 0.15f;

struct ElecConst {
    float thole[5];       // TCC, TCD, TDD, TDDOH, TDDHH
    float alpha;          // Ewald alpha (nm^-1), 0 for NoCutoff
    float rc2;            // real-space cutoff^2 (nm^2); huge for NoCutoff
    float self_term;      // 4 alpha^3 / (3 sqrt(pi))
    int K;                // sites per molecule
    int grid[3];
    float scale[3];       // grid / box
    double box[3], inv[3];
    float boxf[3], invf[3];
    int periodic;         // per-site-pair minimum image (PME)
    float fixed_thole_sign;  // +1 the reference's PME fixed-field Thole term, -1 the consistent one
};
__constant__ ElecConst c_el;

// Site-site vector from the molecule O-O vector and the intramolecular
// offsets, re-imaged per site pair as the reference does
// (getPeriodicDelta, MBPolReferenceElectrostaticsForce.cpp:1226-1231): near
// half the box a site pair's minimum image can differ from its molecules'.
__device__ __forceinline__ f3 site_delta(const f3 dOO, const f3 offb, const f3 offa) {
    f3 d = dOO + offb - offa;
    if (c_el.periodic) {
        d.x -= c_el.boxf[0] * rintf(d.x * c_el.invf[0]);
        d.y -= c_el.boxf[1] * rintf(d.y * c_el.invf[1]);
        d.z -= c_el.boxf[2] * rintf(d.z * c_el.invf[2]);
    }
    return d;
}

// ------------------------------------------------------------ Thole scales
// u = r / (alpha_i alpha_j)^(1/6); x = gamma u^4.  Orders as
// getAndScaleInverseRs (justScale): 1 (charge-charge, incomplete gamma),
// 3, 5, 7.  Returns 1 when undamped (damp == 0).

// Regularized upper incomplete gamma Q(3/4, x): series for x < a+1, Lentz
// continued fraction otherwise (Numerical Recipes, "Incomplete Gamma
// Function"; the same method as the reference's gammq.cpp).
__device__ float gammq34(float x) {
    const float a = 0.75f;
    const float gln = 0.203280951431295f;  // ln Gamma(3/4)
    if (x <= 0.f) return 1.f;
    if (x > 88.f) return 0.f;
    if (x < a + 1.f) {
        float ap = a, sum = 1.f / a, del = sum;
        for (int n = 0; n < 64; ++n) {
            ap += 1.f;
            del *= x / ap;
            sum += del;
            if (fabsf(del) < fabsf(sum) * 1e-8f) break;
        }
        return 1.f - sum * expf(-x + a * logf(x) - gln);
    }
    const float FPMIN = 1e-30f;
    float b = x + 1.f - a, c = 1.f / FPMIN, d = 1.f / b, h = d;
    for (int i = 1; i < 64; ++i) {
        const float an = -i * (i - a);
        b += 2.f;
        d = an * d + b;
        if (fabsf(d) < FPMIN) d = FPMIN;
        c = b + an / c;
        if (fabsf(c) < FPMIN) c = FPMIN;
        d = 1.f / d;
        const float del = d * c;
        h *= del;
        if (fabsf(del - 1.f) <= 1e-7f) break;
    }
    return expf(-x + a * logf(x) - gln) * h;
}

struct Thole {
    float e, u4g, u;  // exp(-gamma u^4), gamma u^4, u
    bool damped;
};

// d6prod = (damp_i damp_j)^(1/6) as the product of the sites' sixth roots
// (stored per site), so no powf per pair.
__device__ __forceinline__ Thole thole(float r, float d6prod, float gamma) {
    Thole t;
    t.damped = d6prod != 0.f;
    if (!t.damped) {
        t.e = 0.f; t.u4g = 0.f; t.u = 0.f;
        return t;
    }
    t.u = r / d6prod;
    const float u2 = t.u * t.u;
    t.u4g = gamma * u2 * u2;
    t.e = expf(-t.u4g);
    return t;
}
__device__ __forceinline__ float s3_of(const Thole& t) { return t.damped ? 1.f - t.e : 1.f; }
__device__ __forceinline__ float s5_of(const Thole& t) {
    return t.damped ? (1.f - t.e) - (4.f / 3.f) * t.u4g * t.e : 1.f;
}
__device__ __forceinline__ float s7_of(const Thole& t, float gamma) {
    // ((1-e) - 4/3 g e u^4) - 4/15 g (4 g u^4 - 1) e u^4
    return t.damped ? s5_of(t) - (4.f / 15.f) * t.u4g * (4.f * t.u4g - 1.f) * t.e : 1.f;
}
__device__ __forceinline__ float s1_of(const Thole& t, float gamma) {
    if (!t.damped) return 1.f;
    const float GAMMA34 = 1.2254167024651776f;  // Gamma(3/4)
    return (1.f - t.e) + powf(gamma, 0.25f) * t.u * GAMMA34 * gammq34(t.u4g);
}

// dipole-dipole Thole parameter for a site pair (reference :294-310)
__device__ __forceinline__ float tdd_gamma(bool same, int ti, int tj) {
    if (!same) return c_el.thole[2];
    return (ti == 0 || tj == 0) ? c_el.thole[3] : c_el.thole[4];
}

// Ewald real-space radial functions bn0..bn3 (reference :2538-2560).
struct Bn {
    float b0, b1, b2, b3;
};
__device__ __forceinline__ Bn ewald_bn(float r, float r2) {
    Bn b;
    const float al = c_el.alpha;
    const float ra = al * r;
    b.b0 = erfcf(ra) / r;
    const float alsq2 = 2.f * al * al;
    float alsq2n = al > 0.f ? 1.f / (kSqrtPiF * al) : 0.f;
    const float exp2a = expf(-(ra * ra));
    alsq2n *= alsq2;
    b.b1 = (b.b0 + alsq2n * exp2a) / r2;
    alsq2n *= alsq2;
    b.b2 = (3.f * b.b1 + alsq2n * exp2a) / r2;
    alsq2n *= alsq2;
    b.b3 = (5.f * b.b2 + alsq2n * exp2a) / r2;
    return b;
}

// Erf parts E_k = (2k-1)!!/r^(2k+1) - bn_k of the real-space functions, for
// the intramolecular pairs whose reciprocal-space interaction has to be taken
// out again.  Formed as rr_k - bn_k they cancel catastrophically when
// alpha r << 1: the M site is 0.025 nm from O, where 1/r^3 ~ 6e4 and
// rr_1 - bn_1 ~ 4 alpha^3 / (3 sqrt(pi)) ~ 37 nm^-3, so FP32 keeps three
// digits.  With D = -(1/r) d/dr, E_k = D^k [erf(alpha r) / r]; the Maclaurin
// series of erf gives, with x = alpha r,
//   E_k = (2 alpha / sqrt(pi)) (2 alpha^2)^k sum_m (-1)^m x^(2m) / (m! (2m+2k+1))
// (= (2 alpha/sqrt(pi)) (2 alpha^2)^k int_0^1 t^(2k) exp(-x^2 t^2) dt), whose
// terms stay below the sum for x < 1.  Larger x (never an intramolecular
// water pair at the usual alpha) falls back to the difference in FP64.
__device__ Bn ewald_erf_part(float r) {
    const float al = c_el.alpha;
    const float x = al * r;
    Bn e;
    if (x < 1.f) {
        const float x2 = x * x;
        float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f, t = 1.f;  // t = (-x^2)^m / m!
        for (int m = 0; m < 16; ++m) {
            const float tm = 2.f * m;
            s0 += t / (tm + 1.f);
            s1 += t / (tm + 3.f);
            s2 += t / (tm + 5.f);
            s3 += t / (tm + 7.f);
            t *= -x2 / (float)(m + 1);
            if (fabsf(t) < 1e-9f) break;
        }
        const float c0 = 2.f * al / kSqrtPiF, a2 = 2.f * al * al;
        e.b0 = c0 * s0;
        e.b1 = c0 * a2 * s1;
        e.b2 = c0 * a2 * a2 * s2;
        e.b3 = c0 * a2 * a2 * a2 * s3;
        return e;
    }
    const double rd = r, r2 = rd * rd, ad = al, ra = ad * rd;
    const double b0 = erfc(ra) / rd, ex = exp(-ra * ra), a2 = 2.0 * ad * ad;
    double a2n = a2 / (kSqrtPi * ad);
    const double b1 = (b0 + a2n * ex) / r2;
    a2n *= a2;
    const double b2 = (3.0 * b1 + a2n * ex) / r2;
    a2n *= a2;
    const double b3 = (5.0 * b2 + a2n * ex) / r2;
    const double q1 = 1.0 / rd, q3 = q1 / r2, q5 = 3.0 * q3 / r2, q7 = 5.0 * q5 / r2;
    e.b0 = (float)(q1 - b0);
    e.b1 = (float)(q3 - b1);
    e.b2 = (float)(q5 - b2);
    e.b3 = (float)(q7 - b3);
    return e;
}

__device__ __forceinline__ f3 ld3(const float* p, int i) { return mk(p[3 * i], p[3 * i + 1], p[3 * i + 2]); }

// ------------------------------------------------------ per-molecule prep
// Charges and their derivatives (reference computeWaterCharge :2793-3096;
// dipole-moment-surface coefficients at :2823-2870), FP64 per water.
__constant__ double c_dms[84];
__constant__ unsigned char c_dms_idx[3][84];

__device__ void water_charges(const double3 O, const double3 H1, const double3 H2, double q[4], double dq[4][3][3]) {
    const double Bohr_A = 0.52917721092;
    const double gammaM = 0.426706882, gamma1 = 1.0 - gammaM, gamma2 = gammaM / 2;
    const double costhe = -0.24780227221366464506, reoh = 0.958649, b1D = 1.0;
    const double a = 0.2999e0, b = -0.6932e0, c0 = 1.0099e0, c1 = -0.1801e0, c2 = 0.0892e0;
    double R1[3] = {(H1.x - O.x) * 10.0, (H1.y - O.y) * 10.0, (H1.z - O.z) * 10.0};
    double R2[3] = {(H2.x - O.x) * 10.0, (H2.y - O.y) * 10.0, (H2.z - O.z) * 10.0};
    const double d1 = sqrt(R1[0] * R1[0] + R1[1] * R1[1] + R1[2] * R1[2]);
    const double d2 = sqrt(R2[0] * R2[0] + R2[1] * R2[1] + R2[2] * R2[2]);
    const double costh = (R1[0] * R2[0] + R1[1] * R2[1] + R1[2] * R2[2]) / (d1 * d2);
    const double efac = exp(-b1D * ((d1 - reoh) * (d1 - reoh) + (d2 - reoh) * (d2 - reoh)));
    const double x1 = (d1 - reoh) / reoh, x2 = (d2 - reoh) / reoh, x3 = costh - costhe;
    double p1f[8], p2f[8], p3f[8];  // x^n, n = 0..7
    p1f[0] = p2f[0] = p3f[0] = 1.0;
    for (int n = 1; n < 8; ++n) {
        p1f[n] = p1f[n - 1] * x1;
        p2f[n] = p2f[n - 1] * x2;
        p3f[n] = p3f[n - 1] * x3;
    }
    double p1 = 0, p2 = 0, dp1dr1 = 0, dp1dr2 = 0, dp1dc = 0, dp2dr1 = 0, dp2dr2 = 0, dp2dc = 0;
    for (int j = 1; j < 84; ++j) {
        const int i0 = c_dms_idx[0][j] - 1, i1 = c_dms_idx[1][j] - 1, i2 = c_dms_idx[2][j] - 1;
        const double cj = c_dms[j];
        p1 += cj * p1f[i0] * p2f[i1] * p3f[i2];
        p2 += cj * p1f[i1] * p2f[i0] * p3f[i2];
        if (i0 > 0) dp1dr1 += cj * i0 * p1f[i0 - 1] * p2f[i1] * p3f[i2];
        if (i1 > 0) dp1dr2 += cj * i1 * p1f[i0] * p2f[i1 - 1] * p3f[i2];
        if (i2 > 0) dp1dc += cj * i2 * p1f[i0] * p2f[i1] * p3f[i2 - 1];
        if (i1 > 0) dp2dr1 += cj * i1 * p1f[i1 - 1] * p2f[i0] * p3f[i2];
        if (i0 > 0) dp2dr2 += cj * i0 * p1f[i1] * p2f[i0 - 1] * p3f[i2];
        if (i2 > 0) dp2dc += cj * i2 * p1f[i1] * p2f[i0] * p3f[i2 - 1];
    }
    const double xx = Bohr_A, xx2 = xx * xx;
    dp1dr1 /= reoh / xx;
    dp1dr2 /= reoh / xx;
    dp2dr1 /= reoh / xx;
    dp2dr2 /= reoh / xx;
    const double pl1 = costh, pl2 = 0.5 * (3 * pl1 * pl1 - 1.0);
    const double pc0 = a * (pow(d1, b) + pow(d2, b)) * (c0 + pl1 * c1 + pl2 * c2);
    const double dpc0dr1 = a * b * pow(d1, b - 1) * (c0 + pl1 * c1 + pl2 * c2) * xx2;
    const double dpc0dr2 = a * b * pow(d2, b - 1) * (c0 + pl1 * c1 + pl2 * c2) * xx2;
    const double dpc0dc = a * (pow(d1, b) + pow(d2, b)) * (c1 + 0.5 * (6.0 * pl1) * c2) * xx;
    const double defacdr1 = -2.0 * b1D * (d1 - reoh) * efac * xx;
    const double defacdr2 = -2.0 * b1D * (d2 - reoh) * efac * xx;
    dp1dr1 = dp1dr1 * efac + p1 * defacdr1 + dpc0dr1;
    dp1dr2 = dp1dr2 * efac + p1 * defacdr2 + dpc0dr2;
    dp1dc = dp1dc * efac + dpc0dc;
    dp2dr1 = dp2dr1 * efac + p2 * defacdr1 + dpc0dr1;
    dp2dr2 = dp2dr2 * efac + p2 * defacdr2 + dpc0dr2;
    dp2dc = dp2dc * efac + dpc0dc;
    p1 = c_dms[0] + p1 * efac + pc0 * xx;
    p2 = c_dms[0] + p2 * efac + pc0 * xx;
    const double qO = -(p1 + p2), qH1 = p1, qH2 = p2;
    const double g21 = gamma2 / gamma1;
    q[0] = 0.0;
    q[1] = qH1 + g21 * (qH1 + qH2);
    q[2] = qH2 + g21 * (qH1 + qH2);
    q[3] = qO / gamma1;
    dp1dr1 /= xx;
    dp1dr2 /= xx;
    dp2dr1 /= xx;
    dp2dr2 /= xx;
    const double f1q1r13 = (dp1dr1 - (dp1dc * costh / d1)) / d1;
    const double f1q1r23 = dp1dc / (d1 * d2);
    const double f2q1r23 = (dp1dr2 - (dp1dc * costh / d2)) / d2;
    const double f2q1r13 = dp1dc / (d2 * d1);
    const double f1q2r13 = (dp2dr1 - (dp2dc * costh / d1)) / d1;
    const double f1q2r23 = dp2dc / (d1 * d2);
    const double f2q2r23 = (dp2dr2 - (dp2dc * costh / d2)) / d2;
    const double f2q2r13 = dp2dc / (d2 * d1);
    // dq[site][s][xyz]: derivative of the charge of other-site s (H1, H2, M)
    // w.r.t. the position of `site` (O=0, H1=1, H2=2, M=3), per nm
    for (int k = 0; k < 3; ++k) {
        const double qh1_h1 = f1q1r13 * R1[k] + f1q1r23 * R2[k];
        const double qh1_h2 = f2q1r13 * R1[k] + f2q1r23 * R2[k];
        const double qh1_o = -(qh1_h1 + qh1_h2);
        const double qh2_h1 = f1q2r13 * R1[k] + f1q2r23 * R2[k];
        const double qh2_h2 = f2q2r13 * R1[k] + f2q2r23 * R2[k];
        const double qh2_o = -(qh2_h1 + qh2_h2);
        const double qo_h1 = -(qh1_h1 + qh2_h1), qo_h2 = -(qh1_h2 + qh2_h2), qo_o = -(qh1_o + qh2_o);
        const double sH1 = g21 * (qh1_h1 + qh2_h1), sH2 = g21 * (qh1_h2 + qh2_h2), sO = g21 * (qh1_o + qh2_o);
        dq[1][0][k] = (qh1_h1 + sH1) * 10.0;
        dq[2][0][k] = (qh1_h2 + sH2) * 10.0;
        dq[0][0][k] = (qh1_o + sO) * 10.0;
        dq[1][1][k] = (qh2_h1 + sH1) * 10.0;
        dq[2][1][k] = (qh2_h2 + sH2) * 10.0;
        dq[0][1][k] = (qh2_o + sO) * 10.0;
        dq[1][2][k] = (qo_h1 - 2 * sH1) * 10.0;
        dq[2][2][k] = (qo_h2 - 2 * sH2) * 10.0;
        dq[0][2][k] = (qo_o - 2 * sO) * 10.0;
        dq[3][0][k] = dq[3][1][k] = dq[3][2][k] = 0.0;
    }
}

// Per molecule: site offsets from the first site (FP64 -> FP32, minimum
// image), charges (static or redistributed), charge derivatives, and the PME
// grid coordinates of every site.
__global__ void elec_prepare_kernel(int nmol, const double* __restrict__ pos, int periodic, int redist,
                                    const float* __restrict__ q_static, float* __restrict__ off,
                                    float* __restrict__ q, float* __restrict__ dq, int pme,
                                    int* __restrict__ gidx, float* __restrict__ gfrac, float* __restrict__ reach,
                                    float4* __restrict__ opos) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmol) return;
    const int K = c_el.K, s0 = K * m;
    const double3 O = load_pos(pos, s0);
    {
        // FP32 first-site position for the neighbour prefilter, wrapped into
        // the box when periodic so that FP32 keeps its absolute precision
        double3 w = O;
        if (periodic) {
            w.x -= c_el.box[0] * floor(w.x * c_el.inv[0]);
            w.y -= c_el.box[1] * floor(w.y * c_el.inv[1]);
            w.z -= c_el.box[2] * floor(w.z * c_el.inv[2]);
        }
        opos[m] = make_float4((float)w.x, (float)w.y, (float)w.z, 0.f);
    }
    double3 S[kMaxK];
    double r2max = 0.0;
    for (int s = 0; s < K; ++s) {
        double3 p = load_pos(pos, s0 + s);
        if (periodic) {
            p.x = O.x + min_image(p.x - O.x, c_el.box[0], c_el.inv[0]);
            p.y = O.y + min_image(p.y - O.y, c_el.box[1], c_el.inv[1]);
            p.z = O.z + min_image(p.z - O.z, c_el.box[2], c_el.inv[2]);
        }
        S[s] = p;
        off[3 * (s0 + s)] = (float)(p.x - O.x);
        off[3 * (s0 + s) + 1] = (float)(p.y - O.y);
        off[3 * (s0 + s) + 2] = (float)(p.z - O.z);
        const double r2 = (p.x - O.x) * (p.x - O.x) + (p.y - O.y) * (p.y - O.y) + (p.z - O.z) * (p.z - O.z);
        r2max = r2 > r2max ? r2 : r2max;
    }
    // largest site distance from the first site: the neighbour list takes
    // molecule pairs with O-O <= cutoff + reach_A + reach_B
    reach[m] = (float)sqrt(r2max) + 1e-4f;
    if (redist) {
        // The reference computes the charges from the raw, unimaged positions
        // (MBPolReferenceElectrostaticsForce.cpp:2873-2884), also for waters
        // split across the periodic boundary; reproduced for parity.
        double qq[4], dd[4][3][3];
        water_charges(load_pos(pos, s0), load_pos(pos, s0 + 1), load_pos(pos, s0 + 2), qq, dd);
        for (int s = 0; s < 4; ++s) {
            q[s0 + s] = (float)qq[s];
            for (int o = 0; o < 3; ++o)
                for (int k = 0; k < 3; ++k) dq[9 * (s0 + s) + 3 * o + k] = (float)dd[s][o][k];
        }
    } else {
        for (int s = 0; s < K; ++s) {
            q[s0 + s] = q_static[s0 + s];
            for (int o = 0; o < 9; ++o) dq[9 * (s0 + s) + o] = 0.f;
        }
    }
    if (pme) {
        // reference computeMBPolBsplines (:1522-1554): wrap into [-L/2, L/2),
        // fr = N (w - (int)(w + 0.5) + 0.5), base index ifr - 4 (mod N)
        for (int s = 0; s < K; ++s) {
            const double pp[3] = {S[s].x, S[s].y, S[s].z};
            for (int d = 0; d < 3; ++d) {
                double x = pp[d] - floor(pp[d] * c_el.inv[d] + 0.5) * c_el.box[d];
                double w = x * c_el.inv[d];
                double fr = c_el.grid[d] * (w - (int)(w + 0.5) + 0.5);
                int ifr = (int)fr;
                float frac = (float)(fr - ifr);
                int ig = ifr - 5 + 1;
                if (ig < 0) ig += c_el.grid[d];
                gidx[3 * (s0 + s) + d] = ig;
                gfrac[3 * (s0 + s) + d] = frac;
            }
        }
    }
}

// Molecule neighbour list: j != i, O-O <= cutoff + reach_i + reach_j (cluster-restricted when
// cluster ids are given), with the FP64 minimum-image O-O vector in FP32.
__global__ void elec_neighbors_kernel(int nmol, const double* __restrict__ pos, const float4* __restrict__ opos,
                                      int periodic, double rc, const float* __restrict__ reach, int cap,
                                      int* __restrict__ nb, float* __restrict__ nbd, int* __restrict__ nnb,
                                      int* __restrict__ overflow, const CandidateSet cs) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= nmol) return;
    const int K = c_el.K;
    const double3 oi = load_pos(pos, K * i);
    const float4 fi = opos[i];
    const float ai = fmaxf(fabsf(fi.x), fmaxf(fabsf(fi.y), fabsf(fi.z)));
    const float rci = (float)rc + reach[i];
    // cells are sized for molecules whose sites lie within kCellReach of
    // their first site; a larger one makes the host scan all pairs instead
    if (cs.mode == 2 && lane == 0 && reach[i] > kCellReach) atomicOr(overflow, 2);
    int n = 0;
    for_candidates(cs, nmol, i, lane, [&](const int j) {
        bool in = false;
        double dx = 0, dy = 0, dz = 0;
        if (j >= 0 && j != i) {
            // FP32 prefilter, padded well above its error (2^-24 of each
            // coordinate): the list only has to contain every molecule pair
            // with a site pair within the cutoff, which the pair kernels test
            const float4 fj = opos[j];
            float fx = fj.x - fi.x, fy = fj.y - fi.y, fz = fj.z - fi.z;
            if (periodic) {
                fx -= c_el.boxf[0] * rintf(fx * c_el.invf[0]);
                fy -= c_el.boxf[1] * rintf(fy * c_el.invf[1]);
                fz -= c_el.boxf[2] * rintf(fz * c_el.invf[2]);
            }
            const float aj = fmaxf(fabsf(fj.x), fmaxf(fabsf(fj.y), fabsf(fj.z)));
            const float rl = rci + reach[j] + 1e-4f + 1e-6f * (ai + aj);
            if (fx * fx + fy * fy + fz * fz <= rl * rl) {
                const double3 oj = load_pos(pos, K * j);
                dx = oj.x - oi.x;
                dy = oj.y - oi.y;
                dz = oj.z - oi.z;
                if (periodic) {
                    dx = min_image(dx, c_el.box[0], c_el.inv[0]);
                    dy = min_image(dy, c_el.box[1], c_el.inv[1]);
                    dz = min_image(dz, c_el.box[2], c_el.inv[2]);
                }
                in = true;
            }
        }
        const unsigned msk = __ballot_sync(0xffffffffu, in);
        if (in) {
            const int slot = n + __popc(msk & ((1u << lane) - 1u));
            if (slot < cap) {
                nb[(size_t)i * cap + slot] = j;
                nbd[3 * ((size_t)i * cap + slot)] = (float)dx;
                nbd[3 * ((size_t)i * cap + slot) + 1] = (float)dy;
                nbd[3 * ((size_t)i * cap + slot) + 2] = (float)dz;
            }
        }
        n += __popc(msk);
    });
    if (lane == 0) {
        nnb[i] = n;
        if (n > cap) atomicOr(overflow, 1);
    }
}

// ---------------------------------------------------------------- B-splines
// Order-5 cardinal B-spline weights at the 5 grid points, and their first and
// second derivatives (Cox-de Boor recursion; derivatives by differencing the
// order-4 and order-3 splines).
__device__ __forceinline__ void bspline5(float w, float th[5], float d1[5], float d2[5]) {
    float A2[2] = {1.f - w, w};
    float A3[3];
    A3[2] = 0.5f * w * A2[1];
    A3[1] = 0.5f * ((1.f + w) * A2[0] + (2.f - w) * A2[1]);
    A3[0] = 0.5f * (1.f - w) * A2[0];
    float A4[4];
    {
        const float dn = 1.f / 3.f;
        A4[3] = dn * w * A3[2];
        A4[2] = dn * ((w + 1.f) * A3[1] + (3.f - w) * A3[2]);
        A4[1] = dn * ((w + 2.f) * A3[0] + (2.f - w) * A3[1]);
        A4[0] = dn * (1.f - w) * A3[0];
    }
    {
        const float dn = 0.25f;
        th[4] = dn * w * A4[3];
        th[3] = dn * ((w + 1.f) * A4[2] + (4.f - w) * A4[3]);
        th[2] = dn * ((w + 2.f) * A4[1] + (3.f - w) * A4[2]);
        th[1] = dn * ((w + 3.f) * A4[0] + (2.f - w) * A4[1]);
        th[0] = dn * (1.f - w) * A4[0];
    }
    // first derivative from the order-4 values
    d1[4] = A4[3];
    d1[3] = A4[2] - A4[3];
    d1[2] = A4[1] - A4[2];
    d1[1] = A4[0] - A4[1];
    d1[0] = -A4[0];
    // second derivative: difference the order-3 values twice
    float E[4];
    E[3] = A3[2];
    E[2] = A3[1] - A3[2];
    E[1] = A3[0] - A3[1];
    E[0] = -A3[0];
    d2[4] = E[3];
    d2[3] = E[2] - E[3];
    d2[2] = E[1] - E[2];
    d2[1] = E[0] - E[1];
    d2[0] = -E[0];
}

// Spread charges (mode 0) or dipoles (mode 1) of every site onto the grid
// as 64-bit fixed point (scale 2^40): integer atomics are order independent,
// so the grid, and the solver, are deterministic.  FP32 atomics left a
// run-to-run noise floor of ~1e-8 D in the dipole convergence measure.
constexpr double kGridFix = 1099511627776.0;  // 2^40
// One warp per site: lane l < 25 takes the grid column (x, y) = (l / 5,
// l % 5) of the 5x5x5 stencil and its 5 z points.  The fixed-point atomics
// make the grid independent of the order of the updates; v * 2^40 is exact
// in FP32 and converts to the same integer as in FP64.
constexpr float kGridFixF = 1099511627776.0f;  // 2^40
__global__ void pme_spread_kernel(int nsite, int mode, const float* __restrict__ q, const float* __restrict__ mu,
                                  const int* __restrict__ gidx, const float* __restrict__ gfrac,
                                  unsigned long long* __restrict__ grid) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= nsite || lane >= 25) return;
    float c0 = 0.f, mx = 0.f, my = 0.f, mz = 0.f;
    if (mode == 0) {
        c0 = q[i];
        if (c0 == 0.f) return;
    } else {
        mx = mu[3 * i] * c_el.scale[0];
        my = mu[3 * i + 1] * c_el.scale[1];
        mz = mu[3 * i + 2] * c_el.scale[2];
        if (mx == 0.f && my == 0.f && mz == 0.f) return;
    }
    float tx[5], ty[5], tz[5], dx[5], dy[5], dz[5], sx[5];
    bspline5(gfrac[3 * i], tx, dx, sx);
    bspline5(gfrac[3 * i + 1], ty, dy, sx);
    bspline5(gfrac[3 * i + 2], tz, dz, sx);
    const int Nx = c_el.grid[0], Ny = c_el.grid[1], Nz = c_el.grid[2];
    const int a = lane / 5, b = lane % 5;
    int x = gidx[3 * i] + a, y = gidx[3 * i + 1] + b;
    if (x >= Nx) x -= Nx;
    if (y >= Ny) y -= Ny;
    const int gz = gidx[3 * i + 2];
    float txa = 0.f, dxa = 0.f, tyb = 0.f, dyb = 0.f;
    #pragma unroll
    for (int k = 0; k < 5; ++k) {
        if (k == a) {
            txa = tx[k];
            dxa = dx[k];
        }
        if (k == b) {
            tyb = ty[k];
            dyb = dy[k];
        }
    }
    const float txy = txa * tyb;
    const float wA = mode == 0 ? c0 * txy : mx * dxa * tyb;
    const float wB = mode == 0 ? 0.f : my * txa * dyb;
    const float wC = mode == 0 ? 0.f : mz * txy;
    unsigned long long* row = grid + ((size_t)x * Ny + y) * Nz;
    #pragma unroll
    for (int c = 0; c < 5; ++c) {
        int z = gz + c;
        if (z >= Nz) z -= Nz;
        const float v = mode == 0 ? wA * tz[c] : (wA + wB) * tz[c] + wC * dz[c];
        atomicAdd(row + z, (unsigned long long)__float2ll_rn(v * kGridFixF));
    }
}

// Fixed-point grid -> FP32 grid for the FFT, and the fixed-point grid back
// to zero for the next spread.  The int64 -> FP32 conversion rounds once and
// the 2^-40 scaling is exact, which equals rounding the exact value; no FP64
// arithmetic (a fraction of the FP32 rate on this part).
__global__ void pme_fix_to_float_kernel(long n, unsigned long long* __restrict__ a, float* __restrict__ b) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        b[i] = __ll2float_rn((long long)a[i]) * (float)(1.0 / kGridFix);
        a[i] = 0ull;
    }
}

// Per-wavevector convolution factor of the reciprocal sum (reference
// :1676-1713), tabulated on the R2C half grid for a box and alpha.
__global__ void pme_eterm_kernel(float* __restrict__ et, const float* __restrict__ bx, const float* __restrict__ by,
                                 const float* __restrict__ bz, float expf_, float scalef, int nzh) {
    const int Nx = c_el.grid[0], Ny = c_el.grid[1], Nz = c_el.grid[2];
    const long total = (long)Nx * Ny * nzh;
    for (long idx = blockIdx.x * (long)blockDim.x + threadIdx.x; idx < total; idx += (long)gridDim.x * blockDim.x) {
        const int kz = (int)(idx % nzh);
        const long rest = idx / nzh;
        const int ky = (int)(rest % Ny);
        const int kx = (int)(rest / Ny);
        if (kx == 0 && ky == 0 && kz == 0) {
            et[idx] = 0.f;
            continue;
        }
        const int mx = kx < (Nx + 1) / 2 ? kx : kx - Nx;
        const int my = ky < (Ny + 1) / 2 ? ky : ky - Ny;
        const int mz = kz < (Nz + 1) / 2 ? kz : kz - Nz;
        const float mhx = mx * (float)c_el.inv[0], mhy = my * (float)c_el.inv[1], mhz = mz * (float)c_el.inv[2];
        const float m2 = mhx * mhx + mhy * mhy + mhz * mhz;
        const float denom = m2 * bx[kx] * by[ky] * bz[kz];
        et[idx] = scalef * expf(-expf_ * m2) / denom;
    }
}

// g *= eterm on the R2C half grid
__global__ void pme_scale_kernel(long total, cufftComplex* __restrict__ g, const float* __restrict__ et) {
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
        const float e = et[i];
        cufftComplex v = g[i];
        v.x *= e;
        v.y *= e;
        g[i] = v;
    }
}


// Gather phi and derivatives (grid units) at every site: ncomp 4 (phi, dx,
// dy, dz) or 10 (+ xx, yy, zz, xy, xz, yz).
// One warp per site: lane l < 25 sums its grid column (x, y) = (l / 5, l % 5)
// over z with the spline weights; the 25 partial sums of each component are
// added by a fixed shuffle tree (the same order every call).
__global__ void pme_gather_kernel(int nsite, int ncomp, const float* __restrict__ grid,
                                  const int* __restrict__ gidx, const float* __restrict__ gfrac,
                                  float* __restrict__ phi) {
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (i >= nsite) return;
    float p[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (lane < 25) {
        float tx[5], ty[5], tz[5], dx[5], dy[5], dz[5], ex[5], ey[5], ez[5];
        bspline5(gfrac[3 * i], tx, dx, ex);
        bspline5(gfrac[3 * i + 1], ty, dy, ey);
        bspline5(gfrac[3 * i + 2], tz, dz, ez);
        const int Nx = c_el.grid[0], Ny = c_el.grid[1], Nz = c_el.grid[2];
        const int a = lane / 5, b = lane % 5;
        int x = gidx[3 * i] + a, y = gidx[3 * i + 1] + b;
        if (x >= Nx) x -= Nx;
        if (y >= Ny) y -= Ny;
        const int gz = gidx[3 * i + 2];
        float txa = 0.f, dxa = 0.f, exa = 0.f, tyb = 0.f, dyb = 0.f, eyb = 0.f;
        #pragma unroll
        for (int k = 0; k < 5; ++k) {
            if (k == a) {
                txa = tx[k];
                dxa = dx[k];
                exa = ex[k];
            }
            if (k == b) {
                tyb = ty[k];
                dyb = dy[k];
                eyb = ey[k];
            }
        }
        const float* row = grid + ((size_t)x * Ny + y) * Nz;
        float t0 = 0.f, t1 = 0.f, t2 = 0.f;
        #pragma unroll
        for (int c = 0; c < 5; ++c) {
            int z = gz + c;
            if (z >= Nz) z -= Nz;
            const float v = row[z];
            t0 += v * tz[c];
            t1 += v * dz[c];
            t2 += v * ez[c];
        }
        p[0] = txa * tyb * t0;
        p[1] = dxa * tyb * t0;
        p[2] = txa * dyb * t0;
        p[3] = txa * tyb * t1;
        p[4] = exa * tyb * t0;
        p[5] = txa * eyb * t0;
        p[6] = txa * tyb * t2;
        p[7] = dxa * dyb * t0;
        p[8] = dxa * tyb * t1;
        p[9] = txa * dyb * t1;
    }
    #pragma unroll
    for (int k = 0; k < 10; ++k) {
        if (k >= ncomp) break;
        float v = p[k];
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) phi[(size_t)ncomp * i + k] = v;
    }
}

// ------------------------------------------------------------ pair kernels
struct MolSites {
    f3 off[kMaxK];
    float q[kMaxK], damp[kMaxK], pol[kMaxK];
    int type[kMaxK];
};

__device__ __forceinline__ void load_mol(int m, const float* __restrict__ off, const float* __restrict__ q,
                                         const float* __restrict__ damp, const float* __restrict__ pol,
                                         const int* __restrict__ type, MolSites& M) {
    const int K = c_el.K;
    #pragma unroll
    for (int s = 0; s < kMaxK; ++s) {
        if (s < K) {
            const int i = K * m + s;
            M.off[s] = ld3(off, i);
            M.q[s] = q[i];
            M.damp[s] = damp[i];
            M.pol[s] = pol[i];
            M.type[s] = type[i];
        } else {
            M.off[s] = mk(0.f, 0.f, 0.f);
            M.q[s] = M.damp[s] = M.pol[s] = 0.f;
            M.type[s] = -1;
        }
    }
}

__device__ __forceinline__ float warp_sum(float v) {
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Dipole-dipole field coefficients (pf1, pf2) of the inter-molecular site
// pair (a of molecule A, b of its neighbour in list slot t): planes
// [A][a][b][c] of cap floats each, so that the lanes of a warp (consecutive
// slots) read consecutive words.  The field at a from mu_b is
// d (mu_b . d) pf2 + mu_b pf1, d = r_b - r_a.
__device__ __forceinline__ size_t pair_coef_index(int A, int a, int b, int c, int t, int cap) {
    return ((((size_t)A * kMaxK + a) * kMaxK + b) * 2 + c) * (size_t)cap + t;
}

// Intramolecular site pairs a < b of a K-site molecule, numbered
// a (2K - a - 1) / 2 + (b - a - 1): (0,1) (0,2) (0,3) (1,2) (1,3) (2,3).
constexpr int kMaxIntra = kMaxK * (kMaxK - 1) / 2;
__device__ __forceinline__ int intra_pair(int a, int b, int K) {
    if (a > b) { const int t = a; a = b; b = t; }
    return a * (2 * K - a - 1) / 2 + (b - a - 1);
}

// Fixed field at the sites of molecule A (one warp).  PME adds E_rec (from
// the gathered potential, -scale * dphi).  Writes E0 and mu0 = alpha E0, and
// the intramolecular dipole-field coefficients of the geometry: for pair
// p = (a, b), intra[2p] = pf1 and intra[2p + 1] = pf2 such that the field at
// a from mu_b is d (mu_b . d) pf2 + mu_b pf1 with d = r_b - r_a (same-water
// Thole parameters; with PME the reciprocal-space part is taken out and
// pairs beyond the cutoff get zeros).  They are used by every solver
// iteration, so the Thole and Ewald functions of these pairs run once.
constexpr int kFFWarps = 4;  // fixed_field_kernel: 128 threads, one warp per molecule
template <bool PME>
__global__ void fixed_field_kernel(int nmol, const float* __restrict__ off, const float* __restrict__ q,
                                   const float* __restrict__ damp, const float* __restrict__ pol,
                                   const int* __restrict__ type, const int* __restrict__ nb,
                                   const float* __restrict__ nbd, const int* __restrict__ nnb, int cap,
                                   const float* __restrict__ phi_fix, float* __restrict__ E0,
                                   float* __restrict__ mu_out, float* __restrict__ intra,
                                   float* __restrict__ pcoef, unsigned long long* __restrict__ npair) {
    // per warp: the queue of the current 32 neighbours' site pairs within the
    // cutoff (source lane << 5 | kind << 4 | a << 2 | b; kind 0: both sites
    // polarisable, dipole-field coefficients; kind 1: charge field), the
    // neighbours' index and O-O vector, and A's site offsets and damping
    __shared__ unsigned short s_item[kFFWarps][32 * 2 * kMaxK * kMaxK];
    __shared__ int s_nbB[kFFWarps][32];
    __shared__ float s_nbd[kFFWarps][32][3];
    __shared__ float s_site[kFFWarps][kMaxK][8];  // off xyz, damp, pol
    const int A = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (A >= nmol) return;  // uniform over the warp
    const int K = c_el.K;
    MolSites MA;
    load_mol(A, off, q, damp, pol, type, MA);
    if (lane < K) {
        const int i = K * A + lane;
        const f3 o = ld3(off, i);
        s_site[wid][lane][0] = o.x;
        s_site[wid][lane][1] = o.y;
        s_site[wid][lane][2] = o.z;
        s_site[wid][lane][3] = damp[i];
        s_site[wid][lane][4] = pol[i];
    }
    __syncwarp();
    #pragma unroll
    for (int a = 0; a < kMaxK; ++a)
    #pragma unroll
    for (int b = a + 1; b < kMaxK; ++b) {
        if (b >= K || lane != intra_pair(a, b, K)) continue;
        const f3 d = MA.off[b] - MA.off[a];
        const float r2 = dot(d, d);
        float pf1 = 0.f, pf2 = 0.f;
        if (!PME || r2 <= c_el.rc2) {
            const float r = sqrtf(r2);
            const Thole th = thole(r, MA.damp[a] * MA.damp[b], tdd_gamma(true, MA.type[a], MA.type[b]));
            const float rr3 = 1.f / (r2 * r), rr5 = 3.f * rr3 / r2;
            if (PME) {
                // (1 - s3) rr3 - bn1 and bn2 - (1 - s5) rr5, as E_k - s rr
                const Bn ek = ewald_erf_part(r);
                pf1 = ek.b1 - s3_of(th) * rr3;
                pf2 = s5_of(th) * rr5 - ek.b2;
            } else {
                pf1 = -s3_of(th) * rr3;
                pf2 = s5_of(th) * rr5;
            }
        }
        intra[(size_t)2 * kMaxIntra * A + 2 * lane] = pf1;
        intra[(size_t)2 * kMaxIntra * A + 2 * lane + 1] = pf2;
    }
    float E[kMaxK][3];
    #pragma unroll
    for (int a = 0; a < kMaxK; ++a) E[a][0] = E[a][1] = E[a][2] = 0.f;
    const int n = min(nnb[A], cap);
    const float gcc = c_el.thole[0], gdd = c_el.thole[2];
    unsigned npol = 0;  // polarisable site pairs within the cutoff
    for (int t0 = 0; t0 < n; t0 += 32) {
        // 1. each lane tests the site pairs of its neighbour: polarisable
        //    pairs within the cutoff and charge pairs within the cutoff are
        //    queued; polarisable pairs beyond it get zero coefficients (pairs
        //    with an unpolarisable site are never read and not written)
        const int t = t0 + lane;
        unsigned mpol = 0, mq = 0;
        if (t < n) {
            const int B = nb[(size_t)A * cap + t];
            const f3 dAB = ld3(nbd, (int)((size_t)A * cap + t));
            s_nbB[wid][lane] = B;
            s_nbd[wid][lane][0] = dAB.x;
            s_nbd[wid][lane][1] = dAB.y;
            s_nbd[wid][lane][2] = dAB.z;
            #pragma unroll
            for (int b = 0; b < kMaxK; ++b) {
                if (b >= K) continue;
                const int jb = K * B + b;
                const f3 offb = ld3(off, jb);
                const bool polb = pol[jb] != 0.f, qb = q[jb] != 0.f;
                #pragma unroll
                for (int a = 0; a < kMaxK; ++a) {
                    if (a >= K) continue;
                    const f3 offa = mk(s_site[wid][a][0], s_site[wid][a][1], s_site[wid][a][2]);
                    const f3 d = site_delta(dAB, offb, offa);
                    const bool in = !PME || dot(d, d) <= c_el.rc2;
                    if (polb && s_site[wid][a][4] != 0.f) {
                        if (in) {
                            mpol |= 1u << (a * kMaxK + b);
                        } else {
                            pcoef[pair_coef_index(A, a, b, 0, t, cap)] = 0.f;
                            pcoef[pair_coef_index(A, a, b, 1, t, cap)] = 0.f;
                        }
                    }
                    if (qb && in) mq |= 1u << (a * kMaxK + b);
                }
            }
        }
        // polarisable items first, then charge items, so that at most one
        // round of the evaluation mixes the two kinds
        const int cp = __popc(mpol), cq = __popc(mq);
        int ip = cp, iq = cq;
        #pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int vp = __shfl_up_sync(0xffffffffu, ip, o);
            const int vq = __shfl_up_sync(0xffffffffu, iq, o);
            if (lane >= o) {
                ip += vp;
                iq += vq;
            }
        }
        const int tp = __shfl_sync(0xffffffffu, ip, 31), tq = __shfl_sync(0xffffffffu, iq, 31);
        int pos = ip - cp;
        while (mpol) {
            const int bit = __ffs(mpol) - 1;
            mpol &= mpol - 1;
            s_item[wid][pos++] = (unsigned short)((lane << 5) | bit);
        }
        pos = tp + iq - cq;
        while (mq) {
            const int bit = __ffs(mq) - 1;
            mq &= mq - 1;
            s_item[wid][pos++] = (unsigned short)((lane << 5) | 16 | bit);
        }
        __syncwarp();
        // 2. the warp evaluates the queued pairs, 32 at a time
        for (int g = lane; g < tp + tq; g += 32) {
            const unsigned item = s_item[wid][g];
            const int src = item >> 5, a = (item >> 2) & 3, b = item & 3;
            const int B = s_nbB[wid][src];
            const f3 dAB = mk(s_nbd[wid][src][0], s_nbd[wid][src][1], s_nbd[wid][src][2]);
            const f3 offa = mk(s_site[wid][a][0], s_site[wid][a][1], s_site[wid][a][2]);
            const float da = s_site[wid][a][3];
            const int jb = K * B + b;
            const f3 d = site_delta(dAB, ld3(off, jb), offa);  // r_b - r_a
            const float r2 = dot(d, d);
            const float r = sqrtf(r2);
            const float dprod = da * damp[jb];
            if (!(item & 16)) {
                // dipole-dipole field coefficients of this geometry for the
                // solver iterations (layout of pair_coef_index)
                ++npol;
                const Thole th = thole(r, dprod, gdd);
                float pf1, pf2;
                if (PME) {
                    const Bn bn = ewald_bn(r, r2);
                    const float rr3 = (1.f - s3_of(th)) / (r2 * r);
                    const float rr5 = 3.f * (1.f - s5_of(th)) / (r2 * r2 * r);
                    pf1 = rr3 - bn.b1;
                    pf2 = bn.b2 - rr5;
                } else {
                    pf1 = -s3_of(th) / (r2 * r);
                    pf2 = 3.f * s5_of(th) / (r2 * r2 * r);
                }
                const int t = t0 + src;
                pcoef[pair_coef_index(A, a, b, 0, t, cap)] = pf1;
                pcoef[pair_coef_index(A, a, b, 1, t, cap)] = pf2;
            } else {
                const Thole th = thole(r, dprod, gcc);
                float fac;
                if (PME) {
                    const Bn bn = ewald_bn(r, r2);
                    // reference :1377-1391 subtracts (s3 - 1)/r^3; the
                    // gradient of its energy wants (1 - s3)/r^3
                    const float rr3 = (s3_of(th) - 1.f) / (r2 * r);
                    fac = bn.b1 - c_el.fixed_thole_sign * rr3;
                } else {
                    fac = s3_of(th) / (r2 * r);
                }
                const float c = -q[jb] * fac;
                #pragma unroll
                for (int k = 0; k < kMaxK; ++k)
                    if (k == a) {
                        E[k][0] += d.x * c;
                        E[k][1] += d.y * c;
                        E[k][2] += d.z * c;
                    }
            }
        }
        __syncwarp();
    }
    #pragma unroll
    for (int a = 0; a < kMaxK; ++a) {
        E[a][0] = warp_sum(E[a][0]);
        E[a][1] = warp_sum(E[a][1]);
        E[a][2] = warp_sum(E[a][2]);
    }
    npol = __reduce_add_sync(0xffffffffu, npol);
    if (lane == 0 && npair) atomicAdd(npair, (unsigned long long)npol);
    if (lane == 0) {
        load_mol(A, off, q, damp, pol, type, MA);
        if (PME) {
            // intramolecular pairs: s3 = 2 (reference :1381-1384), within the cutoff
            #pragma unroll
            for (int a = 0; a < kMaxK; ++a)
                #pragma unroll
                for (int b = 0; b < kMaxK; ++b) {
                    if (a >= K || b >= K || a == b || MA.q[b] == 0.f) continue;
                    const f3 d = MA.off[b] - MA.off[a];
                    const float r2 = dot(d, d);
                    if (r2 > c_el.rc2) continue;
                    const float fac = -ewald_erf_part(sqrtf(r2)).b1;  // bn1 - 1/r^3
                    const float c = -MA.q[b] * fac;
                    E[a][0] += d.x * c;
                    E[a][1] += d.y * c;
                    E[a][2] += d.z * c;
                }
        }
        #pragma unroll
        for (int a = 0; a < kMaxK; ++a) {
            if (a >= K) continue;
            const int i = K * A + a;
            float ex = E[a][0], ey = E[a][1], ez = E[a][2];
            if (PME) {
                ex -= c_el.scale[0] * phi_fix[10 * i + 1];
                ey -= c_el.scale[1] * phi_fix[10 * i + 2];
                ez -= c_el.scale[2] * phi_fix[10 * i + 3];
            }
            E0[3 * i] = ex;
            E0[3 * i + 1] = ey;
            E0[3 * i + 2] = ez;
            mu_out[3 * i] = MA.pol[a] * ex;
            mu_out[3 * i + 1] = MA.pol[a] * ey;
            mu_out[3 * i + 2] = MA.pol[a] * ez;
        }
    }
}

// Induced field from mu_in at the sites of molecule A, then the SOR update
// mu <- mu + 0.55 (alpha (E0 + E_ind) - mu) on the FP64 dipoles and the sum
// of |delta|^2.  Any FP32 evaluation of the field carries rounding noise of
// ~1e-7 |mu|, which can keep the convergence measure from reaching 1e-8 D;
// so once the iteration is close, the current dipoles become an anchor whose
// field is stored once (mode 1) and later iterations evaluate only the field
// of mu - anchor (mode 2), whose rounding noise is smaller by |mu - anchor|/|mu|.
// PME (one box): 7 blocks per SM (at most 72 registers) hold a 4096-water
// box's 1024 blocks in one wave (4096 molecules, one warp each); at 6 blocks
// a second, nearly empty wave made the launch 80 instead of 50 us.
template <bool PME>
__global__ void __launch_bounds__(128, PME ? 7 : 6) induced_update_kernel(int nmol, const float* __restrict__ off, const float* __restrict__ damp,
                                      const float* __restrict__ pol, const int* __restrict__ type,
                                      const int* __restrict__ nb, const float* __restrict__ nbd,
                                      const int* __restrict__ nnb, int cap, const float* __restrict__ E0,
                                      const float* __restrict__ phi_mu, const float* __restrict__ mu_in,
                                      float* __restrict__ mu_out, double* __restrict__ mu_d,
                                      double* __restrict__ eps2, int mode, float* __restrict__ Ebase,
                                      const float* __restrict__ anchor, const float* __restrict__ intra,
                                      const float* __restrict__ pcoef, const int* __restrict__ mcl,
                                      const int* __restrict__ cstate, double* __restrict__ eps2c,
                                      const int* __restrict__ polmask, float* __restrict__ anchor_store,
                                      float* __restrict__ Edir) {
    const int A = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    double d2sum = 0.0;
    // batched clusters (mcl set): each cluster converges on its own, with
    // its own stage of the anchoring (cstate 0 plain, 1 anchoring, 2
    // anchored); a finished cluster (cstate 3) keeps its dipoles (copied
    // through, no field work).  At its anchoring iteration a cluster's
    // dipoles are copied to anchor_store, which mode 2 then reads.
    const int cA = (mcl && A < nmol) ? mcl[A] : -1;
    const bool frozen = cA >= 0 && cstate[cA] >= 3;
    if (cA >= 0 && !frozen) mode = cstate[cA];
    if (A < nmol && frozen && lane == 0) {
        for (int i = c_el.K * A; i < c_el.K * (A + 1); ++i)
            for (int k = 0; k < 3; ++k) mu_out[3 * i + k] = (float)mu_d[3 * i + k];
    }
    if (A < nmol && !frozen) {
        const int K = c_el.K;
        f3 offA[kMaxK];
        float polA[kMaxK];
        #pragma unroll
        for (int a = 0; a < kMaxK; ++a) {
            offA[a] = mk(0.f, 0.f, 0.f);
            polA[a] = 0.f;
            if (a < K) {
                offA[a] = ld3(off, K * A + a);
                polA[a] = pol[K * A + a];
            }
        }
        float E[kMaxK][3];
        #pragma unroll
        for (int a = 0; a < kMaxK; ++a) E[a][0] = E[a][1] = E[a][2] = 0.f;
        const int n = min(nnb[A], cap);
        // the next slot's neighbour index is read one iteration ahead, so the
        // gathers that depend on it do not wait for its load
        int Bn = lane < n ? nb[(size_t)A * cap + lane] : 0;
        for (int t = lane; t < n; t += 32) {
            const int B = Bn;
            if (t + 32 < n) Bn = nb[(size_t)A * cap + t + 32];
            const int pmB = polmask[B];
            const f3 dAB = ld3(nbd, (int)((size_t)A * cap + t));
            #pragma unroll
            for (int b = 0; b < kMaxK; ++b) {
                if (b >= K || !((pmB >> b) & 1)) continue;
                const int jb = K * B + b;
                const f3 mub = ld3(mu_in, jb);
                const f3 offb = ld3(off, jb);
                #pragma unroll
                for (int a = 0; a < kMaxK; ++a) {
                    if (a >= K || polA[a] == 0.f) continue;
                    const f3 d = site_delta(dAB, offb, offA[a]);
                    // coefficients of this geometry from the fixed-field pass
                    // (zero beyond the cutoff)
                    const float pf1 = pcoef[pair_coef_index(A, a, b, 0, t, cap)];
                    const float pf2 = pcoef[pair_coef_index(A, a, b, 1, t, cap)];
                    const float dur = dot(mub, d) * pf2;
                    E[a][0] += d.x * dur + mub.x * pf1;
                    E[a][1] += d.y * dur + mub.y * pf1;
                    E[a][2] += d.z * dur + mub.z * pf1;
                }
            }
        }
        #pragma unroll
        for (int a = 0; a < kMaxK; ++a) {
            E[a][0] = warp_sum(E[a][0]);
            E[a][1] = warp_sum(E[a][1]);
            E[a][2] = warp_sum(E[a][2]);
        }
        // intramolecular pairs: coefficients of this geometry from the
        // fixed-field pass
        const float* pin = intra + (size_t)2 * kMaxIntra * A;
        if (PME) {
            // split form (every PME launch passes Edir): the direct and
            // intramolecular field only; the reciprocal part and the update
            // follow in induced_finish_kernel.  Lane 0 takes every site
            // (compile-time pair indices); this instantiation holds no
            // fused update.
            if (lane == 0) {
                #pragma unroll
                for (int a = 0; a < kMaxK; ++a)
                    #pragma unroll
                    for (int b = 0; b < kMaxK; ++b) {
                        if (a >= K || b >= K || a == b) continue;
                        const int p = intra_pair(a, b, K);
                        const float pf1 = pin[2 * p], pf2 = pin[2 * p + 1];
                        const f3 mub = ld3(mu_in, K * A + b);
                        const f3 d = offA[b] - offA[a];
                        const float dur = dot(mub, d) * pf2;
                        E[a][0] += d.x * dur + mub.x * pf1;
                        E[a][1] += d.y * dur + mub.y * pf1;
                        E[a][2] += d.z * dur + mub.z * pf1;
                    }
                #pragma unroll
                for (int a = 0; a < kMaxK; ++a) {
                    if (a >= K) continue;
                    const int i = K * A + a;
                    Edir[3 * i] = E[a][0];
                    Edir[3 * i + 1] = E[a][1];
                    Edir[3 * i + 2] = E[a][2];
                }
            }
        }
        // fused update: one lane per site a of the molecule (the sites'
        // updates are independent; batched clusters, 4096 clusters: solver
        // 38.6 against 55.6 ms with lane 0 taking every site)
        const int a = lane;
        if (!PME && a < K) {
            float ea[3] = {0.f, 0.f, 0.f};
            f3 offa = mk(0.f, 0.f, 0.f);
            #pragma unroll
            for (int aa = 0; aa < kMaxK; ++aa)
                if (aa == a) {
                    ea[0] = E[aa][0];
                    ea[1] = E[aa][1];
                    ea[2] = E[aa][2];
                    offa = offA[aa];
                }
            #pragma unroll
            for (int b = 0; b < kMaxK; ++b) {
                if (b >= K || a == b) continue;
                const int p = intra_pair(a, b, K);
                const float pf1 = pin[2 * p], pf2 = pin[2 * p + 1];
                const f3 mub = ld3(mu_in, K * A + b);
                const f3 d = offA[b] - offa;
                const float dur = dot(mub, d) * pf2;
                ea[0] += d.x * dur + mub.x * pf1;
                ea[1] += d.y * dur + mub.y * pf1;
                ea[2] += d.z * dur + mub.z * pf1;
            }
            const int i = K * A + a;
            {
                const f3 mu = ld3(mu_in, i);
                const double m0 = mu_d[3 * i], m1 = mu_d[3 * i + 1], m2 = mu_d[3 * i + 2];
                float ex = ea[0], ey = ea[1], ez = ea[2];
                if (PME) {
                    ex += c_el.self_term * mu.x - c_el.scale[0] * phi_mu[4 * i + 1];
                    ey += c_el.self_term * mu.y - c_el.scale[1] * phi_mu[4 * i + 2];
                    ez += c_el.self_term * mu.z - c_el.scale[2] * phi_mu[4 * i + 3];
                }
                // mode 1 (anchoring): mu_in is the anchor; store its field.
                // mode 2 (anchored): mu_in is mu - anchor; add the anchor's field.
                if (mode == 1) {
                    Ebase[3 * i] = ex;
                    Ebase[3 * i + 1] = ey;
                    Ebase[3 * i + 2] = ez;
                    if (anchor_store) {
                        anchor_store[3 * i] = mu_in[3 * i];
                        anchor_store[3 * i + 1] = mu_in[3 * i + 1];
                        anchor_store[3 * i + 2] = mu_in[3 * i + 2];
                    }
                }
                // the anchor's field is added in FP64: an FP32 sum would round
                // the small field of mu - anchor to the anchor field's ulp,
                // a floor of ~1e-9 D under the convergence measure
                double bx = 0.0, by = 0.0, bz = 0.0;
                if (mode == 2) {
                    bx = Ebase[3 * i];
                    by = Ebase[3 * i + 1];
                    bz = Ebase[3 * i + 2];
                }
                const float al = pol[i];
                // reference updateInducedDipole (:516-531); E0 is unscaled here
                const double nx = (double)al * ((double)E0[3 * i] + bx + ex);
                const double ny = (double)al * ((double)E0[3 * i + 1] + by + ey);
                const double nz = (double)al * ((double)E0[3 * i + 2] + bz + ez);
                // the dipole state is FP64: FP32 storage alone would put a
                // floor of ~1e-8 D under the convergence measure
                const double dx = nx - m0, dy = ny - m1, dz = nz - m2;
                const double u0 = m0 + kSOR * dx, u1 = m1 + kSOR * dy, u2 = m2 + kSOR * dz;
                mu_d[3 * i] = u0;
                mu_d[3 * i + 1] = u1;
                mu_d[3 * i + 2] = u2;
                if (mode == 0) {
                    mu_out[3 * i] = (float)u0;
                    mu_out[3 * i + 1] = (float)u1;
                    mu_out[3 * i + 2] = (float)u2;
                } else {
                    const float* an = mode == 1 ? mu_in : anchor;
                    mu_out[3 * i] = (float)(u0 - (double)an[3 * i]);
                    mu_out[3 * i + 1] = (float)(u1 - (double)an[3 * i + 1]);
                    mu_out[3 * i + 2] = (float)(u2 - (double)an[3 * i + 2]);
                }
                d2sum += dx * dx + dy * dy + dz * dz;
            }
        }
    }
    if (!PME && mcl) {  // batched clusters are never periodic
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) d2sum += __shfl_xor_sync(0xffffffffu, d2sum, o);
        if (cA >= 0 && !frozen && lane == 0) atomicAdd(eps2c + cA, d2sum);
        d2sum = 0.0;
    }
    block_sum_atomic<128>(d2sum, eps2);
}

// Second half of a split solver iteration (PME, one system): per site, the
// direct + intramolecular field from induced_update_kernel (Edir) plus the
// self and reciprocal parts, the anchoring stages and the SOR update on the
// FP64 dipoles, as the fused kernel does.  Splitting lets the PME pass of
// the same dipoles run on another stream while the direct field is summed.
__global__ void induced_finish_kernel(int n, const float* __restrict__ Edir, const float* __restrict__ phi_mu,
                                      const float* __restrict__ E0, const float* __restrict__ pol,
                                      const float* mu_in, float* mu_out, double* __restrict__ mu_d,
                                      double* __restrict__ eps2, int mode, float* __restrict__ Ebase,
                                      const float* anchor, const int* __restrict__ d_mode, float* anchor_store) {
    // mu_out may be mu_in (the device-controlled loop updates in place: each
    // site's values are read before they are written); d_mode, when given,
    // holds this iteration's anchoring stage, and at the anchoring iteration
    // the dipoles are copied to anchor_store
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (d_mode) mode = *d_mode;
    double d2 = 0.0;
    if (i < n) {
        const f3 mu = ld3(mu_in, i);
        float ex = Edir[3 * i] + c_el.self_term * mu.x - c_el.scale[0] * phi_mu[4 * i + 1];
        float ey = Edir[3 * i + 1] + c_el.self_term * mu.y - c_el.scale[1] * phi_mu[4 * i + 2];
        float ez = Edir[3 * i + 2] + c_el.self_term * mu.z - c_el.scale[2] * phi_mu[4 * i + 3];
        if (mode == 1) {
            Ebase[3 * i] = ex;
            Ebase[3 * i + 1] = ey;
            Ebase[3 * i + 2] = ez;
            if (anchor_store) {
                anchor_store[3 * i] = mu.x;
                anchor_store[3 * i + 1] = mu.y;
                anchor_store[3 * i + 2] = mu.z;
            }
        }
        // the anchor's field in FP64, as in induced_update_kernel
        double bx = 0.0, by = 0.0, bz = 0.0;
        if (mode == 2) {
            bx = Ebase[3 * i];
            by = Ebase[3 * i + 1];
            bz = Ebase[3 * i + 2];
        }
        const double m0 = mu_d[3 * i], m1 = mu_d[3 * i + 1], m2 = mu_d[3 * i + 2];
        const float al = pol[i];
        const double nx = (double)al * ((double)E0[3 * i] + bx + ex);
        const double ny = (double)al * ((double)E0[3 * i + 1] + by + ey);
        const double nz = (double)al * ((double)E0[3 * i + 2] + bz + ez);
        const double dx = nx - m0, dy = ny - m1, dz = nz - m2;
        const double u0 = m0 + kSOR * dx, u1 = m1 + kSOR * dy, u2 = m2 + kSOR * dz;
        mu_d[3 * i] = u0;
        mu_d[3 * i + 1] = u1;
        mu_d[3 * i + 2] = u2;
        if (mode == 0) {
            mu_out[3 * i] = (float)u0;
            mu_out[3 * i + 1] = (float)u1;
            mu_out[3 * i + 2] = (float)u2;
        } else {
            // the anchor: at the anchoring iteration the input dipoles themselves
            const float a0 = mode == 1 ? mu.x : anchor[3 * i];
            const float a1 = mode == 1 ? mu.y : anchor[3 * i + 1];
            const float a2 = mode == 1 ? mu.z : anchor[3 * i + 2];
            mu_out[3 * i] = (float)(u0 - (double)a0);
            mu_out[3 * i + 1] = (float)(u1 - (double)a1);
            mu_out[3 * i + 2] = (float)(u2 - (double)a2);
        }
        d2 = dx * dx + dy * dy + dz * dz;
    }
    block_sum_atomic<128>(d2, eps2);
}

// State of one system's device-controlled solve (below).
struct SolveState {
    int mode;    // anchoring stage of the next iteration: 0 plain, 1 anchoring, 2 anchored
    int its;     // iterations done
    int conv;    // converged
    int rounds;  // iterations launched (bound on the loop)
    double cur;  // epsilon of the last iteration
};

// Convergence control of one system's solve on the device: the host loop's
// rules (reference convergeInduceDipoles, MBPolReferenceElectrostaticsForce.cpp
// :557-616) applied to the iteration just finished -- epsilon from the sum
// of squared changes, stop on convergence, on an increase or at the
// iteration limit -- then the next iteration's anchoring stage, and the
// condition of the graph's while loop.  One thread.
__global__ void solve_control_kernel(double* __restrict__ eps2, double inv_n, SolveState* __restrict__ s,
                                     double target, int max_it, double switch_eps, cudaGraphConditionalHandle loop) {
    const double e = kSOR * kDebye * sqrt(*eps2 * inv_n);
    *eps2 = 0.0;  // the next iteration's sum
    bool stop = false;
    if (!isfinite(e)) {
        stop = true;
    } else if (e < target) {
        s->conv = 1;
        stop = true;
    } else if (s->cur < e || s->its >= max_it) {
        stop = true;
    }
    s->cur = e;
    s->its += 1;
    s->mode = s->mode == 0 ? (e < switch_eps ? 1 : 0) : 2;
    const int r = ++s->rounds;
    cudaGraphSetConditional(loop, (!stop && r <= max_it + 2) ? 1u : 0u);
}

// Double-float (FP32 pair) helpers for the pair energies: FP64 arithmetic
// runs at a small fraction of the FP32 rate on this part.
struct DFe {
    float h, l;
};
__device__ __forceinline__ void dfe_acc(DFe& a, float p, float q) {  // a += p + q (TwoSum on the leading part)
    const float s = __fadd_rn(a.h, p);
    const float bb = __fsub_rn(s, a.h);
    const float e = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(p, bb));
    a.h = s;
    a.l = __fadd_rn(a.l, __fadd_rn(e, q));
}
__device__ __forceinline__ DFe dfe_prod(float a, float b) {  // exact product
    DFe r;
    r.h = __fmul_rn(a, b);
    r.l = __fmaf_rn(a, b, -r.h);
    return r;
}
__device__ __forceinline__ DFe dfe_mul(const DFe& a, const DFe& b) {
    DFe r;
    r.h = __fmul_rn(a.h, b.h);
    r.l = __fmaf_rn(a.h, b.h, -r.h);
    r.l = __fmaf_rn(a.h, b.l, r.l);
    r.l = __fmaf_rn(a.l, b.h, r.l);
    return r;
}
__device__ __forceinline__ DFe dfe_mulf(const DFe& a, float b) {
    DFe r;
    r.h = __fmul_rn(a.h, b);
    r.l = __fmaf_rn(a.h, b, -r.h);
    r.l = __fmaf_rn(a.l, b, r.l);
    return r;
}
__device__ __forceinline__ DFe dfe_dot(const f3& a, const f3& b) {  // a . b of FP32 vectors
    DFe r = dfe_prod(a.x, b.x);
    const DFe y = dfe_prod(a.y, b.y), z = dfe_prod(a.z, b.z);
    dfe_acc(r, y.h, y.l);
    dfe_acc(r, z.h, z.l);
    return r;
}
// 1/|d| of an FP32 vector to ~1e-14: |d|^2 exactly as a double-float, then
// one Newton step y (1 + (1 - r2 y^2)/2) on rsqrtf with the residual formed
// in double-float.
__device__ __forceinline__ DFe dfe_rinv(const f3& d) {
    const DFe r2 = dfe_dot(d, d);
    const float y = rsqrtf(r2.h);
    DFe t = dfe_mulf(dfe_prod(y, y), r2.h);  // r2.h y^2
    t.l = __fmaf_rn(y * y, r2.l, t.l);       // + r2.l y^2
    const float h = __fadd_rn(__fsub_rn(1.f, t.h), -t.l);
    DFe r;
    r.h = y;
    r.l = 0.5f * y * h;
    return r;
}

// Energy and forces for molecule A (one warp): direct pairs over the full
// list (force on A's sites, half the pair energy), intramolecular pairs, the
// reciprocal and self parts, and the charge-derivative forces through the
// total potential at A's H1, H2, M sites.
constexpr int kEFWarps = 4;  // energy_force_kernel: 128 threads, one warp per molecule
static_assert(kMaxK == 4, "energy_force_kernel packs site indices in two bits");
template <bool PME>
__global__ void energy_force_kernel(int nmol, const float* __restrict__ off, const float* __restrict__ q,
                                    const float* __restrict__ dq, const float* __restrict__ damp,
                                    const int* __restrict__ type, const int* __restrict__ nb,
                                    const float* __restrict__ nbd, const int* __restrict__ nnb, int cap,
                                    const float* __restrict__ mu, const float* __restrict__ phi_fix,
                                    const float* __restrict__ phi_mu, int redist, double* __restrict__ force,
                                    double* __restrict__ energy, ClusterSink cs) {
    // per warp: the queue of site pairs within the cutoff of the current 32
    // neighbours (source lane << 4 | a << 2 | b), those neighbours' index and
    // O-O vector, and A's sites
    __shared__ unsigned short s_item[kEFWarps][32 * kMaxK * kMaxK];
    __shared__ int s_nbB[kEFWarps][32];
    __shared__ float s_nbd[kEFWarps][32][3];
    __shared__ float s_site[kEFWarps][kMaxK][8];  // off xyz, mu xyz, q, damp
    const int A = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    double e_out = 0.0;
    if (A < nmol) {
        const int K = c_el.K;
        const float f = (float)kElectric;
        if (lane < K) {
            const int i = K * A + lane;
            const f3 o = ld3(off, i), m = ld3(mu, i);
            float* sa = s_site[wid][lane];
            sa[0] = o.x; sa[1] = o.y; sa[2] = o.z;
            sa[3] = m.x; sa[4] = m.y; sa[5] = m.z;
            sa[6] = q[i];
            sa[7] = damp[i];
        }
        __syncwarp();
        float F[kMaxK][3], P[kMaxK];  // force on A's sites (before * f), potential (for dq terms)
        #pragma unroll
        for (int a = 0; a < kMaxK; ++a) F[a][0] = F[a][1] = F[a][2] = P[a] = 0.f;
        // the pair energies (tens of kJ/mol each, cancelling to the total)
        // are summed per lane in double-float, then in FP64 across the warp
        DFe el = {0.f, 0.f};
        const int n = min(nnb[A], cap);
        const float gcc = c_el.thole[0], gcd = c_el.thole[1], gdd = c_el.thole[2];
        for (int t0 = 0; t0 < n; t0 += 32) {
            // 1. each lane tests the site pairs of its neighbour against the
            //    cutoff and queues those inside it
            const int t = t0 + lane;
            unsigned msk = 0;
            if (t < n) {
                const int B = nb[(size_t)A * cap + t];
                const f3 dAB = ld3(nbd, (int)((size_t)A * cap + t));
                s_nbB[wid][lane] = B;
                s_nbd[wid][lane][0] = dAB.x;
                s_nbd[wid][lane][1] = dAB.y;
                s_nbd[wid][lane][2] = dAB.z;
                #pragma unroll
                for (int b = 0; b < kMaxK; ++b) {
                    if (b >= K) continue;
                    const f3 offb = ld3(off, K * B + b);
                    #pragma unroll
                    for (int a = 0; a < kMaxK; ++a) {
                        if (a >= K) continue;
                        const f3 offa = mk(s_site[wid][a][0], s_site[wid][a][1], s_site[wid][a][2]);
                        const f3 d = site_delta(dAB, offb, offa);
                        if (!PME || dot(d, d) <= c_el.rc2) msk |= 1u << (a * kMaxK + b);
                    }
                }
            }
            const int cnt = __popc(msk);
            int incl = cnt;
            #pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            const int total = __shfl_sync(0xffffffffu, incl, 31);
            int pos = incl - cnt;
            while (msk) {
                const int bit = __ffs(msk) - 1;
                msk &= msk - 1;
                s_item[wid][pos++] = (unsigned short)((lane << 4) | bit);
            }
            __syncwarp();
            // 2. the warp evaluates the queued pairs, 32 at a time
            for (int g = lane; g < total; g += 32) {
                const unsigned item = s_item[wid][g];
                const int src = item >> 4, a = (item >> 2) & 3, b = item & 3;
                const int B = s_nbB[wid][src];
                const f3 dAB = mk(s_nbd[wid][src][0], s_nbd[wid][src][1], s_nbd[wid][src][2]);
                const float* sa = s_site[wid][a];
                const f3 offa = mk(sa[0], sa[1], sa[2]), mua = mk(sa[3], sa[4], sa[5]);
                const float qa = sa[6], da = sa[7];
                const int jb = K * B + b;
                const f3 offb = ld3(off, jb), mub = ld3(mu, jb);
                const float qb = q[jb], db = damp[jb];
                const f3 d = site_delta(dAB, offb, offa);  // r_b - r_a  (A = i, B = j)
                const float r2 = dot(d, d);
                const float r = sqrtf(r2);
                const float rr1 = 1.f / r, rr3 = rr1 / r2, rr5 = 3.f * rr3 / r2, rr7 = 5.f * rr5 / r2;
                const float dprod = da * db;
                const float sci3 = dot(mua, d), sci4 = dot(mub, d), mumu = dot(mua, mub);
                const float gl0 = qa * qb;
                const float gli = qb * sci3 - qa * sci4;
                const Thole tCC = thole(r, dprod, gcc), tCD = thole(r, dprod, gcd), tDD = thole(r, dprod, gdd);
                f3 fo;
                float pa = 0.f;  // potential at site a from site b (charge-derivative forces)
                if (PME) {
                    const Bn bn = ewald_bn(r, r2);
                    const float s1CC = gl0 != 0.f || qb != 0.f ? s1_of(tCC, gcc) : 1.f;
                    const float s3CD = s3_of(tCD);
                    {
                        // bn0 and bn1 are FP32 (~1e-7), which bounds each term; the
                        // terms are formed in FP32 and summed in double-float
                        const float pe = 0.5f * (bn.b0 * gl0 + 0.5f * bn.b1 * gli -
                                                 rr1 * gl0 * (1.f - s1CC) - 0.5f * rr3 * gli * (1.f - s3CD));
                        dfe_acc(el, pe, 0.f);
                    }
                    pa = qb * (bn.b0 - rr1 * (1.f - s1CC)) - sci4 * (bn.b1 - rr3 * (1.f - s3CD));
                    const float s3CC = s3_of(tCC), s5CD = s5_of(tCD);
                    const float s5DD = s5_of(tDD), s7DD = s7_of(tDD, gdd);
                    const float gf1 = bn.b1 * gl0, gfr1 = (1.f - s3CC) * rr3 * gl0;
                    const float gfi1 = bn.b2 * (gli + mumu) - bn.b3 * sci3 * sci4;
                    const float gfri1 = rr5 * (gli * (1.f - s5CD) + mumu * (1.f - s5DD)) -
                                        rr7 * sci3 * sci4 * (1.f - s7DD);
                    const float c_d = gf1 - gfr1 + gfi1 - gfri1;
                    const float c_i = -qb * bn.b1 - (-qb) * rr3 * (1.f - s3CD);  // mu_i coefficient
                    const float c_j = qa * bn.b1 - qa * rr3 * (1.f - s3CD);
                    const float c_dd = bn.b2 - rr5 * (1.f - s5DD);
                    fo = d * c_d + mua * (c_i + sci4 * c_dd) + mub * (c_j + sci3 * c_dd);
                } else {
                    const float s1CC = s1_of(tCC, gcc), s3CD = s3_of(tCD);
                    {
                        // no cutoff: the charge-charge and charge-dipole terms of a
                        // pair of neutral waters cancel to ~1e-3 of their size, so
                        // 1/r, the products and the dot products are double-float
                        const DFe r1 = dfe_rinv(d);
                        const DFe r3 = dfe_mul(dfe_mul(r1, r1), r1);
                        const DFe cc = dfe_mulf(dfe_mul(dfe_prod(qa, qb), r1), 0.5f * s1CC);
                        DFe glid = dfe_mulf(dfe_dot(mua, d), qb);
                        const DFe t2 = dfe_mulf(dfe_dot(mub, d), -qa);
                        dfe_acc(glid, t2.h, t2.l);
                        const DFe cd = dfe_mulf(dfe_mul(glid, r3), 0.25f * s3CD);
                        dfe_acc(el, cc.h, cc.l);
                        dfe_acc(el, cd.h, cd.l);
                    }
                    const float s3CC = s3_of(tCC), s5CD = s5_of(tCD);
                    const float s5DD = s5_of(tDD), s7DD = s7_of(tDD, gdd);
                    const float gf0 = rr3 * gl0 * s3CC;
                    const float gfi0 = rr5 * gli * s5CD + rr5 * mumu * s5DD - rr7 * sci3 * sci4 * s7DD;
                    fo = d * (gf0 + gfi0) + (mua * sci4 + mub * sci3) * (rr5 * s5DD) +
                         (mub * qa - mua * qb) * (rr3 * s3CD);
                    if (redist) {
                        // potential at A's site from B's site, TCC scaling for both
                        // terms (reference :808-827)
                        const float sc3 = s3_of(tCC);
                        const float sc1 = s1_of(tCC, gcc);
                        pa = qb * sc1 * rr1 - sc3 * sci4 * rr3;
                    }
                }
                // force on site a of A: -force(i, j)
                #pragma unroll
                for (int k = 0; k < kMaxK; ++k)
                    if (k == a) {
                        F[k][0] -= fo.x;
                        F[k][1] -= fo.y;
                        F[k][2] -= fo.z;
                        P[k] += pa;
                    }
            }
            __syncwarp();
        }
        double e = (double)el.h + (double)el.l;
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
        #pragma unroll
        for (int a = 0; a < kMaxK; ++a) {
            F[a][0] = warp_sum(F[a][0]);
            F[a][1] = warp_sum(F[a][1]);
            F[a][2] = warp_sum(F[a][2]);
            P[a] = warp_sum(P[a]);
        }
        if (lane == 0) {
            f3 offA[kMaxK], muA[kMaxK];
            float qA[kMaxK], dA[kMaxK];
            int tA[kMaxK];
            #pragma unroll
            for (int a = 0; a < kMaxK; ++a) {
                if (a < K) {
                    const int i = K * A + a;
                    offA[a] = ld3(off, i);
                    muA[a] = ld3(mu, i);
                    qA[a] = q[i];
                    dA[a] = damp[i];
                    tA[a] = type[i];
                }
            }
            // intramolecular pairs, a < b (both sites are A's)
            #pragma unroll
            for (int a = 0; a < kMaxK; ++a)
                #pragma unroll
                for (int b = a + 1; b < kMaxK; ++b) {
                    if (b >= K) continue;
                    const f3 d = offA[b] - offA[a];
                    const float r2 = dot(d, d);
                    if (PME && r2 > c_el.rc2) continue;
                    const float r = sqrtf(r2);
                    const float rr1 = 1.f / r, rr3 = rr1 / r2, rr5 = 3.f * rr3 / r2, rr7 = 5.f * rr5 / r2;
                    const float sci3 = dot(muA[a], d), sci4 = dot(muA[b], d), mumu = dot(muA[a], muA[b]);
                    const float gdd2 = tdd_gamma(true, tA[a], tA[b]);
                    const Thole tDD = thole(r, dA[a] * dA[b], gdd2);
                    const float s5DD = s5_of(tDD), s7DD = s7_of(tDD, gdd2);
                    f3 fo;
                    if (PME) {
                        // same water: s1CC = s3CD = s3CC = s5CD = 0, so every
                        // term is bn_k - rr_k = -E_k, or bn_k - (1 - s) rr_k
                        // = s rr_k - E_k for the dipole-dipole ones
                        const Bn ek = ewald_erf_part(r);
                        const float gl0 = qA[a] * qA[b];
                        const float gli = qA[b] * sci3 - qA[a] * sci4;
                        e -= (double)ek.b0 * gl0 + 0.5 * (double)ek.b1 * gli;
                        P[a] += sci4 * ek.b1 - qA[b] * ek.b0;
                        P[b] -= qA[a] * ek.b0 + sci3 * ek.b1;
                        const float c_dd = s5DD * rr5 - ek.b2;
                        const float c_d = -ek.b1 * gl0 - ek.b2 * gli + c_dd * mumu - (s7DD * rr7 - ek.b3) * sci3 * sci4;
                        const float c_i = qA[b] * ek.b1;
                        const float c_j = -qA[a] * ek.b1;
                        fo = d * c_d + muA[a] * (c_i + sci4 * c_dd) + muA[b] * (c_j + sci3 * c_dd);
                    } else {
                        // same water: no charge-charge or charge-dipole terms
                        const float gfi0 = rr5 * mumu * s5DD - rr7 * sci3 * sci4 * s7DD;
                        fo = d * gfi0 + (muA[a] * sci4 + muA[b] * sci3) * (rr5 * s5DD);
                    }
                    F[a][0] -= fo.x;
                    F[a][1] -= fo.y;
                    F[a][2] -= fo.z;
                    F[b][0] += fo.x;
                    F[b][1] += fo.y;
                    F[b][2] += fo.z;
                }
            // reciprocal space and self (reference :2113-2265, :2472-2508)
            if (PME) {
                const float sx = c_el.scale[0], sy = c_el.scale[1], sz = c_el.scale[2];
                const float sc[3] = {sx, sy, sz};
                const float ak = c_el.alpha;
                #pragma unroll
                for (int a = 0; a < kMaxK; ++a) {
                    if (a >= K) continue;
                    const int i = K * A + a;
                    const float* pf = phi_fix + 10 * i;
                    const float* pm = phi_mu + 10 * i;
                    // energies: fixed 0.5 q phi, induced 0.5 mu . grad phi_fixed, self -q^2 alpha/sqrt(pi)
                    e += 0.5 * (double)qA[a] * pf[0];
                    e += 0.5 * ((double)sx * muA[a].x * pf[1] + (double)sy * muA[a].y * pf[2] +
                                (double)sz * muA[a].z * pf[3]);
                    e += -(double)qA[a] * qA[a] * ak / kSqrtPi;
                    P[a] += pf[0] + pm[0] - 2.f * qA[a] * ak / kSqrtPiF;
                    // hessian index of (a, k): xx 4, yy 5, zz 6, xy 7, xz 8, yz 9
                    const int H[3][3] = {{4, 7, 8}, {7, 5, 9}, {8, 9, 6}};
                    const float m3[3] = {muA[a].x, muA[a].y, muA[a].z};
                    #pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        float fdip = 0.f;
                        #pragma unroll
                        for (int k = 0; k < 3; ++k) fdip += sc[k] * m3[k] * (pf[H[c][k]] + pm[H[c][k]]);
                        const float fc = sc[c] * (fdip + qA[a] * (pf[1 + c] + pm[1 + c]));
                        F[a][c] -= fc;
                    }
                }
            }
            // charge-derivative forces: F_i -= sum_s dq_i[s] * phi(other site s)
            // (reference :2767-2773 for PME, :791-827 for NoCutoff)
            if (redist && K == 4) {
                #pragma unroll
                for (int a = 0; a < kMaxK; ++a) {
                    const int i = K * A + a;
                    #pragma unroll
                    for (int s = 0; s < 3; ++s) {
                        const float phis = P[s + 1];
                        F[a][0] -= dq[9 * i + 3 * s] * phis;
                        F[a][1] -= dq[9 * i + 3 * s + 1] * phis;
                        F[a][2] -= dq[9 * i + 3 * s + 2] * phis;
                    }
                }
            }
            // atomics: the polynomial, one-body and dispersion kernels add to
            // the same force array from other streams at the same time
            #pragma unroll
            for (int a = 0; a < kMaxK; ++a) {
                if (a >= K) continue;
                add_force(force, K * A + a, (double)F[a][0] * f, (double)F[a][1] * f, (double)F[a][2] * f);
            }
            e_out = e * kElectric;
            cluster_energy(cs, A, e_out);
        }
    }
    block_sum_atomic<128>(e_out, energy);
}

// Starting dipoles from the history of solves (guess 2 and 3): the
// polynomial extrapolation through the last L converged solves r_1 (newest)
// .. r_L, mu = sum_k (-1)^(k+1) C(L, k) r_k (r1; 2 r1 - r2; 3 r1 - 3 r2 + r3;
// ...).  FP64 state and its FP32 copy.  L = 4 gave the fewest solver
// iterations on the 4096-water box at 0.2 fs (22.1 per step, against 26.9
// for L = 3, 23.4 for L = 5 and 25.3 for L = 6; least-squares cubic fits
// through 5-8 solves: 23.2-27.5).
constexpr int kHist = guess::kPredHistory;  // solves kept (the learned predictor's history)
constexpr int kExtrapolate = 4;             // largest L used
struct HistRing {
    const double* r[kHist];
    double c[kHist];
    int levels;
};
__global__ void extrapolated_guess_kernel(int n, const HistRing h, double* __restrict__ mu_d,
                                          float* __restrict__ mu_f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double v = 0.0;
    #pragma unroll
    for (int k = 0; k < kHist; ++k)
        if (k < h.levels) v += h.c[k] * h.r[k][i];
    mu_d[i] = v;
    mu_f[i] = (float)v;
}

// Network start: mu = mu_prev + (m - m_prev) after one solve with a
// prediction, else mu = m; FP64 state and its FP32 copy.
__global__ void learned_guess_kernel(int n, const float* __restrict__ m, const float* __restrict__ m_prev,
                                     const double* __restrict__ mu_prev, double* __restrict__ mu_d,
                                     float* __restrict__ mu_f) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double v = mu_prev ? mu_prev[i] + ((double)m[i] - (double)m_prev[i]) : (double)m[i];
    mu_d[i] = v;
    mu_f[i] = (float)v;
}


__global__ void narrow_kernel(int n, const double* __restrict__ a, float* __restrict__ b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

__global__ void widen_kernel(int n, const float* __restrict__ a, double* __restrict__ b) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) b[i] = a[i];
}

// B-spline moduli with the reference's fixes (:1248-1340), host FP64.
void bspline_moduli(int size, std::vector<double>& mod) {
    const int order = 5;
    double arr[order];
    const double x = 0.0;
    arr[0] = 1.0 - x;
    arr[1] = x;
    for (int k = 2; k < order; ++k) {
        const double dn = 1.0 / k;
        arr[k] = x * arr[k - 1] * dn;
        for (int i = 1; i < k; ++i) arr[k - i] = ((x + i) * arr[k - i - 1] + ((k - i + 1) - x) * arr[k - i]) * dn;
        arr[0] = (1.0 - x) * arr[0] * dn;
    }
    std::vector<double> bs((size_t)size + 1 + order + 2, 0.0);
    for (int i = 2; i <= order + 1; ++i) bs[(size_t)i] = arr[i - 2];
    mod.assign((size_t)size, 0.0);
    const double factor = 2.0 * M_PI / size;
    for (int i = 0; i < size; ++i) {
        double s1 = 0, s2 = 0;
        for (int j = 1; j <= size; ++j) {
            const double arg = factor * i * (j - 1);
            const double bj = j < (int)bs.size() ? bs[(size_t)j] : 0.0;
            s1 += bj * cos(arg);
            s2 += bj * sin(arg);
        }
        mod[(size_t)i] = s1 * s1 + s2 * s2;
    }
    const double eps = 1.0e-7;
    if (mod[0] < eps) mod[0] = 0.5 * mod[1];
    for (int i = 1; i < size - 1; ++i)
        if (mod[(size_t)i] < eps) mod[(size_t)i] = 0.5 * (mod[(size_t)i - 1] + mod[(size_t)i + 1]);
    if (mod[(size_t)size - 1] < eps) mod[(size_t)size - 1] = 0.5 * mod[(size_t)size - 2];
    const int jcut = 50;
    for (int i = 1; i <= size; ++i) {
        int k = i - 1;
        if (i > size / 2) k = k - size;
        double zeta;
        if (k == 0) {
            zeta = 1.0;
        } else {
            double s1 = 1.0, s2 = 1.0;
            const double fac = M_PI * k / size;
            for (int j = 1; j <= jcut; ++j) {
                const double arg = fac / (fac + M_PI * j);
                s1 += pow(arg, order);
                s2 += pow(arg, 2 * order);
            }
            for (int j = 1; j <= jcut; ++j) {
                const double arg = fac / (fac - M_PI * j);
                s1 += pow(arg, order);
                s2 += pow(arg, 2 * order);
            }
            zeta = s2 / s1;
        }
        mod[(size_t)i - 1] *= zeta * zeta;
    }
}

// Dipole-moment-surface fit of the charge redistribution
// (MBPolReferenceElectrostaticsForce.cpp:2823-2870): index triples and coefficients.
const unsigned char kDmsIdx[3][84] = {
    {1, 1, 1, 2, 1, 1, 1, 2, 2, 3, 1, 1, 1, 1, 2, 2, 2, 3, 3, 4, 1, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 4, 4, 5, 1, 1, 1,
     1, 1, 1, 2, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 5, 5, 6, 1, 1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2, 3, 3, 3, 3, 3, 4, 4,
     4, 4, 5, 5, 5, 6, 6, 7},
    {1, 1, 2, 1, 1, 2, 3, 1, 2, 1, 1, 2, 3, 4, 1, 2, 3, 1, 2, 1, 1, 2, 3, 4, 5, 1, 2, 3, 4, 1, 2, 3, 1, 2, 1, 1, 2, 3,
     4, 5, 6, 1, 2, 3, 4, 5, 1, 2, 3, 4, 1, 2, 3, 1, 2, 1, 1, 2, 3, 4, 5, 6, 7, 1, 2, 3, 4, 5, 6, 1, 2, 3, 4, 5, 1, 2,
     3, 4, 1, 2, 3, 1, 2, 1},
    {1, 2, 1, 1, 3, 2, 1, 2, 1, 1, 4, 3, 2, 1, 3, 2, 1, 2, 1, 1, 5, 4, 3, 2, 1, 4, 3, 2, 1, 3, 2, 1, 2, 1, 1, 6, 5, 4,
     3, 2, 1, 5, 4, 3, 2, 1, 4, 3, 2, 1, 3, 2, 1, 2, 1, 1, 7, 6, 5, 4, 3, 2, 1, 6, 5, 4, 3, 2, 1, 5, 4, 3, 2, 1, 4, 3,
     2, 1, 3, 2, 1, 2, 1, 1}};
const double kDmsCoef[84] = {
    -2.1689686086730e-03, 1.4910379754728e-02, 5.3546078430060e-02, -7.4055995388666e-02, -3.7764333017616e-03,
    1.4089887256484e-01,  -6.2584207687264e-02, -1.1260393113022e-01, -5.7824159269319e-02, 1.4360743650655e-02,
    -1.5469680141070e-02, -1.3036350092795e-02, 2.7515837781556e-02, 1.4098478875076e-01, -2.7663168397781e-02,
    -5.2378176254797e-03, -1.0237198381792e-02, 8.9571999265473e-02, 7.2920263098603e-03, -2.6873260551686e-01,
    2.0220870325864e-02,  -7.0764766270927e-02, 1.2140640273760e-01, 2.0978491966341e-02, -1.9443840512668e-01,
    4.0826835370618e-02,  -4.5365190474650e-02, 6.2779900072132e-02, -1.3194351021000e-01, -1.4673032718563e-01,
    1.1894031277247e-01,  -6.4952851564679e-03, 8.8503610374493e-02, 1.4899437409291e-01, 1.3962841511565e-01,
    -2.6459446720450e-02, -5.0128914532773e-02, 1.8329676428116e-01, -1.5559089125095e-01, -4.0176879767592e-02,
    3.6192059996636e-01,  1.0202887240343e-01, 1.9318668580051e-01, -4.3435977107932e-01, -4.2080828803311e-02,
    1.9144626027273e-01,  -1.7851138969948e-01, 1.0524533875070e-01, -1.7954071602185e-02, 5.2022455612120e-02,
    -2.8891891146828e-01, -4.7452036576319e-02, -1.0939400546289e-01, 3.5916564473568e-01, -2.0162789820172e-01,
    -3.5838629543696e-01, 5.6706523551202e-03, 1.3849337488211e-01, -4.1733982195604e-01, 4.1641570764241e-01,
    -1.2243429796296e-01, 4.7141730971228e-02, -1.8224510249551e-01, -1.8880981556620e-01, -3.1992359561800e-01,
    -1.8567550546587e-01, 6.1850530431280e-01, -6.1142756235141e-02, -1.6996135584933e-01, 5.4252879499871e-01,
    6.6128603899427e-01,  1.2107016404639e-02, -1.9633639729189e-01, 2.7652059420824e-03, -2.2684111109778e-01,
    -4.7924491598635e-01, 2.4287790137314e-01, -1.4296023329441e-01, 8.9664665907006e-02, -1.4003228575602e-01,
    -1.3321543452254e-01, -1.8340983193745e-01, 2.3426707273520e-01, 1.5141050914514e-01};

template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    ~DBuf() {
        if (p) cudaFree(p);
    }
    cudaError_t ensure(size_t m) {
        if (m <= n) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
        cudaError_t e = cudaMalloc(&p, sizeof(T) * (m ? m : 1));
        if (e == cudaSuccess) n = m;
        return e;
    }
};

// Convergence control of the batched-cluster solver on the device: after
// each iteration, for every cluster still running, the host loop's rules of
// the single-system solver (reference convergeInduceDipoles :557-616):
// cstate 1 -> 2 after the anchoring iteration; epsilon from the cluster's
// own sum of squared changes and site count; stop on convergence, on an
// increase or at the iteration limit; then the anchoring switch for the
// next iteration.  One block; it sets the condition of the graph's while
// loop (more clusters to run, and a bound on the loop's length).
constexpr int kCtlThreads = 1024;
__global__ void __launch_bounds__(kCtlThreads) cluster_control_kernel(
    int ncl, const double* __restrict__ eps2c, const int* __restrict__ nsites, double* __restrict__ cur,
    int* __restrict__ its, int* __restrict__ cstate, int* __restrict__ cconv, double target, int max_it,
    double switch_eps, int* __restrict__ rounds, cudaGraphConditionalHandle loop) {
    __shared__ int s_active[kCtlThreads / 32];
    int active = 0;
    for (int c = threadIdx.x; c < ncl; c += kCtlThreads) {
        int st = cstate[c];
        if (st >= 3) continue;
        if (st == 1) st = 2;
        const double ec = kSOR * kDebye * sqrt(eps2c[c] / (double)nsites[c]);
        bool stop = false;
        if (!isfinite(ec)) {
            stop = true;
        } else if (ec < target) {
            cconv[c] = 1;
            stop = true;
        } else if (cur[c] < ec || its[c] >= max_it) {
            stop = true;
        }
        cur[c] = ec;
        its[c] += 1;
        if (stop) st = 3;
        else if (st == 0 && ec < switch_eps) st = 1;
        cstate[c] = st;
        if (st < 3) ++active;
    }
    active = __reduce_add_sync(0xffffffffu, active);
    if ((threadIdx.x & 31) == 0) s_active[threadIdx.x >> 5] = active;
    __syncthreads();
    if (threadIdx.x == 0) {
        int total = 0;
        for (int w = 0; w < kCtlThreads / 32; ++w) total += s_active[w];
        const int r = ++(*rounds);
        cudaGraphSetConditional(loop, (total > 0 && r <= max_it + 2) ? 1u : 0u);
    }
}

// FP64 site charges for the electrostatic potential: the charges of
// elec_prepare_kernel (redistribution from the raw positions, as the
// reference) kept in FP64.
__global__ void site_charges_kernel(int nmol, const double* __restrict__ pos, int redist,
                                    const double* __restrict__ q_static, double* __restrict__ qd) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= nmol) return;
    const int K = c_el.K, s0 = K * m;
    if (redist) {
        double qq[4], dd[4][3][3];
        water_charges(load_pos(pos, s0), load_pos(pos, s0 + 1), load_pos(pos, s0 + 2), qq, dd);
        for (int s = 0; s < 4; ++s) qd[s0 + s] = qq[s];
    } else {
        for (int s = 0; s < K; ++s) qd[s0 + s] = q_static[s0 + s];
    }
}

// Electrostatic potential at probe points (reference
// calculateElectrostaticPotential, MBPolReferenceElectrostaticsForce.cpp:
// 1023-1085): phi(g) = 138.9354558456 * sum_i [q_i / r - mu_i . d / r^3] with
// d = r_i - g, minimum-imaged under PME (getPeriodicDelta, :1234-1239), over
// every site, unscreened.  One thread per point, the sites staged through
// shared memory in tiles; FP64 throughout (an analysis call, not part of a
// step).
constexpr int kPotTile = 128;
__global__ void __launch_bounds__(kPotTile) potential_kernel(int n, const double* __restrict__ pos,
                                                             const double* __restrict__ qd,
                                                             const double* __restrict__ mud, int npts,
                                                             const double* __restrict__ pts,
                                                             double* __restrict__ out) {
    __shared__ double sr[3][kPotTile], sq[kPotTile], sm[3][kPotTile];
    const int t = threadIdx.x;
    const int p = blockIdx.x * kPotTile + t;
    const bool live = p < npts;
    double g[3] = {0.0, 0.0, 0.0};
    if (live)
        for (int k = 0; k < 3; ++k) g[k] = pts[3 * (size_t)p + k];
    double acc = 0.0;
    for (int base = 0; base < n; base += kPotTile) {
        const int i = base + t;
        __syncthreads();
        if (i < n) {
            for (int k = 0; k < 3; ++k) {
                sr[k][t] = pos[3 * (size_t)i + k];
                sm[k][t] = mud[3 * (size_t)i + k];
            }
            sq[t] = qd[i];
        }
        __syncthreads();
        const int cnt = min(kPotTile, n - base);
        if (!live) continue;
        for (int j = 0; j < cnt; ++j) {
            double d[3];
            for (int k = 0; k < 3; ++k) {
                d[k] = sr[k][j] - g[k];
                if (c_el.periodic) d[k] -= floor(d[k] * c_el.inv[k] + 0.5) * c_el.box[k];
            }
            const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            const double rinv = 1.0 / sqrt(r2);
            acc += sq[j] * rinv - (sm[0][j] * d[0] + sm[1][j] * d[1] + sm[2][j] * d[2]) * (rinv * rinv * rinv);
        }
    }
    if (live) out[p] = acc * kElectric;
}

// System multipole moments (reference
// calculateMBPolSystemElectrostaticsMoments,
// MBPolReferenceElectrostaticsForce.cpp:923-1021): net charge, dipole and
// traceless quadrupole of the site charges and converged induced dipoles
// about the centre of mass, positions as stored (not wrapped).  Two passes
// of FP64 sums over sites (centre of mass, then the moments), each summed
// per block in a fixed order and then over blocks by one thread, so the
// result is the same from run to run.
constexpr int kMomBlocks = 64, kMomThreads = 256;

template <int NS>
__device__ __forceinline__ void moment_block_sums(double (&v)[NS], double* __restrict__ out) {
    __shared__ double red[kMomThreads / 32][NS];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    #pragma unroll
    for (int k = 0; k < NS; ++k) {
        double x = v[k];
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if (lane == 0) red[warp][k] = x;
    }
    __syncthreads();
    if (threadIdx.x < NS) {
        double x = 0.0;
        for (int w = 0; w < kMomThreads / 32; ++w) x += red[w][threadIdx.x];
        out[threadIdx.x] = x;
    }
}

__global__ void __launch_bounds__(kMomThreads) moments_com_kernel(int n, const double* __restrict__ pos,
                                                                  const double* __restrict__ mass,
                                                                  double* __restrict__ part) {
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    for (int i = blockIdx.x * kMomThreads + threadIdx.x; i < n; i += kMomBlocks * kMomThreads) {
        const double m = mass[i];
        v[0] += m;
        #pragma unroll
        for (int k = 0; k < 3; ++k) v[1 + k] += pos[3 * (size_t)i + k] * m;
    }
    moment_block_sums<4>(v, part + 4 * blockIdx.x);
}

__global__ void __launch_bounds__(kMomThreads) moments_kernel(int n, const double* __restrict__ pos,
                                                              const double* __restrict__ qd,
                                                              const double* __restrict__ mud,
                                                              const double* __restrict__ pcom,
                                                              double* __restrict__ part) {
    __shared__ double com[3];
    if (threadIdx.x == 0) {
        double mt = 0.0, c[3] = {0.0, 0.0, 0.0};
        for (int b = 0; b < kMomBlocks; ++b) {
            mt += pcom[4 * b];
            for (int k = 0; k < 3; ++k) c[k] += pcom[4 * b + 1 + k];
        }
        for (int k = 0; k < 3; ++k) com[k] = mt > 0.0 ? c[k] * (1.0 / mt) : 0.0;
    }
    __syncthreads();
    // q, dipole x y z, Q xx xy xz yy yz zz
    double v[10];
    #pragma unroll
    for (int k = 0; k < 10; ++k) v[k] = 0.0;
    for (int i = blockIdx.x * kMomThreads + threadIdx.x; i < n; i += kMomBlocks * kMomThreads) {
        double r[3], mu[3];
        #pragma unroll
        for (int k = 0; k < 3; ++k) {
            r[k] = pos[3 * (size_t)i + k] - com[k];
            mu[k] = mud[3 * (size_t)i + k];
        }
        const double q = qd[i];
        v[0] += q;
        #pragma unroll
        for (int k = 0; k < 3; ++k) v[1 + k] += r[k] * q + mu[k];
        v[4] += r[0] * r[0] * q + 2.0 * r[0] * mu[0];
        v[5] += r[0] * r[1] * q + r[0] * mu[1] + r[1] * mu[0];
        v[6] += r[0] * r[2] * q + r[0] * mu[2] + r[2] * mu[0];
        v[7] += r[1] * r[1] * q + 2.0 * r[1] * mu[1];
        v[8] += r[1] * r[2] * q + r[1] * mu[2] + r[2] * mu[1];
        v[9] += r[2] * r[2] * q + 2.0 * r[2] * mu[2];
    }
    moment_block_sums<10>(v, part + 10 * blockIdx.x);
}

// out: charge (e), dipole (Debye), traceless quadrupole row by row (the
// reference's units: e nm x 10 x 4.80321, e nm^2 x 100 x 3 x 4.80321)
__global__ void moments_final_kernel(const double* __restrict__ part, double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double v[10];
    for (int k = 0; k < 10; ++k) v[k] = 0.0;
    for (int b = 0; b < kMomBlocks; ++b)
        for (int k = 0; k < 10; ++k) v[k] += part[10 * b + k];
    const double debye = 4.80321, tr = (v[4] + v[7] + v[9]) / 3.0, qs = 0.5 * 100.0 * 3.0 * debye;
    out[0] = v[0];
    for (int k = 0; k < 3; ++k) out[1 + k] = v[1 + k] * 10.0 * debye;
    out[4] = (v[4] - tr) * qs;
    out[5] = v[5] * qs;
    out[6] = v[6] * qs;
    out[7] = v[5] * qs;
    out[8] = (v[7] - tr) * qs;
    out[9] = v[8] * qs;
    out[10] = v[6] * qs;
    out[11] = v[8] * qs;
    out[12] = (v[9] - tr) * qs;
}

}  // namespace

struct ElecImpl {
    int N = 0, K = 4, nmol = 0;
    mbpol_electrostatics_params prm{};
    bool pme = false;
    std::vector<float> q_static, damp, pol;
    std::vector<double> q_static64;  // the caller's charges, for the potential
    DBuf<double> d_qs64, d_qd, d_pts, d_pot, d_mass, d_mom;
    std::vector<int> type;
    DBuf<float> d_qs, d_damp, d_pol, d_off, d_q, d_dq, d_E0, d_mu0, d_mu1, d_mu2, d_mu_prev, d_phi_fix, d_phi_mu, d_nbd,
        d_gfrac, d_reach, d_ebase, d_intra, d_pcoef, d_edir;
    DBuf<int> d_type, d_nb, d_nnb, d_gidx, d_flags, d_polmask;  // polmask: polarisable sites of a molecule, bit s
    DBuf<float4> d_opos;
    DBuf<double> d_eps2, d_mud, d_mud_prev;
    int cap = 0;
    // PME
    int grid[3] = {0, 0, 0};
    double alpha = 0.0;
    DBuf<float> d_grid, d_gridfix, d_bx, d_by, d_bz, d_eterm;
    double eterm_key[4] = {0, 0, 0, 0};  // box and alpha of d_eterm
    DBuf<unsigned long long> d_gridq;
    DBuf<cufftComplex> d_cgrid;
    cufftHandle plan_f = 0, plan_b = 0;
    bool plans = false;
    double box_used[3] = {0, 0, 0};
    // state
    bool converged = true;
    int iterations = 0;
    double epsilon = 0.0;
    bool have_prev = false;
    // learned guess (guess = 2): the cold-start network and the correction
    // network applied on top of the history predictor; `sel` picks the one
    // the mbpol_guess_* calls act on
    GuessNet net;
    GuessNet cnet{1};
    int sel = 0;
    DBuf<float> d_dF, d_mcorr;  // unpredicted field change, correction (lab frame)
    DBuf<double> d_mubase;      // the predictor's dipoles of the last solve
    bool cdesc_valid = false;   // cnet's inputs belong to the last solve
    DBuf<float> d_mguess;
    DBuf<float> d_mprev;  // the network's prediction at the previous solve
    bool have_mprev = false;
    // dipoles of the last (up to) kHist converged solves, a ring of 3n
    // planes (FP64)
    DBuf<double> d_hist;
    DBuf<double> d_pred;  // the predictor's partial sums, then its coefficients
    DBuf<double> d_fhist, d_fnow;  // alpha E0 of the solves in d_hist, and of the current geometry
    int hist_levels = 0, hist_head = 0;
    bool evaluated = false;  // neighbour list, offsets and dipoles are current
    // batched independent clusters (NoCutoff): molecule -> cluster, per-
    // cluster solver state and energy sink
    int ncl = 0, max_cl_mol = 0;
    std::vector<int> cl_nsites, cl_iters;
    std::vector<char> cl_conv;
    DBuf<int> d_mcl, d_cstate;  // d_cstate: per-cluster solver stage (0 plain, 1 anchoring, 2 anchored, 3 done)
    // neighbour candidates: molecules of each cluster (batched clusters), and
    // the cell-binning scratch of periodic boxes
    DBuf<int> d_cl_members, d_cl_start, d_cells;
    CandidateSet cl_candidates;
    bool cells_ok = true;
    DBuf<double> d_eps2c;
    // the batched solver as one graph launch: a while node whose body runs
    // two iterations (ping-pong buffers), each followed by the control kernel
    DBuf<int> d_cl_nsites, d_cl_its, d_cl_conv, d_rounds;
    DBuf<double> d_cl_cur;
    cudaStream_t st_cap = nullptr;
    // one system's PME solve as one graph launch (solver_graph): a while
    // node around one iteration (the PME pass on a forked branch beside the
    // direct field, the update in place, the control kernel)
    cudaStream_t st_cap2 = nullptr;
    cudaEvent_t ev_cfork = nullptr, ev_cjoin = nullptr;
    cudaGraph_t sv_graph = nullptr;
    cudaGraphExec_t sv_exec = nullptr;
    std::vector<uintptr_t> sv_key;
    DBuf<SolveState> d_sstate;
    bool sv_disabled = false;  // the graph could not be built here: host loop
    cudaGraph_t cl_graph = nullptr;
    cudaGraphExec_t cl_exec = nullptr;
    std::vector<uintptr_t> cl_graph_key;
    ClusterSink cl_sink;
    Box last_box{};
    int mu_cur = 0;  // which buffer holds the current dipoles
    // second stream for the solver's PME passes, ordered by two events
    cudaStream_t st2 = nullptr;
    cudaEvent_t ev_in = nullptr, ev_pme = nullptr;
    // the learned predictor is fitted on the second stream right after a
    // solve enters the history (beside the energy/force kernel); the next
    // evaluation waits for ev_fit before it applies the coefficients
    cudaEvent_t ev_hist = nullptr, ev_fit = nullptr;
    bool pred_fitted = false;

    // polarisable site pairs within the cutoff, counted in both directions by
    // the fixed-field kernel
    DBuf<unsigned long long> d_npair;
    unsigned long long* h_npair = nullptr;

    ~ElecImpl() {
        if (sv_exec) cudaGraphExecDestroy(sv_exec);
        if (sv_graph) cudaGraphDestroy(sv_graph);
        if (st_cap2) cudaStreamDestroy(st_cap2);
        if (ev_cfork) cudaEventDestroy(ev_cfork);
        if (ev_cjoin) cudaEventDestroy(ev_cjoin);
        if (cl_exec) cudaGraphExecDestroy(cl_exec);
        if (cl_graph) cudaGraphDestroy(cl_graph);
        if (st_cap) cudaStreamDestroy(st_cap);
        if (h_npair) cudaFreeHost(h_npair);
        if (plans) {
            cufftDestroy(plan_f);
            cufftDestroy(plan_b);
        }
        if (ev_in) cudaEventDestroy(ev_in);
        if (ev_hist) cudaEventDestroy(ev_hist);
        if (ev_fit) cudaEventDestroy(ev_fit);
        if (ev_pme) cudaEventDestroy(ev_pme);
        if (st2) cudaStreamDestroy(st2);
    }
};

ElecEngine::ElecEngine() : impl_(new ElecImpl()) {}
ElecEngine::~ElecEngine() { delete impl_; }

// Per-particle parameters (charges, types, damping, polarisabilities) to the
// device; the molecule layout (I.K, I.nmol) is set.
static mbpol_status upload_particle_params(ElecImpl& I, const double* charge, const int* atom_type,
                                           const double* damping, const double* polarity) {
    const int n = I.N;
    I.q_static.resize(n);
    I.q_static64.resize(n);
    I.damp.resize(n);
    I.pol.resize(n);
    I.type.resize(n);
    for (int i = 0; i < n; ++i) {
        I.q_static[i] = (float)charge[i];
        I.q_static64[i] = charge[i];
        // sixth root of the damping factor: pair kernels use
        // (damp_i damp_j)^(1/6) = damp_i^(1/6) damp_j^(1/6)
        I.damp[i] = (float)std::pow(damping[i], 1.0 / 6.0);
        I.pol[i] = (float)polarity[i];
        I.type[i] = atom_type[i];
    }
    MBPOL_CUDA_OK(I.d_qs.ensure(n));
    MBPOL_CUDA_OK(I.d_damp.ensure(n));
    MBPOL_CUDA_OK(I.d_pol.ensure(n));
    MBPOL_CUDA_OK(I.d_type.ensure(n));
    MBPOL_CUDA_OK(cudaMemcpy(I.d_qs.p, I.q_static.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    MBPOL_CUDA_OK(cudaMemcpy(I.d_damp.p, I.damp.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    MBPOL_CUDA_OK(cudaMemcpy(I.d_pol.p, I.pol.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
    MBPOL_CUDA_OK(cudaMemcpy(I.d_type.p, I.type.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
    {
        std::vector<int> mask(I.nmol, 0);
        for (int m = 0; m < I.nmol; ++m)
            for (int s = 0; s < I.K; ++s)
                if (I.pol[I.K * m + s] != 0.f) mask[m] |= 1 << s;
        MBPOL_CUDA_OK(I.d_polmask.ensure(I.nmol));
        MBPOL_CUDA_OK(cudaMemcpy(I.d_polmask.p, mask.data(), sizeof(int) * I.nmol, cudaMemcpyHostToDevice));
    }
    return MBPOL_OK;
}

// Molecules: consecutive blocks of K = 3 (O, H, H) or 4 (O, H, H, M) sites
// with a common molecule index, different from the previous block's.
static int molecule_layout(int n, const int* molecule) {
    int K = 1;
    while (K < n && molecule[K] == molecule[0]) ++K;
    if (K != 3 && K != 4) return 0;
    if (n % K) return 0;
    for (int i = 0; i < n; ++i)
        if (molecule[i] != molecule[(i / K) * K]) return 0;
    for (int m = 1; m < n / K; ++m)
        if (molecule[m * K] == molecule[(m - 1) * K]) return 0;
    return K;
}

// ---- white-box probes of the device functions above (one thread each),
// for the reference's white-box tests: getAndScaleInverseRs
// (platforms/reference/tests/TestReferenceMBPolElectrostaticsForce.cpp:80-131)
// and computeWaterCharge (:326-417)
namespace {
__global__ void probe_thole_kernel(float r, float d6prod, float gamma, double* out) {
    const Thole th = thole(r, d6prod, gamma);
    const float rI = 1.f / r, r2I = rI * rI;
    out[0] = (double)(s1_of(th, gamma) * rI);
    out[1] = (double)(s3_of(th) * rI * r2I);
    out[2] = (double)(s5_of(th) * 3.f * rI * r2I * r2I);
    out[3] = (double)(s7_of(th, gamma) * 15.f * rI * r2I * r2I * r2I);
}

__global__ void probe_water_charges_kernel(const double* pos, double* out) {
    double q[4], dq[4][3][3];
    water_charges(make_double3(pos[0], pos[1], pos[2]), make_double3(pos[3], pos[4], pos[5]),
                  make_double3(pos[6], pos[7], pos[8]), q, dq);
    for (int s = 0; s < 4; ++s) out[s] = q[s];
    for (int x = 0; x < 3; ++x)
        for (int o = 0; o < 3; ++o)
            for (int k = 0; k < 3; ++k) out[4 + 9 * x + 3 * o + k] = dq[x][o][k];
}
}  // namespace

mbpol_status probe_thole(double r, double damp_i, double damp_j, double gamma, double* rr) {
    DBuf<double> d;
    MBPOL_CUDA_OK(d.ensure(4));
    // the sites' sixth roots of the damping factors, as the field kernels store them
    const float d6 = (float)(std::pow(damp_i, 1.0 / 6.0)) * (float)(std::pow(damp_j, 1.0 / 6.0));
    probe_thole_kernel<<<1, 1>>>((float)r, d6, (float)gamma, d.p);
    MBPOL_CUDA_OK(cudaGetLastError());
    MBPOL_CUDA_OK(cudaMemcpy(rr, d.p, 4 * sizeof(double), cudaMemcpyDeviceToHost));
    return MBPOL_OK;
}

mbpol_status probe_water_charges(const double* pos9, double* out31) {
    DBuf<double> d;
    MBPOL_CUDA_OK(d.ensure(9 + 31));
    MBPOL_CUDA_OK(cudaMemcpyToSymbol(c_dms, kDmsCoef, sizeof(kDmsCoef)));
    MBPOL_CUDA_OK(cudaMemcpyToSymbol(c_dms_idx, kDmsIdx, sizeof(kDmsIdx)));
    MBPOL_CUDA_OK(cudaMemcpy(d.p, pos9, 9 * sizeof(double), cudaMemcpyHostToDevice));
    probe_water_charges_kernel<<<1, 1>>>(d.p, d.p + 9);
    MBPOL_CUDA_OK(cudaGetLastError());
    MBPOL_CUDA_OK(cudaMemcpy(out31, d.p + 9, 31 * sizeof(double), cudaMemcpyDeviceToHost));
    return MBPOL_OK;
}

mbpol_status ElecEngine::update_parameters(const double* charge, const int* molecule, const int* atom_type,
                                           const double* damping, const double* polarity) {
    ElecImpl& I = *impl_;
    if (molecule_layout(I.N, molecule) != I.K)
        return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "updateParametersInContext: the molecule layout has changed");
    if (I.prm.include_charge_redistribution)
        for (int m = 0; m < I.nmol; ++m)
            if (atom_type[4 * m] != 0 || atom_type[4 * m + 1] != 1 || atom_type[4 * m + 2] != 1 ||
                atom_type[4 * m + 3] != 2)
                return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT,
                                  "charge redistribution needs O, H1, H2, M order (types 0,1,1,2)");
    // the neighbour lists, the dipoles of the last solves and the history
    // predictor stay; the next evaluation recomputes every parameter-dependent
    // quantity
    return upload_particle_params(I, charge, atom_type, damping, polarity);
}

mbpol_status ElecEngine::init(int n, const mbpol_electrostatics_params& p, const double* charge, const int* molecule,
                              const int* atom_type, const double* damping, const double* polarity) {
    ElecImpl& I = *impl_;
    I.N = n;
    I.prm = p;
    I.pme = p.nonbonded_method == MBPOL_ELEC_PME;
    if (p.nonbonded_method != MBPOL_ELEC_PME && p.nonbonded_method != MBPOL_ELEC_NOCUTOFF)
        return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "unknown electrostatics nonbonded method");
    // molecules: consecutive blocks of K sites with a common molecule index
    int K = 1;
    while (K < n && molecule[K] == molecule[0]) ++K;
    if (K != 3 && K != 4)
        return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "electrostatics expects molecules of 3 (O,H,H) or 4 (O,H,H,M) consecutive sites");
    if (n % K) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "particle count is not a multiple of the molecule size");
    for (int i = 0; i < n; ++i) {
        if (molecule[i] != molecule[(i / K) * K])
            return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "molecule indices must be constant over consecutive blocks");
        if (i % K && molecule[i] == molecule[i - 1] && false) return MBPOL_ERR_INVALID_ARGUMENT;
    }
    for (int m = 1; m < n / K; ++m)
        if (molecule[m * K] == molecule[(m - 1) * K])
            return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "molecule sizes differ");
    if (p.include_charge_redistribution) {
        if (K != 4) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "charge redistribution needs O, H1, H2, M sites");
        for (int m = 0; m < n / 4; ++m)
            if (atom_type[4 * m] != 0 || atom_type[4 * m + 1] != 1 || atom_type[4 * m + 2] != 1 || atom_type[4 * m + 3] != 2)
                return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "charge redistribution needs O, H1, H2, M order (types 0,1,1,2)");
    }
    if (p.max_iterations < 0 || !(p.target_epsilon > 0))
        return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "bad solver parameters");
    I.K = K;
    I.nmol = n / K;
    {
        mbpol_status s = upload_particle_params(I, charge, atom_type, damping, polarity);
        if (s) return s;
    }
    for (auto* b : {&I.d_off, &I.d_E0, &I.d_mu0, &I.d_mu1, &I.d_mu2, &I.d_mu_prev, &I.d_gfrac, &I.d_ebase, &I.d_edir})
        MBPOL_CUDA_OK(b->ensure(3 * (size_t)n));
    MBPOL_CUDA_OK(I.d_q.ensure(n));
    MBPOL_CUDA_OK(I.d_dq.ensure(9 * (size_t)n));
    MBPOL_CUDA_OK(I.d_phi_fix.ensure(10 * (size_t)n));
    MBPOL_CUDA_OK(I.d_phi_mu.ensure(10 * (size_t)n));
    MBPOL_CUDA_OK(I.d_gidx.ensure(3 * (size_t)n));
    MBPOL_CUDA_OK(I.d_nnb.ensure(I.nmol));
    MBPOL_CUDA_OK(I.d_reach.ensure(I.nmol));
    MBPOL_CUDA_OK(I.d_opos.ensure(I.nmol));
    MBPOL_CUDA_OK(I.d_intra.ensure((size_t)2 * kMaxIntra * I.nmol));
    MBPOL_CUDA_OK(I.d_flags.ensure(4));
    MBPOL_CUDA_OK(I.d_eps2.ensure(1));
    MBPOL_CUDA_OK(I.d_mud.ensure(3 * (size_t)n));
    MBPOL_CUDA_OK(I.d_mud_prev.ensure(3 * (size_t)n));
    if (!I.st2) {
        MBPOL_CUDA_OK(cudaStreamCreateWithFlags(&I.st2, cudaStreamNonBlocking));
        MBPOL_CUDA_OK(cudaEventCreateWithFlags(&I.ev_in, cudaEventDisableTiming));
        MBPOL_CUDA_OK(cudaEventCreateWithFlags(&I.ev_pme, cudaEventDisableTiming));
        MBPOL_CUDA_OK(cudaEventCreateWithFlags(&I.ev_hist, cudaEventDisableTiming));
        MBPOL_CUDA_OK(cudaEventCreateWithFlags(&I.ev_fit, cudaEventDisableTiming));
    }
    MBPOL_CUDA_OK(I.d_mguess.ensure(3 * (size_t)n));
    MBPOL_CUDA_OK(I.d_dF.ensure(3 * (size_t)n));
    MBPOL_CUDA_OK(I.d_mcorr.ensure(3 * (size_t)n));
    MBPOL_CUDA_OK(I.d_mubase.ensure(3 * (size_t)n));
    MBPOL_CUDA_OK(I.d_hist.ensure(3 * kHist * (size_t)n));
    MBPOL_CUDA_OK(I.d_fhist.ensure(3 * kHist * (size_t)n));
    MBPOL_CUDA_OK(I.d_fnow.ensure(3 * (size_t)n));
    MBPOL_CUDA_OK(I.d_mprev.ensure(3 * (size_t)n));
    MBPOL_CUDA_OK(cudaMemcpyToSymbol(c_dms, kDmsCoef, sizeof(kDmsCoef)));
    MBPOL_CUDA_OK(cudaMemcpyToSymbol(c_dms_idx, kDmsIdx, sizeof(kDmsIdx)));
    I.have_prev = false;
    I.have_mprev = false;
    I.hist_levels = 0;
    I.evaluated = false;
    return MBPOL_OK;
}

static mbpol_status pme_setup(ElecImpl& I, const Box& box) {
    // alpha / grid: explicit values, or chosen from the error tolerance
    // (alpha = sqrt(-ln(2 tol)) / rc, n = ceil(2 alpha L / (3 tol^0.2)) rounded up to 2,3,5,7-smooth)
    double alpha = I.prm.ewald_alpha;
    const double tol = I.prm.ewald_error_tolerance;
    if (!(alpha > 0)) alpha = sqrt(-log(2.0 * tol)) / I.prm.cutoff;
    int g[3];
    for (int d = 0; d < 3; ++d) {
        g[d] = I.prm.pme_grid[d];
        if (g[d] <= 0) {
            int nn = (int)ceil(2.0 * alpha * box.L[d] / (3.0 * pow(tol, 0.2)));
            for (;; ++nn) {
                int m = nn;
                for (int pf : {2, 3, 5, 7})
                    while (m % pf == 0) m /= pf;
                if (m == 1) break;
            }
            g[d] = nn < 6 ? 6 : nn;
        }
    }
    const bool changed = g[0] != I.grid[0] || g[1] != I.grid[1] || g[2] != I.grid[2];
    I.alpha = alpha;
    if (changed) {
        if (I.plans) {
            cufftDestroy(I.plan_f);
            cufftDestroy(I.plan_b);
            I.plans = false;
        }
        for (int d = 0; d < 3; ++d) I.grid[d] = g[d];
        if (cufftPlan3d(&I.plan_f, g[0], g[1], g[2], CUFFT_R2C) != CUFFT_SUCCESS ||
            cufftPlan3d(&I.plan_b, g[0], g[1], g[2], CUFFT_C2R) != CUFFT_SUCCESS)
            return mbpol_fail(MBPOL_ERR_CUDA, "cufftPlan3d failed");
        I.plans = true;
        const size_t nreal = (size_t)g[0] * g[1] * g[2];
        const size_t ncplx = (size_t)g[0] * g[1] * (g[2] / 2 + 1);
        MBPOL_CUDA_OK(I.d_grid.ensure(2 * ncplx));  // in-place friendly size
        MBPOL_CUDA_OK(I.d_gridq.ensure(nreal));
        // zero once: every spread is followed by the conversion, which
        // returns the fixed-point grid to zero
        MBPOL_CUDA_OK(cudaMemset(I.d_gridq.p, 0, sizeof(unsigned long long) * nreal));
        MBPOL_CUDA_OK(I.d_gridfix.ensure(nreal));
        MBPOL_CUDA_OK(I.d_cgrid.ensure(ncplx));
        MBPOL_CUDA_OK(I.d_eterm.ensure(ncplx));
        I.eterm_key[3] = 0.0;
        std::vector<double> mod;
        DBuf<float>* bb[3] = {&I.d_bx, &I.d_by, &I.d_bz};
        for (int d = 0; d < 3; ++d) {
            bspline_moduli(g[d], mod);
            std::vector<float> mf(mod.begin(), mod.end());
            MBPOL_CUDA_OK(bb[d]->ensure(g[d]));
            MBPOL_CUDA_OK(cudaMemcpy(bb[d]->p, mf.data(), sizeof(float) * g[d], cudaMemcpyHostToDevice));
        }
    }
    return MBPOL_OK;
}

// spread (fixed point) and convert to the FP32 grid d_grid
static cudaError_t pme_spread(ElecImpl& I, cudaStream_t st, int mode, const float* mu, int n, size_t nreal) {
    count_launch();
    pme_spread_kernel<<<(n * 32 + 127) / 128, 128, 0, st>>>(n, mode, I.d_q.p, mu, I.d_gidx.p, I.d_gfrac.p, I.d_gridq.p);
    count_launch();
    pme_fix_to_float_kernel<<<(int)std::min<size_t>((nreal + 255) / 256, 152 * 16), 256, 0, st>>>(
        (long)nreal, I.d_gridq.p, I.d_grid.p);
    return cudaGetLastError();
}

// grid (real) -> FFT -> convolution -> inverse FFT, in place in d_grid
static mbpol_status pme_convolve(ElecImpl& I, cudaStream_t st, const Box& box) {
    if (cufftSetStream(I.plan_f, st) != CUFFT_SUCCESS || cufftSetStream(I.plan_b, st) != CUFFT_SUCCESS)
        return mbpol_fail(MBPOL_ERR_CUDA, "cufftSetStream failed");
    if (cufftExecR2C(I.plan_f, I.d_grid.p, I.d_cgrid.p) != CUFFT_SUCCESS)
        return mbpol_fail(MBPOL_ERR_CUDA, "cufftExecR2C failed");
    const int nzh = I.grid[2] / 2 + 1;
    const float expf_ = (float)(M_PI * M_PI / (I.alpha * I.alpha));
    const float scalef = (float)(1.0 / (M_PI * box.L[0] * box.L[1] * box.L[2]));
    const long total = (long)I.grid[0] * I.grid[1] * nzh;
    int blocks = (int)std::min<long>((total + 255) / 256, 152L * 16);
    if (I.eterm_key[0] != box.L[0] || I.eterm_key[1] != box.L[1] || I.eterm_key[2] != box.L[2] ||
        I.eterm_key[3] != I.alpha) {
        count_launch();
        pme_eterm_kernel<<<blocks, 256, 0, st>>>(I.d_eterm.p, I.d_bx.p, I.d_by.p, I.d_bz.p, expf_, scalef, nzh);
        I.eterm_key[0] = box.L[0];
        I.eterm_key[1] = box.L[1];
        I.eterm_key[2] = box.L[2];
        I.eterm_key[3] = I.alpha;
    }
    count_launch();
    pme_scale_kernel<<<blocks, 256, 0, st>>>(total, I.d_cgrid.p, I.d_eterm.p);
    if (cufftExecC2R(I.plan_b, I.d_cgrid.p, I.d_grid.p) != CUFFT_SUCCESS)
        return mbpol_fail(MBPOL_ERR_CUDA, "cufftExecC2R failed");
    return MBPOL_OK;
}

namespace {

uintptr_t key_bits(double v) {
    uint64_t u;
    std::memcpy(&u, &v, sizeof u);
    return (uintptr_t)u;
}

// The batched-cluster solver as one graph: a while node whose body runs two
// iterations (buffers a -> b, then b -> a), each a zeroing of the
// per-cluster sums, the field + update kernel and the control kernel, which
// decides on the device whether the loop goes on.  Rebuilt when a buffer,
// size or solver parameter it captured changes.
mbpol_status cluster_solver_graph(ElecImpl& I, int nmol, int wblocks, float* buf_a, float* buf_b, float* anchor_buf,
                                  double switch_eps) {
    const std::vector<uintptr_t> key = {
        (uintptr_t)nmol, (uintptr_t)wblocks, (uintptr_t)I.cap, (uintptr_t)I.ncl, (uintptr_t)buf_a, (uintptr_t)buf_b,
        (uintptr_t)anchor_buf, (uintptr_t)I.d_off.p, (uintptr_t)I.d_damp.p, (uintptr_t)I.d_pol.p,
        (uintptr_t)I.d_type.p, (uintptr_t)I.d_nb.p, (uintptr_t)I.d_nbd.p, (uintptr_t)I.d_nnb.p, (uintptr_t)I.d_E0.p,
        (uintptr_t)I.d_mud.p, (uintptr_t)I.d_eps2.p, (uintptr_t)I.d_ebase.p, (uintptr_t)I.d_intra.p,
        (uintptr_t)I.d_pcoef.p, (uintptr_t)I.d_mcl.p, (uintptr_t)I.d_cstate.p, (uintptr_t)I.d_eps2c.p,
        (uintptr_t)I.d_polmask.p, (uintptr_t)I.d_cl_nsites.p, (uintptr_t)I.d_cl_cur.p, (uintptr_t)I.d_cl_its.p,
        (uintptr_t)I.d_cl_conv.p, (uintptr_t)I.d_rounds.p, key_bits(I.prm.target_epsilon),
        (uintptr_t)I.prm.max_iterations, key_bits(switch_eps)};
    if (I.cl_exec && key == I.cl_graph_key) return MBPOL_OK;
    if (I.cl_exec) cudaGraphExecDestroy(I.cl_exec);
    if (I.cl_graph) cudaGraphDestroy(I.cl_graph);
    I.cl_exec = nullptr;
    I.cl_graph = nullptr;
    I.cl_graph_key.clear();
    if (!I.st_cap) MBPOL_CUDA_OK(cudaStreamCreateWithFlags(&I.st_cap, cudaStreamNonBlocking));
    MBPOL_CUDA_OK(cudaGraphCreate(&I.cl_graph, 0));
    cudaGraphConditionalHandle loop;
    MBPOL_CUDA_OK(cudaGraphConditionalHandleCreate(&loop, I.cl_graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = loop;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    MBPOL_CUDA_OK(cudaGraphAddNode(&node, I.cl_graph, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    cudaStream_t sc = I.st_cap;
    MBPOL_CUDA_OK(cudaStreamBeginCaptureToGraph(sc, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    for (int half = 0; half < 2; ++half) {
        const float* mu_in = half ? buf_b : buf_a;
        float* mu_out = half ? buf_a : buf_b;
        cudaMemsetAsync(I.d_eps2c.p, 0, sizeof(double) * I.ncl, sc);
        induced_update_kernel<false><<<wblocks, 128, 0, sc>>>(
            nmol, I.d_off.p, I.d_damp.p, I.d_pol.p, I.d_type.p, I.d_nb.p, I.d_nbd.p, I.d_nnb.p, I.cap, I.d_E0.p,
            nullptr, mu_in, mu_out, I.d_mud.p, I.d_eps2.p, 0, I.d_ebase.p, anchor_buf, I.d_intra.p, I.d_pcoef.p,
            I.d_mcl.p, I.d_cstate.p, I.d_eps2c.p, I.d_polmask.p, anchor_buf, nullptr);
        cluster_control_kernel<<<1, kCtlThreads, 0, sc>>>(I.ncl, I.d_eps2c.p, I.d_cl_nsites.p, I.d_cl_cur.p,
                                                           I.d_cl_its.p, I.d_cstate.p, I.d_cl_conv.p,
                                                           I.prm.target_epsilon, I.prm.max_iterations, switch_eps,
                                                           I.d_rounds.p, loop);
    }
    cudaGraph_t captured = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(sc, &captured);
    MBPOL_CUDA_OK(ce);
    MBPOL_CUDA_OK(cudaGetLastError());
    MBPOL_CUDA_OK(cudaGraphInstantiate(&I.cl_exec, I.cl_graph, 0));
    I.cl_graph_key = key;
    return MBPOL_OK;
}

// One system's PME solve as one graph: a while node whose body is one
// iteration -- the reciprocal-space pass of the dipoles on a forked branch
// beside their direct field (induced_update_kernel), the self and
// reciprocal parts and the SOR update in place (induced_finish_kernel, the
// anchoring stage read from the device), and solve_control_kernel, which
// applies the reference's stopping rules and sets the loop's condition.
// The host reads the state once, after the launch.  Rebuilt when a buffer,
// size, plan or solver parameter it captured changes.
mbpol_status solver_graph(ElecImpl& I, int nmol, int wblocks, int n, size_t nreal, float* mu, float* anchor_buf,
                          double switch_eps, const Box& box) {
    const std::vector<uintptr_t> key = {
        (uintptr_t)nmol, (uintptr_t)wblocks, (uintptr_t)n, (uintptr_t)nreal, (uintptr_t)I.cap, (uintptr_t)mu,
        (uintptr_t)anchor_buf, (uintptr_t)I.d_off.p, (uintptr_t)I.d_damp.p, (uintptr_t)I.d_pol.p,
        (uintptr_t)I.d_type.p, (uintptr_t)I.d_nb.p, (uintptr_t)I.d_nbd.p, (uintptr_t)I.d_nnb.p, (uintptr_t)I.d_E0.p,
        (uintptr_t)I.d_phi_mu.p, (uintptr_t)I.d_mud.p, (uintptr_t)I.d_eps2.p, (uintptr_t)I.d_ebase.p,
        (uintptr_t)I.d_intra.p, (uintptr_t)I.d_pcoef.p, (uintptr_t)I.d_polmask.p, (uintptr_t)I.d_edir.p,
        (uintptr_t)I.d_q.p, (uintptr_t)I.d_gidx.p, (uintptr_t)I.d_gfrac.p, (uintptr_t)I.d_gridq.p,
        (uintptr_t)I.d_grid.p, (uintptr_t)I.d_cgrid.p, (uintptr_t)I.d_eterm.p, (uintptr_t)I.plan_f,
        (uintptr_t)I.plan_b, (uintptr_t)I.d_sstate.p, key_bits(I.prm.target_epsilon),
        (uintptr_t)I.prm.max_iterations, key_bits(switch_eps)};
    if (I.sv_exec && key == I.sv_key) return MBPOL_OK;
    if (I.sv_exec) cudaGraphExecDestroy(I.sv_exec);
    if (I.sv_graph) cudaGraphDestroy(I.sv_graph);
    I.sv_exec = nullptr;
    I.sv_graph = nullptr;
    I.sv_key.clear();
    if (!I.st_cap) MBPOL_CUDA_OK(cudaStreamCreateWithFlags(&I.st_cap, cudaStreamNonBlocking));
    if (!I.st_cap2) MBPOL_CUDA_OK(cudaStreamCreateWithFlags(&I.st_cap2, cudaStreamNonBlocking));
    if (!I.ev_cfork) MBPOL_CUDA_OK(cudaEventCreateWithFlags(&I.ev_cfork, cudaEventDisableTiming));
    if (!I.ev_cjoin) MBPOL_CUDA_OK(cudaEventCreateWithFlags(&I.ev_cjoin, cudaEventDisableTiming));
    MBPOL_CUDA_OK(cudaGraphCreate(&I.sv_graph, 0));
    cudaGraphConditionalHandle loop;
    MBPOL_CUDA_OK(cudaGraphConditionalHandleCreate(&loop, I.sv_graph, 1, cudaGraphCondAssignDefault));
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = loop;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    cudaGraphNode_t node;
    MBPOL_CUDA_OK(cudaGraphAddNode(&node, I.sv_graph, nullptr, nullptr, 0, &cp));
    cudaGraph_t body = cp.conditional.phGraph_out[0];
    cudaStream_t sc = I.st_cap, sc2 = I.st_cap2;
    MBPOL_CUDA_OK(cudaStreamBeginCaptureToGraph(sc, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
    // fork: the PME pass of mu on the second branch
    cudaError_t ce = cudaEventRecord(I.ev_cfork, sc);
    if (ce == cudaSuccess) ce = cudaStreamWaitEvent(sc2, I.ev_cfork, 0);
    mbpol_status ps = MBPOL_OK;
    if (ce == cudaSuccess) ce = pme_spread(I, sc2, 1, mu, n, nreal);
    if (ce == cudaSuccess) ps = pme_convolve(I, sc2, box);
    if (ce == cudaSuccess && ps == MBPOL_OK) {
        pme_gather_kernel<<<(n * 32 + 127) / 128, 128, 0, sc2>>>(n, 4, I.d_grid.p, I.d_gidx.p, I.d_gfrac.p,
                                                                I.d_phi_mu.p);
        ce = cudaEventRecord(I.ev_cjoin, sc2);
    }
    if (ce == cudaSuccess && ps == MBPOL_OK) {
        induced_update_kernel<true><<<wblocks, 128, 0, sc>>>(
            nmol, I.d_off.p, I.d_damp.p, I.d_pol.p, I.d_type.p, I.d_nb.p, I.d_nbd.p, I.d_nnb.p, I.cap, I.d_E0.p,
            I.d_phi_mu.p, mu, mu, I.d_mud.p, I.d_eps2.p, 0, I.d_ebase.p, anchor_buf, I.d_intra.p, I.d_pcoef.p,
            nullptr, nullptr, nullptr, I.d_polmask.p, nullptr, I.d_edir.p);
        ce = cudaStreamWaitEvent(sc, I.ev_cjoin, 0);
    }
    if (ce == cudaSuccess && ps == MBPOL_OK) {
        induced_finish_kernel<<<(n + 127) / 128, 128, 0, sc>>>(n, I.d_edir.p, I.d_phi_mu.p, I.d_E0.p, I.d_pol.p,
                                                               mu, mu, I.d_mud.p, I.d_eps2.p, 0, I.d_ebase.p,
                                                               anchor_buf, reinterpret_cast<const int*>(I.d_sstate.p),
                                                               anchor_buf);
        solve_control_kernel<<<1, 1, 0, sc>>>(I.d_eps2.p, 1.0 / (double)n, I.d_sstate.p, I.prm.target_epsilon,
                                              I.prm.max_iterations, switch_eps, loop);
    }
    cudaGraph_t captured = nullptr;
    const cudaError_t ee = cudaStreamEndCapture(sc, &captured);
    if (ps) return ps;
    MBPOL_CUDA_OK(ce);
    MBPOL_CUDA_OK(ee);
    MBPOL_CUDA_OK(cudaGetLastError());
    MBPOL_CUDA_OK(cudaGraphInstantiate(&I.sv_exec, I.sv_graph, 0));
    I.sv_key = key;
    return MBPOL_OK;
}

}  // namespace

mbpol_status ElecEngine::compute(cudaStream_t st, const double* pos, const Box& box, double* force, double* energy) {
    ElecImpl& I = *impl_;
    const int n = I.N, K = I.K, nmol = I.nmol;
    if (I.pme) {
        if (!box.periodic) return mbpol_fail(MBPOL_ERR_STATE, "PME requires a periodic box");
        for (int d = 0; d < 3; ++d)
            if (box.L[d] < 1.999999 * I.prm.cutoff)
                return mbpol_fail(MBPOL_ERR_BOX_TOO_SMALL,
                                  "The periodic box size has decreased to less than twice the nonbonded cutoff.");
        mbpol_status s = pme_setup(I, box);
        if (s) return s;
    }
    ElecConst c{};
    for (int k = 0; k < 5; ++k) c.thole[k] = (float)I.prm.thole[k];
    c.alpha = I.pme ? (float)I.alpha : 0.f;
    c.rc2 = I.pme ? (float)(I.prm.cutoff * I.prm.cutoff) : 3.0e38f;
    c.self_term = I.pme ? (float)((4.0 / 3.0) * I.alpha * I.alpha * I.alpha / kSqrtPi) : 0.f;
    c.K = K;
    for (int d = 0; d < 3; ++d) {
        c.grid[d] = I.grid[d];
        c.box[d] = box.periodic ? box.L[d] : 1.0;
        c.inv[d] = box.periodic ? box.inv[d] : 1.0;
        c.scale[d] = I.pme ? (float)(I.grid[d] * box.inv[d]) : 0.f;
        c.boxf[d] = (float)c.box[d];
        c.invf[d] = (float)c.inv[d];
    }
    c.periodic = I.pme ? 1 : 0;
    c.fixed_thole_sign = I.prm.pme_fixed_field == MBPOL_PME_FIELD_CONSISTENT ? -1.f : 1.f;
    MBPOL_CUDA_OK(cudaMemcpyToSymbolAsync(c_el, &c, sizeof(c), 0, cudaMemcpyHostToDevice, st));
    const int redist = I.prm.include_charge_redistribution ? 1 : 0;
    count_launch();
    elec_prepare_kernel<<<(nmol + 127) / 128, 128, 0, st>>>(nmol, pos, box.periodic, redist, I.d_qs.p, I.d_off.p,
                                                            I.d_q.p, I.d_dq.p, I.pme ? 1 : 0, I.d_gidx.p, I.d_gfrac.p, I.d_reach.p,
                                                            I.d_opos.p);
    // neighbour list
    const double rcut = I.pme ? I.prm.cutoff : 1e30;
    if (I.cap == 0) I.cap = I.pme ? 256 : ((((I.ncl > 0 ? I.max_cl_mol : nmol)) + 31) / 32) * 32;
    // candidates: the molecule's cluster, or the cells around it (edges >=
    // the cutoff plus twice kCellReach), else all molecules
    CandidateSet cands;
    Box cbox = box;
    cbox.periodic = box.periodic && I.pme;
    if (I.ncl > 0) {
        cands = I.cl_candidates;
    } else if (I.cells_ok) {
        const double rcell = rcut + 2.0 * kCellReach;
        const size_t ints = cell_scratch_ints(nmol, cbox, rcell);
        if (ints) {
            MBPOL_CUDA_OK(I.d_cells.ensure(ints));
            mbpol_status cs = launch_cell_binning(st, nmol, I.d_opos.p, cbox, rcell, I.d_cells.p, &cands);
            if (cs) return cs;
        }
    }
    for (int attempt = 0;; ++attempt) {
        MBPOL_CUDA_OK(I.d_nb.ensure((size_t)nmol * I.cap));
        MBPOL_CUDA_OK(I.d_nbd.ensure((size_t)nmol * I.cap * 3));
        MBPOL_CUDA_OK(cudaMemsetAsync(I.d_flags.p, 0, sizeof(int), st));
        count_launch();
        elec_neighbors_kernel<<<(nmol * 32 + 127) / 128, 128, 0, st>>>(
            nmol, pos, I.d_opos.p, cbox.periodic, rcut, I.d_reach.p, I.cap, I.d_nb.p, I.d_nbd.p, I.d_nnb.p,
            I.d_flags.p, cands);
        int ovf = 0;
        MBPOL_CUDA_OK(cudaMemcpyAsync(&ovf, I.d_flags.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        MBPOL_CUDA_OK(cudaStreamSynchronize(st));
        if (!ovf) break;
        if (ovf & 2) {
            // a molecule reaches beyond kCellReach: scan all pairs from now on
            I.cells_ok = false;
            cands = CandidateSet();
            continue;
        }
        if (attempt > 6) return mbpol_fail(MBPOL_ERR_CAPACITY, "electrostatics neighbour capacity");
        I.cap *= 2;
    }
    MBPOL_CUDA_OK(I.d_pcoef.ensure((size_t)nmol * kMaxK * kMaxK * 2 * I.cap));
    MBPOL_CUDA_OK(I.d_npair.ensure(1));
    if (!I.h_npair) MBPOL_CUDA_OK(cudaMallocHost(&I.h_npair, sizeof(unsigned long long)));
    MBPOL_CUDA_OK(cudaMemsetAsync(I.d_npair.p, 0, sizeof(unsigned long long), st));
    const int wblocks = (nmol * 32 + 127) / 128;
    const size_t nreal = I.pme ? (size_t)I.grid[0] * I.grid[1] * I.grid[2] : 0;
    // fixed field
    if (I.pme) {
        MBPOL_CUDA_OK(pme_spread(I, st, 0, nullptr, n, nreal));
        mbpol_status s = pme_convolve(I, st, box);
        if (s) return s;
        MBPOL_CUDA_OK(cudaMemcpyAsync(I.d_gridfix.p, I.d_grid.p, sizeof(float) * nreal, cudaMemcpyDeviceToDevice, st));
        count_launch();
        pme_gather_kernel<<<(n * 32 + 127) / 128, 128, 0, st>>>(n, 10, I.d_gridfix.p, I.d_gidx.p, I.d_gfrac.p, I.d_phi_fix.p);
        prof_begin(st, K_ELEC_FIXED);
        count_launch();
        fixed_field_kernel<true><<<wblocks, 128, 0, st>>>(nmol, I.d_off.p, I.d_q.p, I.d_damp.p, I.d_pol.p, I.d_type.p,
                                                           I.d_nb.p, I.d_nbd.p, I.d_nnb.p, I.cap, I.d_phi_fix.p,
                                                           I.d_E0.p, I.d_mu0.p, I.d_intra.p, I.d_pcoef.p,
                                                           I.d_npair.p);
        prof_end(st, K_ELEC_FIXED);
    } else {
        count_launch();
        fixed_field_kernel<false><<<wblocks, 128, 0, st>>>(nmol, I.d_off.p, I.d_q.p, I.d_damp.p, I.d_pol.p,
                                                            I.d_type.p, I.d_nb.p, I.d_nbd.p, I.d_nnb.p, I.cap,
                                                            nullptr, I.d_E0.p, I.d_mu0.p, I.d_intra.p,
                                                            I.d_pcoef.p, I.d_npair.p);
    }
    // directed pair count -> host (pinned), read after the solver's first wait
    MBPOL_CUDA_OK(cudaMemcpyAsync(I.h_npair, I.d_npair.p, sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
    // d_mu0 holds float(mu) of the starting dipoles (alpha*E0 from the
    // fixed-field kernel, or the previous call's dipoles)
    float* bufs[3] = {I.d_mu0.p, I.d_mu1.p, I.d_mu2.p};
    // starting dipoles: 3 polynomial extrapolation of the last solves; 2 the
    // same once two solves exist, before that the network (cold start, or
    // mu_prev + m - m_prev after one solve); 1 previous solve; 0 alpha E0
    // (the reference).  In a smooth trajectory the extrapolation error
    // (~1e-4 of mu) is below what a BF16 network resolves, so the network
    // serves the first steps and single-point evaluations.
    const bool learned = I.prm.guess == 2 && I.net.ready() && (I.K == 3 || I.K == 4);
    const bool history = I.prm.guess >= 2;
    const bool extrapolate = history && (I.hist_levels >= 2 || (I.prm.guess == 3 && I.hist_levels >= 1));
    // guess 2 with a full history: the learned linear predictor, refitted on
    // the last steps (predictor.cu)
    const bool predictor = I.prm.guess == 2 && I.hist_levels >= guess::kPredHistory;
    if (learned && !extrapolate) {
        MBPOL_CUDA_OK(I.net.descriptors(st, nmol, I.K, I.d_off.p, I.d_nb.p, I.d_nbd.p, I.d_nnb.p, I.cap, box.L,
                                        box.periodic && I.pme, I.d_E0.p));
        MBPOL_CUDA_OK(I.net.predict(st, nmol, I.K, I.d_mguess.p));
    }
    const bool used_net = learned && !extrapolate;
    I.cdesc_valid = false;
    if (history) MBPOL_CUDA_OK(scaled_field(st, 3 * n, I.d_E0.p, I.d_pol.p, I.d_fnow.p));
    if (predictor) {
        PredictorRing ring{};
        for (int k = 0; k < guess::kPredHistory; ++k) {
            const size_t slot = 3 * (size_t)n * ((I.hist_head + kHist - k) % kHist);
            ring.r[k] = I.d_hist.p + slot;
            ring.f[k] = I.d_fhist.p + slot;
        }
        MBPOL_CUDA_OK(
            I.d_pred.ensure((size_t)predictor_partial_blocks() * guess::kPredStats + guess::kPredRegressors));
        double* coef = I.d_pred.p + (size_t)predictor_partial_blocks() * guess::kPredStats;
        if (I.pred_fitted)
            MBPOL_CUDA_OK(cudaStreamWaitEvent(st, I.ev_fit, 0));  // fitted after the last solve
        else
            MBPOL_CUDA_OK(predictor_fit(st, 3 * n, ring, I.d_pred.p, coef));
        // the correction network: its inputs whenever it is trained or being
        // trained (selected), its output added when it is trained
        const bool corr = (I.cnet.ready() || I.sel == 1) && (I.K == 3 || I.K == 4);
        MBPOL_CUDA_OK(predictor_apply(st, 3 * n, ring, I.d_fnow.p, coef, I.d_mud.p, I.d_mu0.p,
                                      corr ? I.d_dF.p : nullptr));
        if (corr) {
            MBPOL_CUDA_OK(I.cnet.descriptors(st, nmol, I.K, I.d_off.p, I.d_nb.p, I.d_nbd.p, I.d_nnb.p, I.cap,
                                             box.L, box.periodic && I.pme, I.d_dF.p));
            MBPOL_CUDA_OK(cudaMemcpyAsync(I.d_mubase.p, I.d_mud.p, sizeof(double) * 3 * (size_t)n,
                                          cudaMemcpyDeviceToDevice, st));
            I.cdesc_valid = true;
            if (I.cnet.ready()) {
                MBPOL_CUDA_OK(I.cnet.predict(st, nmol, I.K, I.d_mcorr.p));
                MBPOL_CUDA_OK(add_correction(st, 3 * n, I.d_mcorr.p, I.d_mud.p, I.d_mu0.p));
            }
        }
    } else if (extrapolate) {
        const size_t plane = 3 * (size_t)n;
        HistRing h{};
        h.levels = std::min(I.hist_levels, kExtrapolate);
        double binom = 1.0;  // C(L, k), k = 1 .. L
        for (int k = 0; k < h.levels; ++k) {
            binom = binom * (h.levels - k) / (k + 1);
            h.r[k] = I.d_hist.p + plane * ((I.hist_head + kHist - k) % kHist);
            h.c[k] = (k % 2 ? -1.0 : 1.0) * binom;
        }
        count_launch();
        extrapolated_guess_kernel<<<(3 * n + 255) / 256, 256, 0, st>>>(3 * n, h, I.d_mud.p, I.d_mu0.p);
    } else if (used_net) {
        const bool prev = I.have_prev && I.have_mprev;
        count_launch();
        learned_guess_kernel<<<(3 * n + 255) / 256, 256, 0, st>>>(3 * n, I.d_mguess.p, prev ? I.d_mprev.p : nullptr,
                                                                  prev ? I.d_mud_prev.p : nullptr, I.d_mud.p,
                                                                  I.d_mu0.p);
    } else if (I.prm.guess >= 1 && I.have_prev) {
        MBPOL_CUDA_OK(cudaMemcpyAsync(I.d_mu0.p, I.d_mu_prev.p, sizeof(float) * 3 * (size_t)n,
                                      cudaMemcpyDeviceToDevice, st));
        MBPOL_CUDA_OK(cudaMemcpyAsync(I.d_mud.p, I.d_mud_prev.p, sizeof(double) * 3 * (size_t)n,
                                      cudaMemcpyDeviceToDevice, st));
    } else {
        count_launch();
        widen_kernel<<<(3 * n + 255) / 256, 256, 0, st>>>(3 * n, I.d_mu0.p, I.d_mud.p);
    }
    // solver (reference convergeInduceDipoles :557-616); the anchoring switch
    // is taken once the measure is 100x above the target (at most 1e-6 D)
    const double switch_eps = std::min(1e-6, 100.0 * I.prm.target_epsilon);
    double current = 1.0e+50;
    int it = 0;
    bool done = false, conv = false;
    double eps = 0.0;
    float* mu_in = bufs[0];
    float* anchor = nullptr;
    int mode = 0;
    if (I.ncl > 0) {
        // batched clusters: each cluster runs the reference's loop on its own
        // epsilon (its own site count) and stops on its own while the others
        // go on; the whole loop is one graph launch, its control on the device
        const int ncl = I.ncl;
        std::vector<int> cstate(ncl, 0), cconv(ncl, 0), its(ncl, 0);
        std::vector<double> cur(ncl, 1.0e+50);
        for (int c = 0; c < ncl; ++c)
            if (I.cl_nsites[c] == 0) {
                cstate[c] = 3;
                cconv[c] = 1;
            }
        MBPOL_CUDA_OK(cudaMemcpyAsync(I.d_cstate.p, cstate.data(), sizeof(int) * ncl, cudaMemcpyHostToDevice, st));
        MBPOL_CUDA_OK(cudaMemcpyAsync(I.d_cl_conv.p, cconv.data(), sizeof(int) * ncl, cudaMemcpyHostToDevice, st));
        MBPOL_CUDA_OK(cudaMemcpyAsync(I.d_cl_cur.p, cur.data(), sizeof(double) * ncl, cudaMemcpyHostToDevice, st));
        MBPOL_CUDA_OK(cudaMemsetAsync(I.d_cl_its.p, 0, sizeof(int) * ncl, st));
        MBPOL_CUDA_OK(cudaMemsetAsync(I.d_rounds.p, 0, sizeof(int), st));
        mbpol_status gs = cluster_solver_graph(I, nmol, wblocks, bufs[0], bufs[1], bufs[2], switch_eps);
        if (gs) return gs;
        prof_begin(st, K_ELEC_INDUCED);
        MBPOL_CUDA_OK(cudaGraphLaunch(I.cl_exec, st));
        prof_end(st, K_ELEC_INDUCED);
        int rounds = 0;
        MBPOL_CUDA_OK(cudaMemcpyAsync(its.data(), I.d_cl_its.p, sizeof(int) * ncl, cudaMemcpyDeviceToHost, st));
        MBPOL_CUDA_OK(cudaMemcpyAsync(cconv.data(), I.d_cl_conv.p, sizeof(int) * ncl, cudaMemcpyDeviceToHost, st));
        MBPOL_CUDA_OK(cudaMemcpyAsync(cur.data(), I.d_cl_cur.p, sizeof(double) * ncl, cudaMemcpyDeviceToHost, st));
        MBPOL_CUDA_OK(cudaMemcpyAsync(&rounds, I.d_rounds.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        MBPOL_CUDA_OK(cudaStreamSynchronize(st));
        for (int r = 0; r < 2 * rounds; ++r) count_launch();  // field + control kernels per iteration
        I.cl_iters = its;
        I.cl_conv.assign(cconv.begin(), cconv.end());
        it = 0;
        conv = true;
        current = 0.0;
        for (int c = 0; c < ncl; ++c) {
            it = std::max(it, its[c]);
            conv = conv && cconv[c];
            if (I.cl_nsites[c] > 0) current = std::max(current, cur[c]);
        }
        done = true;
    }
    if (!done && I.pme && !prof_on() && !I.sv_disabled) {
        MBPOL_CUDA_OK(I.d_sstate.ensure(1));
        if (solver_graph(I, nmol, wblocks, n, nreal, bufs[0], bufs[2], switch_eps, box) != MBPOL_OK) {
            // a capture this driver does not support: keep the host loop
            I.sv_disabled = true;
            cudaGetLastError();
        }
    }
    if (!done && I.pme && !prof_on() && !I.sv_disabled) {
        // one graph launch; the host reads the solve's state once
        const SolveState s0 = {0, 0, 0, 0, 1.0e+50};
        MBPOL_CUDA_OK(cudaMemcpyAsync(I.d_sstate.p, &s0, sizeof s0, cudaMemcpyHostToDevice, st));
        MBPOL_CUDA_OK(cudaMemsetAsync(I.d_eps2.p, 0, sizeof(double), st));
        MBPOL_CUDA_OK(cudaGraphLaunch(I.sv_exec, st));
        SolveState sr{};
        MBPOL_CUDA_OK(cudaMemcpyAsync(&sr, I.d_sstate.p, sizeof sr, cudaMemcpyDeviceToHost, st));
        MBPOL_CUDA_OK(cudaStreamSynchronize(st));
        for (int r = 0; r < 7 * sr.rounds; ++r) count_launch();  // spread, conversion, scale, gather, field, update, control
        it = sr.its;
        conv = sr.conv != 0;
        current = sr.cur;
        done = true;
    }
    while (!done) {
        int kmode = mode;
        if (mode == 0 && current < switch_eps) kmode = 1;
        float* mu_out = nullptr;
        for (float* b : bufs)
            if (b != mu_in && b != anchor) {
                mu_out = b;
                break;
            }
        if (I.pme) {
            // the reciprocal-space pass of mu_in runs on the second stream
            // while the direct field of the same dipoles is summed here
            MBPOL_CUDA_OK(cudaEventRecord(I.ev_in, st));
            MBPOL_CUDA_OK(cudaStreamWaitEvent(I.st2, I.ev_in, 0));
            prof_begin(I.st2, K_ELEC_PME);
            MBPOL_CUDA_OK(pme_spread(I, I.st2, 1, mu_in, n, nreal));
            mbpol_status s = pme_convolve(I, I.st2, box);
            if (s) return s;
            count_launch();
            pme_gather_kernel<<<(n * 32 + 127) / 128, 128, 0, I.st2>>>(n, 4, I.d_grid.p, I.d_gidx.p, I.d_gfrac.p,
                                                                   I.d_phi_mu.p);
            prof_end(I.st2, K_ELEC_PME);
            MBPOL_CUDA_OK(cudaEventRecord(I.ev_pme, I.st2));
        }
        MBPOL_CUDA_OK(cudaMemsetAsync(I.d_eps2.p, 0, sizeof(double), st));
        prof_begin(st, K_ELEC_INDUCED);
        count_launch();
        prof_begin(st, K_ELEC_FIELD);
        if (I.pme) {
            induced_update_kernel<true><<<wblocks, 128, 0, st>>>(nmol, I.d_off.p, I.d_damp.p, I.d_pol.p, I.d_type.p,
                                                                  I.d_nb.p, I.d_nbd.p, I.d_nnb.p, I.cap, I.d_E0.p,
                                                                  I.d_phi_mu.p, mu_in, mu_out, I.d_mud.p, I.d_eps2.p,
                                                                  kmode, I.d_ebase.p, anchor, I.d_intra.p,
                                                                  I.d_pcoef.p, nullptr, nullptr, nullptr,
                                                                  I.d_polmask.p, nullptr, I.d_edir.p);
            prof_end(st, K_ELEC_FIELD);
            MBPOL_CUDA_OK(cudaStreamWaitEvent(st, I.ev_pme, 0));
            count_launch();
            induced_finish_kernel<<<(n + 127) / 128, 128, 0, st>>>(n, I.d_edir.p, I.d_phi_mu.p, I.d_E0.p, I.d_pol.p,
                                                                   mu_in, mu_out, I.d_mud.p, I.d_eps2.p, kmode,
                                                                   I.d_ebase.p, anchor, nullptr, nullptr);
        } else
            induced_update_kernel<false><<<wblocks, 128, 0, st>>>(nmol, I.d_off.p, I.d_damp.p, I.d_pol.p, I.d_type.p,
                                                                   I.d_nb.p, I.d_nbd.p, I.d_nnb.p, I.cap, I.d_E0.p,
                                                                   nullptr, mu_in, mu_out, I.d_mud.p, I.d_eps2.p,
                                                                   kmode, I.d_ebase.p, anchor, I.d_intra.p,
                                                                  I.d_pcoef.p, nullptr, nullptr, nullptr,
                                                                  I.d_polmask.p, nullptr, nullptr);
        if (!I.pme) prof_end(st, K_ELEC_FIELD);
        prof_end(st, K_ELEC_INDUCED);
        if (kmode == 1) anchor = mu_in;
        mode = kmode == 0 ? 0 : 2;
        mu_in = mu_out;
        double e2 = 0.0;
        MBPOL_CUDA_OK(cudaMemcpyAsync(&e2, I.d_eps2.p, sizeof(double), cudaMemcpyDeviceToHost, st));
        MBPOL_CUDA_OK(cudaStreamSynchronize(st));
        eps = kSOR * kDebye * sqrt(e2 / (double)n);
        if (!std::isfinite(eps)) {
            done = true;
        } else if (eps < I.prm.target_epsilon) {
            conv = true;
            done = true;
        } else if (current < eps || it >= I.prm.max_iterations) {
            done = true;
        }
        current = eps;
        ++it;
    }
    I.iterations = it;
    I.epsilon = current;
    I.converged = conv;
    // final dipoles (FP32 copy of the FP64 state) for the energy and forces
    float* mu_final = bufs[0];
    count_launch();
    narrow_kernel<<<(3 * n + 255) / 256, 256, 0, st>>>(3 * n, I.d_mud.p, mu_final);
    if (conv) {
        MBPOL_CUDA_OK(cudaMemcpyAsync(I.d_mu_prev.p, mu_final, sizeof(float) * 3 * (size_t)n,
                                      cudaMemcpyDeviceToDevice, st));
        MBPOL_CUDA_OK(cudaMemcpyAsync(I.d_mud_prev.p, I.d_mud.p, sizeof(double) * 3 * (size_t)n,
                                      cudaMemcpyDeviceToDevice, st));
        if (history) {
            I.hist_head = (I.hist_head + 1) % kHist;
            MBPOL_CUDA_OK(cudaMemcpyAsync(I.d_hist.p + 3 * (size_t)n * I.hist_head, I.d_mud.p,
                                          sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToDevice, st));
            MBPOL_CUDA_OK(cudaMemcpyAsync(I.d_fhist.p + 3 * (size_t)n * I.hist_head, I.d_fnow.p,
                                          sizeof(double) * 3 * (size_t)n, cudaMemcpyDeviceToDevice, st));
            I.hist_levels = std::min(I.hist_levels + 1, kHist);
        }
        // the next evaluation's predictor, fitted now beside the energy and
        // forces (the ring is not written again before that evaluation's
        // start, which waits for the fit)
        I.pred_fitted = false;
        if (history && I.prm.guess == 2 && I.hist_levels >= guess::kPredHistory) {
            PredictorRing ring{};
            for (int k = 0; k < guess::kPredHistory; ++k) {
                const size_t slot = 3 * (size_t)n * ((I.hist_head + kHist - k) % kHist);
                ring.r[k] = I.d_hist.p + slot;
                ring.f[k] = I.d_fhist.p + slot;
            }
            MBPOL_CUDA_OK(
                I.d_pred.ensure((size_t)predictor_partial_blocks() * guess::kPredStats + guess::kPredRegressors));
            MBPOL_CUDA_OK(cudaEventRecord(I.ev_hist, st));
            MBPOL_CUDA_OK(cudaStreamWaitEvent(I.st2, I.ev_hist, 0));
            MBPOL_CUDA_OK(predictor_fit(I.st2, 3 * n, ring, I.d_pred.p,
                                        I.d_pred.p + (size_t)predictor_partial_blocks() * guess::kPredStats));
            MBPOL_CUDA_OK(cudaEventRecord(I.ev_fit, I.st2));
            I.pred_fitted = true;
        }
        if (used_net)
            MBPOL_CUDA_OK(cudaMemcpyAsync(I.d_mprev.p, I.d_mguess.p, sizeof(float) * 3 * (size_t)n,
                                          cudaMemcpyDeviceToDevice, st));
    }
    I.have_prev = conv;
    I.have_mprev = conv && used_net;
    if (!conv || !history) I.hist_levels = 0;
    I.evaluated = true;
    I.last_box = box;
    if (I.pme) {
        MBPOL_CUDA_OK(pme_spread(I, st, 1, mu_final, n, nreal));
        mbpol_status s = pme_convolve(I, st, box);
        if (s) return s;
        count_launch();
        pme_gather_kernel<<<(n * 32 + 127) / 128, 128, 0, st>>>(n, 10, I.d_grid.p, I.d_gidx.p, I.d_gfrac.p, I.d_phi_mu.p);
        prof_begin(st, K_ELEC_FORCES);
        count_launch();
        energy_force_kernel<true><<<wblocks, 128, 0, st>>>(nmol, I.d_off.p, I.d_q.p, I.d_dq.p, I.d_damp.p, I.d_type.p,
                                                            I.d_nb.p, I.d_nbd.p, I.d_nnb.p, I.cap, mu_final,
                                                            I.d_phi_fix.p, I.d_phi_mu.p, redist, force, energy,
                                                            I.cl_sink);
        prof_end(st, K_ELEC_FORCES);
    } else {
        count_launch();
        energy_force_kernel<false><<<wblocks, 128, 0, st>>>(nmol, I.d_off.p, I.d_q.p, I.d_dq.p, I.d_damp.p,
                                                             I.d_type.p, I.d_nb.p, I.d_nbd.p, I.d_nnb.p, I.cap,
                                                             mu_final, nullptr, nullptr, redist, force, energy,
                                                             I.cl_sink);
    }
    MBPOL_CUDA_OK(cudaGetLastError());
    return MBPOL_OK;
}

mbpol_status ElecEngine::get_dipoles(cudaStream_t st, double* dipoles, int* iterations, double* epsilon) {
    ElecImpl& I = *impl_;
    std::vector<double> h(3 * (size_t)I.N);
    MBPOL_CUDA_OK(cudaMemcpyAsync(h.data(), I.d_mud.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, st));
    MBPOL_CUDA_OK(cudaStreamSynchronize(st));
    if (dipoles)
        for (size_t i = 0; i < h.size(); ++i) dipoles[i] = h[i];
    if (iterations) *iterations = I.iterations;
    if (epsilon) *epsilon = I.epsilon;
    return MBPOL_OK;
}

mbpol_status ElecEngine::potential(cudaStream_t st, const double* pos, int npts, const double* points,
                                   double* potential) {
    ElecImpl& I = *impl_;
    if (!I.evaluated) return mbpol_fail(MBPOL_ERR_STATE, "no electrostatics evaluation yet");
    if (npts <= 0) return MBPOL_OK;
    const int n = I.N;
    MBPOL_CUDA_OK(I.d_qd.ensure(n));
    if (!I.prm.include_charge_redistribution) {
        MBPOL_CUDA_OK(I.d_qs64.ensure(n));
        MBPOL_CUDA_OK(cudaMemcpyAsync(I.d_qs64.p, I.q_static64.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
    }
    MBPOL_CUDA_OK(I.d_pts.ensure(3 * (size_t)npts));
    MBPOL_CUDA_OK(I.d_pot.ensure(npts));
    MBPOL_CUDA_OK(cudaMemcpyAsync(I.d_pts.p, points, sizeof(double) * 3 * npts, cudaMemcpyHostToDevice, st));
    count_launch();
    site_charges_kernel<<<(I.nmol + 127) / 128, 128, 0, st>>>(I.nmol, pos, I.prm.include_charge_redistribution ? 1 : 0,
                                                              I.d_qs64.p, I.d_qd.p);
    count_launch();
    potential_kernel<<<(npts + kPotTile - 1) / kPotTile, kPotTile, 0, st>>>(n, pos, I.d_qd.p, I.d_mud.p, npts,
                                                                          I.d_pts.p, I.d_pot.p);
    MBPOL_CUDA_OK(cudaGetLastError());
    MBPOL_CUDA_OK(cudaMemcpyAsync(potential, I.d_pot.p, sizeof(double) * npts, cudaMemcpyDeviceToHost, st));
    MBPOL_CUDA_OK(cudaStreamSynchronize(st));
    return MBPOL_OK;
}

mbpol_status ElecEngine::moments(cudaStream_t st, const double* pos, const double* masses, double* out) {
    ElecImpl& I = *impl_;
    if (!I.evaluated) return mbpol_fail(MBPOL_ERR_STATE, "no electrostatics evaluation yet");
    const int n = I.N;
    MBPOL_CUDA_OK(I.d_qd.ensure(n));
    if (!I.prm.include_charge_redistribution) {
        MBPOL_CUDA_OK(I.d_qs64.ensure(n));
        MBPOL_CUDA_OK(cudaMemcpyAsync(I.d_qs64.p, I.q_static64.data(), sizeof(double) * n, cudaMemcpyHostToDevice, st));
    }
    MBPOL_CUDA_OK(I.d_mass.ensure(n));
    MBPOL_CUDA_OK(I.d_mom.ensure(14 * (size_t)kMomBlocks + 13));
    MBPOL_CUDA_OK(cudaMemcpyAsync(I.d_mass.p, masses, sizeof(double) * n, cudaMemcpyHostToDevice, st));
    double* pcom = I.d_mom.p;
    double* part = pcom + 4 * kMomBlocks;
    double* res = part + 10 * kMomBlocks;
    count_launch();
    site_charges_kernel<<<(I.nmol + 127) / 128, 128, 0, st>>>(I.nmol, pos, I.prm.include_charge_redistribution ? 1 : 0,
                                                              I.d_qs64.p, I.d_qd.p);
    count_launch();
    moments_com_kernel<<<kMomBlocks, kMomThreads, 0, st>>>(n, pos, I.d_mass.p, pcom);
    count_launch();
    moments_kernel<<<kMomBlocks, kMomThreads, 0, st>>>(n, pos, I.d_qd.p, I.d_mud.p, pcom, part);
    count_launch();
    moments_final_kernel<<<1, 32, 0, st>>>(part, res);
    MBPOL_CUDA_OK(cudaGetLastError());
    MBPOL_CUDA_OK(cudaMemcpyAsync(out, res, sizeof(double) * 13, cudaMemcpyDeviceToHost, st));
    MBPOL_CUDA_OK(cudaStreamSynchronize(st));
    return MBPOL_OK;
}

mbpol_status ElecEngine::guess_fit_predictor(cudaStream_t st, const double* history, const double* field,
                                             const double* field_now, int n3, double* coef, double* prediction) {
    if (!history || !field || !field_now || n3 <= 0) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "bad argument");
    DBuf<double> h, fh, fn, pred, out;
    DBuf<float> outf;
    const size_t hn = (size_t)guess::kPredHistory * n3;
    MBPOL_CUDA_OK(h.ensure(hn));
    MBPOL_CUDA_OK(fh.ensure(hn));
    MBPOL_CUDA_OK(fn.ensure(n3));
    MBPOL_CUDA_OK(pred.ensure((size_t)predictor_partial_blocks() * guess::kPredStats + guess::kPredRegressors));
    MBPOL_CUDA_OK(out.ensure(n3));
    MBPOL_CUDA_OK(outf.ensure(n3));
    MBPOL_CUDA_OK(cudaMemcpyAsync(h.p, history, sizeof(double) * hn, cudaMemcpyHostToDevice, st));
    MBPOL_CUDA_OK(cudaMemcpyAsync(fh.p, field, sizeof(double) * hn, cudaMemcpyHostToDevice, st));
    MBPOL_CUDA_OK(cudaMemcpyAsync(fn.p, field_now, sizeof(double) * (size_t)n3, cudaMemcpyHostToDevice, st));
    PredictorRing ring{};
    for (int k = 0; k < guess::kPredHistory; ++k) {
        ring.r[k] = h.p + (size_t)k * n3;
        ring.f[k] = fh.p + (size_t)k * n3;
    }
    double* c = pred.p + (size_t)predictor_partial_blocks() * guess::kPredStats;
    MBPOL_CUDA_OK(predictor_fit(st, n3, ring, pred.p, c));
    MBPOL_CUDA_OK(predictor_apply(st, n3, ring, fn.p, c, out.p, outf.p));
    if (coef)
        MBPOL_CUDA_OK(
            cudaMemcpyAsync(coef, c, sizeof(double) * guess::kPredRegressors, cudaMemcpyDeviceToHost, st));
    if (prediction)
        MBPOL_CUDA_OK(cudaMemcpyAsync(prediction, out.p, sizeof(double) * (size_t)n3, cudaMemcpyDeviceToHost, st));
    MBPOL_CUDA_OK(cudaStreamSynchronize(st));
    return MBPOL_OK;
}

mbpol_status ElecEngine::guess_select(int which) {
    if (which != 0 && which != 1) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "network 0 (cold start) or 1 (correction)");
    impl_->sel = which;
    return MBPOL_OK;
}

mbpol_status ElecEngine::guess_descriptors(cudaStream_t st, float* host_out) {
    ElecImpl& I = *impl_;
    if (!I.evaluated) return mbpol_fail(MBPOL_ERR_STATE, "no electrostatics evaluation yet");
    if (I.K != 3 && I.K != 4) return mbpol_fail(MBPOL_ERR_STATE, "the learned guess needs water molecules");
    GuessNet& net = I.sel ? I.cnet : I.net;
    if (I.sel == 1) {
        // the correction network's inputs are those of the last solve
        if (!I.cdesc_valid)
            return mbpol_fail(MBPOL_ERR_STATE, "the last solve did not start from the history predictor");
    } else {
        MBPOL_CUDA_OK(I.net.descriptors(st, I.nmol, I.K, I.d_off.p, I.d_nb.p, I.d_nbd.p, I.d_nnb.p, I.cap,
                                        I.last_box.L, I.last_box.periodic && I.pme, I.d_E0.p));
    }
    if (host_out) {
        MBPOL_CUDA_OK(cudaMemcpyAsync(host_out, net.d_desc(), sizeof(float) * guess::kIn * (size_t)I.nmol,
                                      cudaMemcpyDeviceToHost, st));
        MBPOL_CUDA_OK(cudaStreamSynchronize(st));
    }
    return MBPOL_OK;
}

mbpol_status ElecEngine::guess_collect(cudaStream_t st) {
    ElecImpl& I = *impl_;
    if (!I.converged) return mbpol_fail(MBPOL_ERR_STATE, "the last solve did not converge; nothing to collect");
    mbpol_status s = guess_descriptors(st, nullptr);
    if (s) return s;
    if (I.sel == 1)
        MBPOL_CUDA_OK(I.cnet.collect(st, I.nmol, I.K, I.d_mud.p, I.d_mubase.p));
    else
        MBPOL_CUDA_OK(I.net.collect(st, I.nmol, I.K, I.d_mud.p));
    return MBPOL_OK;
}

mbpol_status ElecEngine::guess_train(cudaStream_t st, int steps, int batch, double lr, unsigned long long seed,
                                     double* loss) {
    GuessNet& net = impl_->sel ? impl_->cnet : impl_->net;
    if (net.num_samples() <= 0) return mbpol_fail(MBPOL_ERR_STATE, "no training samples collected");
    if (steps <= 0 || batch <= 0 || !(lr > 0)) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "bad training arguments");
    MBPOL_CUDA_OK(net.train(st, steps, batch, lr, seed, loss));
    return MBPOL_OK;
}

mbpol_status ElecEngine::guess_get_params(float* block) {
    GuessNet& net = impl_->sel ? impl_->cnet : impl_->net;
    if (!block) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null parameter block");
    if (!net.ready()) return mbpol_fail(MBPOL_ERR_STATE, "the network has no parameters yet");
    MBPOL_CUDA_OK(net.get_params(block));
    return MBPOL_OK;
}

mbpol_status ElecEngine::guess_set_params(const float* block) {
    if (!block) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null parameter block");
    if (impl_->sel == 1) {
        MBPOL_CUDA_OK(impl_->cnet.set_params(block));
        return MBPOL_OK;
    }
    MBPOL_CUDA_OK(impl_->net.set_params(block));
    impl_->hist_levels = 0;
    impl_->have_mprev = false;
    return MBPOL_OK;
}

mbpol_status ElecEngine::guess_loss_grad(cudaStream_t st, const float* X, const float* T, int n, double* loss,
                                         float* grad, float* Y) {
    GuessNet& net = impl_->sel ? impl_->cnet : impl_->net;
    if (!X || !T || !loss || !grad || !Y || n <= 0) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "bad arguments");
    if (!net.ready()) return mbpol_fail(MBPOL_ERR_STATE, "the network has no parameters yet");
    MBPOL_CUDA_OK(net.loss_grad(st, X, T, n, loss, grad, Y));
    return MBPOL_OK;
}

long ElecEngine::guess_num_samples() const { return (impl_->sel ? impl_->cnet : impl_->net).num_samples(); }

bool ElecEngine::converged() const { return impl_->converged; }
int ElecEngine::iterations() const { return impl_->iterations; }
long ElecEngine::num_site_pairs() const { return impl_->h_npair ? (long)(*impl_->h_npair / 2) : 0; }
std::string ElecEngine::convergence_message() const {
    std::ostringstream m;
    m << "Induced dipoles did not converge:  iterations=" << impl_->iterations << " eps=" << impl_->epsilon;
    for (size_t c = 0; c < impl_->cl_conv.size(); ++c)
        if (!impl_->cl_conv[c]) {
            m << " (cluster " << c << " after " << impl_->cl_iters[c] << " iterations)";
            break;
        }
    return m.str();
}

mbpol_status ElecEngine::set_clusters(const int* cluster_of_particle, int ncl, double* cluster_energy, int stride) {
    ElecImpl& I = *impl_;
    I.ncl = 0;
    I.cl_sink = ClusterSink();
    I.cl_iters.clear();
    I.cl_conv.clear();
    I.cap = 0;
    I.have_prev = false;
    I.have_mprev = false;
    I.hist_levels = 0;
    if (ncl <= 0 || !cluster_of_particle) return MBPOL_OK;
    if (I.pme) return mbpol_fail(MBPOL_ERR_STATE, "batched clusters need the NoCutoff electrostatics method");
    std::vector<int> mcl(I.nmol), count(ncl, 0);
    I.cl_nsites.assign(ncl, 0);
    for (int m = 0; m < I.nmol; ++m) {
        const int c = cluster_of_particle[I.K * m];
        if (c < 0 || c >= ncl) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "cluster index out of range");
        for (int a = 1; a < I.K; ++a)
            if (cluster_of_particle[I.K * m + a] != c)
                return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "the sites of one molecule are in different clusters");
        mcl[m] = c;
        ++count[c];
        I.cl_nsites[c] += I.K;
    }
    I.max_cl_mol = 0;
    for (int c = 0; c < ncl; ++c) I.max_cl_mol = std::max(I.max_cl_mol, count[c]);
    MBPOL_CUDA_OK(I.d_mcl.ensure(I.nmol));
    MBPOL_CUDA_OK(cudaMemcpy(I.d_mcl.p, mcl.data(), sizeof(int) * (size_t)I.nmol, cudaMemcpyHostToDevice));
    MBPOL_CUDA_OK(I.d_cstate.ensure(ncl));
    MBPOL_CUDA_OK(I.d_eps2c.ensure(ncl));
    MBPOL_CUDA_OK(I.d_cl_nsites.ensure(ncl));
    MBPOL_CUDA_OK(I.d_cl_its.ensure(ncl));
    MBPOL_CUDA_OK(I.d_cl_conv.ensure(ncl));
    MBPOL_CUDA_OK(I.d_cl_cur.ensure(ncl));
    MBPOL_CUDA_OK(I.d_rounds.ensure(1));
    MBPOL_CUDA_OK(cudaMemcpy(I.d_cl_nsites.p, I.cl_nsites.data(), sizeof(int) * (size_t)ncl, cudaMemcpyHostToDevice));
    std::vector<int> members, start;
    cluster_members(mcl.data(), I.nmol, ncl, members, start);
    MBPOL_CUDA_OK(I.d_cl_members.ensure(members.size()));
    MBPOL_CUDA_OK(I.d_cl_start.ensure(start.size()));
    MBPOL_CUDA_OK(cudaMemcpy(I.d_cl_members.p, members.data(), sizeof(int) * members.size(), cudaMemcpyHostToDevice));
    MBPOL_CUDA_OK(cudaMemcpy(I.d_cl_start.p, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice));
    I.cl_candidates = CandidateSet();
    I.cl_candidates.mode = 1;
    I.cl_candidates.members = I.d_cl_members.p;
    I.cl_candidates.start = I.d_cl_start.p;
    I.cl_candidates.group = I.d_mcl.p;
    I.ncl = ncl;
    I.cl_sink.wcl = I.d_mcl.p;
    I.cl_sink.e = cluster_energy;
    I.cl_sink.stride = stride;
    return MBPOL_OK;
}

const std::vector<int>& ElecEngine::cluster_iterations() const { return impl_->cl_iters; }

}  // namespace mbpol
