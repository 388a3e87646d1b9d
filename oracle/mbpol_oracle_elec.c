/*
 * Oracle C port, electrostatics (TEST INFRASTRUCTURE ONLY; see mbpol_oracle.c).
 * FP64 restatement of platforms/reference/src/MBPolReferenceElectrostaticsForce.cpp
 * for water systems laid out O, H1, H2, M (4 sites per molecule) with charge
 * redistribution:
 *   charges + derivatives  computeWaterCharge :2793-3096
 *   Thole scale factors    getAndScaleInverseRs :261-334, ...justScaleTCC :336-359,
 *                          incomplete gamma (gammq.cpp:133-178: series / Lentz CF)
 *   fixed field            NoCutoff :361-420; PME real space :1342-1407, reciprocal :1409-1439
 *   induced dipoles        SOR (omega 0.55) :488-616; PME pair term :2369-2470, self :2357-2364
 *   energy, forces         NoCutoff :649-836; PME direct :2510-2716, reciprocal :2113-2265,
 *                          self :2472-2508, charge derivatives :2767-2773
 *   PME                    moduli :1248-1340, splines :1446-1554, potentials :1715-2111
 * The reference's two identical dipole sets are one set here.  Pair loops are
 * O(N^2) with a cutoff test, as in the reference.  `row_stride` > 1 restricts
 * the outer loop of the direct-space sums to every row_stride-th site (timing
 * samples only; results are then partial).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

static double o_now(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

#define ELECTRIC 138.9354558456
#define DEBYE 48.033324
#define SOR 0.55
#define SQRT_PI 1.77245385091

typedef struct {
    double r[3], q, damp, pol;
    int mol, type;
    double dq[3][3];
} OSite;

typedef struct {
    int n, pme, grid[3], row_stride;
    double alpha, rc2, box[3], thole[5];
    OSite* s;
} OCtx;

/* --- incomplete gamma Q(a, x) (Numerical Recipes: series / Lentz) --- */
static double o_gammln(double xx) {
    /* Lanczos approximation, g = 5, n = 6 (Numerical Recipes 2nd ed. 6.1) */
    static const double cof[6] = {76.18009172947146, -86.50532032941677, 24.01409824083091,
                                  -1.231739572450155, 0.1208650973866179e-2, -0.5395239384953e-5};
    double x = xx, y = xx, tmp = x + 5.5;
    tmp -= (x + 0.5) * log(tmp);
    double ser = 1.000000000190015;
    for (int j = 0; j < 6; ++j) ser += cof[j] / ++y;
    return -tmp + log(2.5066282746310005 * ser / x);
}
static double o_gammq(double a, double x) {
    if (x <= 0.0) return 1.0;
    const double gln = o_gammln(a), EPS = 2.2e-16, FPMIN = 1e-300;
    if (x < a + 1.0) {
        double ap = a, sum = 1.0 / a, del = sum;
        for (int n = 0; n < 1000; ++n) {
            ap += 1.0;
            del *= x / ap;
            sum += del;
            if (fabs(del) < fabs(sum) * EPS) break;
        }
        return 1.0 - sum * exp(-x + a * log(x) - gln);
    }
    double b = x + 1.0 - a, c = 1.0 / FPMIN, d = 1.0 / b, h = d;
    for (int i = 1; i < 1000; ++i) {
        const double an = -i * (i - a);
        b += 2.0;
        d = an * d + b;
        if (fabs(d) < FPMIN) d = FPMIN;
        c = b + an / c;
        if (fabs(c) < FPMIN) c = FPMIN;
        d = 1.0 / d;
        const double del = d * c;
        h *= del;
        if (fabs(del - 1.0) <= EPS) break;
    }
    return exp(-x + a * log(x) - gln) * h;
}

enum { TCC = 0, TCD = 1, TDD = 2, TDDOH = 3, TDDHH = 4 };

/* Thole scale (justScale form) of order 1/3/5/7 for site pair (i, k). */
static double o_scale(const OCtx* C, const OSite* a, const OSite* b, double r, int order, int itype) {
    double g = C->thole[itype];
    if (itype == TDD) {
        if (a->mol == b->mol) g = (a->type == 0 || b->type == 0) ? C->thole[TDDOH] : C->thole[TDDHH];
        else g = C->thole[TDD];
    }
    const double damp = pow(a->damp * b->damp, 1.0 / 6.0);
    if (!(damp != 0.0 && damp > -50.0)) return 1.0;
    const double ratio = pow(r / damp, 4), e = exp(-g * ratio);
    switch (order) {
        case 1: return 1.0 - e + pow(g, 0.25) * (r / damp) * exp(o_gammln(0.75)) * o_gammq(0.75, g * ratio);
        case 3: return 1.0 - e;
        case 5: return (1.0 - e) - (4. / 3.) * g * e * ratio;
        default: return ((1.0 - e) - (4. / 3.) * g * e * ratio) - (4. / 15.) * g * (4. * g * ratio - 1.) * e * ratio;
    }
}

static void o_delta(const OCtx* C, const OSite* a, const OSite* b, double* d) {
    for (int k = 0; k < 3; ++k) {
        d[k] = b->r[k] - a->r[k];
        if (C->pme) d[k] -= floor(d[k] / C->box[k] + 0.5) * C->box[k];
    }
}

static void o_bn(double alpha, double r, double bn[4]) {
    const double r2 = r * r, ra = alpha * r;
    bn[0] = erfc(ra) / r;
    const double al2 = 2.0 * alpha * alpha, ex = exp(-ra * ra);
    double a2n = alpha > 0 ? 1.0 / (SQRT_PI * alpha) : 0.0;
    a2n *= al2;
    bn[1] = (bn[0] + a2n * ex) / r2;
    a2n *= al2;
    bn[2] = (3.0 * bn[1] + a2n * ex) / r2;
    a2n *= al2;
    bn[3] = (5.0 * bn[2] + a2n * ex) / r2;
}

/* ---------------------------------------------------------------- PME */
typedef struct {
    double re, im;
} ocplx;

static int o_smallest_factor(int n) {
    for (int p = 2; p * p <= n; ++p)
        if (n % p == 0) return p;
    return n;
}
/* out[k] = sum_j in[j*stride] exp(sign 2 pi i j k / n), mixed radix */
static void o_fft1(const ocplx* in, int stride, ocplx* out, int n, int sign) {
    if (n == 1) {
        out[0] = in[0];
        return;
    }
    const int p = o_smallest_factor(n), m = n / p;
    ocplx* sub = (ocplx*)malloc(sizeof(ocplx) * (size_t)n);
    if (p == n) {
        for (int j = 0; j < n; ++j) sub[j] = in[j * stride];
    } else {
        for (int r = 0; r < p; ++r) o_fft1(in + r * stride, stride * p, sub + (size_t)r * m, m, sign);
    }
    for (int k = 0; k < n; ++k) {
        double sr = 0, si = 0;
        for (int r = 0; r < p; ++r) {
            const ocplx v = p == n ? sub[r] : sub[(size_t)r * m + (k % m)];
            const double a = sign * 2.0 * M_PI * (double)((long)r * k % n) / n;
            const double c = cos(a), s = sin(a);
            sr += v.re * c - v.im * s;
            si += v.re * s + v.im * c;
        }
        out[k].re = sr;
        out[k].im = si;
    }
    free(sub);
}
static void o_fft3(ocplx* g, const int* N, int sign) {
    const int nx = N[0], ny = N[1], nz = N[2];
    int nm = nx > ny ? nx : ny;
    nm = nm > nz ? nm : nz;
    ocplx* res = (ocplx*)malloc(sizeof(ocplx) * (size_t)nm);
    for (int x = 0; x < nx; ++x)
        for (int y = 0; y < ny; ++y) {
            ocplx* b = g + ((size_t)x * ny + y) * nz;
            o_fft1(b, 1, res, nz, sign);
            memcpy(b, res, sizeof(ocplx) * (size_t)nz);
        }
    for (int x = 0; x < nx; ++x)
        for (int z = 0; z < nz; ++z) {
            ocplx* b = g + (size_t)x * ny * nz + z;
            o_fft1(b, nz, res, ny, sign);
            for (int y = 0; y < ny; ++y) b[(size_t)y * nz] = res[y];
        }
    for (int y = 0; y < ny; ++y)
        for (int z = 0; z < nz; ++z) {
            ocplx* b = g + (size_t)y * nz + z;
            o_fft1(b, ny * nz, res, nx, sign);
            for (int x = 0; x < nx; ++x) b[(size_t)x * ny * nz] = res[x];
        }
    free(res);
}

/* order-5 B-spline weights and first/second derivatives at fraction w */
static void o_bspline(double w, double th[5], double d1[5], double d2[5]) {
    double A2[2] = {1 - w, w}, A3[3], A4[4];
    A3[2] = 0.5 * w * A2[1];
    A3[1] = 0.5 * ((1 + w) * A2[0] + (2 - w) * A2[1]);
    A3[0] = 0.5 * (1 - w) * A2[0];
    A4[3] = w * A3[2] / 3;
    A4[2] = ((w + 1) * A3[1] + (3 - w) * A3[2]) / 3;
    A4[1] = ((w + 2) * A3[0] + (2 - w) * A3[1]) / 3;
    A4[0] = (1 - w) * A3[0] / 3;
    th[4] = w * A4[3] / 4;
    th[3] = ((w + 1) * A4[2] + (4 - w) * A4[3]) / 4;
    th[2] = ((w + 2) * A4[1] + (3 - w) * A4[2]) / 4;
    th[1] = ((w + 3) * A4[0] + (2 - w) * A4[1]) / 4;
    th[0] = (1 - w) * A4[0] / 4;
    d1[4] = A4[3];
    for (int i = 3; i >= 1; --i) d1[i] = A4[i - 1] - A4[i];
    d1[0] = -A4[0];
    double E[4];
    E[3] = A3[2];
    E[2] = A3[1] - A3[2];
    E[1] = A3[0] - A3[1];
    E[0] = -A3[0];
    d2[4] = E[3];
    for (int i = 3; i >= 1; --i) d2[i] = E[i - 1] - E[i];
    d2[0] = -E[0];
}

static void o_moduli(int size, double* mod) {
    double bs[8] = {0, 0, 0, 0, 0, 0, 0, 0}, arr[5];
    const double x = 0.0;
    arr[0] = 1.0 - x;
    arr[1] = x;
    for (int k = 2; k < 5; ++k) {
        const double dn = 1.0 / k;
        arr[k] = x * arr[k - 1] * dn;
        for (int i = 1; i < k; ++i) arr[k - i] = ((x + i) * arr[k - i - 1] + ((k - i + 1) - x) * arr[k - i]) * dn;
        arr[0] = (1.0 - x) * arr[0] * dn;
    }
    for (int i = 2; i <= 6; ++i) bs[i] = arr[i - 2];
    for (int i = 0; i < size; ++i) {
        double s1 = 0, s2 = 0;
        for (int j = 1; j <= size && j < 8; ++j) {
            const double a = 2.0 * M_PI / size * i * (j - 1);
            s1 += bs[j] * cos(a);
            s2 += bs[j] * sin(a);
        }
        mod[i] = s1 * s1 + s2 * s2;
    }
    if (mod[0] < 1e-7) mod[0] = 0.5 * mod[1];
    for (int i = 1; i < size - 1; ++i)
        if (mod[i] < 1e-7) mod[i] = 0.5 * (mod[i - 1] + mod[i + 1]);
    if (mod[size - 1] < 1e-7) mod[size - 1] = 0.5 * mod[size - 2];
    for (int i = 1; i <= size; ++i) {
        int k = i - 1;
        if (i > size / 2) k -= size;
        double z = 1.0;
        if (k) {
            double s1 = 1, s2 = 1;
            const double fac = M_PI * k / size;
            for (int j = 1; j <= 50; ++j) {
                double a = fac / (fac + M_PI * j);
                s1 += pow(a, 5);
                s2 += pow(a, 10);
                a = fac / (fac - M_PI * j);
                s1 += pow(a, 5);
                s2 += pow(a, 10);
            }
            z = s2 / s1;
        }
        mod[i - 1] *= z * z;
    }
}

typedef struct {
    int ig[3];
    double th[3][5], d1[3][5], d2[3][5];
} OSpl;

static void o_splines(const OCtx* C, OSpl* sp) {
    for (int i = 0; i < C->n; ++i)
        for (int d = 0; d < 3; ++d) {
            const double x = C->s[i].r[d] - floor(C->s[i].r[d] / C->box[d] + 0.5) * C->box[d];
            const double w = x / C->box[d];
            const double fr = C->grid[d] * (w - (int)(w + 0.5) + 0.5);
            const int ifr = (int)fr;
            int ig = ifr - 4;
            if (ig < 0) ig += C->grid[d];
            sp[i].ig[d] = ig;
            o_bspline(fr - ifr, sp[i].th[d], sp[i].d1[d], sp[i].d2[d]);
        }
}

/* spread charges (mode 0) or dipoles (mode 1), convolve, and gather the
 * potential and its derivatives up to second order (phi[10*i..]). */
static void o_recip(const OCtx* C, const OSpl* sp, int mode, const double* mu, const double* mods[3], double* phi) {
    const int* N = C->grid;
    const size_t G = (size_t)N[0] * N[1] * N[2];
    ocplx* g = (ocplx*)calloc(G, sizeof(ocplx));
    double sc[3];
    for (int d = 0; d < 3; ++d) sc[d] = N[d] / C->box[d];
    for (int i = 0; i < C->n; ++i) {
        const OSpl* p = sp + i;
        for (int a = 0; a < 5; ++a)
            for (int b = 0; b < 5; ++b)
                for (int c = 0; c < 5; ++c) {
                    double v;
                    if (mode == 0) v = C->s[i].q * p->th[0][a] * p->th[1][b] * p->th[2][c];
                    else
                        v = sc[0] * mu[3 * i] * p->d1[0][a] * p->th[1][b] * p->th[2][c] +
                            sc[1] * mu[3 * i + 1] * p->th[0][a] * p->d1[1][b] * p->th[2][c] +
                            sc[2] * mu[3 * i + 2] * p->th[0][a] * p->th[1][b] * p->d1[2][c];
                    const int x = (p->ig[0] + a) % N[0], y = (p->ig[1] + b) % N[1], z = (p->ig[2] + c) % N[2];
                    g[((size_t)x * N[1] + y) * N[2] + z].re += v;
                }
    }
    o_fft3(g, N, -1);
    const double ef = M_PI * M_PI / (C->alpha * C->alpha);
    const double sf = 1.0 / (M_PI * C->box[0] * C->box[1] * C->box[2]);
    for (int kx = 0; kx < N[0]; ++kx)
        for (int ky = 0; ky < N[1]; ++ky)
            for (int kz = 0; kz < N[2]; ++kz) {
                const size_t idx = ((size_t)kx * N[1] + ky) * N[2] + kz;
                if (!kx && !ky && !kz) {
                    g[idx].re = g[idx].im = 0.0;
                    continue;
                }
                const int mx = kx < (N[0] + 1) / 2 ? kx : kx - N[0];
                const int my = ky < (N[1] + 1) / 2 ? ky : ky - N[1];
                const int mz = kz < (N[2] + 1) / 2 ? kz : kz - N[2];
                const double hx = mx / C->box[0], hy = my / C->box[1], hz = mz / C->box[2];
                const double m2 = hx * hx + hy * hy + hz * hz;
                const double et = sf * exp(-ef * m2) / (m2 * mods[0][kx] * mods[1][ky] * mods[2][kz]);
                g[idx].re *= et;
                g[idx].im *= et;
            }
    o_fft3(g, N, 1);
    for (int i = 0; i < C->n; ++i) {
        const OSpl* p = sp + i;
        double* P = phi + 10 * i;
        memset(P, 0, 10 * sizeof(double));
        for (int a = 0; a < 5; ++a)
            for (int b = 0; b < 5; ++b)
                for (int c = 0; c < 5; ++c) {
                    const int x = (p->ig[0] + a) % N[0], y = (p->ig[1] + b) % N[1], z = (p->ig[2] + c) % N[2];
                    const double v = g[((size_t)x * N[1] + y) * N[2] + z].re;
                    const double tx = p->th[0][a], ty = p->th[1][b], tz = p->th[2][c];
                    P[0] += v * tx * ty * tz;
                    P[1] += v * p->d1[0][a] * ty * tz;
                    P[2] += v * tx * p->d1[1][b] * tz;
                    P[3] += v * tx * ty * p->d1[2][c];
                    P[4] += v * p->d2[0][a] * ty * tz;
                    P[5] += v * tx * p->d2[1][b] * tz;
                    P[6] += v * tx * ty * p->d2[2][c];
                    P[7] += v * p->d1[0][a] * p->d1[1][b] * tz;
                    P[8] += v * p->d1[0][a] * ty * p->d1[2][c];
                    P[9] += v * tx * p->d1[1][b] * p->d1[2][c];
                }
    }
    free(g);
}

/* ------------------------------------------------------------- charges */
static void o_water_charge(OSite* O, OSite* H1, OSite* H2, OSite* M);
#include "oracle_dms.h"

/* fixed (permanent) field of the last orc_electrostatics call, FP64
 * [n][3], before multiplication by the polarisabilities (the field the
 * solver starts from; reference :361-420, :1342-1439) */
static double* o_last_E0 = NULL;
static int o_last_n = 0;
int orc_last_fixed_field(int n, double* out) {
    if (!o_last_E0 || n != o_last_n) return 1;
    memcpy(out, o_last_E0, 3 * (size_t)n * sizeof(double));
    return 0;
}

/* PME fixed-field Thole sign: 1 the reference's (s3 - 1)/r^3 subtraction
 * (MBPolReferenceElectrostaticsForce.cpp:1377-1391), -1 the form whose
 * forces are the gradient of the energy, bn1 - (1 - s3)/r^3 (the same
 * damping as the energy, :2609-2626).  Intramolecular pairs are unaffected. */
static double o_fixed_thole_sign = 1.0;
void orc_set_pme_fixed_field(int consistent) { o_fixed_thole_sign = consistent ? -1.0 : 1.0; }

/* positions, charges (after redistribution) and converged induced dipoles
 * of the last orc_electrostatics call: [n][7] = r[3], q, mu[3] */
static double* o_last_state = NULL;
static int o_last_state_n = 0, o_last_pme = 0;
static double o_last_box[3];

/* Electrostatic potential at npts points from the last orc_electrostatics
 * call (MBPolReferenceElectrostaticsForce.cpp:1023-1085): for every point g
 * the sum over all sites of q/r - mu.(r_i - g)/r^3 with d = r_i - g
 * minimum-imaged under PME, times 138.9354558456 (kJ/mol/e). */
int orc_electrostatic_potential(int npts, const double* points, double* out) {
    if (!o_last_state) return 1;
    for (int p = 0; p < npts; ++p) {
        double acc = 0.0;
        for (int i = 0; i < o_last_state_n; ++i) {
            const double* S = o_last_state + 7 * i;
            double d[3];
            for (int k = 0; k < 3; ++k) {
                d[k] = S[k] - points[3 * p + k];
                if (o_last_pme) d[k] -= floor(d[k] / o_last_box[k] + 0.5) * o_last_box[k];
            }
            const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2], r = sqrt(r2);
            acc += S[3] / r - (S[4] * d[0] + S[5] * d[1] + S[6] * d[2]) / (r2 * r);
        }
        out[p] = acc * ELECTRIC;
    }
    return 0;
}

/* System multipole moments from the last orc_electrostatics call
 * (calculateMBPolSystemElectrostaticsMoments,
 * MBPolReferenceElectrostaticsForce.cpp:923-1021), about the centre of mass
 * of `mass` (none when the total mass is 0): out[0] net charge (e),
 * out[1..3] dipole (Debye: e nm x 10 x 4.80321), out[4..12] the traceless
 * quadrupole 0.5 (Q_ab - delta_ab tr/3) row by row, Q_ab = sum q r_a r_b +
 * r_a mu_b + r_b mu_a, in e nm^2 x 100 x 3 x 4.80321. */
int orc_system_moments(const double* mass, double* out) {
    if (!o_last_state) return 1;
    const int n = o_last_state_n;
    double mt = 0.0, com[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < n; ++i) {
        mt += mass[i];
        for (int k = 0; k < 3; ++k) com[k] += o_last_state[7 * i + k] * mass[i];
    }
    if (mt > 0.0)
        for (int k = 0; k < 3; ++k) com[k] *= 1.0 / mt;
    double q = 0.0, dp[3] = {0.0, 0.0, 0.0}, Q[3][3] = {{0.0}};
    for (int i = 0; i < n; ++i) {
        const double* S = o_last_state + 7 * i;
        double r[3];
        for (int k = 0; k < 3; ++k) r[k] = S[k] - com[k];
        q += S[3];
        for (int k = 0; k < 3; ++k) dp[k] += r[k] * S[3] + S[4 + k];
        for (int a = 0; a < 3; ++a)
            for (int b = a; b < 3; ++b) Q[a][b] += r[a] * r[b] * S[3] + r[a] * S[4 + b] + r[b] * S[4 + a];
    }
    const double debye = 4.80321, tr = (Q[0][0] + Q[1][1] + Q[2][2]) / 3.0;
    out[0] = q;
    for (int k = 0; k < 3; ++k) out[1 + k] = dp[k] * 10.0 * debye;
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < 3; ++b) {
            const double v = a <= b ? Q[a][b] : Q[b][a];
            out[4 + 3 * a + b] = 0.5 * (v - (a == b ? tr : 0.0)) * 100.0 * 3.0 * debye;
        }
    return 0;
}

/* -------------------------------------------------------------- solver */
int orc_electrostatics(int n, const double* pos, const double* box, int pme, double alpha, const int* grid,
                       double rc, double target_eps, int maxiter, const double* thole, int row_stride, double* f,
                       double* energy, double* dip_out, int* iters, double* timing) {
    /* timing (optional, 6 doubles): [0] charges+splines+fixed reciprocal,
     * [1] fixed-field direct loop, [2] reciprocal per iteration (summed),
     * [3] induced direct loops (summed), [4] energy/force direct loop,
     * [5] final reciprocal + per-site terms */
    double tm[6] = {0, 0, 0, 0, 0, 0}, t0 = o_now();
    OCtx C;
    memset(&C, 0, sizeof C);
    C.n = n;
    C.pme = pme;
    C.alpha = alpha;
    C.rc2 = pme ? rc * rc : 1e300;
    C.row_stride = row_stride > 0 ? row_stride : 1;
    for (int k = 0; k < 5; ++k) C.thole[k] = thole[k];
    if (pme)
        for (int k = 0; k < 3; ++k) {
            C.box[k] = box[k];
            C.grid[k] = grid[k];
        }
    C.s = (OSite*)calloc((size_t)n, sizeof(OSite));
    static const double qd[4] = {-5.1966000e-01, 2.5983000e-01, 2.5983000e-01, 0.0};
    static const double dd[4] = {0.00131, 0.000294, 0.000294, 0.00131};
    static const double pl[4] = {0.00131, 0.000294, 0.000294, 0.0};
    for (int i = 0; i < n; ++i) {
        memcpy(C.s[i].r, pos + 3 * i, 24);
        C.s[i].q = qd[i % 4];
        C.s[i].damp = dd[i % 4];
        C.s[i].pol = pl[i % 4];
        C.s[i].mol = i / 4;
        C.s[i].type = (i % 4 == 0) ? 0 : (i % 4 == 3 ? 2 : 1);
    }
    for (int m = 0; m < n / 4; ++m) o_water_charge(&C.s[4 * m], &C.s[4 * m + 1], &C.s[4 * m + 2], &C.s[4 * m + 3]);
    double* E0 = (double*)calloc(3 * (size_t)n, sizeof(double));
    double* Ei = (double*)calloc(3 * (size_t)n, sizeof(double));
    double* mu = (double*)calloc(3 * (size_t)n, sizeof(double));
    double* phif = NULL, *phim = NULL, *mods[3] = {NULL, NULL, NULL};
    OSpl* sp = NULL;
    double sc[3] = {0, 0, 0};
    if (pme) {
        phif = (double*)calloc(10 * (size_t)n, sizeof(double));
        phim = (double*)calloc(10 * (size_t)n, sizeof(double));
        sp = (OSpl*)calloc((size_t)n, sizeof(OSpl));
        for (int d = 0; d < 3; ++d) {
            mods[d] = (double*)malloc(sizeof(double) * (size_t)grid[d]);
            o_moduli(grid[d], mods[d]);
            sc[d] = grid[d] / box[d];
        }
        o_splines(&C, sp);
        o_recip(&C, sp, 0, NULL, (const double**)mods, phif);
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) E0[3 * i + k] = -sc[k] * phif[10 * i + 1 + k];
    }
    tm[0] = o_now() - t0;
    t0 = o_now();
    /* fixed field, direct space */
    for (int i = 0; i < n; i += C.row_stride)
        for (int j = i + 1; j < n; ++j) {
            OSite *a = &C.s[i], *b = &C.s[j];
            const int same = a->mol == b->mol;
            if (!pme && same) continue;
            double d[3];
            o_delta(&C, a, b, d);
            const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (r2 > C.rc2) continue;
            const double r = sqrt(r2);
            double fac;
            if (pme) {
                double bn[4];
                o_bn(alpha, r, bn);
                const double s3 = same ? 2.0 : o_scale(&C, a, b, r, 3, TCC);
                fac = bn[1] - (same ? 1.0 : o_fixed_thole_sign) * (s3 - 1.0) / (r2 * r);
            } else {
                fac = o_scale(&C, a, b, r, 3, TCC) / (r2 * r);
            }
            for (int k = 0; k < 3; ++k) {
                E0[3 * i + k] -= d[k] * fac * b->q;
                E0[3 * j + k] += d[k] * fac * a->q;
            }
        }
    for (int i = 0; i < n; ++i)
        for (int k = 0; k < 3; ++k) mu[3 * i + k] = C.s[i].pol * E0[3 * i + k];
    /* keep the fixed field for orc_last_fixed_field */
    free(o_last_E0);
    o_last_E0 = (double*)malloc(3 * (size_t)n * sizeof(double));
    memcpy(o_last_E0, E0, 3 * (size_t)n * sizeof(double));
    o_last_n = n;
    tm[1] = o_now() - t0;
    /* SOR iterations */
    const double self = pme ? (4.0 / 3.0) * alpha * alpha * alpha / SQRT_PI : 0.0;
    double current = 1e50, eps = 0.0;
    int it = 0, done = 0, conv = 0;
    while (!done) {
        memset(Ei, 0, sizeof(double) * 3 * (size_t)n);
        t0 = o_now();
        if (pme) {
            o_recip(&C, sp, 1, mu, (const double**)mods, phim);
            for (int i = 0; i < n; ++i)
                for (int k = 0; k < 3; ++k) Ei[3 * i + k] = -sc[k] * phim[10 * i + 1 + k] + self * mu[3 * i + k];
        }
        tm[2] += o_now() - t0;
        t0 = o_now();
        for (int i = 0; i < n; i += C.row_stride)
            for (int j = i + 1; j < n; ++j) {
                OSite *a = &C.s[i], *b = &C.s[j];
                double d[3];
                o_delta(&C, a, b, d);
                const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
                if (r2 > C.rc2) continue;
                const double r = sqrt(r2);
                const double s3 = o_scale(&C, a, b, r, 3, TDD), s5 = o_scale(&C, a, b, r, 5, TDD);
                double p1, p2;
                if (pme) {
                    double bn[4];
                    o_bn(alpha, r, bn);
                    p1 = (1.0 - s3) / (r2 * r) - bn[1];
                    p2 = bn[2] - 3.0 * (1.0 - s5) / (r2 * r2 * r);
                } else {
                    p1 = -s3 / (r2 * r);
                    p2 = 3.0 * s5 / (r2 * r2 * r);
                }
                const double dj = mu[3 * j] * d[0] + mu[3 * j + 1] * d[1] + mu[3 * j + 2] * d[2];
                const double di = mu[3 * i] * d[0] + mu[3 * i + 1] * d[1] + mu[3 * i + 2] * d[2];
                for (int k = 0; k < 3; ++k) {
                    Ei[3 * i + k] += d[k] * dj * p2 + mu[3 * j + k] * p1;
                    Ei[3 * j + k] += d[k] * di * p2 + mu[3 * i + k] * p1;
                }
            }
        tm[3] += o_now() - t0;
        double e2 = 0.0;
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < 3; ++k) {
                const double nv = C.s[i].pol * (E0[3 * i + k] + Ei[3 * i + k]);
                const double dl = nv - mu[3 * i + k];
                mu[3 * i + k] += SOR * dl;
                e2 += dl * dl;
            }
        eps = SOR * DEBYE * sqrt(e2 / n);
        if (eps < target_eps) {
            conv = 1;
            done = 1;
        } else if (current < eps || it >= maxiter) {
            done = 1;
        }
        current = eps;
        ++it;
    }
    /* energy and forces */
    t0 = o_now();
    double e = 0.0;
    double* phi = (double*)calloc((size_t)n, sizeof(double)); /* potential for charge derivatives */
    for (int i = 0; i < n; i += C.row_stride)
        for (int j = i + 1; j < n; ++j) {
            OSite *a = &C.s[i], *b = &C.s[j];
            const int same = a->mol == b->mol;
            double d[3];
            o_delta(&C, a, b, d);
            const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (r2 > C.rc2) continue;
            const double r = sqrt(r2), rr1 = 1.0 / r, rr3 = rr1 / r2, rr5 = 3.0 * rr3 / r2, rr7 = 5.0 * rr5 / r2;
            const double *mi = mu + 3 * i, *mj = mu + 3 * j;
            const double si = mi[0] * d[0] + mi[1] * d[1] + mi[2] * d[2];
            const double sj = mj[0] * d[0] + mj[1] * d[1] + mj[2] * d[2];
            const double mm = mi[0] * mj[0] + mi[1] * mj[1] + mi[2] * mj[2];
            double gl0 = a->q * b->q, gli = b->q * si - a->q * sj;
            const double s5DD = o_scale(&C, a, b, r, 5, TDD), s7DD = o_scale(&C, a, b, r, 7, TDD);
            double fo[3];
            if (pme) {
                double bn[4];
                o_bn(alpha, r, bn);
                const double s1CC = same ? 0.0 : o_scale(&C, a, b, r, 1, TCC);
                const double s3CD = same ? 0.0 : o_scale(&C, a, b, r, 3, TCD);
                const double s3CC = same ? 0.0 : o_scale(&C, a, b, r, 3, TCC);
                const double s5CD = same ? 0.0 : o_scale(&C, a, b, r, 5, TCD);
                e += bn[0] * gl0 + 0.5 * bn[1] * gli - rr1 * gl0 * (1 - s1CC) - 0.5 * rr3 * gli * (1 - s3CD);
                phi[i] += b->q * (bn[0] - rr1 * (1 - s1CC)) - sj * (bn[1] - rr3 * (1 - s3CD));
                phi[j] += a->q * (bn[0] - rr1 * (1 - s1CC)) + si * (bn[1] - rr3 * (1 - s3CD));
                const double cd = bn[1] * gl0 - (1 - s3CC) * rr3 * gl0 + bn[2] * (gli + mm) - bn[3] * si * sj -
                                  (rr5 * (gli * (1 - s5CD) + mm * (1 - s5DD)) - rr7 * si * sj * (1 - s7DD));
                const double ci = -b->q * bn[1] + b->q * rr3 * (1 - s3CD), cj = a->q * bn[1] - a->q * rr3 * (1 - s3CD);
                const double cdd = bn[2] - rr5 * (1 - s5DD);
                for (int k = 0; k < 3; ++k) fo[k] = d[k] * cd + mi[k] * (ci + sj * cdd) + mj[k] * (cj + si * cdd);
            } else {
                if (same) gl0 = gli = 0.0;
                const double s1CC = o_scale(&C, a, b, r, 1, TCC), s3CD = o_scale(&C, a, b, r, 3, TCD);
                const double s3CC = o_scale(&C, a, b, r, 3, TCC), s5CD = o_scale(&C, a, b, r, 5, TCD);
                e += rr1 * gl0 * s1CC + 0.5 * rr3 * gli * s3CD;
                const double g0 = rr3 * gl0 * s3CC + rr5 * gli * s5CD + rr5 * mm * s5DD - rr7 * si * sj * s7DD;
                for (int k = 0; k < 3; ++k) {
                    fo[k] = d[k] * g0 + (mi[k] * sj + mj[k] * si) * rr5 * s5DD;
                    if (!same) fo[k] += (mj[k] * a->q - mi[k] * b->q) * rr3 * s3CD;
                }
                if (!same) {
                    /* potential at each site from the other (TCC scaling), for the charge derivatives */
                    const double q3 = o_scale(&C, a, b, r, 3, TCC);
                    phi[i] += b->q * s1CC * rr1 - q3 * sj * rr3;
                    phi[j] += a->q * s1CC * rr1 + q3 * si * rr3;
                }
            }
            for (int k = 0; k < 3; ++k) {
                f[3 * i + k] -= ELECTRIC * fo[k];
                f[3 * j + k] += ELECTRIC * fo[k];
            }
        }
    tm[4] = o_now() - t0;
    t0 = o_now();
    if (pme) {
        o_recip(&C, sp, 1, mu, (const double**)mods, phim);
        static const int H[3][3] = {{4, 7, 8}, {7, 5, 9}, {8, 9, 6}};
        for (int i = 0; i < n; ++i) {
            const double* pf = phif + 10 * i;
            const double* pm = phim + 10 * i;
            const double q = C.s[i].q;
            e += 0.5 * q * pf[0];
            e += 0.5 * (sc[0] * mu[3 * i] * pf[1] + sc[1] * mu[3 * i + 1] * pf[2] + sc[2] * mu[3 * i + 2] * pf[3]);
            e += -q * q * alpha / SQRT_PI;
            phi[i] += pf[0] + pm[0] - 2.0 * q * alpha / SQRT_PI;
            for (int c = 0; c < 3; ++c) {
                double fd = 0.0;
                for (int k = 0; k < 3; ++k) fd += sc[k] * mu[3 * i + k] * (pf[H[c][k]] + pm[H[c][k]]);
                f[3 * i + c] -= ELECTRIC * sc[c] * (fd + q * (pf[1 + c] + pm[1 + c]));
            }
        }
    }
    /* charge-derivative forces: F_i -= f * sum_s dq_i[s] * phi(H1, H2, M of i's water) */
    for (int i = 0; i < n; ++i) {
        const int base = 4 * (i / 4);
        for (int s = 0; s < 3; ++s)
            for (int k = 0; k < 3; ++k) f[3 * i + k] -= ELECTRIC * C.s[i].dq[s][k] * phi[base + 1 + s];
    }
    tm[5] = o_now() - t0;
    if (timing) memcpy(timing, tm, sizeof tm);
    *energy = e * ELECTRIC;
    if (iters) *iters = it;
    if (dip_out) memcpy(dip_out, mu, sizeof(double) * 3 * (size_t)n);
    /* the state the electrostatic potential is evaluated from */
    free(o_last_state);
    o_last_state = (double*)malloc(7 * (size_t)n * sizeof(double));
    for (int i = 0; i < n; ++i) {
        memcpy(o_last_state + 7 * i, C.s[i].r, 24);
        o_last_state[7 * i + 3] = C.s[i].q;
        memcpy(o_last_state + 7 * i + 4, mu + 3 * i, 24);
    }
    o_last_state_n = n;
    o_last_pme = pme;
    if (pme) memcpy(o_last_box, box, 24);
    free(C.s);
    free(E0);
    free(Ei);
    free(mu);
    free(phi);
    if (pme) {
        free(phif);
        free(phim);
        free(sp);
        for (int d = 0; d < 3; ++d) free(mods[d]);
    }
    return conv ? 0 : 1;
}

/* White-box probes for the reference's own white-box tests
 * (platforms/reference/tests/TestReferenceMBPolElectrostaticsForce.cpp):
 * getAndScaleInverseRs (:80-131) as rr[0..3] = scale_k / r^k times the
 * reference's factors 1, 1, 3, 15 (orders 1, 3, 5, 7; thole parameter index
 * TCC with every parameter equal to `thole`), and computeWaterCharge
 * (:326-417): charges O, H1, H2, M and derivatives [particle O, H1, H2]
 * [charge of H1, H2, M][xyz] in e/nm. */
void orc_probe_thole(double r, double damp_i, double damp_j, double thole, double* rr) {
    OCtx C;
    memset(&C, 0, sizeof C);
    for (int k = 0; k < 5; ++k) C.thole[k] = thole;
    OSite a, b;
    memset(&a, 0, sizeof a);
    memset(&b, 0, sizeof b);
    a.damp = damp_i;
    b.damp = damp_j;
    b.mol = 1;
    const double rI = 1.0 / r, r2I = rI * rI;
    rr[0] = o_scale(&C, &a, &b, r, 1, TCC) * rI;
    rr[1] = o_scale(&C, &a, &b, r, 3, TCC) * rI * r2I;
    rr[2] = o_scale(&C, &a, &b, r, 5, TCC) * 3.0 * rI * r2I * r2I;
    rr[3] = o_scale(&C, &a, &b, r, 7, TCC) * 15.0 * rI * r2I * r2I * r2I;
}

void orc_probe_water_charges(const double* pos9, double* q4, double* d27) {
    OSite s[4];
    memset(s, 0, sizeof s);
    for (int i = 0; i < 3; ++i)
        for (int k = 0; k < 3; ++k) s[i].r[k] = pos9[3 * i + k];
    o_water_charge(&s[0], &s[1], &s[2], &s[3]);
    for (int i = 0; i < 4; ++i) q4[i] = s[i].q;
    for (int i = 0; i < 3; ++i)
        for (int o = 0; o < 3; ++o)
            for (int k = 0; k < 3; ++k) d27[9 * i + 3 * o + k] = s[i].dq[o][k];
}
