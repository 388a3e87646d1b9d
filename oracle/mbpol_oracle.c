/*
 * The oracle's C port: an FP64, single-threaded CPU restatement of the MB-pol
 * reference's algorithms.  TEST INFRASTRUCTURE ONLY -- it is the checker
 * (tests/, __graft_entry__.smoke()) and the timed CPU baseline (bench.py),
 * never part of the product library.
 *
 * It follows the reference's Reference platform:
 *   one-body     platforms/reference/src/MBPolReferenceOneBodyForce.cpp:69-221
 *   two-body     platforms/reference/src/MBPolReferenceTwoBodyForce.cpp:66-323,
 *                mbpol_2body_constants.cpp:10-111
 *   three-body   platforms/reference/src/MBPolReferenceThreeBodyForce.cpp:67-322,
 *                trimer list ReferenceThreeNeighborList.cpp:181-226 (chain rule)
 *   electrostatics platforms/reference/src/MBPolReferenceElectrostaticsForce.cpp
 *                (charges :2793-3096, Thole :261-359, fields :361-420 and
 *                :1342-1439, solver :438-647 and :2280-2470, energy/forces
 *                :649-836 and :2510-2777, PME :1248-2278), with the O(N^2)
 *                direct-space loops of the reference
 *   dispersion   python/mbpol.xml:37-108
 * The two- and three-body polynomials are evaluated from the extracted
 * monomial basis (data/poly*_basis.txt), walked as a trie (oracle/gen/),
 * which equals the reference's generated code to ~1e-15.
 * Units: nm, kJ/mol, kJ/mol/nm; forces are accumulated.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct {
    int level, var;
    double c;
} mbpol_prog_entry;

#include "poly2b_prog.h"
#include "poly3b_prog.h"

#define NM2A 10.0
#define CAL2J 4.184

/* ------------------------------------------------------------ utilities */
static void image_to(const double* a, double* b, const double* box) {
    if (!box) return;
    for (int k = 0; k < 3; ++k) b[k] += box[k] * floor((a[k] - b[k]) / box[k] + 0.5);
}
static double mimg(double d, double L) { return d - L * floor(d / L + 0.5); }
static double dot3(const double* a, const double* b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
static void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

/* Trie walk in FP64: value and gradient of sum_m c_m x^m. */
static double poly_eval(const mbpol_prog_entry* prog, int nprog, int nv, const double* x, double* g) {
    double P[6], V[6];
    int var[6], d = 0;
    P[0] = 1.0;
    V[0] = 0.0;
    for (int v = 0; v < nv; ++v) g[v] = 0.0;
    for (int e = 0; e < nprog; ++e) {
        while (d >= prog[e].level) {
            V[d - 1] += V[d] * x[var[d]];
            g[var[d]] += V[d] * P[d - 1];
            --d;
        }
        d = prog[e].level;
        var[d] = prog[e].var;
        P[d] = P[d - 1] * x[var[d]];
        V[d] = prog[e].c;
    }
    while (d > 0) {
        V[d - 1] += V[d] * x[var[d]];
        g[var[d]] += V[d] * P[d - 1];
        --d;
    }
    return V[0];
}

/* ------------------------------------------------------------- one-body */
/* Combined PES coefficients and index tables are passed in once
 * (orc_set_onebody_tables) from data/onebody_tables.txt. */
static double g_c5z[245];
static int g_idx[3][245];

void orc_set_onebody_tables(const double* c5z, const int* idx3) {
    memcpy(g_c5z, c5z, sizeof(g_c5z));
    for (int k = 0; k < 3; ++k)
        for (int j = 0; j < 245; ++j) g_idx[k][j] = idx3[245 * k + j];
}

static double onebody_one(const double* O, const double* H1, const double* H2, double* fO, double* fH1,
                          double* fH2) {
    const double Eh_J = 4.35974434e-18, Na = 6.02214129e+23, kcal_J = 4184.0, c0 = 299792458.0,
                 h_Js = 6.62606957e-34;
    const double cm1_kcalmol = (Eh_J * Na / kcal_J) / (1.0e-2 * Eh_J / (c0 * h_Js));
    const double f5z = 0.999677885, reoh = 0.958649, b1 = 2.0, roh = 0.9519607159623009,
                 alphaoh = 2.587949757553683, deoh = f5z * 42290.92019288289, phh2 = 12.66426998162947;
    const double phh1 = f5z * 16.94879431193463 * exp(phh2), costhe = -.24780227221366464506;
    double r1[3], r2[3], rh[3];
    for (int k = 0; k < 3; ++k) {
        r1[k] = (H1[k] - O[k]) * 10.0;
        r2[k] = (H2[k] - O[k]) * 10.0;
        rh[k] = (H1[k] - H2[k]) * 10.0;
    }
    const double d1 = sqrt(dot3(r1, r1)), d2 = sqrt(dot3(r2, r2)), dh = sqrt(dot3(rh, rh));
    const double costh = dot3(r1, r2) / (d1 * d2);
    const double e1 = exp(-alphaoh * (d1 - roh)), e2 = exp(-alphaoh * (d2 - roh));
    const double Va = deoh * (e1 * (e1 - 2.0) + e2 * (e2 - 2.0)), Vb = phh1 * exp(-phh2 * dh);
    const double dVa1 = 2.0 * alphaoh * deoh * e1 * (1.0 - e1) / d1, dVa2 = 2.0 * alphaoh * deoh * e2 * (1.0 - e2) / d2;
    const double dVb = -phh2 * Vb / dh;
    const double x1 = (d1 - reoh) / reoh, x2 = (d2 - reoh) / reoh, x3 = costh - costhe;
    double fm[3][16];
    for (int i = 0; i < 3; ++i) {
        fm[i][0] = 0.0;
        fm[i][1] = 1.0;
    }
    for (int j = 2; j < 16; ++j) {
        fm[0][j] = fm[0][j - 1] * x1;
        fm[1][j] = fm[1][j - 1] * x2;
        fm[2][j] = fm[2][j - 1] * x3;
    }
    const double efac = exp(-b1 * (pow(d1 - reoh, 2) + pow(d2 - reoh, 2)));
    double s0 = 0, s1 = 0, s2 = 0, s3 = 0;
    for (int j = 1; j < 245; ++j) {
        const int I = g_idx[0][j], J = g_idx[1][j], K = g_idx[2][j];
        const double c = g_c5z[j];
        s0 += c * (fm[0][I] * fm[1][J] + fm[0][J] * fm[1][I]) * fm[2][K];
        s1 += c * ((I - 1) * fm[0][I - 1] * fm[1][J] + (J - 1) * fm[0][J - 1] * fm[1][I]) * fm[2][K];
        s2 += c * ((J - 1) * fm[0][I] * fm[1][J - 1] + (I - 1) * fm[0][J] * fm[1][I - 1]) * fm[2][K];
        s3 += c * (fm[0][I] * fm[1][J] + fm[0][J] * fm[1][I]) * (K - 1) * fm[2][K - 1];
    }
    const double Vc = 2 * g_c5z[0] + efac * s0;
    const double e = (Va + Vb + Vc + 0.44739574026257) * cm1_kcalmol;
    const double dr1 = (-2 * b1 * efac * (d1 - reoh) * s0 + efac * s1 / reoh) / d1;
    const double dr2 = (-2 * b1 * efac * (d2 - reoh) * s0 + efac * s2 / reoh) / d2;
    const double dc = efac * s3;
    for (int k = 0; k < 3; ++k) {
        const double a = (dVa1 * r1[k] + dVb * rh[k] + dr1 * r1[k] + dc * (r2[k] / (d1 * d2) - costh * r1[k] / (d1 * d1))) *
                         cm1_kcalmol * CAL2J * 10;
        const double b = (dVa2 * r2[k] - dVb * rh[k] + dr2 * r2[k] + dc * (r1[k] / (d1 * d2) - costh * r2[k] / (d2 * d2))) *
                         cm1_kcalmol * CAL2J * 10;
        fH1[k] -= a;
        fH2[k] -= b;
        fO[k] += a + b;
    }
    return e * CAL2J;
}

double orc_onebody(int nw, const int* w, const double* pos, const double* box, double* f) {
    double e = 0.0;
    for (int i = 0; i < nw; ++i) {
        double O[3], H1[3], H2[3];
        memcpy(O, pos + 3 * w[3 * i], sizeof O);
        memcpy(H1, pos + 3 * w[3 * i + 1], sizeof H1);
        memcpy(H2, pos + 3 * w[3 * i + 2], sizeof H2);
        image_to(O, H1, box);
        image_to(O, H2, box);
        e += onebody_one(O, H1, H2, f + 3 * w[3 * i], f + 3 * w[3 * i + 1], f + 3 * w[3 * i + 2]);
    }
    return e;
}

/* ------------------------------------------------------------- two-body */
static const int V2[31][3] = {{1, 2, 0}, {4, 5, 0}, {0, 1, 0}, {0, 2, 0}, {3, 4, 0}, {3, 5, 0}, {1, 4, 1},
                              {1, 5, 1}, {2, 4, 1}, {2, 5, 1}, {0, 4, 1}, {0, 5, 1}, {3, 1, 1}, {3, 2, 1},
                              {0, 3, 1}, {6, 4, 0}, {6, 5, 0}, {7, 4, 0}, {7, 5, 0}, {8, 1, 0}, {8, 2, 0},
                              {9, 1, 0}, {9, 2, 0}, {0, 8, 0}, {0, 9, 0}, {3, 6, 0}, {3, 7, 0}, {6, 8, 0},
                              {6, 9, 0}, {7, 8, 0}, {7, 9, 0}};
/* mbpol_2body_constants.h:33-48 */
static const double K2[31] = {-6.480884773303821e-01, -6.480884773303821e-01, 1.674518993682975e+00, 1.674518993682975e+00,
                              1.674518993682975e+00,  1.674518993682975e+00,  1.148231864355956e+00, 1.148231864355956e+00,
                              1.148231864355956e+00,  1.148231864355956e+00,  1.205989761123099e+00, 1.205989761123099e+00,
                              1.205989761123099e+00,  1.205989761123099e+00,  1.395357065790959e+00, 7.347036852042255e-01,
                              7.347036852042255e-01,  7.347036852042255e-01,  7.347036852042255e-01, 7.347036852042255e-01,
                              7.347036852042255e-01,  7.347036852042255e-01,  7.347036852042255e-01, 7.998249864422826e-01,
                              7.998249864422826e-01,  7.998249864422826e-01,  7.998249864422826e-01, 7.960663960630585e-01,
                              7.960663960630585e-01,  7.960663960630585e-01,  7.960663960630585e-01};

static double twobody_pair(const int* wa, const int* wb, const double* pos, const double* box, double* f) {
    const double gi = -9.721486914088159e-02, go = 9.859272078406150e-02, r2i = 4.5, r2f = 6.5;
    double S[10][3];
    memcpy(S[0], pos + 3 * wa[0], 24);
    memcpy(S[1], pos + 3 * wa[1], 24);
    memcpy(S[2], pos + 3 * wa[2], 24);
    memcpy(S[3], pos + 3 * wb[0], 24);
    memcpy(S[4], pos + 3 * wb[1], 24);
    memcpy(S[5], pos + 3 * wb[2], 24);
    image_to(S[0], S[1], box);
    image_to(S[0], S[2], box);
    image_to(S[0], S[3], box);
    image_to(S[3], S[4], box);
    image_to(S[3], S[5], box);
    for (int i = 0; i < 6; ++i)
        for (int k = 0; k < 3; ++k) S[i][k] *= NM2A;
    double dOO[3] = {S[0][0] - S[3][0], S[0][1] - S[3][1], S[0][2] - S[3][2]};
    const double rOO = sqrt(dot3(dOO, dOO));
    if (rOO > r2f || rOO < 2.0) return 0.0;
    double oh[2][2][3];
    for (int m = 0; m < 2; ++m) {
        double a[3], b[3], c[3];
        for (int k = 0; k < 3; ++k) {
            a[k] = S[3 * m + 1][k] - S[3 * m][k];
            b[k] = S[3 * m + 2][k] - S[3 * m][k];
        }
        cross3(a, b, c);
        for (int k = 0; k < 3; ++k) {
            const double inp = S[3 * m][k] + (a[k] + b[k]) * 0.5 * gi;
            S[6 + 2 * m][k] = inp + c[k] * go;
            S[7 + 2 * m][k] = inp - c[k] * go;
            oh[m][0][k] = a[k];
            oh[m][1][k] = b[k];
        }
    }
    double x[31], gv[31][3], g[31];
    for (int n = 0; n < 31; ++n) {
        double d[3];
        for (int k = 0; k < 3; ++k) d[k] = S[V2[n][0]][k] - S[V2[n][1]][k];
        const double r = sqrt(dot3(d, d));
        const double r0 = n < 6 ? 1.0 : 4.0;
        const double e = exp(K2[n] * (r0 - r));
        double gg;
        if (V2[n][2]) {
            x[n] = e / r;
            gg = -(K2[n] + 1.0 / r) * x[n] / r;
        } else {
            x[n] = e;
            gg = -K2[n] * e / r;
        }
        for (int k = 0; k < 3; ++k) gv[n][k] = d[k] * gg;
    }
    const double E = poly_eval(poly2b_prog, POLY2B_NPROG, 31, x, g);
    double G[10][3];
    memset(G, 0, sizeof G);
    for (int n = 0; n < 31; ++n)
        for (int k = 0; k < 3; ++k) {
            G[V2[n][0]][k] += gv[n][k] * g[n];
            G[V2[n][1]][k] -= gv[n][k] * g[n];
        }
    for (int m = 0; m < 2; ++m) {
        double gm[3], t1[3], t2[3];
        for (int k = 0; k < 3; ++k) gm[k] = G[6 + 2 * m][k] - G[7 + 2 * m][k];
        cross3(oh[m][1], gm, t1);
        cross3(oh[m][0], gm, t2);
        for (int k = 0; k < 3; ++k) {
            const double gs = G[6 + 2 * m][k] + G[7 + 2 * m][k];
            const double inp = gs * 0.5 * gi;
            const double gh1 = inp + t1[k] * go, gh2 = inp - t2[k] * go;
            G[3 * m][k] += gs - (gh1 + gh2);
            G[3 * m + 1][k] += gh1;
            G[3 * m + 2][k] += gh2;
        }
    }
    double sw = 1.0, gsw = 0.0;
    if (rOO > r2i) {
        const double t1 = M_PI / (r2f - r2i), xx = (rOO - r2i) * t1;
        gsw = -sin(xx) * t1 / 2.0;
        sw = (1.0 + cos(xx)) / 2.0;
    }
    const int idx[6] = {wa[0], wa[1], wa[2], wb[0], wb[1], wb[2]};
    for (int i = 0; i < 6; ++i)
        for (int k = 0; k < 3; ++k) f[3 * idx[i] + k] += G[i][k] * sw * CAL2J * -10.;
    gsw *= E / rOO;
    for (int k = 0; k < 3; ++k) {
        f[3 * wa[0] + k] += gsw * dOO[k] * CAL2J * -10.;
        f[3 * wb[0] + k] -= gsw * dOO[k] * CAL2J * -10.;
    }
    return sw * E * CAL2J;
}

static double oo_dist(const int* w, int i, int j, const double* pos, const double* box) {
    double d2 = 0.0;
    for (int k = 0; k < 3; ++k) {
        double d = pos[3 * w[3 * j] + k] - pos[3 * w[3 * i] + k];
        if (box) d = mimg(d, box[k]);
        d2 += d * d;
    }
    return sqrt(d2);
}

double orc_twobody(int nw, const int* w, const double* pos, const double* box, double rc, double* f, long* npairs) {
    double e = 0.0;
    long np = 0;
    for (int i = 0; i < nw; ++i)
        for (int j = i + 1; j < nw; ++j)
            if (oo_dist(w, i, j, pos, box) <= rc) {
                e += twobody_pair(w + 3 * j, w + 3 * i, pos, box, f);
                ++np;
            }
    if (npairs) *npairs = np;
    return e;
}

/* Two-body over a subset of the pair list (for timing samples): pairs
 * p0, p0+stride, ... of the enumeration order above. */
double orc_twobody_sample(int nw, const int* w, const double* pos, const double* box, double rc, long stride,
                          double* f, long* npairs_total, long* nsampled) {
    double e = 0.0;
    long np = 0, ns = 0;
    for (int i = 0; i < nw; ++i)
        for (int j = i + 1; j < nw; ++j)
            if (oo_dist(w, i, j, pos, box) <= rc) {
                if (np % stride == 0) {
                    e += twobody_pair(w + 3 * j, w + 3 * i, pos, box, f);
                    ++ns;
                }
                ++np;
            }
    *npairs_total = np;
    *nsampled = ns;
    return e;
}

/* ----------------------------------------------------------- three-body */
static const int V3[36][3] = {{1, 2, 0}, {4, 5, 0}, {7, 8, 0}, {0, 1, 1}, {0, 2, 1}, {3, 4, 1}, {3, 5, 1}, {6, 7, 1},
                              {6, 8, 1}, {1, 4, 2}, {1, 5, 2}, {1, 7, 2}, {1, 8, 2}, {2, 4, 2}, {2, 5, 2}, {2, 7, 2},
                              {2, 8, 2}, {4, 7, 2}, {4, 8, 2}, {5, 7, 2}, {5, 8, 2}, {0, 4, 3}, {0, 5, 3}, {0, 7, 3},
                              {0, 8, 3}, {3, 1, 3}, {3, 2, 3}, {3, 7, 3}, {3, 8, 3}, {6, 1, 3}, {6, 2, 3}, {6, 4, 3},
                              {6, 5, 3}, {0, 3, 4}, {0, 6, 4}, {3, 6, 4}};
/* mbpol_3body_constants.h:5-20: k and d0 per class HH_intra, OH_intra, HH, OH, OO */
static const double K3[5] = {-2.254303257872797e+00, -2.564771901404151e-01, 4.247920544074333e-01,
                             8.128985941165371e-01, 3.749457984616480e-02};
static const double D3[5] = {1.690594510379166e+00, -2.999999868517452e+00, 3.499031358429095e+00,
                             4.854042963514281e+00, 4.816312044947604e-08};

static double sw3(double r, double* g) {
    const double r3f = 4.5;
    if (r > r3f) {
        *g = 0.0;
        return 0.0;
    }
    const double t1 = M_PI / r3f, x = r * t1;
    *g = -sin(x) * t1 / 2.0;
    return (1.0 + cos(x)) / 2.0;
}

static double threebody_trip(const int* wa, const int* wb, const int* wc, const double* pos, const double* box,
                             double* f) {
    double S[9][3];
    const int* W[3] = {wa, wb, wc};
    for (int m = 0; m < 3; ++m)
        for (int s = 0; s < 3; ++s) memcpy(S[3 * m + s], pos + 3 * W[m][s], 24);
    image_to(S[0], S[1], box);
    image_to(S[0], S[2], box);
    image_to(S[0], S[3], box);
    image_to(S[3], S[4], box);
    image_to(S[3], S[5], box);
    image_to(S[0], S[6], box);
    image_to(S[6], S[7], box);
    image_to(S[6], S[8], box);
    double rab[3], rac[3], rbc[3];
    for (int k = 0; k < 3; ++k) {
        rab[k] = (S[0][k] - S[3][k]) * NM2A;
        rac[k] = (S[0][k] - S[6][k]) * NM2A;
        rbc[k] = (S[3][k] - S[6][k]) * NM2A;
    }
    const double dab = sqrt(dot3(rab, rab)), dac = sqrt(dot3(rac, rac)), dbc = sqrt(dot3(rbc, rbc));
    if (dab < 2 || dac < 2 || dbc < 2) return 0.0;
    double x[36], g[36], dx[36][3], dd[36];
    for (int n = 0; n < 36; ++n) {
        const int c = V3[n][2];
        for (int k = 0; k < 3; ++k) dx[n][k] = (S[V3[n][0]][k] - S[V3[n][1]][k]) * NM2A;
        dd[n] = sqrt(dot3(dx[n], dx[n]));
        x[n] = exp(-K3[c] * (dd[n] - D3[c]));
    }
    double E = poly_eval(poly3b_prog, POLY3B_NPROG, 36, x, g);
    double gab, gac, gbc;
    const double sab = sw3(dab, &gab), sac = sw3(dac, &gac), sbc = sw3(dbc, &gbc);
    const double s = sab * sac + sab * sbc + sac * sbc;
    double F[9][3];
    memset(F, 0, sizeof F);
    for (int n = 0; n < 36; ++n) {
        const int c = V3[n][2];
        const double gg = -K3[c] * g[n] * s * x[n] / dd[n] * CAL2J * 10. * -1;
        for (int k = 0; k < 3; ++k) {
            F[V3[n][0]][k] += gg * dx[n][k];
            F[V3[n][1]][k] -= gg * dx[n][k];
        }
    }
    gab *= (sac + sbc) * E / dab;
    gac *= (sab + sbc) * E / dac;
    gbc *= (sab + sac) * E / dbc;
    for (int k = 0; k < 3; ++k) {
        F[0][k] += (gab * rab[k] + gac * rac[k]) * CAL2J * -NM2A;
        F[3][k] += (gbc * rbc[k] - gab * rab[k]) * CAL2J * -NM2A;
        F[6][k] -= (gac * rac[k] + gbc * rbc[k]) * CAL2J * -NM2A;
    }
    for (int m = 0; m < 3; ++m)
        for (int s2 = 0; s2 < 3; ++s2)
            for (int k = 0; k < 3; ++k) f[3 * W[m][s2] + k] += F[3 * m + s2][k];
    return E * s * CAL2J;
}

/* Trimers by the reference's chain rule: (I, J, K), J < I within rc of I,
 * K < J within rc of J.  With stride > 1 only every stride-th trimer is
 * evaluated (timing samples). */
double orc_threebody(int nw, const int* w, const double* pos, const double* box, double rc, long stride, double* f,
                     long* ntrip, long* nsampled) {
    int* cnt = (int*)calloc((size_t)nw, sizeof(int));
    int cap = 64;
    int* low = (int*)malloc(sizeof(int) * (size_t)nw * cap);
    for (int i = 0; i < nw; ++i)
        for (int j = 0; j < i; ++j)
            if (oo_dist(w, i, j, pos, box) <= rc && cnt[i] < cap) low[(size_t)i * cap + cnt[i]++] = j;
    double e = 0.0;
    long nt = 0, ns = 0;
    for (int i = 0; i < nw; ++i)
        for (int a = 0; a < cnt[i]; ++a) {
            const int j = low[(size_t)i * cap + a];
            for (int b = 0; b < cnt[j]; ++b) {
                const int k = low[(size_t)j * cap + b];
                if (nt % stride == 0) {
                    e += threebody_trip(w + 3 * i, w + 3 * j, w + 3 * k, pos, box, f);
                    ++ns;
                }
                ++nt;
            }
        }
    free(cnt);
    free(low);
    if (ntrip) *ntrip = nt;
    if (nsampled) *nsampled = ns;
    return e;
}

/* ----------------------------------------------------------- dispersion */
double orc_dispersion(int nw, const int* w, const double* pos, const double* box, double rc, double* f) {
    static const double C6[2][2] = {{9.92951990e-4, 3.49345451e-4}, {3.49345451e-4, 8.40715638e-5}};
    static const double D6[2][2] = {{9.29548582e+01, 9.77520243e+01}, {9.77520243e+01, 9.40647517e+01}};
    double e = 0.0;
    for (int i = 0; i < nw; ++i)
        for (int j = i + 1; j < nw; ++j)
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) {
                    const int pa = w[3 * i + a], pb = w[3 * j + b];
                    double d[3];
                    for (int k = 0; k < 3; ++k) {
                        d[k] = pos[3 * pb + k] - pos[3 * pa + k];
                        if (box) d[k] = mimg(d[k], box[k]);
                    }
                    const double r2 = dot3(d, d);
                    if (r2 > rc * rc) continue;
                    const double r = sqrt(r2);
                    const int ca = a ? 1 : 0, cb = b ? 1 : 0;
                    const double c6 = C6[ca][cb], d6 = D6[ca][cb], x = d6 * r;
                    double s = 1.0, t = 1.0;
                    for (int n = 1; n <= 6; ++n) {
                        t *= x / n;
                        s += t;
                    }
                    const double tt = 1.0 - exp(-x) * s, dtt = d6 * exp(-x) * pow(x, 6) / 720.0;
                    e += -c6 * tt / pow(r, 6);
                    const double dEdr = -c6 * (dtt / pow(r, 6) - 6.0 * tt / pow(r, 7));
                    for (int k = 0; k < 3; ++k) {
                        f[3 * pb + k] += -dEdr * d[k] / r;
                        f[3 * pa + k] -= -dEdr * d[k] / r;
                    }
                }
    return e;
}

/* Dispersion of chloride ions (class CL, python/mbpol.xml:52-83): every ion
 * with the O and H sites of every water and with every other ion (C6 Cl-Cl
 * = 0 in the table), site distances within rc (minimum image with a box);
 * the same damped -C6 tt6 / r^6 as the water pairs.  Returns the energy
 * (kJ/mol) and adds the forces into f. */
double orc_dispersion_ions(int nw, const int* w, int nion, const int* ions, const double* pos, const double* box,
                           double rc, double* f) {
    /* [class of the partner: O, H, CL] against CL */
    static const double C6[3] = {0.00456078851, 0.00085979832, 0.0};
    static const double D6[3] = {1.638868407461115e+02, 5.778854012725382e+01, 0.0};
    double e = 0.0;
    for (int i = 0; i < nion; ++i) {
        const int pi = ions[i];
        for (int j = 0; j < 3 * nw + nion; ++j) {
            int pj, c;
            if (j < 3 * nw) {
                pj = w[j];
                c = j % 3 ? 1 : 0;
            } else {
                if (j - 3 * nw <= i) continue;
                pj = ions[j - 3 * nw];
                c = 2;
            }
            if (C6[c] == 0.0) continue;
            double d[3];
            for (int k = 0; k < 3; ++k) {
                d[k] = pos[3 * pj + k] - pos[3 * pi + k];
                if (box) d[k] = mimg(d[k], box[k]);
            }
            const double r2 = dot3(d, d);
            if (r2 > rc * rc) continue;
            const double r = sqrt(r2), x = D6[c] * r;
            double s = 1.0, t = 1.0;
            for (int n = 1; n <= 6; ++n) {
                t *= x / n;
                s += t;
            }
            const double tt = 1.0 - exp(-x) * s, dtt = D6[c] * exp(-x) * pow(x, 6) / 720.0;
            e += -C6[c] * tt / pow(r, 6);
            const double dEdr = -C6[c] * (dtt / pow(r, 6) - 6.0 * tt / pow(r, 7));
            for (int k = 0; k < 3; ++k) {
                f[3 * pj + k] += -dEdr * d[k] / r;
                f[3 * pi + k] -= -dEdr * d[k] / r;
            }
        }
    }
    return e;
}
