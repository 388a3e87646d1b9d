/*
 * Oracle C port (TEST INFRASTRUCTURE ONLY): geometry-dependent charges of a
 * water and their derivatives, restating
 * platforms/reference/src/MBPolReferenceElectrostaticsForce.cpp:2793-3096
 * (dipole-moment-surface fit, TTM2.1-F M site gammaM = 0.426706882).
 * dq[s][k]: derivative of the charge of other-site s (H1, H2, M) with respect
 * to coordinate k of the site that owns the array, per nm.
 */
static const int O_DMS_IDX[3][84] = {
    {1, 1, 1, 2, 1, 1, 1, 2, 2, 3, 1, 1, 1, 1, 2, 2, 2, 3, 3, 4, 1, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 4, 4, 5, 1, 1, 1,
     1, 1, 1, 2, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 5, 5, 6, 1, 1, 1, 1, 1, 1, 1, 2, 2, 2, 2, 2, 2, 3, 3, 3, 3, 3, 4, 4,
     4, 4, 5, 5, 5, 6, 6, 7},
    {1, 1, 2, 1, 1, 2, 3, 1, 2, 1, 1, 2, 3, 4, 1, 2, 3, 1, 2, 1, 1, 2, 3, 4, 5, 1, 2, 3, 4, 1, 2, 3, 1, 2, 1, 1, 2, 3,
     4, 5, 6, 1, 2, 3, 4, 5, 1, 2, 3, 4, 1, 2, 3, 1, 2, 1, 1, 2, 3, 4, 5, 6, 7, 1, 2, 3, 4, 5, 6, 1, 2, 3, 4, 5, 1, 2,
     3, 4, 1, 2, 3, 1, 2, 1},
    {1, 2, 1, 1, 3, 2, 1, 2, 1, 1, 4, 3, 2, 1, 3, 2, 1, 2, 1, 1, 5, 4, 3, 2, 1, 4, 3, 2, 1, 3, 2, 1, 2, 1, 1, 6, 5, 4,
     3, 2, 1, 5, 4, 3, 2, 1, 4, 3, 2, 1, 3, 2, 1, 2, 1, 1, 7, 6, 5, 4, 3, 2, 1, 6, 5, 4, 3, 2, 1, 5, 4, 3, 2, 1, 4, 3,
     2, 1, 3, 2, 1, 2, 1, 1}};
static const double O_DMS_C[84] = {
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

static void o_water_charge(OSite* O, OSite* H1, OSite* H2, OSite* M) {
    const double Bohr_A = 0.52917721092, gammaM = 0.426706882, gamma1 = 1.0 - gammaM, gamma2 = gammaM / 2;
    const double costhe = -0.24780227221366464506, reoh = 0.958649, b1D = 1.0;
    const double a = 0.2999e0, b = -0.6932e0, c0 = 1.0099e0, c1 = -0.1801e0, c2 = 0.0892e0;
    double R1[3], R2[3];
    for (int k = 0; k < 3; ++k) {
        R1[k] = H1->r[k] * 10. - O->r[k] * 10.;
        R2[k] = H2->r[k] * 10. - O->r[k] * 10.;
    }
    const double d1 = sqrt(R1[0] * R1[0] + R1[1] * R1[1] + R1[2] * R1[2]);
    const double d2 = sqrt(R2[0] * R2[0] + R2[1] * R2[1] + R2[2] * R2[2]);
    const double costh = (R1[0] * R2[0] + R1[1] * R2[1] + R1[2] * R2[2]) / (d1 * d2);
    const double efac = exp(-b1D * (pow(d1 - reoh, 2) + pow(d2 - reoh, 2)));
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
    double p1 = 0, p2 = 0, dp1dr1 = 0, dp1dr2 = 0, dp1dc = 0, dp2dr1 = 0, dp2dr2 = 0, dp2dc = 0;
    for (int j = 1; j < 84; ++j) {
        const int I = O_DMS_IDX[0][j], J = O_DMS_IDX[1][j], K = O_DMS_IDX[2][j];
        const double c = O_DMS_C[j];
        p1 += c * fm[0][I] * fm[1][J] * fm[2][K];
        p2 += c * fm[0][J] * fm[1][I] * fm[2][K];
        dp1dr1 += c * (I - 1) * fm[0][I - 1] * fm[1][J] * fm[2][K];
        dp1dr2 += c * (J - 1) * fm[0][I] * fm[1][J - 1] * fm[2][K];
        dp1dc += c * (K - 1) * fm[0][I] * fm[1][J] * fm[2][K - 1];
        dp2dr1 += c * (J - 1) * fm[0][J - 1] * fm[1][I] * fm[2][K];
        dp2dr2 += c * (I - 1) * fm[0][J] * fm[1][I - 1] * fm[2][K];
        dp2dc += c * (K - 1) * fm[0][J] * fm[1][I] * fm[2][K - 1];
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
    const double de1 = -2.0 * b1D * (d1 - reoh) * efac * xx, de2 = -2.0 * b1D * (d2 - reoh) * efac * xx;
    dp1dr1 = dp1dr1 * efac + p1 * de1 + dpc0dr1;
    dp1dr2 = dp1dr2 * efac + p1 * de2 + dpc0dr2;
    dp1dc = dp1dc * efac + dpc0dc;
    dp2dr1 = dp2dr1 * efac + p2 * de1 + dpc0dr1;
    dp2dr2 = dp2dr2 * efac + p2 * de2 + dpc0dr2;
    dp2dc = dp2dc * efac + dpc0dc;
    p1 = O_DMS_C[0] + p1 * efac + pc0 * xx;
    p2 = O_DMS_C[0] + p2 * efac + pc0 * xx;
    const double g21 = gamma2 / gamma1;
    O->q = 0.0;
    H1->q = p1 + g21 * (p1 + p2);
    H2->q = p2 + g21 * (p1 + p2);
    M->q = -(p1 + p2) / gamma1;
    dp1dr1 /= xx;
    dp1dr2 /= xx;
    dp2dr1 /= xx;
    dp2dr2 /= xx;
    const double f1q1r13 = (dp1dr1 - (dp1dc * costh / d1)) / d1, f1q1r23 = dp1dc / (d1 * d2);
    const double f2q1r23 = (dp1dr2 - (dp1dc * costh / d2)) / d2, f2q1r13 = dp1dc / (d2 * d1);
    const double f1q2r13 = (dp2dr1 - (dp2dc * costh / d1)) / d1, f1q2r23 = dp2dc / (d1 * d2);
    const double f2q2r23 = (dp2dr2 - (dp2dc * costh / d2)) / d2, f2q2r13 = dp2dc / (d2 * d1);
    for (int k = 0; k < 3; ++k) {
        const double a11 = f1q1r13 * R1[k] + f1q1r23 * R2[k], a12 = f2q1r13 * R1[k] + f2q1r23 * R2[k];
        const double a1o = -(a11 + a12);
        const double a21 = f1q2r13 * R1[k] + f1q2r23 * R2[k], a22 = f2q2r13 * R1[k] + f2q2r23 * R2[k];
        const double a2o = -(a21 + a22);
        const double o1 = -(a11 + a21), o2 = -(a12 + a22), oo = -(a1o + a2o);
        const double sH1 = g21 * (a11 + a21), sH2 = g21 * (a12 + a22), sO = g21 * (a1o + a2o);
        H1->dq[0][k] = (a11 + sH1) * 10;
        H2->dq[0][k] = (a12 + sH2) * 10;
        O->dq[0][k] = (a1o + sO) * 10;
        H1->dq[1][k] = (a21 + sH1) * 10;
        H2->dq[1][k] = (a22 + sH2) * 10;
        O->dq[1][k] = (a2o + sO) * 10;
        H1->dq[2][k] = (o1 - 2 * sH1) * 10;
        H2->dq[2][k] = (o2 - 2 * sH2) * 10;
        O->dq[2][k] = (oo - 2 * sO) * 10;
        M->dq[0][k] = M->dq[1][k] = M->dq[2][k] = 0.0;
    }
}
