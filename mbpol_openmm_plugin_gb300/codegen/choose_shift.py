"""Choose the expansion points of the MB-pol polynomials for the tensor-core
evaluation (codegen/gen_poly_tc.py, csrc/poly_tc.cu).

The polynomial E(x) = sum_m c_m x^m cancels by a factor ~5e5 at typical
inputs (monomial terms of 1e2-1e5 kcal/mol summing to ~1).  Most of that is
structural: the intramolecular variables are nearly constant (x ~ 2.76 for
the three-body O-H ones) and their powers carry large coefficients of both
signs.  Re-expanded about a point x0 near the typical inputs,
E = sum_m c'_m (x - x0)^m has ~250x less cancellation, which is what lets
FP32-accumulated tensor-core products reach the accuracy the double-float
walk needed before.

x0 is the median of each variable over seeded synthetic configurations (the
4096-water jittered lattice and 14-water clusters of systems.py); the
largest |x - x0| seen there sets the power-of-two scale of each fp16
operand row (inputs beyond it are rescaled per unit by the kernel).  The
variables are restated here in numpy from
platforms/reference/src/mbpol_2body_constants.cpp:10-77 (two-body, with the
lone-pair X sites) and MBPolReferenceThreeBodyForce.cpp:67-104 (three-body).

    python -m mbpol_openmm_plugin_gb300.codegen.choose_shift
writes data/poly2b_shift.txt and data/poly3b_shift.txt (committed).
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
DATA = os.path.join(PKG, "data")

# two-body variables: (site a, site b, kind, k, r0); kind 0 exp(k(r0-r)),
# kind 1 exp(k(r0-r))/r.  Sites 0 Oa 1 Ha1 2 Ha2 3 Ob 4 Hb1 5 Hb2 6 Xa1 7 Xa2
# 8 Xb1 9 Xb2 (mbpol_2body_constants.h:33-48, mbpol_2body_constants.cpp:10-60).
K2 = dict(HHi=-6.480884773303821e-01, OHi=1.674518993682975e+00, HHc=1.148231864355956e+00,
          OHc=1.205989761123099e+00, OOc=1.395357065790959e+00, XH=7.347036852042255e-01,
          XO=7.998249864422826e-01, XX=7.960663960630585e-01)
V2 = [(1, 2, 0, "HHi", 1.0), (4, 5, 0, "HHi", 1.0), (0, 1, 0, "OHi", 1.0), (0, 2, 0, "OHi", 1.0),
      (3, 4, 0, "OHi", 1.0), (3, 5, 0, "OHi", 1.0), (1, 4, 1, "HHc", 4.0), (1, 5, 1, "HHc", 4.0),
      (2, 4, 1, "HHc", 4.0), (2, 5, 1, "HHc", 4.0), (0, 4, 1, "OHc", 4.0), (0, 5, 1, "OHc", 4.0),
      (3, 1, 1, "OHc", 4.0), (3, 2, 1, "OHc", 4.0), (0, 3, 1, "OOc", 4.0), (6, 4, 0, "XH", 4.0),
      (6, 5, 0, "XH", 4.0), (7, 4, 0, "XH", 4.0), (7, 5, 0, "XH", 4.0), (8, 1, 0, "XH", 4.0),
      (8, 2, 0, "XH", 4.0), (9, 1, 0, "XH", 4.0), (9, 2, 0, "XH", 4.0), (0, 8, 0, "XO", 4.0),
      (0, 9, 0, "XO", 4.0), (3, 6, 0, "XO", 4.0), (3, 7, 0, "XO", 4.0), (6, 8, 0, "XX", 4.0),
      (6, 9, 0, "XX", 4.0), (7, 8, 0, "XX", 4.0), (7, 9, 0, "XX", 4.0)]
GAMMA_IN, GAMMA_OUT = -9.721486914088159e-02, 9.859272078406150e-02

# three-body variables x = exp(-k (d - d0)) (mbpol_3body_constants.h:5-20)
K3 = dict(HHi=(-2.254303257872797e+00, 1.690594510379166e+00), OHi=(-2.564771901404151e-01, -2.999999868517452e+00),
          HH=(4.247920544074333e-01, 3.499031358429095e+00), OH=(8.128985941165371e-01, 4.854042963514281e+00),
          OO=(3.749457984616480e-02, 4.816312044947604e-08))
V3 = ([(1, 2, "HHi"), (4, 5, "HHi"), (7, 8, "HHi")] +
      [(0, 1, "OHi"), (0, 2, "OHi"), (3, 4, "OHi"), (3, 5, "OHi"), (6, 7, "OHi"), (6, 8, "OHi")] +
      [(a, b, "HH") for a, b in ((1, 4), (1, 5), (1, 7), (1, 8), (2, 4), (2, 5), (2, 7), (2, 8), (4, 7), (4, 8),
                                 (5, 7), (5, 8))] +
      [(a, b, "OH") for a, b in ((0, 4), (0, 5), (0, 7), (0, 8), (3, 1), (3, 2), (3, 7), (3, 8), (6, 1), (6, 2),
                                 (6, 4), (6, 5))] +
      [(0, 3, "OO"), (0, 6, "OO"), (3, 6, "OO")])


def _mi(d, L):
    return d if L is None else d - L * np.round(d / L)


def _sites(ws):
    pos = ws.positions.reshape(-1, 4, 3)[:, :3] * 10.0
    L = None if ws.box is None else ws.box * 10.0
    return pos, L


def var2(kind, k, r0, r):
    e = np.exp(k * (r0 - r))
    return e / r if kind else e


def twobody_samples(ws, rc=6.5, maxn=20000, rng=None):
    pos, L = _sites(ws)
    O = pos[:, 0]
    out = []
    idx = np.arange(len(O)) if rng is None else rng.permutation(len(O))
    for i in idx:
        d = np.linalg.norm(_mi(O - O[i], L), axis=1)
        for j in np.nonzero((d <= rc) & (d >= 2.0) & (np.arange(len(O)) > i))[0]:
            S = np.zeros((10, 3))
            S[0:3] = pos[i]
            S[3:6] = pos[j]
            for m in range(1, 6):
                S[m] = S[0] + _mi(S[m] - S[0], L)
            for m in range(2):
                o, h1, h2 = S[3 * m], S[3 * m + 1], S[3 * m + 2]
                a, b = h1 - o, h2 - o
                inp = o + (a + b) * 0.5 * GAMMA_IN
                out_ = np.cross(a, b) * GAMMA_OUT
                S[6 + 2 * m] = inp + out_
                S[7 + 2 * m] = inp - out_
            out.append([var2(kind, K2[c], r0, np.linalg.norm(S[a] - S[b])) for a, b, kind, c, r0 in V2])
            if len(out) >= maxn:
                return np.array(out)
    return np.array(out)


def threebody_samples(ws, rc=4.5, maxn=20000, rng=None):
    pos, L = _sites(ws)
    O = pos[:, 0]
    out = []
    idx = np.arange(len(O)) if rng is None else rng.permutation(len(O))
    for i in idx:
        d = np.linalg.norm(_mi(O[:i] - O[i], L), axis=1)
        for j in np.nonzero(d <= rc)[0]:
            dj = np.linalg.norm(_mi(O[:j] - O[j], L), axis=1)
            for k in np.nonzero(dj <= rc)[0]:
                S = np.concatenate([pos[i], pos[j], pos[k]])
                for m in (1, 2, 3, 6):
                    S[m] = S[0] + _mi(S[m] - S[0], L)
                for m in (4, 5):
                    S[m] = S[3] + _mi(S[m] - S[3], L)
                for m in (7, 8):
                    S[m] = S[6] + _mi(S[m] - S[6], L)
                out.append([np.exp(-K3[c][0] * (np.linalg.norm(S[a] - S[b]) - K3[c][1])) for a, b, c in V3])
                if len(out) >= maxn:
                    return np.array(out)
    return np.array(out)


def write(name, x0, bnd):
    path = os.path.join(DATA, "%s_shift.txt" % name)
    with open(path, "w") as f:
        f.write("# expansion point x0 and the sampled maximum of |x - x0| per variable, written by codegen/choose_shift.py\n")
        f.write("# columns: variable x0 max|x-x0| over the samples\n")
        for v, (a, b) in enumerate(zip(x0, bnd)):
            f.write("%d %.17e %.17e\n" % (v, a, b))
    print("wrote", path)


def main():
    import sys
    sys.path.insert(0, os.path.dirname(PKG))
    from mbpol_openmm_plugin_gb300 import systems
    rng = np.random.default_rng(7)
    box = systems.workload("box4096", 0)
    clusters = [systems.cluster(14, s) for s in range(4)]
    s2 = np.concatenate([twobody_samples(box, rng=rng)] + [twobody_samples(c) for c in clusters])
    s3 = np.concatenate([threebody_samples(box, rng=rng)] + [threebody_samples(c) for c in clusters])
    x0_2 = np.median(s2, axis=0)
    x0_3 = np.median(s3, axis=0)
    b2 = np.abs(s2 - x0_2).max(axis=0)
    b3 = np.abs(s3 - x0_3).max(axis=0)
    write("poly2b", x0_2, b2)
    write("poly3b", x0_3, b3)


if __name__ == "__main__":
    main()
