"""Oracle for the learned induced-dipole guess (TEST INFRASTRUCTURE ONLY:
imported by tests/ as the checker of the CUDA kernels in
mbpol_openmm_plugin_gb300/csrc/guess.cu, never by the product path).

The reference has no learned guess: its solver always starts from
alpha * E_fixed (MBPolReferenceElectrostaticsForce.cpp:438-486, initial
dipoles in calculateInducedDipoleFields' caller :557-616).  This file states
in numpy, FP64, the exact descriptor, network and loss that the CUDA kernels
compute, so the kernels can be checked value by value and gradient by
gradient.

Descriptor of water i (48 numbers), all in the water's own frame:
  O, H1, H2 of water i; u1 = H1 - O, u2 = H2 - O (minimum image);
  e1 = unit(u1/|u1| + u2/|u2|)           (bisector)
  e2 = unit of (u1/|u1| - u2/|u2|) minus its e1 part (in plane, toward H1)
  e3 = e1 x e2
  for every O and H atom a of another water with r = |x_a - O_i| < RC
  (minimum image), g_k(r) = exp(-((r - R_k) / SIGMA)^2) * fc(r),
  fc(r) = (cos(pi r / RC) + 1) / 2, and
     D[s, k, 0] += g_k(r)
     D[s, k, c] += g_k(r) * (x_a - O_i) . e_c / r      c = 1, 2, 3
  s = 0 for O atoms, 1 for H atoms; k = 0..5; flat index s*24 + k*4 + c.

Field features of water i (9 numbers): the permanent field (the solver's
starting field, before the polarisabilities) at its O, H1, H2 sites in the
same frame, flat index 3*site + c.  Network input (64): the 48 descriptors,
the 9 field features, 7 zeros.

Network (weights BF16, accumulation FP32 on the GPU):
  x = bf16((input - mean) / std)
  h1 = SiLU(W1 x + b1)  (64);  h2 = SiLU(W2 bf16(h1) + b2)  (64)
  y = W3 bf16(h2) + b3  (9): the O, H1, H2 dipoles in the frame (e1, e2, e3),
  in units of OUT_SCALE e nm.
Loss: mean over samples of sum_c (y_c - t_c)^2 / 2, t the solver's converged
dipoles in the same frame and units.
"""
import numpy as np

RC = 0.6          # nm, descriptor cutoff (6 Angstrom)
NRAD = 6
R0 = 0.15         # nm, first radial centre
DR = 0.09         # nm, spacing of the radial centres
SIGMA = 0.09      # nm, Gaussian width
NFEAT = 48        # neighbourhood descriptors
NFIELD = 9        # permanent field at O, H1, H2 in the water's frame
NIN = 64          # network input: descriptors, field, zero padding
HIDDEN = 64
NOUT = 9
OUT_SCALE = 1e-3  # e nm per output unit


def bf16(a):
    """Round FP32 values to BF16 (round to nearest even), returned as FP64."""
    a = np.asarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return u.view(np.float32).astype(np.float64)


def _mi(d, box):
    if box is None:
        return d
    return d - box * np.round(d / box)


def frames(pos, box=None):
    """Local frames (nw, 3, 3), rows e1, e2, e3, of waters [O, H1, H2, M]."""
    O, H1, H2 = pos[0::4], pos[1::4], pos[2::4]
    u1 = _mi(H1 - O, box)
    u2 = _mi(H2 - O, box)
    a = u1 / np.linalg.norm(u1, axis=1, keepdims=True)
    b = u2 / np.linalg.norm(u2, axis=1, keepdims=True)
    e1 = a + b
    e1 /= np.linalg.norm(e1, axis=1, keepdims=True)
    p = a - b
    p -= (p * e1).sum(1, keepdims=True) * e1
    e2 = p / np.linalg.norm(p, axis=1, keepdims=True)
    e3 = np.cross(e1, e2)
    return np.stack([e1, e2, e3], 1)


def descriptors(pos, box=None):
    """(nw, 48) descriptors of waters laid out [O, H1, H2, M] per water."""
    pos = np.asarray(pos, np.float64)
    nw = pos.shape[0] // 4
    E = frames(pos, box)
    O = pos[0::4]
    D = np.zeros((nw, 2, NRAD, 4))
    centres = R0 + DR * np.arange(NRAD)
    for s, sites in ((0, [0]), (1, [1, 2])):
        for site in sites:
            X = pos[site::4]
            for i in range(nw):
                d = _mi(X - O[i], box)
                r = np.linalg.norm(d, axis=1)
                m = (r < RC) & (np.arange(nw) != i)
                if not m.any():
                    continue
                d, r = d[m], r[m]
                fc = 0.5 * (np.cos(np.pi * r / RC) + 1.0)
                g = np.exp(-((r[:, None] - centres[None, :]) / SIGMA) ** 2) * fc[:, None]
                proj = (d @ E[i].T) / r[:, None]
                D[i, s, :, 0] += g.sum(0)
                D[i, s, :, 1:] += g.T @ proj
    return D.reshape(nw, NFEAT)


def field_features(E0, pos, box=None):
    """(nw, 9) permanent field at O, H1, H2 in each water's frame."""
    F = frames(pos, box)
    E0 = np.asarray(E0, np.float64)
    out = np.zeros((F.shape[0], NFIELD))
    for s in range(3):
        out[:, 3 * s:3 * s + 3] = np.einsum("wcd,wd->wc", F, E0[s::4])
    return out


def inputs(pos, E0, box=None):
    """(nw, 64) network inputs: descriptors, field features, zeros."""
    nw = np.asarray(pos).shape[0] // 4
    return np.concatenate([descriptors(pos, box), field_features(E0, pos, box),
                           np.zeros((nw, NIN - NFEAT - NFIELD))], axis=1)


def neighbour_field_features(dF, pos, box=None):
    """(nw, 6) the correction network's neighbour features: over waters B
    whose O lies within RC of A's O, sum fc(r) dF_O(B) and
    fc(r) (dF_H1(B) + dF_H2(B)), in A's frame (csrc/guess.cu,
    descriptor_kernel, mode 1)."""
    pos = np.asarray(pos, np.float64)
    dF = np.asarray(dF, np.float64)
    nw = pos.shape[0] // 4
    E = frames(pos, box)
    O = pos[0::4]
    out = np.zeros((nw, 6))
    for i in range(nw):
        d = _mi(O - O[i], box)
        r = np.linalg.norm(d, axis=1)
        m = (r < RC) & (np.arange(nw) != i)
        fc = 0.5 * (np.cos(np.pi * r[m] / RC) + 1.0)
        so = (fc[:, None] * dF[0::4][m]).sum(0)
        sh = (fc[:, None] * (dF[1::4][m] + dF[2::4][m])).sum(0)
        out[i, :3] = E[i] @ so
        out[i, 3:] = E[i] @ sh
    return out


def correction_inputs(pos, dF, box=None):
    """(nw, 64) inputs of the correction network: descriptors, the water's
    own unpredicted field change dF at O, H1, H2 in its frame, the neighbour
    features, one zero."""
    nw = np.asarray(pos).shape[0] // 4
    return np.concatenate([descriptors(pos, box), field_features(dF, pos, box),
                           neighbour_field_features(dF, pos, box), np.zeros((nw, 1))], axis=1)


def targets(dipoles, pos, box=None):
    """(nw, 9) solver dipoles of O, H1, H2 in each water's frame / OUT_SCALE."""
    E = frames(pos, box)
    mu = np.asarray(dipoles, np.float64)
    out = np.zeros((E.shape[0], NOUT))
    for s in range(3):
        out[:, 3 * s:3 * s + 3] = np.einsum("wcd,wd->wc", E, mu[s::4]) / OUT_SCALE
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    sg = 1.0 / (1.0 + np.exp(-z))
    return sg * (1.0 + z * (1.0 - sg))


def forward_backward(X, T, params, mean, std, rounding=True):
    """Loss and its gradients with the GPU kernels' BF16 roundings (operands
    of every tensor-core product: inputs, activations, output and hidden
    gradients, weights).  params: dict W1 (64,64), b1, W2 (64,64), b2,
    W3 (9,64), b3 (FP32 masters).  rounding=False gives the exact FP64
    network (for finite-difference checks).  Returns (loss, grads, Y)."""
    R = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    W1, W2, W3 = R(params["W1"]), R(params["W2"]), R(params["W3"])
    b1, b2, b3 = (np.asarray(params[k], np.float64) for k in ("b1", "b2", "b3"))
    x = R((np.asarray(X, np.float64) - mean) / std)
    z1 = x @ W1.T + b1
    a1 = R(silu(z1))
    z2 = a1 @ W2.T + b2
    a2 = R(silu(z2))
    y = a2 @ W3.T + b3
    n = X.shape[0]
    r = y - T
    loss = 0.5 * (r * r).sum() / n
    dy = R(r / n)
    g = {"W3": dy.T @ a2, "b3": (r / n).sum(0)}
    dz2 = (dy @ W3) * dsilu(z2)
    g["b2"] = dz2.sum(0)
    dz2 = R(dz2)
    g["W2"] = dz2.T @ a1
    dz1 = (dz2 @ W2) * dsilu(z1)
    g["b1"] = dz1.sum(0)
    dz1 = R(dz1)
    g["W1"] = dz1.T @ x
    return loss, g, y


def predict(X, params, mean, std):
    """Network output (n, 9) with the kernels' roundings."""
    return forward_backward(X, np.zeros((X.shape[0], NOUT)), params, mean, std)[2]


def init_params(seed):
    """He-style initialisation shared with the GPU trainer's host side."""
    rng = np.random.default_rng(seed)
    p = {
        "W1": rng.normal(0, np.sqrt(2.0 / NIN), (HIDDEN, NIN)),
        "b1": np.zeros(HIDDEN),
        "W2": rng.normal(0, np.sqrt(2.0 / HIDDEN), (HIDDEN, HIDDEN)),
        "b2": np.zeros(HIDDEN),
        "W3": rng.normal(0, np.sqrt(1.0 / HIDDEN), (NOUT, HIDDEN)),
        "b3": np.zeros(NOUT),
    }
    return {k: v.astype(np.float32) for k, v in p.items()}


# ------------------------------------------------- learned linear predictor
PRED_ORDER = 7    # backward differences of the dipoles in the model
PRED_REGRESSORS = PRED_ORDER
PRED_WINDOW = 4   # past steps it is fitted on
PRED_HISTORY = PRED_ORDER + 1 + PRED_WINDOW
FIELD_GAIN = 2.4  # weight of the unpredicted permanent-field change


def backward_differences(x):
    """nabla^1 .. nabla^J of the sequence x[0 .. J] (x[0] the newest; rows
    of any trailing shape), by repeated differencing."""
    t = np.array(x, dtype=np.float64)
    out = []
    for j in range(1, t.shape[0]):
        t = t[:-1] - t[1:]
        out.append(t[0])
    return np.array(out)


def predictor_fit(history, stride=None):
    """Coefficients a_1..a_J of P(Y) = Y0 + sum_j a_j nabla^j Y0, fitted by
    least squares on the last PRED_WINDOW steps of the dipoles: X_w - X_{w+1}
    from the differences at X_{w+1}.  history: [PRED_HISTORY, n3], newest
    first.  Normal equations scaled by their diagonal, vanishing columns left
    out, ridge 1e-6 on the scaled system, as the CUDA kernel (which solves
    the scaled system in FP32; here FP64)."""
    h = np.asarray(history, np.float64)
    if stride is None:  # the CUDA kernel's subsample: about 8k components
        stride = h.shape[1] // 8192 if h.shape[1] > 8192 else 1
    h = h[:, ::stride]
    J = PRED_ORDER
    G = np.zeros((J, J))
    b = np.zeros(J)
    for w in range(PRED_WINDOW):
        D = backward_differences(h[w + 1:w + 2 + J])
        y = h[w] - h[w + 1]
        G += D @ D.T
        b += D @ y
    gmax = np.max(np.diag(G))
    keep = (np.diag(G) > 1e-24 * gmax) & (np.diag(G) > 0)
    sc = np.where(keep, 1.0 / np.sqrt(np.where(keep, np.diag(G), 1.0)), 0.0)
    Gs = np.where(np.outer(keep, keep), G * np.outer(sc, sc), np.eye(J)) + 1e-6 * np.eye(J)
    bs = np.where(keep, b * sc, 0.0)
    return np.linalg.solve(Gs, bs) * sc


def predictor_apply(history, field, field_now, a, gain=FIELD_GAIN):
    """mu = P(X) + gain (F_new - P(F)) with P(Y) = Y0 + sum_j a_j nabla^j Y0."""
    h = np.asarray(history, np.float64)
    f = np.asarray(field, np.float64)
    P = lambda y: y[0] + np.tensordot(a, backward_differences(y[:PRED_ORDER + 1]), axes=1)  # noqa: E731
    return P(h) + gain * (np.asarray(field_now, np.float64) - P(f))
