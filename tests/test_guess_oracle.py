"""CPU: the oracle of the learned dipole guess (oracle/dipole_guess.py).
Descriptors are invariant under rotation, translation and relabelling of the
other waters; the network's analytic gradients match finite differences
(exact FP64 network); the BF16-rounded network stays close to it."""
import numpy as np
import pytest

from mbpol_openmm_plugin_gb300 import systems

dg = pytest.importorskip("dipole_guess")


def _cluster(n=14, seed=0):
    return systems.cluster(n, seed).positions


def _rot(seed):
    q = np.random.default_rng(seed).normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([[a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
                     [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
                     [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d]])


def test_descriptors_invariant_under_rotation_translation_and_relabelling():
    pos = _cluster()
    D = dg.descriptors(pos)
    assert D.shape == (14, 48) and np.abs(D).sum() > 0
    R = _rot(3)
    moved = pos @ R.T + np.array([1.3, -0.7, 2.1])
    assert np.allclose(dg.descriptors(moved), D, atol=1e-12)
    perm = np.random.default_rng(1).permutation(14)
    idx = (4 * perm[:, None] + np.arange(4)[None, :]).ravel()
    assert np.allclose(dg.descriptors(pos[idx]), D[perm], atol=1e-12)


def test_targets_rotate_with_the_water():
    pos = _cluster()
    mu = np.random.default_rng(2).normal(size=pos.shape) * 1e-3
    R = _rot(5)
    t0 = dg.targets(mu, pos)
    t1 = dg.targets(mu @ R.T, pos @ R.T)
    assert np.allclose(t0, t1, atol=1e-10)


def test_periodic_descriptors_match_an_explicit_image():
    ws = systems.workload("box256", 0)
    D = dg.descriptors(ws.positions, ws.box)
    shifted = ws.positions + ws.box * np.array([1.0, -2.0, 0.0])
    assert np.allclose(dg.descriptors(shifted, ws.box), D, atol=1e-9)


def test_field_features_rotate_with_the_water():
    pos = _cluster()
    E0 = np.random.default_rng(4).normal(size=pos.shape)
    R = _rot(9)
    assert np.allclose(dg.field_features(E0, pos), dg.field_features(E0 @ R.T, pos @ R.T), atol=1e-10)
    X = dg.inputs(pos, E0)
    assert X.shape == (14, 64) and np.all(X[:, 57:] == 0)


def test_network_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    X = rng.normal(size=(40, 64))
    T = rng.normal(size=(40, 9))
    p = {k: v.astype(np.float64) for k, v in dg.init_params(7).items()}
    mean, std = np.zeros(64), np.ones(64)
    loss, g, _ = dg.forward_backward(X, T, p, mean, std, rounding=False)
    h = 1e-6
    for k, idx in (("W1", (3, 5)), ("W2", (10, 20)), ("W3", (4, 7)), ("b1", (6,)), ("b2", (1,)), ("b3", (8,))):
        q = {kk: vv.copy() for kk, vv in p.items()}
        q[k][idx] += h
        lp = dg.forward_backward(X, T, q, mean, std, rounding=False)[0]
        q[k][idx] -= 2 * h
        lm = dg.forward_backward(X, T, q, mean, std, rounding=False)[0]
        assert abs((lp - lm) / (2 * h) - g[k][idx]) <= 1e-6 * max(1.0, abs(g[k][idx])), k


def test_bf16_network_close_to_exact():
    rng = np.random.default_rng(1)
    X = rng.normal(size=(64, 64))
    T = rng.normal(size=(64, 9))
    p = dg.init_params(3)
    l0, g0, y0 = dg.forward_backward(X, T, p, np.zeros(64), np.ones(64), rounding=False)
    l1, g1, y1 = dg.forward_backward(X, T, p, np.zeros(64), np.ones(64), rounding=True)
    assert abs(l1 - l0) <= 2e-2 * l0
    assert np.linalg.norm(y1 - y0) <= 2e-2 * np.linalg.norm(y0)
    for k in g0:
        assert np.linalg.norm(g1[k] - g0[k]) <= 5e-2 * np.linalg.norm(g0[k]), k


def _oscillation_history(n3=600, steps=None, seed=0):
    """Superposed slow oscillations sampled at unit steps, newest first."""
    steps = steps or dg.PRED_HISTORY + 1
    rng = np.random.default_rng(seed)
    A = rng.normal(size=(4, n3)) * 1e-2
    w = np.array([0.03, 0.05, 0.08, 0.13])
    ph = rng.uniform(0, 2 * np.pi, size=(4, n3))
    t = np.arange(steps)[::-1].astype(float)  # newest first
    return np.einsum("mn,tmn->tn", A, np.cos(w[None, :, None] * t[:, None, None] + ph[None]))


def test_predictor_exact_on_polynomial_history():
    """A cubic trajectory without a field: the higher differences vanish,
    are left out, and the prediction is the cubic's continuation (to the
    1e-6 ridge on the scaled normal equations)."""
    t = np.arange(dg.PRED_HISTORY + 1)[::-1].astype(float)
    c = np.random.default_rng(1).normal(size=(4, 50))
    X = c[0] + np.outer(t, c[1]) + np.outer(t ** 2, c[2]) * 1e-2 + np.outer(t ** 3, c[3]) * 1e-4
    F = np.zeros_like(X)
    a = dg.predictor_fit(X[1:])
    p = dg.predictor_apply(X[1:], F[1:], F[0], a)
    assert np.max(np.abs(p - X[0])) <= 1e-6 * np.max(np.abs(X))


def test_predictor_beats_polynomial_extrapolation():
    """On smooth oscillations the fitted predictor is closer to the next
    value than the 4-point polynomial extrapolation (a = 1, 1, 1, 0, ...)."""
    X = _oscillation_history()
    F = np.zeros_like(X)
    hist = X[1:]
    p = dg.predictor_apply(hist, F[1:], F[0], dg.predictor_fit(hist))
    p4 = dg.predictor_apply(hist, F[1:], F[0], np.array([1.0, 1.0, 1.0, 0, 0, 0, 0]))
    assert np.sqrt(np.mean((p - X[0]) ** 2)) < 0.5 * np.sqrt(np.mean((p4 - X[0]) ** 2))


def test_predictor_field_term():
    """Dipoles that respond with the field gain to an unpredictable field
    change at the new step: the field term adds exactly that response."""
    X = _oscillation_history(seed=2)
    F = 0.3 * _oscillation_history(seed=3)
    a = dg.predictor_fit(X[1:])
    kick = 1e-4 * np.random.default_rng(4).normal(size=X.shape[1])
    p0 = dg.predictor_apply(X[1:], F[1:], F[0], a)
    p1 = dg.predictor_apply(X[1:], F[1:], F[0] + kick, a)
    assert np.allclose(p1 - p0, dg.FIELD_GAIN * kick, rtol=1e-10, atol=1e-15)
