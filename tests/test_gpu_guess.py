"""GPU: the learned induced-dipole guess against its oracle
(oracle/dipole_guess.py): descriptors on the periodic 256-water box and the
14-water cluster; network loss, outputs and gradients (BF16 tensor-core
kernels, FP32 accumulation) against the oracle's FP64 network with the same
BF16 roundings.

Tolerances: descriptors 1e-4 relative to each feature's scale (FP32 pair
arithmetic); loss 1e-3 relative; outputs and each gradient tensor 2e-2
relative RMS (a product near a BF16 rounding boundary may round the other
way in FP32 than in FP64, which moves that operand by one BF16 unit)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_rms
import mbpol_openmm_plugin_gb300 as mb
from mbpol_openmm_plugin_gb300 import systems

pytestmark = pytest.mark.gpu
dg = pytest.importorskip("dipole_guess")


def _context(pos, box, alpha=0.0, grid=None):
    ws = systems.WaterSystem(pos, box, 0, "fixture")
    s = mb.create_mbpol_system(ws, terms=("electrostatics",), target_epsilon=1e-8, ewald_alpha=alpha,
                               pme_grid=grid, guess=2)
    ctx = mb.Context(s)
    ctx.setPositions(pos)
    ctx.getState()
    return ctx


@pytest.mark.parametrize("name", ["elec_box256_seed0", "elec_cluster14_seed0"])
def test_network_inputs_match_oracle(name):
    """Columns 0-47: neighbourhood descriptors; 48-56: the permanent field at
    O, H1, H2 in the water's frame (against the oracle port's FP64 field);
    57-63: zero."""
    oracle = pytest.importorskip("oracle")
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    periodic = bool(d["periodic"])
    box = d["box"] if periodic else None
    alpha = float(d["alpha"])
    grid = [int(v) for v in d["grid"]] if periodic else None
    ctx = _context(d["positions"], box, alpha, grid)
    D = ctx.getDipoleGuessDescriptors()
    ref = dg.descriptors(d["positions"], box)
    scale = np.maximum(np.abs(ref).max(0), 1e-3)
    err = np.abs(D[:, :48] - ref) / scale
    E0 = oracle.fixed_field(d["positions"], box, alpha, grid if periodic else (0, 0, 0))
    fref = dg.field_features(E0, d["positions"], box)
    ferr = np.abs(D[:, 48:57] - fref).max() / np.abs(fref).max()
    print(name, "descriptor max rel err %.2e, field max rel err %.2e" % (err.max(), ferr))
    assert err.max() <= 1e-4
    assert ferr <= 1e-5
    assert np.all(D[:, 57:] == 0)


def _params_block(p, mean, inv):
    return np.concatenate([p["W1"].ravel(), p["b1"], p["W2"].ravel(), p["b2"], p["W3"].ravel(), p["b3"],
                           mean, inv]).astype(np.float32)


def test_network_loss_and_gradients_match_oracle():
    d = np.load(os.path.join(GOLDEN, "elec_box256_seed0.npz"))
    ctx = _context(d["positions"], d["box"], float(d["alpha"]), [int(v) for v in d["grid"]])
    X = ctx.getDipoleGuessDescriptors().astype(np.float64)
    T = dg.targets(d["dipoles"], d["positions"], d["box"])
    mean = X.mean(0).astype(np.float32)
    sd = X.std(0)
    inv = np.where(sd > 1e-10, 1.0 / np.where(sd > 1e-10, sd, 1.0), 1.0).astype(np.float32)
    p = dg.init_params(11)
    p["b1"] = (0.1 * np.random.default_rng(2).normal(size=64)).astype(np.float32)
    p["b3"] = np.linspace(-0.5, 0.5, 9).astype(np.float32)
    ctx.setDipoleGuessParameters(_params_block(p, mean, inv))
    loss, g, Y = ctx.dipoleGuessLossGrad(X, T)
    lref, gref, yref = dg.forward_backward(X.astype(np.float32), T, p, mean.astype(np.float64),
                                           1.0 / inv.astype(np.float64))
    print("loss %.6e ref %.6e | Y relrms %.2e" % (loss, lref, rel_rms(Y, yref)))
    assert abs(loss - lref) <= 1e-3 * abs(lref)
    assert rel_rms(Y, yref) <= 2e-2
    flat = np.concatenate([gref[k].ravel() for k in ("W1", "b1", "W2", "b2", "W3", "b3")])
    offs = {"W1": (0, 4096), "b1": (4096, 4160), "W2": (4160, 8256), "b2": (8256, 8320), "W3": (8320, 8896),
            "b3": (8896, 8905)}
    for k, (a, b) in offs.items():
        e = np.linalg.norm(g[a:b] - flat[a:b]) / np.linalg.norm(flat[a:b])
        print("grad %s relrms %.2e" % (k, e))
        assert e <= 2e-2, k


def test_trained_network_cuts_solver_iterations():
    """What the trained network gains over the method without it, on the
    256-water PME box: trained on the GPU on 120 NVT frames (300 K, 0.2 fs)
    of solver-converged dipoles, then evaluated on later configurations it
    has not seen.  Cold starts (no previous solve): the network's guess
    against the reference's alpha * E_fixed start.  MD: the learned mode
    (network, then extrapolation of the solves) against the plain
    previous-step guess.  Both at the same 1e-8 D threshold."""
    import ctypes
    from mbpol_openmm_plugin_gb300 import _capi
    lib = _capi.load()
    ws = systems.workload("box256", 1)
    alpha, grid = mb.pme_parameters(ws.box, 0.9, 1e-5)

    def context(guess):
        s = mb.create_mbpol_system(ws, target_epsilon=1e-8, ewald_alpha=alpha, pme_grid=grid, guess=guess)
        c = mb.Context(s)
        c.setPositions(ws.positions)
        c._build()
        return c, s

    ctx, sysm = context(1)
    h = ctx._h
    masses = np.ascontiguousarray(sysm.masses, np.float64)
    rng = np.random.default_rng(3)
    vel = np.zeros((masses.size, 3))
    live = masses > 0
    vel[live] = rng.normal(size=(int(live.sum()), 3)) * np.sqrt(2.494 / masses[live])[:, None]
    box = np.ascontiguousarray(ws.box, np.float64)
    _capi.check(lib.mbpol_set_positions(h, _capi.ptr(np.ascontiguousarray(ws.positions)), _capi.ptr(box)))
    _capi.check(lib.mbpol_set_masses(h, _capi.ptr(masses)))
    _capi.check(lib.mbpol_set_velocities(h, _capi.ptr(vel)))
    ms, it, en = ctypes.c_double(), ctypes.c_long(), np.zeros(6)

    def run(hh, n, seed, T=300.0):
        _capi.check(lib.mbpol_md_run(hh, n, 0.0002, T, 1.0 if T > 0 else 0.0, seed, ctypes.byref(ms), _capi.ptr(en),
                                     ctypes.byref(it)))
        return it.value

    for f in range(120):
        run(h, 1, 10 + f)
        ctx.collectDipoleGuessSample()
    loss = ctx.trainDipoleGuess(4000, 2048, 2e-3, 5)
    params = ctx.getDipoleGuessParameters()
    # later, unseen configurations
    confs = []
    for k in range(4):
        run(h, 40, 500 + k)
        q = np.zeros_like(ws.positions)
        v = np.zeros_like(ws.positions)
        _capi.check(lib.mbpol_get_state(h, _capi.ptr(q), _capi.ptr(v), None))
        confs.append((q, v))
    cold = {}
    for name, guess in (("alphaE", 0), ("learned", 2)):
        c, _ = context(guess)
        its = []
        for q, _ in confs:
            if guess == 2:
                c.setDipoleGuessParameters(params)  # no previous solve: a cold start
            c.setPositions(q)
            c.getState()
            its.append(int(c.getCounts()[3]))
        cold[name] = np.mean(its)
    md = {}
    for name, guess in (("plain", 1), ("learned", 2)):
        c, _ = context(guess)
        if guess == 2:
            c.setDipoleGuessParameters(params)
        q, v = confs[-1]
        _capi.check(lib.mbpol_set_positions(c._h, _capi.ptr(q), _capi.ptr(box)))
        _capi.check(lib.mbpol_set_masses(c._h, _capi.ptr(masses)))
        _capi.check(lib.mbpol_set_velocities(c._h, _capi.ptr(v)))
        run(c._h, 4, 1, 0.0)
        md[name] = run(c._h, 10, 1, 0.0) / 10.0
    print("train loss %.3f | cold start iterations: alpha*E %.1f, network %.1f | MD iterations/step: "
          "previous-step %.1f, learned %.1f" % (loss, cold["alphaE"], cold["learned"], md["plain"], md["learned"]))
    assert cold["learned"] <= cold["alphaE"] - 3
    assert md["learned"] <= md["plain"] - 5


def test_predictor_fit_matches_oracle():
    """The learned linear predictor's least-squares fit and prediction
    (predictor.cu: FP64 normal equations, FP32 solve of the scaled system,
    the permanent-field term) against the oracle (FP64 throughout).
    Dipoles: 12 consecutive converged solves of an MD run of the 4096-water
    box (tests/golden/make_dipole_history.py); field: a seeded smooth signal
    standing in for alpha E0.  Coefficients
    within 2e-3, the predicted change within 1e-3 of its size; with the
    field set to zero, the prediction is closer to the next solve than the
    4-point polynomial extrapolation."""
    import ctypes
    from mbpol_openmm_plugin_gb300 import _capi
    lib = _capi.load()
    d = np.load(os.path.join(GOLDEN, "elec_cluster14_seed0.npz"))
    ctx = _context(d["positions"], None)
    f = np.load(os.path.join(GOLDEN, "dipole_history_box4096.npz"))
    hist = np.ascontiguousarray(f["history"])
    n3 = hist.shape[1]
    rng = np.random.default_rng(11)
    steps = np.arange(dg.PRED_HISTORY + 1)[::-1].astype(float)
    field_all = 1e-3 * np.cos(0.07 * steps[:, None] + rng.uniform(0, 6.3, size=n3)[None]) \
        * rng.normal(size=n3)[None]
    cases = {"field": (np.ascontiguousarray(field_all[1:]), np.ascontiguousarray(field_all[0])),
             "no field": (np.zeros_like(hist), np.zeros(n3))}
    for name, (field, now) in cases.items():
        coef = np.zeros(dg.PRED_REGRESSORS)
        pred = np.zeros(n3)
        _capi.check(lib.mbpol_guess_fit_predictor(ctx._h, _capi.ptr(hist), _capi.ptr(field), _capi.ptr(now), n3,
                                                  _capi.ptr(coef), _capi.ptr(pred)))
        a_ref = dg.predictor_fit(hist)
        p_ref = dg.predictor_apply(hist, field, now, a_ref)
        print(name, "coefficients", np.round(coef, 6), "oracle", np.round(a_ref, 6))
        assert np.max(np.abs(coef - a_ref)) <= 2e-3 * max(1.0, np.max(np.abs(a_ref)))
        step = np.max(np.abs(p_ref - hist[0]))
        assert np.max(np.abs(pred - p_ref)) <= 1e-3 * step
        if name == "no field":
            p4 = dg.predictor_apply(hist, field, now, np.array([1.0, 1.0, 1.0, 0, 0, 0, 0]))
            err, err4 = np.sqrt(np.mean((pred - f["next"]) ** 2)), np.sqrt(np.mean((p4 - f["next"]) ** 2))
            print("error %.3e, 4-point %.3e" % (err, err4))
            assert err < err4


def test_learned_predictor_cuts_md_iterations():
    """MD on the 256-water PME box from the same state: guess 2 (without a
    network: extrapolation, then the learned predictor with its permanent-
    field term once 12 solves exist) against guess 3 (4-point polynomial
    extrapolation), iterations per step over steps 16-40 at the same 1e-8 D
    threshold."""
    import ctypes
    from mbpol_openmm_plugin_gb300 import _capi
    lib = _capi.load()
    ws = systems.workload("box256", 2)
    alpha, grid = mb.pme_parameters(ws.box, 0.9, 1e-5)
    masses = None
    its = {}
    for name, guess in (("extrapolation", 3), ("learned", 2)):
        s = mb.create_mbpol_system(ws, target_epsilon=1e-8, ewald_alpha=alpha, pme_grid=grid, guess=guess)
        c = mb.Context(s)
        c.setPositions(ws.positions)
        c._build()
        masses = np.ascontiguousarray(s.masses, np.float64)
        rng = np.random.default_rng(4)
        vel = np.zeros((masses.size, 3))
        live = masses > 0
        vel[live] = rng.normal(size=(int(live.sum()), 3)) * np.sqrt(2.494 / masses[live])[:, None]
        box = np.ascontiguousarray(ws.box, np.float64)
        _capi.check(lib.mbpol_set_positions(c._h, _capi.ptr(np.ascontiguousarray(ws.positions)), _capi.ptr(box)))
        _capi.check(lib.mbpol_set_masses(c._h, _capi.ptr(masses)))
        _capi.check(lib.mbpol_set_velocities(c._h, _capi.ptr(vel)))
        ms, it, en = ctypes.c_double(), ctypes.c_long(), np.zeros(6)
        _capi.check(lib.mbpol_md_run(c._h, 16, 0.0002, 0.0, 0.0, 0, ctypes.byref(ms), _capi.ptr(en),
                                     ctypes.byref(it)))
        _capi.check(lib.mbpol_md_run(c._h, 24, 0.0002, 0.0, 0.0, 0, ctypes.byref(ms), _capi.ptr(en),
                                     ctypes.byref(it)))
        its[name] = it.value / 24.0
    print("MD iterations/step: extrapolation %.2f, learned predictor %.2f" % (its["extrapolation"], its["learned"]))
    assert its["learned"] <= its["extrapolation"] - 2.0


def _md_context(ws, guess, seed=4):
    import ctypes
    from mbpol_openmm_plugin_gb300 import _capi
    lib = _capi.load()
    alpha, grid = mb.pme_parameters(ws.box, 0.9, 1e-5)
    s = mb.create_mbpol_system(ws, target_epsilon=1e-8, ewald_alpha=alpha, pme_grid=grid, guess=guess)
    c = mb.Context(s)
    c.setPositions(ws.positions)
    c._build()
    masses = np.ascontiguousarray(s.masses, np.float64)
    rng = np.random.default_rng(seed)
    vel = np.zeros((masses.size, 3))
    live = masses > 0
    vel[live] = rng.normal(size=(int(live.sum()), 3)) * np.sqrt(2.494 / masses[live])[:, None]
    box = np.ascontiguousarray(ws.box, np.float64)
    _capi.check(lib.mbpol_set_positions(c._h, _capi.ptr(np.ascontiguousarray(ws.positions)), _capi.ptr(box)))
    _capi.check(lib.mbpol_set_masses(c._h, _capi.ptr(masses)))
    _capi.check(lib.mbpol_set_velocities(c._h, _capi.ptr(vel)))

    def run(n):
        ms, it, en = ctypes.c_double(), ctypes.c_long(), np.zeros(6)
        _capi.check(lib.mbpol_md_run(c._h, n, 0.0002, 0.0, 0.0, 0, ctypes.byref(ms), _capi.ptr(en),
                                     ctypes.byref(it)))
        return it.value
    return c, run


def test_correction_network_inputs_match_oracle():
    """The correction network's inputs of the last solve (box256, MD with the
    history predictor): the 48 descriptors, and the neighbour features of the
    unpredicted field change against the oracle's, computed from the
    water's own dF (read back from its frame components)."""
    from mbpol_openmm_plugin_gb300 import _capi
    ws = systems.workload("box256", 2)
    c, run = _md_context(ws, 2)
    c.selectDipoleGuessNetwork(mb.Context.CorrectionNetwork)
    run(14)   # the predictor starts at the 13th solve
    D = c.getDipoleGuessDescriptors()
    lib = _capi.load()
    pos = np.zeros_like(ws.positions)
    _capi.check(lib.mbpol_get_state(c._h, _capi.ptr(pos), None, None))
    ref = dg.descriptors(pos, ws.box)
    scale = np.maximum(np.abs(ref).max(0), 1e-3)
    derr = (np.abs(D[:, :48] - ref) / scale).max()
    F = dg.frames(pos, ws.box)
    dF = np.zeros_like(pos)
    for s in range(3):
        dF[s::4] = np.einsum("wcd,wc->wd", F, D[:, 48 + 3 * s:51 + 3 * s].astype(np.float64))
    nref = dg.neighbour_field_features(dF, pos, ws.box)
    nerr = np.abs(D[:, 57:63] - nref).max() / np.abs(nref).max()
    print("correction inputs: descriptors %.1e, neighbour features %.1e, |dF| ~ %.1e" % (
        derr, nerr, np.abs(dF).max()))
    assert derr <= 1e-4
    assert nerr <= 1e-4
    assert np.all(D[:, 63] == 0)


def test_correction_network_cuts_md_iterations():
    """What the trained correction network (the committed block, trained on
    2000 NVE frames of a different 4096-water trajectory, seed 1) gains over
    the history predictor alone on the benchmark's trajectory: iterations per
    step over 300 NVE steps after 200, at the same 1e-8 D."""
    block = np.load(os.path.join(os.path.dirname(mb.__file__), "data", "dipole_correction_box4096.npy"))
    ws = systems.workload("box4096", 0)
    its = {}
    for use in (False, True):
        c, run = _md_context(ws, 2, seed=0)
        if use:
            c.selectDipoleGuessNetwork(mb.Context.CorrectionNetwork)
            c.setDipoleGuessParameters(block)
            c.selectDipoleGuessNetwork(mb.Context.ColdStartNetwork)
        run(200)
        its[use] = run(300) / 300.0
        del c
    print("MD iterations/step: predictor %.3f, predictor + correction network %.3f" % (its[False], its[True]))
    assert its[True] <= its[False] - 0.05
