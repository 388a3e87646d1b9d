"""Train the learned induced-dipole guess on a seeded water box.

    python -m mbpol_openmm_plugin_gb300.train_guess --workload box4096 \
        --frames 2000 --steps 20000 --out dipole_guess_box4096.npy
    python -m mbpol_openmm_plugin_gb300.train_guess --network correction \
        --seed 1 --frames 2000 --steps 20000 --out dipole_correction_box4096.npy

NVT molecular dynamics (velocity Verlet, Andersen thermostat at 300 K,
0.2 fs) at 1e-8 D; after every step the network's inputs and targets are
collected on the device, and the network is trained there with the
library's own forward/backward kernels and Adam.  The cold-start network
learns the converged dipoles from the plain solver's frames (previous-step
guess); the correction network learns the history predictor's remaining
error (guess 2, from the 13th frame on, when the predictor runs).  The
parameter block (weights, biases and input standardisation;
mbpol_guess_get_params) is saved as float32 .npy.
"""
import argparse
import ctypes
import time

import numpy as np

from . import _capi
from .plugin import Context, create_mbpol_system, pme_parameters
from .systems import workload

DT_PS = 0.0002  # 0.2 fs
KT_PER_AMU = 0.00831446261815324 * 300.0  # kJ/mol per amu (nm/ps)^2 at 300 K


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="box4096")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--frames", type=int, default=2000)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--batch", type=int, default=4096)
    ap.add_argument("--lr", type=float, default=2e-3)
    ap.add_argument("--collision-rate", type=float, default=1.0, help="Andersen collisions per ps")
    ap.add_argument("--network", default="cold-start", choices=["cold-start", "correction"])
    ap.add_argument("--out", required=True)
    a = ap.parse_args(argv)
    correction = a.network == "correction"

    ws = workload(a.workload, a.seed)
    alpha, grid = pme_parameters(ws.box, 0.9, 1e-5) if ws.box is not None else (0.0, None)
    sysm = create_mbpol_system(ws, target_epsilon=1e-8, ewald_alpha=alpha, pme_grid=grid, guess=2 if correction else 1)
    ctx = Context(sysm)
    ctx.setPositions(ws.positions)
    ctx._build()
    if correction:
        ctx.selectDipoleGuessNetwork(Context.CorrectionNetwork)
    lib = _capi.load()
    h = ctx._h
    masses = np.ascontiguousarray(sysm.masses, np.float64)
    rng = np.random.default_rng(a.seed)
    vel = np.zeros((masses.size, 3))
    live = masses > 0
    vel[live] = rng.normal(size=(int(live.sum()), 3)) * np.sqrt(KT_PER_AMU / masses[live])[:, None]
    box = None if ws.box is None else np.ascontiguousarray(ws.box, np.float64)
    _capi.check(lib.mbpol_set_positions(h, _capi.ptr(np.ascontiguousarray(ws.positions)), _capi.ptr(box)))
    _capi.check(lib.mbpol_set_masses(h, _capi.ptr(masses)))
    _capi.check(lib.mbpol_set_velocities(h, _capi.ptr(vel)))
    ms, it, en = ctypes.c_double(), ctypes.c_long(), np.zeros(6)
    t0 = time.time()
    iters = 0
    for f in range(a.frames):
        _capi.check(lib.mbpol_md_run(h, 1, DT_PS, 300.0, a.collision_rate, a.seed * 1000003 + f, ctypes.byref(ms),
                                     _capi.ptr(en), ctypes.byref(it)))
        iters += it.value
        if not correction or f >= 12:   # the predictor needs 12 solves of history
            ctx.collectDipoleGuessSample()
    t1 = time.time()
    loss = ctx.trainDipoleGuess(a.steps, a.batch, a.lr, a.seed + 1)
    t2 = time.time()
    block = ctx.getDipoleGuessParameters()
    np.save(a.out, block)
    print("frames %d (%d samples, %.1f solver iterations/frame, %.1f s), training %d steps of %d: "
          "tail loss %.4g (%.1f s) -> %s" % (a.frames, ctx.getNumDipoleGuessSamples(), iters / max(a.frames, 1),
                                             t1 - t0, a.steps, a.batch, loss, t2 - t1, a.out))


if __name__ == "__main__":
    main()
