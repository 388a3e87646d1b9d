"""Generate tests/golden/dipole_history_box4096.npz: converged induced
dipoles of consecutive MD steps, the input of the learned predictor's
parity test (tests/test_gpu_guess.py).  Needs a CUDA device.

    python tests/golden/make_dipole_history.py

The 4096-water box (mbpol_openmm_plugin_gb300.systems.workload("box4096")),
PME as in bench.py, 1e-8 D, extrapolated guess; 200 NVT steps (Andersen,
300 K, 0.2 fs), then NVE steps, reading the dipoles after each.  Saved:
the 12 solves before step 120 (newest first) and the solve of step 120,
first 3000 components of the O and H1 dipoles of the first 1024 waters.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
import bench  # noqa: E402
import mbpol_openmm_plugin_gb300 as mb  # noqa: E402
from mbpol_openmm_plugin_gb300 import _capi  # noqa: E402


def main():
    lib = _capi.load()
    ws, sysm, alpha, grid = bench.build_workload("box4096", 0, 3)
    ctx = mb.Context(sysm)
    ctx.setPositions(ws.positions)
    ctx._build()
    h = ctx._h
    box = np.ascontiguousarray(ws.box, np.float64)
    masses = np.array(sysm.masses)
    _capi.check(lib.mbpol_set_positions(h, _capi.ptr(np.ascontiguousarray(ws.positions)), _capi.ptr(box)))
    _capi.check(lib.mbpol_set_masses(h, _capi.ptr(np.ascontiguousarray(masses))))
    _capi.check(lib.mbpol_set_velocities(h, _capi.ptr(np.ascontiguousarray(bench.maxwell_boltzmann(masses, 300.0, 0)))))
    ms, it, en = ctypes.c_double(), ctypes.c_long(), np.zeros(6)
    _capi.check(lib.mbpol_md_run(h, 200, bench.DT_PS, 300.0, 10.0, 5, ctypes.byref(ms), _capi.ptr(en),
                                 ctypes.byref(it)))
    n = ws.positions.shape[0]
    sel = np.arange(0, n, 4)[:1024]
    sel = np.concatenate([sel, sel + 1])
    hist = []
    for _ in range(121):
        _capi.check(lib.mbpol_md_run(h, 1, bench.DT_PS, 0.0, 0.0, 0, ctypes.byref(ms), _capi.ptr(en),
                                     ctypes.byref(it)))
        d, _, _ = ctx.getInducedDipoles()
        hist.append(d[sel].reshape(-1))
    X = np.array(hist)
    t = 120
    np.savez_compressed(os.path.join(HERE, "dipole_history_box4096.npz"),
                        history=np.ascontiguousarray(X[t - 1::-1][:12][:, :3000]), next=X[t, :3000])


if __name__ == "__main__":
    main()
