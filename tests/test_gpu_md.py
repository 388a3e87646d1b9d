"""GPU: the molecular-dynamics driver (mbpol_md_run), the role OpenMM's
integrators play for the reference plugin (python/example_nvt_nve.py:
VerletIntegrator for NVE, a thermostat for NVT).

  * one NVE step against a velocity-Verlet step done here in numpy on the
    library's own forces (mbpol_compute of a second context): positions and
    velocities to 1e-12 relative; the massless M sites are placed from
    their parents (python/mbpol.xml:14);
  * the Andersen thermostat: with frequent collisions the kinetic
    temperature averages to the bath's and each atom type's velocity
    variance to kT/m (Maxwell-Boltzmann)."""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN
import mbpol_openmm_plugin_gb300 as mb
from mbpol_openmm_plugin_gb300 import _capi, systems

pytestmark = pytest.mark.gpu
KB = 0.00831446261815324  # kJ/mol/K
MW = np.array([0.573293118, 0.213353441, 0.213353441])


def _context(ws, positions, masses, velocities):
    s = mb.create_mbpol_system(ws)
    ctx = mb.Context(s)
    ctx.setPositions(positions)
    ctx._build()
    lib = _capi.load()
    _capi.check(lib.mbpol_set_positions(ctx._h, _capi.ptr(np.ascontiguousarray(positions)), None))
    _capi.check(lib.mbpol_set_masses(ctx._h, _capi.ptr(np.ascontiguousarray(masses))))
    _capi.check(lib.mbpol_set_velocities(ctx._h, _capi.ptr(np.ascontiguousarray(velocities))))
    return ctx, s


def _forces(ctx, pos):
    lib = _capi.load()
    f = np.zeros_like(pos)
    e = np.zeros(5)
    _capi.check(lib.mbpol_set_positions(ctx._h, _capi.ptr(np.ascontiguousarray(pos)), None))
    _capi.check(lib.mbpol_compute(ctx._h, _capi.ALL_TERMS, _capi.ptr(e), _capi.ptr(f)))
    return f


def _place_m(p):
    p = p.copy()
    p[3::4] = MW[0] * p[0::4] + MW[1] * p[1::4] + MW[2] * p[2::4]
    return p


def test_nve_step_matches_velocity_verlet():
    d = np.load(os.path.join(GOLDEN, "cluster14_seed0.npz"))
    pos0 = _place_m(d["positions"])
    ws = systems.WaterSystem(pos0, None, 0, "cluster14")
    masses = np.tile([15.99943, 1.007947, 1.007947, 0.0], ws.num_waters)
    rng = np.random.default_rng(3)
    vel0 = rng.normal(size=pos0.shape) * np.sqrt(KB * 300.0 / np.where(masses > 0, masses, 1.0))[:, None]
    vel0[masses == 0] = 0.0
    dt = 0.0002
    ctx, _ = _context(ws, pos0, masses, vel0)
    lib = _capi.load()
    ms, it, en = ctypes.c_double(), ctypes.c_long(), np.zeros(6)
    _capi.check(lib.mbpol_md_run(ctx._h, 1, dt, 0.0, 0.0, 0, ctypes.byref(ms), _capi.ptr(en), ctypes.byref(it)))
    p_dev, v_dev, f_dev = (np.zeros_like(pos0) for _ in range(3))
    _capi.check(lib.mbpol_get_state(ctx._h, _capi.ptr(p_dev), _capi.ptr(v_dev), _capi.ptr(f_dev)))
    # the same step in numpy on a second context's forces
    ref, _ = _context(ws, pos0, masses, vel0)
    live = masses > 0
    invm = np.where(live, 1.0 / np.where(live, masses, 1.0), 0.0)[:, None]
    f0 = _forces(ref, pos0)
    vh = vel0 + 0.5 * dt * f0 * invm
    p1 = pos0 + dt * vh * live[:, None]
    p1 = _place_m(p1)
    f1 = _forces(ref, p1)
    v1 = vh + 0.5 * dt * f1 * invm
    perr = np.abs(p_dev - p1).max() / np.abs(p1).max()
    verr = np.abs(v_dev - v1).max() / np.abs(v1).max()
    ferr = np.abs(f_dev - f1).max() / np.abs(f1).max()
    print("one NVE step: positions %.1e, velocities %.1e, forces %.1e (max relative)" % (perr, verr, ferr))
    assert perr <= 1e-12 and verr <= 1e-12 and ferr <= 1e-10
    ekin = 0.5 * np.sum(masses[:, None] * v1 ** 2)
    assert abs(en[5] - ekin) <= 1e-10 * ekin


def test_andersen_thermostat_maxwell_boltzmann():
    d = np.load(os.path.join(GOLDEN, "cluster14_seed0.npz"))
    pos0 = _place_m(d["positions"])
    ws = systems.WaterSystem(pos0, None, 0, "cluster14")
    masses = np.tile([15.99943, 1.007947, 1.007947, 0.0], ws.num_waters)
    T, dt, nu = 300.0, 0.0002, 1000.0   # a collision per atom every ~5 steps
    ctx, _ = _context(ws, pos0, masses, np.zeros_like(pos0))
    lib = _capi.load()
    ms, it, en = ctypes.c_double(), ctypes.c_long(), np.zeros(6)
    _capi.check(lib.mbpol_md_run(ctx._h, 200, dt, T, nu, 11, ctypes.byref(ms), _capi.ptr(en), ctypes.byref(it)))
    temps, vO, vH = [], [], []
    p, v, f = (np.zeros_like(pos0) for _ in range(3))
    for k in range(300):
        _capi.check(lib.mbpol_md_run(ctx._h, 10, dt, T, nu, 11, ctypes.byref(ms), _capi.ptr(en), ctypes.byref(it)))
        temps.append(2.0 * en[5] / (3 * 3 * ws.num_waters * KB))
        _capi.check(lib.mbpol_get_state(ctx._h, None, _capi.ptr(v), None))
        vO.append(v[0::4].copy())
        vH.append(np.concatenate([v[1::4], v[2::4]]))
    Tm = float(np.mean(temps))
    sO = np.var(np.concatenate(vO)) * masses[0] / (KB * T)
    sH = np.var(np.concatenate(vH)) * masses[1] / (KB * T)
    print("Andersen: mean kinetic temperature %.1f K (bath %.0f K); m<v^2>/kT: O %.3f, H %.3f" % (Tm, T, sO, sH))
    assert abs(Tm - T) <= 0.05 * T
    assert abs(sO - 1.0) <= 0.1 and abs(sH - 1.0) <= 0.1
