"""GPU: updateParametersInContext through mbpol_update_parameters
(copyParametersToContext, MBPolReferenceKernels.cpp:116-126, 306-322,
401-411, 485-495).  A live context given new parameters evaluates as a
context built fresh with them (to rounding: forces are summed with FP64
atomics in no fixed order), keeps its solver state, and refuses a changed
count with the reference's message."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_rms
import mbpol_openmm_plugin_gb300 as mb
from mbpol_openmm_plugin_gb300 import _capi, systems

pytestmark = pytest.mark.gpu


def _elec(system):
    return next(f for f in system.forces if isinstance(f, mb.MBPolElectrostaticsForce))


def _evaluate(ctx, pos):
    ctx.setPositions(pos)
    st = ctx.getState()
    dip, it, _ = ctx.getInducedDipoles()
    return st.getPotentialEnergy(), np.asarray(st.getForces()), it


def test_electrostatics_parameters_match_fresh_context():
    d = np.load(os.path.join(GOLDEN, "elec_box256_seed0.npz"))
    ws = systems.WaterSystem(d["positions"], d["box"], 0, "box256")
    s = mb.create_mbpol_system(ws, terms=("electrostatics",), ewald_alpha=float(d["alpha"]),
                               pme_grid=[int(v) for v in d["grid"]])
    ctx = mb.Context(s)
    e0, f0, _ = _evaluate(ctx, d["positions"])
    # new polarisabilities and damping factors of the O sites
    f = _elec(s)
    for i in range(0, f.getNumElectrostatics(), 4):
        q, mol, typ, damp, pol = f.getElectrostaticsParameters(i)
        f.setElectrostaticsParameters(i, q, mol, typ, damp * 1.05, pol * 1.1)
    f.updateParametersInContext(ctx)
    e1, f1, it1 = _evaluate(ctx, d["positions"])
    fresh = mb.Context(s)
    e2, f2, it2 = _evaluate(fresh, d["positions"])
    print("E before %.8f, updated %.10f, fresh %.10f; iterations %d / %d; F relrms %.1e" % (
        e0, e1, e2, it1, it2, rel_rms(f1, f2)))
    assert abs(e1 - e0) > 1e-3 * abs(e0)          # the update took effect
    assert it1 == it2
    assert abs(e1 - e2) <= 1e-12 * abs(e2)
    assert rel_rms(f1, f2) <= 1e-10


def test_water_indices_match_fresh_context():
    d = np.load(os.path.join(GOLDEN, "cluster14_seed0.npz"))
    ws = systems.WaterSystem(d["positions"], None, 0, "cluster14")
    s = mb.create_mbpol_system(ws, terms=("onebody", "twobody", "threebody"))
    ctx = mb.Context(s)

    def _evaluate_terms(c):
        st = c.getState()
        return st.getPotentialEnergy(), np.asarray(st.getForces())

    ctx.setPositions(d["positions"])
    e0, _ = _evaluate_terms(ctx)
    one = next(f for f in s.forces if isinstance(f, mb.MBPolOneBodyForce))
    two = next(f for f in s.forces if isinstance(f, mb.MBPolTwoBodyForce))
    # the first two waters exchange their second H atoms
    a, b = one.getOneBodyParameters(0), one.getOneBodyParameters(1)
    a2, b2 = [a[0], a[1], b[2]], [b[0], b[1], a[2]]
    one.setOneBodyParameters(0, a2)
    one.setOneBodyParameters(1, b2)
    two.setParticleParameters(0, a2)
    two.setParticleParameters(1, b2)
    one.updateParametersInContext(ctx)
    two.updateParametersInContext(ctx)
    e1, f1 = _evaluate_terms(ctx)
    fresh = mb.Context(s)
    fresh.setPositions(d["positions"])
    e2, f2 = _evaluate_terms(fresh)
    print("E before %.8f, updated %.10f, fresh %.10f" % (e0, e1, e2))
    assert abs(e1 - e0) > 1.0
    assert abs(e1 - e2) <= 1e-12 * abs(e2)
    assert rel_rms(f1, f2) <= 1e-10


def test_changed_count_is_refused():
    d = np.load(os.path.join(GOLDEN, "cluster14_seed0.npz"))
    ws = systems.WaterSystem(d["positions"], None, 0, "cluster14")
    s = mb.create_mbpol_system(ws, terms=("onebody",))
    ctx = mb.Context(s)
    ctx.setPositions(d["positions"])
    ctx.getState()
    w = np.array(s.forces[0]._waters[:-1], np.int32)
    lib = _capi.load()
    rc = lib.mbpol_update_parameters(ctx._h, 0, w.shape[0], _capi.ptr(w), None, None, None, None, None)
    assert rc == 1  # MBPOL_ERR_INVALID_ARGUMENT
    assert b"number of one-body molecules has changed" in lib.mbpol_last_error()
