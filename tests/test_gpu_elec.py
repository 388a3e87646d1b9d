"""GPU parity: electrostatics (charge redistribution, Thole-damped induced
dipoles, NoCutoff and PME) through the C ABI vs the FP64 reference.

Tolerances: energy relative error <= 1e-6; forces relative RMS error <= 1e-4;
induced dipoles relative RMS error <= 1e-4 (FP32 pair arithmetic, FP64
accumulation and convergence test, same solver threshold)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_rms
import mbpol_openmm_plugin_gb300 as mb
from mbpol_openmm_plugin_gb300 import systems

pytestmark = pytest.mark.gpu
KCAL = 4.184


def elec_system(pos, box, alpha=0.0, grid=None, eps=1e-8):
    ws = systems.WaterSystem(pos, box, 0, "fixture")
    s = mb.create_mbpol_system(ws, terms=("electrostatics",), target_epsilon=eps, ewald_alpha=alpha,
                               pme_grid=grid)
    return s


@pytest.mark.parametrize("name", ["elec_cluster14_seed0", "elec_cluster14_seed1", "elec_box256_seed0"])
def test_electrostatics_vs_reference(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    periodic = bool(d["periodic"])
    box = d["box"] if periodic else None
    s = elec_system(d["positions"], box, float(d["alpha"]), [int(v) for v in d["grid"]] if periodic else None)
    ctx = mb.Context(s)
    ctx.setPositions(d["positions"])
    st = ctx.getState()
    e, eref = st.getPotentialEnergy(), float(d["eelec"])
    f, fref = st.getForces(), d["felec"]
    dip, it, eps = ctx.getInducedDipoles()
    derr = rel_rms(dip, d["dipoles"])
    print(name, "E %.8f ref %.8f rel %.2e | F relrms %.2e | dipoles relrms %.2e | iters %d ref %d" % (
        e, eref, abs(e - eref) / abs(eref), rel_rms(f, fref), derr, it, int(d["iterations"])))
    assert abs(e - eref) <= 1e-6 * abs(eref)
    assert rel_rms(f, fref) <= 1e-4
    assert derr <= 1e-4
    assert abs(it - int(d["iterations"])) <= 2


def test_water3_virtual_site_known_answer():
    """TestReferenceMBPolElectrostaticsForce.cpp:419-546 (NoCutoff, M sites,
    charge redistribution): E = -15.818784 kcal/mol."""
    k = json.load(open(os.path.join(GOLDEN, "elec_water3_virtualsite.json")))
    pos = np.array(k["positions_A"]) * 0.1
    s = elec_system(pos, None, eps=1e-7)
    ctx = mb.Context(s)
    ctx.setPositions(pos)
    st = ctx.getState()
    assert abs(st.getPotentialEnergy() / KCAL - k["expected_energy_kcal"]) < 1e-4
    assert abs(st.getPotentialEnergy() - k["oracle_energy_kJ"]) <= 1e-6 * abs(k["oracle_energy_kJ"])
    assert rel_rms(st.getForces(), np.array(k["oracle_forces_kJ_nm"])) <= 1e-4


def test_not_converged_status():
    """max_iterations too small: the call reports non-convergence, as the
    reference throws (MBPolReferenceElectrostaticsForce.cpp:888-894)."""
    d = np.load(os.path.join(GOLDEN, "elec_cluster14_seed0.npz"))
    s = elec_system(d["positions"], None)
    s.forces[0].setMutualInducedMaxIterations(2)
    ctx = mb.Context(s)
    ctx.setPositions(d["positions"])
    with pytest.raises(mb.MBPolError) as ei:
        ctx.getState()
    assert ei.value.status == 3


@pytest.mark.parametrize("name", ["potential_cluster14_seed0", "potential_box256_seed0"])
def test_electrostatic_potential_vs_reference(name):
    """MBPolElectrostaticsForce::getElectrostaticPotential against the compiled
    reference (MBPolReferenceElectrostaticsForce.cpp:1023-1085) on seeded probe
    points: max |error| <= 1e-5 of the largest |potential| (the induced
    dipoles carry the solver's FP32-field error, ~1e-6 relative)."""
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    periodic = bool(d["periodic"])
    box = d["box"] if periodic else None
    s = elec_system(d["positions"], box, float(d["alpha"]), [int(v) for v in d["grid"]] if periodic else None)
    ctx = mb.Context(s)
    ctx.setPositions(d["positions"])
    out = []
    phi = s.forces[0].getElectrostaticPotential(d["points"], ctx, out)
    ref = d["potential"]
    err = np.max(np.abs(phi - ref)) / np.max(np.abs(ref))
    print(name, "max |error| / max |potential| %.2e" % err)
    assert len(out) == len(ref)
    assert err <= 1e-5


@pytest.mark.parametrize("name", ["moments_cluster14_seed0", "moments_box256_seed0"])
def test_system_moments_vs_reference(name):
    """getSystemElectrostaticsMoments (mbpolKernels.h:121,
    MBPolReferenceElectrostaticsForce.cpp:923-1021) against the compiled
    reference, with the mbpol.xml masses: max |error| <= 1e-5 of the largest
    |moment| (the induced dipoles carry the solver's FP32-field error, ~1e-6
    relative); the net charge of neutral waters vanishes."""
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    periodic = bool(d["periodic"])
    box = d["box"] if periodic else None
    s = elec_system(d["positions"], box, float(d["alpha"]), [int(v) for v in d["grid"]] if periodic else None)
    assert np.allclose(s.masses, d["masses"])
    ctx = mb.Context(s)
    ctx.setPositions(d["positions"])
    out = []
    mom = s.forces[0].getSystemElectrostaticsMoments(ctx, out)
    ref = d["moments"]
    err = np.max(np.abs(mom - ref)) / np.max(np.abs(ref))
    print(name, "max |error| / max |moment| %.2e" % err)
    assert len(out) == 13
    assert err <= 1e-5
    assert abs(mom[0]) <= 1e-10
    # the quadrupole is symmetric and traceless
    Q = np.asarray(mom[4:]).reshape(3, 3)
    assert np.allclose(Q, Q.T) and abs(np.trace(Q)) <= 1e-9 * np.max(np.abs(Q))


def test_solver_graph_matches_host_loop():
    """A periodic system's solve runs as one graph launch with its stopping
    rules on the device; with the per-kernel timers on it runs the host loop
    instead (one host round trip per iteration).  Both take the reference's
    rules, so they agree: same iteration count, energies and forces to
    rounding (the residual sums use FP64 atomics in no fixed order)."""
    from mbpol_openmm_plugin_gb300 import _capi
    d = np.load(os.path.join(GOLDEN, "elec_box256_seed0.npz"))
    s = elec_system(d["positions"], d["box"], float(d["alpha"]), [int(v) for v in d["grid"]])
    res = []
    lib = _capi.load()
    for timers in (0, 1):
        lib.mbpol_profile_enable(timers)
        try:
            ctx = mb.Context(s)
            ctx.setPositions(d["positions"])
            st = ctx.getState()
            dip, it, eps = ctx.getInducedDipoles()
            res.append((st.getPotentialEnergy(), st.getForces(), it, eps))
        finally:
            lib.mbpol_profile_enable(0)
    (e0, f0, i0, p0), (e1, f1, i1, p1) = res
    print("graph E %.10f it %d eps %.3e | host loop E %.10f it %d eps %.3e | F relrms %.1e" % (
        e0, i0, p0, e1, i1, p1, rel_rms(f0, f1)))
    assert i0 == i1
    assert abs(e0 - e1) <= 1e-10 * abs(e1)
    assert rel_rms(f0, f1) <= 1e-9
