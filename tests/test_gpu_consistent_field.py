"""GPU: the consistent PME permanent field (MBPOL_PME_FIELD_CONSISTENT,
bn1 - (1 - s3)/r^3 for intermolecular pairs) against the oracle port in the
same mode, and the forces in both modes against the energy's gradient.

Tolerances: parity as for the reference mode (energy relative error <= 1e-6,
forces and induced dipoles relative RMS error <= 1e-4); finite differences
(central, h = 3e-4 nm along a random unit displacement of O and H, solver
converged to 1e-8 D) on the 14-water PME box: consistent mode within 2e-3 of
-F.D (the FP64 oracle: 6e-7), the reference's sign off by more than 0.5%
(the oracle: 1.1%; MBPolReferenceElectrostaticsForce.cpp:1377-1391).  In
larger boxes the hard real-space cutoff, which the reference shares, makes
the energy jump as pairs cross it and limits such a check to about 1%."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_rms
import mbpol_openmm_plugin_gb300 as mb
from mbpol_openmm_plugin_gb300 import systems

pytestmark = pytest.mark.gpu
oracle = pytest.importorskip("oracle")


def _context(pos, box, alpha, grid, mode, eps):
    ws = systems.WaterSystem(pos, box, 0, "fixture")
    s = mb.create_mbpol_system(ws, terms=("electrostatics",), target_epsilon=eps, ewald_alpha=alpha, pme_grid=grid,
                               max_iterations=400, pme_fixed_field=mode)
    ctx = mb.Context(s)
    ctx.setPositions(pos)
    return ctx


@pytest.mark.parametrize("name", ["pdb_water14_pme", "elec_box256_seed0"])
def test_consistent_field_vs_oracle(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    pos, box, alpha, grid = d["positions"], d["box"], float(d["alpha"]), [int(v) for v in d["grid"]]
    ctx = _context(pos, box, alpha, grid, mb.MBPolElectrostaticsForce.ConsistentPmeField, 1e-8)
    st = ctx.getState()
    dip, it, _ = ctx.getInducedDipoles()
    oracle.set_pme_fixed_field(True)
    try:
        r = oracle.full_model(pos, box, alpha, tuple(grid), eps=1e-8)
    finally:
        oracle.set_pme_fixed_field(False)
    e, eref = st.getPotentialEnergy(), r["eelec"]
    ferr, derr = rel_rms(st.getForces(), r["felec"]), rel_rms(dip, r["dipoles"])
    print(name, "E %.8f oracle %.8f rel %.2e | F relrms %.2e | dipoles relrms %.2e | iters %d oracle %d" % (
        e, eref, abs(e - eref) / abs(eref), ferr, derr, it, r["iterations"]))
    assert abs(e - eref) <= 1e-6 * abs(eref)
    assert ferr <= 1e-4
    assert derr <= 1e-4
    assert abs(it - r["iterations"]) <= 2


def test_forces_against_energy_gradient():
    d = np.load(os.path.join(GOLDEN, "pdb_water14_pme.npz"))
    pos, box, alpha, grid = d["positions"], d["box"], float(d["alpha"]), [int(v) for v in d["grid"]]
    D = np.random.default_rng(3).normal(size=pos.shape)
    D[3::4] = 0.0  # M sites follow O, H1, H2
    D /= np.linalg.norm(D)
    h = 3e-4
    mismatch = {}
    for mode in (mb.MBPolElectrostaticsForce.ReferencePmeField, mb.MBPolElectrostaticsForce.ConsistentPmeField):
        ctx = _context(pos, box, alpha, grid, mode, 1e-8)
        fdot = -np.sum(ctx.getState().getForces() * D)
        ctx.setPositions(pos + h * D)
        ep = ctx.getState().getPotentialEnergy()
        ctx.setPositions(pos - h * D)
        em = ctx.getState().getPotentialEnergy()
        mismatch[mode] = abs((ep - em) / (2 * h) - fdot) / abs(fdot)
        print("mode %d: -F.D %.6e dE/dh %.6e mismatch %.2e" % (mode, fdot, (ep - em) / (2 * h), mismatch[mode]))
    assert mismatch[mb.MBPolElectrostaticsForce.ConsistentPmeField] < 2e-3
    assert mismatch[mb.MBPolElectrostaticsForce.ReferencePmeField] > 5e-3
