"""GPU: systems built by ForceField().createSystem (the mbpol.xml flow of
python/tests/TestReferenceMBPolIntegrationTest.py and TestCustomDispersion.py)
against the reference fixtures.  Tolerances as the full-model tests: energy
relative error <= 1e-6, forces relative RMS <= 1e-4."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_rms
import mbpol_openmm_plugin_gb300 as mb
from mbpol_openmm_plugin_gb300.forcefield import water_topology

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["water3", "water256_pme"])
def test_integration_through_forcefield(name):
    d = np.load(os.path.join(GOLDEN, "pdb_%s.npz" % name))
    periodic = bool(d["periodic"])
    nw = d["positions"].shape[0] // 4
    top = water_topology(nw, 0, d["box"] if periodic else None)
    s = mb.ForceField().createSystem(top, nonbondedMethod=mb.PME if periodic else mb.NoCutoff,
                                     nonbondedCutoff=0.9)
    elec = s.getForce(0)
    elec.setMutualInducedTargetEpsilon(1e-8)
    if periodic:
        elec.setAEwald(float(d["alpha"]))
        elec.setPmeGridDimensions([int(v) for v in d["grid"]])
    ctx = mb.Context(s)
    ctx.setPositions(d["positions"])
    st = ctx.getState()
    e, eref = st.getPotentialEnergy(), float(d["etotal"])
    ferr = rel_rms(np.asarray(st.getForces()), d["ftotal"])
    print(name, "E %.8f ref %.8f rel %.2e | F relrms %.2e" % (e, eref, abs(e - eref) / abs(eref), ferr))
    assert abs(e - eref) <= 1e-6 * abs(eref)
    assert ferr <= 1e-4
    assert abs(e / 4.184 - float(d["expected_kcal"])) <= float(d["expected_tol_kcal"])


def test_custom_dispersion_water_and_ion():
    """python/tests/TestCustomDispersion.py:49-83: createSystem, remove the
    forces before the dispersion, evaluate."""
    d = np.load(os.path.join(GOLDEN, "disp_water_and_ion.npz"))
    s = mb.ForceField().createSystem(water_topology(1, 1), nonbondedMethod=mb.CutoffNonPeriodic,
                                     nonbondedCutoff=1e3)
    for _ in range(5):
        s.removeForce(0)
    ctx = mb.Context(s)
    ctx.setPositions(d["positions"])
    st = ctx.getState()
    e = st.getPotentialEnergy()
    print("water_and_ion E %.8f kcal/mol (reference test %.8f)" % (e / 4.184, float(d["expected_kcal"])))
    assert abs(e - float(d["edisp"])) <= 1e-6 * abs(float(d["edisp"]))
    assert rel_rms(np.asarray(st.getForces()), d["fdisp"]) <= 1e-4
    assert abs(e / 4.184 - float(d["expected_kcal"])) <= float(d["expected_tol_kcal"])
