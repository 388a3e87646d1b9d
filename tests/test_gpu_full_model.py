"""GPU parity of the full MB-pol model (one-, two-, three-body,
electrostatics, dispersion) on the reference's integration-test
configurations (python/tests/pdb_files), against the FP64 reference.

Tolerances (the project's acceptance bar): total energy relative error
<= 1e-6; total forces relative RMS error <= 1e-4."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_rms
import mbpol_openmm_plugin_gb300 as mb
from mbpol_openmm_plugin_gb300 import systems

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["water3", "water14", "water14_pme", "water50_pme", "water256_pme"])
def test_full_model(name):
    d = np.load(os.path.join(GOLDEN, "pdb_%s.npz" % name))
    periodic = bool(d["periodic"])
    ws = systems.WaterSystem(d["positions"], d["box"] if periodic else None, 0, name)
    s = mb.create_mbpol_system(ws, target_epsilon=1e-8, ewald_alpha=float(d["alpha"]),
                               pme_grid=[int(v) for v in d["grid"]] if periodic else None)
    ctx = mb.Context(s)
    ctx.setPositions(d["positions"])
    st = ctx.getState()
    e, eref = st.getPotentialEnergy(), float(d["etotal"])
    terms = dict(zip(["e1", "e2", "e3", "eelec", "edisp"], st.term_energies))
    for k, v in terms.items():
        print("  %s %.8f ref %.8f diff %.2e" % (k, v, float(d[k]), v - float(d[k])))
    ferr = rel_rms(st.getForces(), d["ftotal"])
    print(name, "E %.8f ref %.8f rel %.2e | F relrms %.2e" % (e, eref, abs(e - eref) / abs(eref), ferr))
    if not np.isnan(float(d["expected_kcal"])):
        assert abs(e / 4.184 - float(d["expected_kcal"])) <= float(d["expected_tol_kcal"])
    assert abs(e - eref) <= 1e-6 * abs(eref)
    assert ferr <= 1e-4
