"""GPU dispersion with chloride ions (python/mbpol.xml:37-108, Cl class of
the C6/d6 tables :52-83) against the oracle's FP64 port, which is pinned to
the reference's own known answers (python/tests/TestCustomDispersion.py).

Tolerances: energy relative error <= 1e-6, forces relative RMS <= 1e-4 (the
acceptance bar of the model); the reference test's own bar on the energy is
0.01 kcal/mol."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, rel_rms
import mbpol_openmm_plugin_gb300 as mb
from mbpol_openmm_plugin_gb300 import systems
from mbpol_openmm_plugin_gb300.plugin import ThreeParticleAverageSite

oracle = pytest.importorskip("oracle")

pytestmark = pytest.mark.gpu

CL_MASS = 35.4532  # python/mbpol.xml:6


def ion_system(nw, nion, box=None, cutoff=0.9):
    """Waters (O, H1, H2, M) followed by chloride ions, dispersion only."""
    s = mb.System()
    for _ in range(nw):
        for m in (15.99943, 1.007947, 1.007947, 0.0):
            s.addParticle(m)
    for _ in range(nion):
        s.addParticle(CL_MASS)
    for w in range(nw):
        s.setVirtualSite(4 * w + 3, ThreeParticleAverageSite(4 * w, 4 * w + 1, 4 * w + 2, 0.573293118,
                                                             0.213353441, 0.213353441))
    f = mb.MBPolDispersionForce()
    if box is not None:
        s.setDefaultPeriodicBoxVectors((box[0], 0, 0), (0, box[1], 0), (0, 0, box[2]))
        f.setNonbondedMethod(mb.MBPolDispersionForce.CutoffPeriodic)
        f.setCutoff(cutoff)
    else:
        f.setNonbondedMethod(mb.MBPolDispersionForce.NoCutoff)
    for w in range(nw):
        f.addParticle([4 * w, 4 * w + 1, 4 * w + 2])
    for i in range(nion):
        f.addIon(4 * nw + i)
    s.addForce(f)
    return s


@pytest.mark.parametrize("name", ["disp_water3", "disp_water_and_ion"])
def test_dispersion_known_answers(name):
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    nw, nion = len(d["waters"]), len(d["ions"])
    ctx = mb.Context(ion_system(nw, nion))
    ctx.setPositions(d["positions"])
    st = ctx.getState()
    e, f = st.getPotentialEnergy(), np.asarray(st.getForces())
    eref = float(d["edisp"])
    ferr = rel_rms(f, d["fdisp"])
    print(name, "E %.8f kcal/mol (port %.8f, reference test %.8f) | F relrms %.2e" % (
        e / 4.184, eref / 4.184, float(d["expected_kcal"]), ferr))
    assert abs(e - eref) <= 1e-6 * abs(eref)
    assert ferr <= 1e-4
    assert abs(e / 4.184 - float(d["expected_kcal"])) <= float(d["expected_tol_kcal"])


def test_dispersion_ions_in_periodic_box():
    """box256 (PME-sized box, cutoff 0.9 nm, minimum image) with six seeded
    chloride ions at least 0.25 nm from every site."""
    ws = systems.workload("box256", 0)
    pos = ws.positions.copy()
    nw = pos.shape[0] // 4
    for w in range(nw):
        pos[4 * w + 3] = 0.573293118 * pos[4 * w] + 0.213353441 * (pos[4 * w + 1] + pos[4 * w + 2])
    box = np.asarray(ws.box, float)
    rng = np.random.default_rng(7)
    ions = []
    while len(ions) < 6:
        g = box * rng.random(3)
        d = np.concatenate([pos, np.array(ions).reshape(-1, 3)]) - g
        d -= box * np.round(d / box)
        if np.sqrt((d * d).sum(1)).min() >= 0.25:
            ions.append(g)
    allpos = np.concatenate([pos, np.array(ions)])
    ctx = mb.Context(ion_system(nw, len(ions), box))
    ctx.setPositions(allpos)
    st = ctx.getState()
    e, f = st.getPotentialEnergy(), np.asarray(st.getForces())
    waters = np.stack([4 * np.arange(nw), 4 * np.arange(nw) + 1, 4 * np.arange(nw) + 2], 1)
    eref, fref = oracle.dispersion(allpos, waters, np.arange(4 * nw, 4 * nw + len(ions)), box, 0.9)
    ferr = rel_rms(f, fref)
    fion = rel_rms(f[4 * nw:], fref[4 * nw:])
    print("box256 + 6 Cl: E %.6f port %.6f rel %.2e | F relrms %.2e (ions %.2e)" % (
        e, eref, abs(e - eref) / abs(eref), ferr, fion))
    assert abs(e - eref) <= 1e-6 * abs(eref)
    assert ferr <= 1e-4 and fion <= 1e-4
