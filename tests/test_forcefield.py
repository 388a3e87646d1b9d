"""CPU: the PDB reader/writer and the mbpol.xml force field loader
(mbpol_openmm_plugin_gb300.forcefield), against python/mbpol.py's
generators and python/mbpol.xml."""
import io
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
import mbpol_openmm_plugin_gb300 as mb
from mbpol_openmm_plugin_gb300 import systems
from mbpol_openmm_plugin_gb300.forcefield import water_topology



def test_pdb_round_trip():
    d = np.load(os.path.join(GOLDEN, "pdb_water14.npz"))
    pos = np.round(d["positions"] * 10.0, 3) / 10.0
    top = water_topology(14, 1, np.array([2.5, 2.6, 2.7]))
    pos = np.concatenate([pos, [[0.1, 0.2, 0.3]]])
    buf = io.StringIO()
    mb.PDBFile.writeFile(top, pos, buf)
    pdb = mb.PDBFile(io.StringIO(buf.getvalue()))
    assert np.allclose(pdb.positions, pos, rtol=0, atol=1e-12)
    assert np.allclose(pdb.topology.getUnitCellDimensions(), [2.5, 2.6, 2.7])
    res = list(pdb.topology.residues())
    assert [r.name for r in res] == ["HOH"] * 14 + ["Cl"]
    assert [a.name for a in res[0].atoms()] == ["O", "H1", "H2", "M"]


def test_builtin_parameters_match_reference_xml():
    """The built-in parameters against the reference's python/mbpol.xml as
    the loader read it (tests/golden/mbpol_xml_params.json, written by
    make_golden.py mbpol_xml)."""
    a = json.load(open(os.path.join(GOLDEN, "mbpol_xml_params.json")))
    b = mb.ForceField()
    rt = lambda v: json.loads(json.dumps(v))  # tuples as JSON lists
    assert a["thole"] == b.thole
    assert a["elec"] == rt(b.elec)
    assert a["masses"] == rt(b.masses)
    assert (a["cutoff2"], a["cutoff3"]) == (b.cutoff2, b.cutoff3)
    assert np.array_equal(a["c6"], b.c6) and np.array_equal(a["d6"], b.d6)
    assert a["templates"] == rt(b.templates)
    assert all(a["elements"].values())


def _summary(s):
    out = []
    for f in s.forces:
        if isinstance(f, mb.MBPolElectrostaticsForce):
            out.append(("elec", f._method, f._cutoff, tuple(f._thole), tuple(f._particles)))
        elif isinstance(f, mb.CMMotionRemover):
            continue
        else:
            out.append((type(f).__name__, f._method, getattr(f, "_cutoff", None),
                        tuple(tuple(w) for w in f._waters)))
    return sorted(out, key=str)


@pytest.mark.parametrize("method", ["NoCutoff", "PME"])
def test_create_system_matches_builder(method):
    """ForceField().createSystem gives the same System as
    create_mbpol_system (which follows python/mbpol.py for the waters)."""
    ws = systems.workload("box256" if method == "PME" else "cluster14", 0)
    nw = ws.num_waters
    top = water_topology(nw, 0, ws.box)
    s = mb.ForceField().createSystem(top, nonbondedMethod=method, nonbondedCutoff=0.9)
    ref = mb.create_mbpol_system(ws, nonbonded_method=method if method == "PME" else "NoCutoff",
                                 nonbonded_cutoff=0.9, target_epsilon=1e-7)
    for f in ref.forces:
        if isinstance(f, mb.MBPolElectrostaticsForce):
            f.setEwaldErrorTolerance(1e-4)
    assert s.masses == ref.masses
    assert sorted(s.vsites) == sorted(ref.vsites)
    assert [type(f).__name__ for f in s.forces] == [
        "MBPolElectrostaticsForce", "MBPolOneBodyForce", "MBPolTwoBodyForce", "MBPolThreeBodyForce",
        "CMMotionRemover", "MBPolDispersionForce"]
    if method == "NoCutoff":
        # app.NoCutoff gives the two- and three-body forces NoCutoff
        # (python/mbpol.py:118-121, 191-194); the builder gives clusters
        # CutoffNonPeriodic.  Their switching functions vanish beyond the
        # cutoffs, so the energies are the same.
        for f in s.forces[2:4]:
            assert f._method == type(f).NoCutoff
        for f in ref.forces:
            if isinstance(f, (mb.MBPolTwoBodyForce, mb.MBPolThreeBodyForce)):
                f.setNonbondedMethod(type(f).NoCutoff)
    assert _summary(s) == _summary(ref)


def test_method_maps():
    """python/mbpol.py:46-49, 118-121, 191-194, 291-293 and the script's map."""
    top = water_topology(3, 0, np.array([3.0, 3.0, 3.0]))
    ff = mb.ForceField()
    s = ff.createSystem(top, nonbondedMethod=mb.CutoffNonPeriodic, nonbondedCutoff=1.0)
    e, one, two, three, cm, disp = s.forces
    assert e._method == mb.MBPolElectrostaticsForce.NoCutoff
    assert one._method == mb.MBPolOneBodyForce.NonPeriodic
    assert two._method == mb.MBPolTwoBodyForce.CutoffNonPeriodic and two._cutoff == 0.65
    assert three._method == mb.MBPolThreeBodyForce.CutoffNonPeriodic and three._cutoff == 0.45
    assert disp._method == mb.MBPolDispersionForce.CutoffNonPeriodic and disp._cutoff == 1.0
    s = ff.createSystem(top, nonbondedMethod=mb.PME, nonbondedCutoff=0.9)
    assert s.forces[0]._method == mb.MBPolElectrostaticsForce.PME and s.forces[0]._cutoff == 0.9
    assert s.forces[1]._method == mb.MBPolOneBodyForce.Periodic
    assert s.forces[5]._method == mb.MBPolDispersionForce.CutoffPeriodic
    with pytest.raises(ValueError):
        ff.createSystem(top, nonbondedMethod=mb.CutoffPeriodic)
    with pytest.raises(ValueError):
        ff.createSystem(water_topology(3), nonbondedMethod=mb.PME)


def test_water_and_ion_system():
    """The flow of python/tests/TestCustomDispersion.py:49-83: the forces
    before the dispersion are removed by index."""
    s = mb.ForceField().createSystem(water_topology(1, 1), nonbondedMethod=mb.CutoffNonPeriodic,
                                     nonbondedCutoff=1e3)
    for _ in range(5):
        s.removeForce(0)
    assert s.getNumForces() == 1
    assert mb.CMMotionRemover().getForceGroup() == 0
    f = s.getForce(0)
    assert isinstance(f, mb.MBPolDispersionForce)
    assert f.getNumParticles() == 1 and f.getNumIons() == 1
    assert s.getParticleMass(4) == 35.4532
