"""GPU: scripts of the mbpol_builder workflow (INI -> script, python/bin/
mbpol_builder) run on the package's MD driver, on a seeded 14-water cluster
written as a PDB: the energy-only script reports the energy of a direct
evaluation; an NVE run writes its energy log and trajectory at the INI's
intervals and conserves the total energy; the local minimizer lowers the
energy; an NVT run of the 256-water PME box keeps a plausible temperature."""
import configparser
import os

import numpy as np
import pytest

from conftest import GOLDEN
import mbpol_openmm_plugin_gb300 as mb
from mbpol_openmm_plugin_gb300 import builder, systems
from mbpol_openmm_plugin_gb300.forcefield import water_topology
from mbpol_openmm_plugin_gb300.simulation import LocalEnergyMinimizer, Simulation, VerletIntegrator

pytestmark = pytest.mark.gpu


def cfg(text):
    c = configparser.ConfigParser()
    c.read_string(text)
    return c


@pytest.fixture()
def cluster_pdb(tmp_path, monkeypatch):
    ws = systems.cluster(14, 3)
    path = tmp_path / "cluster14.pdb"
    mb.PDBFile.writeFile(water_topology(14), ws.positions, str(path))
    monkeypatch.chdir(tmp_path)
    return path


def log_rows(path):
    rows = [ln.split(",") for ln in open(path) if not ln.startswith("#")]
    return [[float(v.strip().rstrip("%")) for v in r] for r in rows]


def test_energy_only_script(cluster_pdb):
    builder.run(cfg("""
[system]
pdb_filename = cluster14.pdb
simulation_name = c14
nonbonded = CutoffNonPeriodic
temperature_k = 300
[logging]
save_energy_every = 1
"""))
    pdb = mb.PDBFile(str(cluster_pdb))
    s = mb.ForceField().createSystem(pdb.topology, nonbondedMethod=mb.CutoffNonPeriodic, nonbondedCutoff=0.9,
                                     ewaldErrorTolerance=1e-8)
    ctx = mb.Context(s)
    ctx.setPositions(pdb.getPositions())
    e = ctx.getState().getPotentialEnergy()
    (row,) = log_rows("c14.log")
    print("script", row[1], "direct", e)
    assert abs(row[1] - e) <= 1e-6 * abs(e) + 1e-6


def test_nve_script_logs_and_conserves(cluster_pdb):
    builder.run(cfg("""
[system]
pdb_filename = cluster14.pdb
simulation_name = c14nve
nonbonded = CutoffNonPeriodic
temperature_k = 200
[integrator]
timestep_fs = 0.2
equilibration_steps = 4
production_steps = 40
[logging]
save_energy_every = 10
save_positions_every = 20
"""))
    rows = log_rows("c14nve.log")
    steps = [int(r[0]) for r in rows]
    assert steps == [10, 20, 30, 40]          # production reporting starts after the equilibration steps' count
    etot = np.array([r[3] for r in rows])
    print("total energies", etot, "temperatures", [r[4] for r in rows])
    assert np.ptp(etot) <= 2e-3 * np.abs(etot).max() + 0.05
    traj = open("c14nve_trajectory.pdb").read()
    assert traj.count("MODEL") == 2 and traj.count("ENDMDL") == 2


def test_local_minimizer_lowers_energy(cluster_pdb):
    pdb = mb.PDBFile(str(cluster_pdb))
    s = mb.ForceField().createSystem(pdb.topology, nonbondedMethod=mb.CutoffNonPeriodic, nonbondedCutoff=0.9)
    sim = Simulation(pdb.topology, s, VerletIntegrator(0.2))
    sim.setPositions(pdb.getPositions())
    e0 = sim.context.getState().getPotentialEnergy()
    res = LocalEnergyMinimizer.minimize(sim.context, tolerance=10.0, maxIterations=40)
    st = sim.context.getState()
    print("minimizer: %.4f -> %.4f kJ/mol in %d iterations" % (e0, st.getPotentialEnergy(), res["iterations"]))
    assert st.getPotentialEnergy() < e0 - 1.0
    # the virtual sites follow their parents through the minimizer and MD
    sim.step(1)
    p = sim.context._pos.reshape(-1, 4, 3)
    m = 0.573293118 * p[:, 0] + 0.213353441 * (p[:, 1] + p[:, 2])
    assert np.abs(p[:, 3] - m).max() < 1e-9


def test_nvt_pme_box(tmp_path, monkeypatch):
    d = np.load(os.path.join(GOLDEN, "box256_seed0.npz"))
    monkeypatch.chdir(tmp_path)
    mb.PDBFile.writeFile(water_topology(256, box=np.asarray(d["box"])), d["positions"], "box256.pdb")
    builder.run(cfg("""
[system]
pdb_filename = box256.pdb
simulation_name = b256
nonbonded = PME
pme_box_size_nm = %.6f
ewald_error_tolerance = 1e-5
temperature_k = 300
[integrator]
timestep_fs = 0.2
equilibration_steps = 0
production_steps = 30
[logging]
save_energy_every = 10
[thermostat]
collision_rate_1overps = 1.0
""" % float(d["box"][0])))
    rows = log_rows("b256.log")
    temps = [r[4] for r in rows]
    print("b256 temperatures", temps)
    assert len(rows) == 3 and all(150.0 < t < 600.0 for t in temps)
