"""CPU: the mbpol_builder workflow (python/bin/mbpol_builder): INI -> script.
The configurations here exercise every key of the reference's INI format
(python/mbpol_config.ini): each generated script must compile, carry the
settings through, and fail loudly where the package has no counterpart
(pressure coupling)."""
import configparser

import numpy as np

import pytest

from mbpol_openmm_plugin_gb300 import builder


def cfg(text):
    c = configparser.ConfigParser()
    c.read_string(text)
    return c


NVT_PME = """
[system]
pdb_filename = box.pdb
simulation_name = box_nvt
nonbonded = PME
pme_box_size_nm = 1.9
ewald_error_tolerance = 1e-5
temperature_k = 310
[integrator]
timestep_fs = 0.2
equilibration_steps = 3
production_steps = 7
[logging]
save_positions_every = 5
save_energy_every = 2
[thermostat]
collision_rate_1overps = 2.5
"""

CLUSTER_MIN = """
[system]
pdb_filename = cluster.pdb
simulation_name = cluster_min
nonbonded = CutoffNonPeriodic
temperature_k = 300
local_minimization = true
[logging]
save_energy_every = 1
"""


def test_nvt_pme_script():
    code = builder.build_script(cfg(NVT_PME))
    compile(code, "<nvt>", "exec")
    for piece in ('mb.PDBFile("box.pdb")', "nonbonded = mb.PME", "box = float(1.9)", "ewaldErrorTolerance=1e-05",
                  "AndersenThermostat(temperature, float(2.5))", "VerletIntegrator(0.2)", "temperature = float(310)",
                  "equilibration_steps = 3", "simulation_steps = 7", 'PDBReporter(simulation_name + "_trajectory.pdb", 5)',
                  'StateDataReporter(simulation_name + ".log", 2', "totalSteps=10", "setVelocitiesToTemperature"):
        assert piece in code, piece
    assert "LocalEnergyMinimizer.minimize" not in code.split("import")[-1].split("\n", 1)[1]


def test_cluster_minimization_energy_only():
    code = builder.build_script(cfg(CLUSTER_MIN))
    compile(code, "<min>", "exec")
    assert "LocalEnergyMinimizer.minimize(simulation.context, 1e-1)" in code
    assert "Computing forces and energy" in code and "simulation.step" not in code
    assert "setUnitCellDimensions" not in code and "ewaldErrorTolerance=1e-08" in code


def test_barostat_and_bad_input():
    c = cfg(NVT_PME + "\n[barostat]\npressure_atm = 1.0\nbarostat_interval = 25\n")
    code = builder.build_script(c)
    assert "MonteCarloBarostat(float(1.0), temperature, int(25))" in code
    from mbpol_openmm_plugin_gb300.simulation import MonteCarloBarostat
    with pytest.raises(NotImplementedError):
        MonteCarloBarostat(1.0, 300.0, 25)
    with pytest.raises(ValueError):
        builder.build_script(cfg("[logging]\nsave_energy_every = 1\n"))
    with pytest.raises(ValueError):
        builder.build_script(cfg(CLUSTER_MIN.replace("CutoffNonPeriodic", "Ewald")))


def test_main_writes_script(tmp_path):
    ini = tmp_path / "c.ini"
    ini.write_text(NVT_PME)
    out = tmp_path / "run.py"
    assert builder.main([str(ini), str(out)]) == 0
    compile(out.read_text(), str(out), "exec")
    assert builder.main([]) == 1


class _FakeState:
    def __init__(self, e, f):
        self.e, self.f = e, f

    def getPotentialEnergy(self):
        return self.e

    def getForces(self):
        return self.f


class _FakeContext:
    """A context whose energy is an anisotropic quadratic well around x0
    (the fourth particle massless, like an M site) and whose evaluation
    fails (as a diverging dipole solve does) for large displacements."""

    def __init__(self, x0, k):
        class S:
            masses = [15.99, 1.008, 1.008, 0.0]
        self.system = S()
        self.x0, self.k = x0, k
        self._pos = x0 + 0.3
        self.calls = 0

    def setPositions(self, p):
        self._pos = np.array(p, float)

    def getState(self):
        from mbpol_openmm_plugin_gb300._capi import MBPolError
        self.calls += 1
        d = self._pos - self.x0
        if np.abs(d).max() > 2.0:
            raise MBPolError(3, "diverged")
        d[3] = 0.0
        return _FakeState(float((self.k * d * d).sum()), -2 * self.k * d)


def test_local_minimizer_on_a_quadratic_well():
    import numpy as np  # noqa: F811
    from mbpol_openmm_plugin_gb300.simulation import LocalEnergyMinimizer
    rng = np.random.default_rng(0)
    x0 = rng.normal(size=(4, 3))
    k = 10.0 ** rng.uniform(0, 4, size=(4, 3))
    ctx = _FakeContext(x0, k)
    m0 = ctx._pos[3].copy()
    res = LocalEnergyMinimizer.minimize(ctx, tolerance=1e-3, max_step=0.05)
    assert res["converged"], res
    assert np.abs(ctx._pos[:3] - x0[:3]).max() < 5e-4  # |force| < 1e-3 with stiffness >= 2
    assert np.all(ctx._pos[3] == m0)  # massless sites are not moved by the minimizer
