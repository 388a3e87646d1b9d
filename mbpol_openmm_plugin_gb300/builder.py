"""The mbpol_builder workflow of the reference (python/bin/mbpol_builder):
an INI file describing a water system and a run is turned into a Python
script that sets the run up and executes it, here with this package in place
of OpenMM and the plugin.  Sections and keys are the reference's
(python/mbpol_config.ini, python/example_ini/*.ini):

  [system]      pdb_filename, simulation_name, nonbonded (NoCutoff,
                CutoffNonPeriodic, CutoffPeriodic or PME), pme_box_size_nm
                (PME), ewald_error_tolerance (default 1e-8), temperature_k,
                local_minimization (default false)
  [thermostat]  collision_rate_1overps (Andersen)
  [barostat]    pressure_atm, barostat_interval: pressure coupling is not
                part of this package; the script raises NotImplementedError
  [integrator]  timestep_fs (default 1), equilibration_steps,
                production_steps; without this section the script evaluates
                energy and forces once
  [logging]     save_energy_every, save_positions_every (PDB trajectory),
                save_velocities_every (NetCDF through ParmEd in the
                reference: reported as unavailable, as the reference does
                without ParmEd)

The generated script uses the nonbonded cutoff of the reference's script
(0.9 nm) and runs on CUDA device 0.

    python -m mbpol_openmm_plugin_gb300.builder config.ini [script.py]

writes the script (or prints it without a second argument); `run(config)`
executes a configuration directly."""
import configparser
import sys

TEMPLATE = '''#!/usr/bin/env python
# Generated by mbpol_openmm_plugin_gb300.builder from {config_name}
import sys

import mbpol_openmm_plugin_gb300 as mb
from mbpol_openmm_plugin_gb300.simulation import (AndersenThermostat, LocalEnergyMinimizer, MonteCarloBarostat,
                                                  PDBReporter, Simulation, StateDataReporter, VerletIntegrator)

simulation_name = "{name}"
pdb = mb.PDBFile("{pdb}")
forcefield = mb.ForceField()
nonbonded = mb.{nonbonded}{pme}

system = forcefield.createSystem(pdb.topology, nonbondedMethod=nonbonded, nonbondedCutoff=0.9,
                                 ewaldErrorTolerance={ewald_tol})
temperature = float({temperature})
{thermostat}{barostat}
integrator = VerletIntegrator({timestep})

simulation = Simulation(pdb.topology, system, integrator)
simulation.setPositions(pdb.getPositions())

simulation_steps = {production}
equilibration_steps = {equilibration}

reporters = []{pdb_reporter}{state_reporter}
{minimization}
{integration}
'''


def _cfg(config):
    if isinstance(config, configparser.ConfigParser):
        return config
    c = configparser.ConfigParser()
    if not c.read(config):
        raise FileNotFoundError(config)
    return c


def build_script(config, config_name="configuration"):
    """The script text for an INI path or a ConfigParser."""
    c = _cfg(config)
    if "system" not in c.sections():
        raise ValueError("The configuration file needs a [system] section")
    s = c["system"]
    nonbonded = s["nonbonded"]
    if nonbonded not in ("NoCutoff", "CutoffNonPeriodic", "CutoffPeriodic", "PME"):
        raise ValueError("unknown nonbonded method %r" % nonbonded)
    save_energy = c.getint("logging", "save_energy_every", fallback=0)
    save_pos = c.getint("logging", "save_positions_every", fallback=0)
    save_vel = c.getint("logging", "save_velocities_every", fallback=0)
    pme = ""
    if nonbonded in ("PME", "CutoffPeriodic"):
        pme = ("\nbox = float({0})\npdb.topology.setUnitCellDimensions([box, box, box])".format(s["pme_box_size_nm"]))
    thermostat = ("\nsystem.addForce(AndersenThermostat(temperature, float({0})))".format(
        c["thermostat"]["collision_rate_1overps"]) if "thermostat" in c.sections() else "")
    barostat = ("\nsystem.addForce(MonteCarloBarostat(float({0}), temperature, int({1})))".format(
        c["barostat"]["pressure_atm"], c["barostat"]["barostat_interval"]) if "barostat" in c.sections() else "")
    production = c.getint("integrator", "production_steps", fallback=0)
    equilibration = c.getint("integrator", "equilibration_steps", fallback=0)
    total = max(production + equilibration, 1)
    pdb_reporter = ('\nreporters.append(PDBReporter(simulation_name + "_trajectory.pdb", {0}))'.format(save_pos)
                    if save_pos > 0 else "")
    state_reporter = ('\nreporters.append(StateDataReporter(simulation_name + ".log", {0}, step=True,\n'
                      '    potentialEnergy=True, temperature=True, progress=True, totalEnergy=True,\n'
                      '    kineticEnergy=True, totalSteps={1}, separator=","))'.format(save_energy, total)
                      if save_energy > 0 else "")
    minimization = ('\nprint("Running geometry optimization")\n'
                    'LocalEnergyMinimizer.minimize(simulation.context, 1e-1)\n'
                    'simulation.setPositions(simulation.context._pos)'
                    if c.getboolean("system", "local_minimization", fallback=False) else "")
    if c.has_section("integrator"):
        integration = '''
print("Setting random velocities based on temperature")
simulation.setVelocitiesToTemperature(temperature)
simulation.reporters.append(StateDataReporter(sys.stdout, max(1, int((simulation_steps + equilibration_steps) / 10)),
    step=True, progress=True, totalSteps=max(simulation_steps + equilibration_steps, 1), separator=","))
print("Running equilibration")
simulation.step(equilibration_steps)
print("Running simulation")
if {save_vel} > 0:
    print("Saving velocities to file requires the ParmEd python package")
for r in reporters:
    simulation.reporters.append(r)
simulation.step(simulation_steps)'''.format(save_vel=save_vel)
    else:
        integration = '''print("Computing forces and energy")
state = simulation.context.getState()
print("Potential energy %.6f kJ/mol" % state.getPotentialEnergy())
for r in reporters:
    r.report(simulation, simulation.getState())'''
    return TEMPLATE.format(config_name=config_name, name=s["simulation_name"], pdb=s["pdb_filename"],
                           nonbonded=nonbonded, pme=pme,
                           ewald_tol=c.getfloat("system", "ewald_error_tolerance", fallback=1e-8),
                           temperature=s["temperature_k"], thermostat=thermostat, barostat=barostat,
                           timestep=c.getfloat("integrator", "timestep_fs", fallback=1.0),
                           production=production, equilibration=equilibration, pdb_reporter=pdb_reporter,
                           state_reporter=state_reporter, minimization=minimization, integration=integration)


def run(config):
    """Build and execute the script of a configuration in this process."""
    code = build_script(config)
    exec(compile(code, "<mbpol_builder>", "exec"), {"__name__": "__main__"})


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    if not argv:
        print("usage: python -m mbpol_openmm_plugin_gb300.builder configuration_filename.ini [script_filename.py]")
        return 1
    text = build_script(argv[0], config_name=argv[0])
    if len(argv) > 1:
        with open(argv[1], "w") as fh:
            fh.write(text)
    else:
        print(text)
    return 0


if __name__ == "__main__":
    sys.exit(main())
