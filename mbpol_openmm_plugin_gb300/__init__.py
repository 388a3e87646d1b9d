"""GB300-native MB-pol force and energy evaluation with the MB-pol OpenMM
plugin's API (MBPolOneBodyForce, MBPolTwoBodyForce, MBPolThreeBodyForce,
MBPolElectrostaticsForce, MBPolDispersionForce).  Compute runs in the CUDA
library built from csrc/ (include/mbpol_gb300.h is its C ABI)."""
from .plugin import (  # noqa: F401
    MBPolOneBodyForce, MBPolTwoBodyForce, MBPolThreeBodyForce, MBPolElectrostaticsForce, MBPolDispersionForce,
    ThreeParticleAverageSite, System, Context, State, create_mbpol_system, pme_parameters,
)
from ._capi import MBPolError  # noqa: F401
from .forcefield import (  # noqa: F401
    ForceField, PDBFile, CMMotionRemover, NoCutoff, CutoffNonPeriodic, CutoffPeriodic, PME,
)
from .simulation import (  # noqa: F401
    VerletIntegrator, AndersenThermostat, MonteCarloBarostat, Simulation, StateDataReporter, PDBReporter,
    LocalEnergyMinimizer,
)

