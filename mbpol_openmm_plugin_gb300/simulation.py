"""Molecular dynamics in OpenMM's shape on this package's MD kernels
(csrc/md.cu: velocity Verlet with an Andersen thermostat, all state on the
device).  These are the OpenMM pieces that the scripts of the reference's
python/bin/mbpol_builder and python/example_nvt_nve.py use: VerletIntegrator,
AndersenThermostat, app.Simulation with StateDataReporter and PDBReporter,
Context.setVelocitiesToTemperature and LocalEnergyMinimizer.  Units: nm, ps,
kJ/mol, K (the integrator's step in fs, as the builder's INI gives it)."""
import ctypes

import numpy as np

from . import _capi
from .forcefield import CMMotionRemover, PDBFile
from .plugin import Context, check, ptr

KB = 0.00831446261815324  # kJ/mol/K


class VerletIntegrator:
    """Velocity Verlet with a fixed step (OpenMM's VerletIntegrator)."""

    def __init__(self, stepSize_fs):
        self.dt_ps = float(stepSize_fs) * 1e-3

    def getStepSize(self):
        return self.dt_ps


class AndersenThermostat:
    """Andersen collisions at `collision_rate` per ps toward `temperature`
    (OpenMM's AndersenThermostat, added to the System as a force).  Applied
    by the MD kernels at the end of each step."""
    _no_kernel = True

    def __init__(self, temperature, collision_rate):
        self.temperature = float(temperature)
        self.collision_rate = float(collision_rate)
        self._group = 0

    def getDefaultTemperature(self):
        return self.temperature

    def getDefaultCollisionFrequency(self):
        return self.collision_rate

    def setForceGroup(self, g):
        self._group = int(g)

    def getForceGroup(self):
        return self._group


class MonteCarloBarostat:
    """Pressure coupling is not part of this package: constructing one is an
    error (the reference builder adds OpenMM's MonteCarloBarostat for its
    [barostat] section)."""

    def __init__(self, *args, **kwargs):
        raise NotImplementedError("MonteCarloBarostat: pressure coupling is not available in this package")


class MDState:
    """Positions, velocities and energies of a Simulation after a step."""

    def __init__(self, step, positions, velocities, energies, kinetic, dof):
        self.step = step
        self._pos = positions
        self._vel = velocities
        self.term_energies = energies
        self._kin = kinetic
        self.dof = dof

    def getPositions(self, asNumpy=True):
        return self._pos

    def getVelocities(self, asNumpy=True):
        return self._vel

    def getPotentialEnergy(self):
        return float(np.sum(self.term_energies))

    def getKineticEnergy(self):
        return self._kin

    def getTemperature(self):
        return 2.0 * self._kin / (self.dof * KB) if self.dof > 0 else 0.0


def degrees_of_freedom(system):
    """3 per particle with mass, minus 3 with a centre-of-mass motion
    remover (OpenMM's count; no constraints here)."""
    n = sum(1 for m in system.masses if m > 0)
    dof = 3 * n
    if any(isinstance(f, CMMotionRemover) for f in system.forces):
        dof -= 3
    return dof


def maxwell_boltzmann(masses, temperature, seed):
    rng = np.random.default_rng(seed)
    v = np.zeros((len(masses), 3))
    for i, m in enumerate(masses):
        if m > 0:
            v[i] = rng.normal(0.0, np.sqrt(KB * temperature / m), 3)
    return v


class Simulation:
    """app.Simulation: a Context of `system` on one device driven by
    `integrator`; step(n) runs n MD steps on the device, stopping only at
    the reporters' intervals (positions and velocities are read back there)."""

    def __init__(self, topology, system, integrator, device=0, seed=1):
        self.topology = topology
        self.system = system
        self.integrator = integrator
        self.context = Context(system, device)
        self.reporters = []
        self.currentStep = 0
        self.seed = int(seed)
        self._thermostat = next((f for f in system.forces if isinstance(f, AndersenThermostat)), None)
        self._vel = None
        self._uploaded = False
        self._state = None
        self.dof = degrees_of_freedom(system)

    # -- state set by the user
    def setPositions(self, positions):
        self.context.setPositions(positions)
        self._uploaded = False

    def setVelocities(self, velocities):
        self._vel = np.ascontiguousarray(np.asarray(velocities, float).reshape(-1, 3))
        self._uploaded = False

    def setVelocitiesToTemperature(self, temperature, randomSeed=None):
        self.setVelocities(maxwell_boltzmann(self.system.masses, float(temperature),
                                             self.seed if randomSeed is None else int(randomSeed)))

    # -- device
    def _upload(self):
        ctx = self.context
        if ctx._h is None:
            ctx._build()
        lib = _capi.load()
        if ctx._pos is None:
            raise _capi.MBPolError(6, "positions have not been set")
        box = None if ctx._box is None else np.ascontiguousarray(ctx._box, np.float64)
        check(lib.mbpol_set_positions(ctx._h, ptr(ctx._pos), ptr(box)))
        check(lib.mbpol_set_masses(ctx._h, ptr(np.ascontiguousarray(self.system.masses, np.float64))))
        if self._vel is None:
            self._vel = np.zeros((self.system.getNumParticles(), 3))
        check(lib.mbpol_set_velocities(ctx._h, ptr(self._vel)))
        ctx._pos_dirty = False
        self._uploaded = True

    def _run(self, n):
        lib = _capi.load()
        T, rate = (self._thermostat.temperature, self._thermostat.collision_rate) if self._thermostat else (0.0, 0.0)
        ms, iters, en = ctypes.c_double(), ctypes.c_long(), np.zeros(_capi.NUM_TERMS + 1)
        check(lib.mbpol_md_run(self.context._h, int(n), self.integrator.dt_ps, T, rate,
                               self.seed * 1000003 + self.currentStep, ctypes.byref(ms), ptr(en),
                               ctypes.byref(iters)))
        self.currentStep += int(n)
        n_part = self.system.getNumParticles()
        pos, vel = np.zeros((n_part, 3)), np.zeros((n_part, 3))
        check(lib.mbpol_get_state(self.context._h, ptr(pos), ptr(vel), None))
        self.context._pos = np.ascontiguousarray(pos)
        self._vel = vel
        self._state = MDState(self.currentStep, pos, vel, en[:_capi.NUM_TERMS].copy(), float(en[_capi.NUM_TERMS]),
                              self.dof)
        self._uploaded = True

    def step(self, steps):
        if not self._uploaded or self.context._pos_dirty:
            self._upload()
        remaining = int(steps)
        while remaining > 0:
            k = remaining
            for r in self.reporters:
                k = min(k, r.stepsUntilReport(self.currentStep))
            k = max(1, k)
            self._run(k)
            remaining -= k
            for r in self.reporters:
                if self.currentStep % r.interval == 0:
                    r.report(self, self._state)

    def getState(self):
        """The last MD state (after step()); before any step, an evaluation
        of the current positions."""
        if self._state is None:
            st = self.context.getState()
            v = self._vel if self._vel is not None else np.zeros((self.system.getNumParticles(), 3))
            m = np.array(self.system.masses)[:, None]
            return MDState(self.currentStep, self.context._pos, v, st.term_energies, 0.5 * float((m * v * v).sum()),
                           self.dof)
        return self._state


class StateDataReporter:
    """Comma-separated step, energies (kJ/mol), temperature (K), and
    progress every reportInterval steps (OpenMM's StateDataReporter with the
    builder's columns; `file` a path or an open text file)."""

    def __init__(self, file, reportInterval, step=True, potentialEnergy=True, kineticEnergy=False,
                 totalEnergy=False, temperature=False, progress=False, totalSteps=None, separator=",", **ignored):
        self._out = open(file, "w") if isinstance(file, str) else file
        self._own = isinstance(file, str)
        self.interval = int(reportInterval)
        self.cols = [(k, v) for k, v in (("Step", step), ("Potential Energy (kJ/mole)", potentialEnergy),
                                         ("Kinetic Energy (kJ/mole)", kineticEnergy),
                                         ("Total Energy (kJ/mole)", totalEnergy), ("Temperature (K)", temperature),
                                         ("Progress (%)", progress and totalSteps)) if v]
        self.total = totalSteps
        self.sep = separator
        self._header = False

    def stepsUntilReport(self, current_step):
        return self.interval - current_step % self.interval

    def report(self, simulation, state):
        if not self._header:
            self._out.write("#" + self.sep.join('"%s"' % k for k, _ in self.cols) + "\n")
            self._header = True
        vals = {"Step": "%d" % state.step, "Potential Energy (kJ/mole)": "%.6f" % state.getPotentialEnergy(),
                "Kinetic Energy (kJ/mole)": "%.6f" % state.getKineticEnergy(),
                "Total Energy (kJ/mole)": "%.6f" % (state.getPotentialEnergy() + state.getKineticEnergy()),
                "Temperature (K)": "%.4f" % state.getTemperature()}
        if self.total:
            vals["Progress (%)"] = "%.1f%%" % (100.0 * state.step / self.total)
        self._out.write(self.sep.join(vals[k] for k, _ in self.cols) + "\n")
        self._out.flush()

    def __del__(self):
        if getattr(self, "_own", False):
            try:
                self._out.close()
            except Exception:
                pass


class PDBReporter:
    """One MODEL per report with the positions (OpenMM's PDBReporter)."""

    def __init__(self, file, reportInterval):
        self.path = file
        self.interval = int(reportInterval)
        self._models = 0
        open(file, "w").close()

    def stepsUntilReport(self, current_step):
        return self.interval - current_step % self.interval

    def report(self, simulation, state):
        import io
        buf = io.StringIO()
        PDBFile.writeFile(simulation.topology, state.getPositions(), buf)
        self._models += 1
        body = [ln for ln in buf.getvalue().splitlines() if ln and ln != "END"]
        with open(self.path, "a") as fh:
            fh.write("MODEL     %4d\n" % self._models)
            fh.write("\n".join(b for b in body if not b.startswith("CRYST1") or self._models == 1) + "\n")
            fh.write("ENDMDL\n")


class LocalEnergyMinimizer:
    """OpenMM's LocalEnergyMinimizer: limited-memory BFGS (Nocedal & Wright,
    Numerical Optimization, Algorithm 7.4: the two-loop recursion, memory 8)
    on the positions of the particles with mass, the virtual sites following
    their parents (the context places them and projects their forces).  Each
    step moves no atom by more than `max_step` nm and backtracks (Armijo)
    while the energy does not decrease or cannot be evaluated; the search
    stops when the largest force component is below `tolerance` (kJ/mol/nm)
    or after maxIterations (0: no limit)."""

    @staticmethod
    def minimize(context, tolerance=10.0, maxIterations=0, max_step=0.02, memory=8):
        sysm = context.system
        free = np.array([m > 0 for m in sysm.masses])
        pos = np.array(context._pos, float).reshape(-1, 3)

        def evaluate(x):
            p = pos.copy()
            p[free] = x.reshape(-1, 3)
            context.setPositions(p)
            try:
                st = context.getState()
            except _capi.MBPolError:
                return np.inf, None
            e = st.getPotentialEnergy()
            if not np.isfinite(e):
                return np.inf, None
            return e, -np.asarray(st.getForces())[free].reshape(-1)

        x = pos[free].reshape(-1)
        e, g = evaluate(x)
        if g is None:
            raise _capi.MBPolError(3, "the starting geometry cannot be evaluated")
        hist_s, hist_y = [], []
        it = 0
        limit = int(maxIterations) if maxIterations else 1 << 30
        while np.abs(g).max() > tolerance and it < limit:
            # two-loop recursion: d = -H g
            q = g.copy()
            alphas = []
            for s_, y_ in reversed(list(zip(hist_s, hist_y))):
                a = s_.dot(q) / y_.dot(s_)
                alphas.append(a)
                q -= a * y_
            if hist_s:
                q *= hist_s[-1].dot(hist_y[-1]) / hist_y[-1].dot(hist_y[-1])
            for (s_, y_), a in zip(zip(hist_s, hist_y), reversed(alphas)):
                b = y_.dot(q) / y_.dot(s_)
                q += (a - b) * s_
            d = -q
            if d.dot(g) >= 0:  # not a descent direction: restart from steepest descent
                hist_s, hist_y = [], []
                d = -g
            step = min(1.0, max_step / max(np.abs(d.reshape(-1, 3)).max(), 1e-30))
            while True:
                x_new = x + step * d
                e_new, g_new = evaluate(x_new)
                if g_new is not None and e_new <= e + 1e-4 * step * d.dot(g):
                    break
                step *= 0.5
                if step < 1e-12:
                    p = pos.copy()
                    p[free] = x.reshape(-1, 3)
                    context.setPositions(p)
                    return {"energy": e, "iterations": it, "converged": False}
            s_k, y_k = x_new - x, g_new - g
            if s_k.dot(y_k) > 1e-12:
                hist_s.append(s_k)
                hist_y.append(y_k)
                if len(hist_s) > memory:
                    hist_s.pop(0)
                    hist_y.pop(0)
            x, e, g = x_new, e_new, g_new
            it += 1
        p = pos.copy()
        p[free] = x.reshape(-1, 3)
        context.setPositions(p)
        return {"energy": e, "iterations": it, "converged": bool(np.abs(g).max() <= tolerance)}
