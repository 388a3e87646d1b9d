"""Python mirror of the MB-pol plugin's API (python/mbpolplugin.i:42-171 and
openmmapi/include/openmm/MBPol*Force.h), running on the GB300 library.

OpenMM itself is not part of this package, so the few OpenMM pieces that
the plugin's tests use (System with masses and three-particle-average virtual
sites, Context.setPositions / getState) are provided as small stand-ins.
Units: nm, kJ/mol, kJ/mol/nm."""
import ctypes

import numpy as np

from . import _capi
from ._capi import as_c, check, ptr

# --------------------------------------------------------------------------
# parameters of python/mbpol.xml
MBPOL_THOLE = [0.4, 0.4, 0.055, 0.626, 0.055]        # mbpol.xml:22 (TCC, TCD, TDD, TDDOH, TDDHH)
MBPOL_CHARGE = {0: -5.1966000e-01, 1: 2.5983000e-01, 2: 0.0}   # mbpol.xml:24-26 (O, H, M)
MBPOL_DAMPING = {0: 0.00131, 1: 0.000294, 2: 0.00131}
MBPOL_POLARITY = {0: 0.00131, 1: 0.000294, 2: 0.0}
MBPOL_2B_CUTOFF = 0.65                                # mbpol.xml:31
MBPOL_3B_CUTOFF = 0.45                                # mbpol.xml:34
MBPOL_MASS = {0: 15.99943, 1: 1.007947, 2: 0.0}       # mbpol.xml:3-5
# dispersion tables, classes O=0, H=1, M=2, Cl=3 (mbpol.xml:52-83)
DISP_C6 = np.array([9.92951990e-4, 3.49345451e-4, 0, 0.00456078851,
                    3.49345451e-4, 8.40715638e-5, 0, 0.00085979832,
                    0, 0, 0, 0,
                    0.00456078851, 0.00085979832, 0, 0], float)
DISP_D6 = np.array([9.29548582e+01, 9.77520243e+01, 0, 1.638868407461115e+02,
                    9.77520243e+01, 9.40647517e+01, 0, 5.778854012725382e+01,
                    0, 0, 0, 0,
                    1.638868407461115e+02, 5.778854012725382e+01, 0, 0], float)


class _WaterForce:
    def __init__(self):
        self._waters = []
        self._method = 0
        self._group = 0

    def getNumMolecules(self):
        return len(self._waters)

    def setNonbondedMethod(self, m):
        self._method = int(m)

    def getNonbondedMethod(self):
        return self._method

    def setForceGroup(self, g):
        self._group = int(g)

    def getForceGroup(self):
        return self._group

    def _add(self, indices):
        idx = [int(v) for v in indices]
        if len(idx) != 3:
            raise ValueError("a water needs exactly 3 particle indices (O, H1, H2)")
        self._waters.append(idx)
        return len(self._waters) - 1

    def updateParametersInContext(self, context):
        """copyParametersToContext (MBPolReferenceKernels.cpp:116-126,
        401-411, 485-495): the waters' particle indices into a live context
        (mbpol_update_parameters), which keeps its lists, dipole history and
        predictor; the number of waters may not change."""
        if context._h is None:
            return
        w = as_c(np.array(self._waters, dtype=np.int32).reshape(-1, 3), np.int32)
        check(_capi.load().mbpol_update_parameters(context._h, self._term, w.shape[0], ptr(w), None, None, None,
                                                   None, None))


class MBPolOneBodyForce(_WaterForce):
    """openmmapi/include/openmm/MBPolOneBodyForce.h"""
    _term = 0
    NonPeriodic, Periodic = 0, 1

    def addOneBody(self, particleIndices):
        return self._add(particleIndices)

    def getNumOneBodys(self):
        return len(self._waters)

    def getOneBodyParameters(self, i):
        return list(self._waters[i])

    def setOneBodyParameters(self, i, particleIndices):
        self._waters[i] = [int(v) for v in particleIndices]

    def usesPeriodicBoundaryConditions(self):
        return self._method == self.Periodic


class _CutoffWaterForce(_WaterForce):
    NoCutoff, CutoffNonPeriodic, CutoffPeriodic = 0, 1, 2

    def __init__(self, cutoff):
        super().__init__()
        self._cutoff = cutoff

    def addParticle(self, particleIndices):
        return self._add(particleIndices)

    def getNumParticles(self):
        return len(self._waters)

    def getParticleParameters(self, i):
        return list(self._waters[i])

    def setParticleParameters(self, i, particleIndices):
        self._waters[i] = [int(v) for v in particleIndices]

    def setCutoff(self, c):
        self._cutoff = float(c)

    def getCutoff(self):
        return self._cutoff

    def usesPeriodicBoundaryConditions(self):
        return self._method == self.CutoffPeriodic


class MBPolTwoBodyForce(_CutoffWaterForce):
    """openmmapi/include/openmm/MBPolTwoBodyForce.h"""
    _term = 1

    def __init__(self):
        super().__init__(1.0)


class MBPolThreeBodyForce(_CutoffWaterForce):
    """openmmapi/include/openmm/MBPolThreeBodyForce.h.  setTrimerRule chooses
    between the reference's enumeration (default) and the complete one;
    setPolynomialEvaluator between the tensor-core evaluation of the
    polynomial (tcgen05; TensorCoresMmaSync for the legacy mma.sync path),
    the double-float walk and the automatic choice by size (default;
    mbpol_set_threebody_evaluator)."""
    _term = 2
    ReferenceTrimers, CompleteTrimers = 0, 1
    TensorCores, DoubleFloatWalk, AutomaticEvaluator, TensorCoresMmaSync = 0, 1, 2, 3

    def __init__(self):
        super().__init__(1.0)
        self._rule = 0
        self._evaluator = 2

    def setTrimerRule(self, r):
        self._rule = int(r)

    def getTrimerRule(self):
        return self._rule

    def setPolynomialEvaluator(self, kind):
        self._evaluator = int(kind)

    def getPolynomialEvaluator(self):
        return self._evaluator


class MBPolDispersionForce(_CutoffWaterForce):
    """Dispersion as built by the <Script> of python/mbpol.xml:37-108
    (-C6 tt6/r^6 over O/H pairs of different waters)."""
    _term = 4

    def __init__(self):
        super().__init__(0.9)
        self.c6 = DISP_C6.copy()
        self.d6 = DISP_D6.copy()
        self._ions = []

    def addIon(self, particleIndex):
        """A chloride ion (class Cl of the tables, python/mbpol.xml:52-83):
        it interacts with the O and H sites of every water and with the
        other ions, as the xml's CustomNonbondedForce does for a Cl residue."""
        self._ions.append(int(particleIndex))
        return len(self._ions) - 1

    def getNumIons(self):
        return len(self._ions)


class MBPolElectrostaticsForce:
    """openmmapi/include/openmm/MBPolElectrostaticsForce.h"""
    NoCutoff, PME = 0, 1
    # initial guess for the induced dipoles (this library's addition)
    DirectGuess, PreviousGuess, LearnedGuess = 0, 1, 2

    def __init__(self):
        self._particles = []
        self._method = 0
        self._cutoff = 0.9
        self._alpha = 0.0
        self._grid = [0, 0, 0]
        self._tol = 1e-4
        self._maxiter = 200
        self._eps = 1e-7
        self._thole = list(MBPOL_THOLE)
        self._redist = True
        self._guess = 0
        self._pme_field = 0
        self._group = 0

    def addElectrostatics(self, charge, moleculeIndex, atomType, dampingFactor, polarity):
        self._particles.append((float(charge), int(moleculeIndex), int(atomType), float(dampingFactor), float(polarity)))
        return len(self._particles) - 1

    def getNumElectrostatics(self):
        return len(self._particles)

    def getElectrostaticsParameters(self, i):
        return self._particles[i]

    def setElectrostaticsParameters(self, i, charge, moleculeIndex, atomType, dampingFactor, polarity):
        self._particles[i] = (float(charge), int(moleculeIndex), int(atomType), float(dampingFactor), float(polarity))

    def setNonbondedMethod(self, m):
        self._method = int(m)

    def getNonbondedMethod(self):
        return self._method

    def setCutoffDistance(self, d):
        self._cutoff = float(d)

    def getCutoffDistance(self):
        return self._cutoff

    def setAEwald(self, a):
        self._alpha = float(a)

    def getAEwald(self):
        return self._alpha

    def getPmeBSplineOrder(self):
        return 5

    def setPmeGridDimensions(self, g):
        self._grid = [int(v) for v in g]

    def getPmeGridDimensions(self):
        return list(self._grid)

    def setEwaldErrorTolerance(self, t):
        self._tol = float(t)

    def getEwaldErrorTolerance(self):
        return self._tol

    def setMutualInducedMaxIterations(self, n):
        self._maxiter = int(n)

    def getMutualInducedMaxIterations(self):
        return self._maxiter

    def setMutualInducedTargetEpsilon(self, e):
        self._eps = float(e)

    def getMutualInducedTargetEpsilon(self):
        return self._eps

    def setTholeParameters(self, t):
        self._thole = [float(v) for v in t]

    def getTholeParameters(self):
        return list(self._thole)

    def setIncludeChargeRedistribution(self, b):
        self._redist = bool(b)

    def getIncludeChargeRedistribution(self):
        return self._redist

    def setInducedDipoleGuess(self, g):
        self._guess = int(g)

    def getInducedDipoleGuess(self):
        return self._guess

    # Thole term of the PME permanent field: the reference's sign (default)
    # or the one whose forces are the gradient of the energy; no reference
    # counterpart (MBPolReferenceElectrostaticsForce.cpp:1377-1391)
    ReferencePmeField, ConsistentPmeField = 0, 1

    def setPmeFixedField(self, m):
        self._pme_field = int(m)

    def getPmeFixedField(self):
        return self._pme_field

    def setForceGroup(self, g):
        self._group = int(g)

    def getForceGroup(self):
        return self._group

    def updateParametersInContext(self, context):
        """copyParametersToContext (MBPolReferenceKernels.cpp:306-322): the
        per-particle charges, types, damping factors and polarities into a
        live context (mbpol_update_parameters), which keeps its lists, dipole
        history and predictor; the particles and molecules may not change."""
        if context._h is None:
            return
        q = as_c([p[0] for p in self._particles], np.float64)
        mol = as_c([p[1] for p in self._particles], np.int32)
        typ = as_c([p[2] for p in self._particles], np.int32)
        dmp = as_c([p[3] for p in self._particles], np.float64)
        pol = as_c([p[4] for p in self._particles], np.float64)
        check(_capi.load().mbpol_update_parameters(context._h, 3, len(self._particles), None, ptr(q), ptr(mol),
                                                   ptr(typ), ptr(dmp), ptr(pol)))

    def getElectrostaticPotential(self, inputGrid, context, outputElectrostaticPotential=None):
        """MBPolElectrostaticsForce.h:267: potential (kJ/mol/e) at the points
        of inputGrid (nm) from the charges and converged induced dipoles at
        the context's current positions.  Returns the values; when a list is
        passed as outputElectrostaticPotential it is filled as well."""
        pts = as_c(np.asarray(inputGrid, float).reshape(-1, 3), np.float64)
        if context._h is None:
            context._build()
        lib = _capi.load()
        box = None if context._box is None else as_c(context._box, np.float64)
        check(lib.mbpol_set_positions(context._h, ptr(context._pos), ptr(box)))
        out = np.zeros(pts.shape[0])
        check(lib.mbpol_get_electrostatic_potential(context._h, pts.shape[0], ptr(pts), ptr(out)))
        if outputElectrostaticPotential is not None:
            outputElectrostaticPotential[:] = out.tolist()
        return out

    def getSystemElectrostaticsMoments(self, context, outputElectrostaticsMoments=None):
        """mbpolKernels.h:121 (MBPolReferenceElectrostaticsForce.cpp:923-1021):
        the 13 system moments of the charges and converged induced dipoles
        at the context's current positions, about the System's centre of
        mass: net charge (e), dipole (Debye), traceless quadrupole
        xx xy xz yx yy yz zx zy zz (e nm^2 x 300 x 4.80321 / 2).  Returns
        the values; a list passed as outputElectrostaticsMoments is filled
        as well."""
        if context._h is None:
            context._build()
        lib = _capi.load()
        box = None if context._box is None else as_c(context._box, np.float64)
        check(lib.mbpol_set_positions(context._h, ptr(context._pos), ptr(box)))
        masses = as_c(context.system.masses, np.float64)
        out = np.zeros(13)
        check(lib.mbpol_get_system_multipole_moments(context._h, ptr(masses), ptr(out)))
        if outputElectrostaticsMoments is not None:
            outputElectrostaticsMoments[:] = out.tolist()
        return out

    def _params(self):
        p = _capi.ElectrostaticsParams()
        _capi.load().mbpol_electrostatics_params_default(ctypes.byref(p))
        p.nonbonded_method = self._method
        p.cutoff = self._cutoff
        p.ewald_alpha = self._alpha
        for k in range(3):
            p.pme_grid[k] = self._grid[k]
        p.ewald_error_tolerance = self._tol
        p.max_iterations = self._maxiter
        p.target_epsilon = self._eps
        for k in range(5):
            p.thole[k] = self._thole[k]
        p.include_charge_redistribution = 1 if self._redist else 0
        p.guess = self._guess
        p.pme_fixed_field = self._pme_field
        return p


class ThreeParticleAverageSite:
    def __init__(self, p1, p2, p3, w1, w2, w3):
        self.particles = (int(p1), int(p2), int(p3))
        self.weights = (float(w1), float(w2), float(w3))


class System:
    """Minimal stand-in for OpenMM's System."""

    def __init__(self):
        self.masses = []
        self.forces = []
        self.vsites = {}
        self.box = None

    def addParticle(self, mass):
        self.masses.append(float(mass))
        return len(self.masses) - 1

    def getNumParticles(self):
        return len(self.masses)

    def setVirtualSite(self, index, site):
        self.vsites[int(index)] = site

    def isVirtualSite(self, index):
        return int(index) in self.vsites

    def addForce(self, f):
        self.forces.append(f)
        return len(self.forces) - 1

    def getNumForces(self):
        return len(self.forces)

    def getForce(self, i):
        return self.forces[i]

    def removeForce(self, i):
        del self.forces[i]

    def getParticleMass(self, i):
        return self.masses[i]

    def setDefaultPeriodicBoxVectors(self, a, b, c):
        self.box = np.array([a[0], b[1], c[2]], float)


class State:
    def __init__(self, energy, forces, terms):
        self._energy = energy
        self._forces = forces
        self.term_energies = terms

    def getPotentialEnergy(self):
        return self._energy

    def getForces(self, asNumpy=True):
        return self._forces


TERM_OF = {MBPolOneBodyForce: _capi.TERM_ONEBODY, MBPolTwoBodyForce: _capi.TERM_TWOBODY,
           MBPolThreeBodyForce: _capi.TERM_THREEBODY, MBPolElectrostaticsForce: _capi.TERM_ELECTROSTATICS,
           MBPolDispersionForce: _capi.TERM_DISPERSION}


class Context:
    """Stand-in for OpenMM's Context on the GB300 library (one CUDA device)."""

    def __init__(self, system, device=0):
        self.system = system
        self.device = device
        self._h = None
        self._pos = None
        self._pos_dirty = False
        self._box = None if system.box is None else np.array(system.box, float)

    def _invalidate(self):
        self._destroy()

    def _destroy(self):
        if self._h is not None:
            _capi.load().mbpol_context_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self._destroy()
        except Exception:
            pass

    def _build(self):
        lib = _capi.load()
        n = self.system.getNumParticles()
        h = ctypes.c_void_p()
        check(lib.mbpol_context_create(n, self.device, ctypes.byref(h)))
        self._h = h
        for idx, vs in sorted(self.system.vsites.items()):
            check(lib.mbpol_add_average3_site(h, idx, *vs.particles, *vs.weights))
        for f in self.system.forces:
            if getattr(f, "_no_kernel", False):  # e.g. the centre-of-mass motion remover
                continue
            if isinstance(f, MBPolElectrostaticsForce):
                if f.getNumElectrostatics() != n:
                    raise _capi.MBPolError(1, "MBPolElectrostaticsForce must have exactly as many particles as the System")
                a = np.array(f._particles, dtype=object)
                q = as_c([p[0] for p in f._particles], np.float64)
                mol = as_c([p[1] for p in f._particles], np.int32)
                typ = as_c([p[2] for p in f._particles], np.int32)
                dmp = as_c([p[3] for p in f._particles], np.float64)
                pol = as_c([p[4] for p in f._particles], np.float64)
                prm = f._params()
                check(lib.mbpol_add_electrostatics_force(h, ctypes.byref(prm), ptr(q), ptr(mol), ptr(typ), ptr(dmp), ptr(pol)))
                del a
                continue
            w = as_c(np.array(f._waters, dtype=np.int32).reshape(-1, 3), np.int32)
            nw = w.shape[0]
            if isinstance(f, MBPolOneBodyForce):
                check(lib.mbpol_add_onebody_force(h, nw, ptr(w), f._method))
            elif isinstance(f, MBPolTwoBodyForce):
                check(lib.mbpol_add_twobody_force(h, nw, ptr(w), f._method, f._cutoff))
            elif isinstance(f, MBPolThreeBodyForce):
                check(lib.mbpol_add_threebody_force(h, nw, ptr(w), f._method, f._cutoff, f._rule))
                check(lib.mbpol_set_threebody_evaluator(h, f._evaluator))
            elif isinstance(f, MBPolDispersionForce):
                c6 = as_c(f.c6, np.float64)
                d6 = as_c(f.d6, np.float64)
                check(lib.mbpol_add_dispersion_force(h, nw, ptr(w), f._method, f._cutoff, ptr(c6), ptr(d6)))
                if f._ions:
                    ions = as_c(f._ions, np.int32)
                    check(lib.mbpol_add_dispersion_ions(h, len(f._ions), ptr(ions)))
            else:
                raise TypeError("unsupported force %r" % (f,))

    def setPositions(self, positions):
        self._pos = as_c(np.asarray(positions, float).reshape(-1, 3), np.float64)
        self._pos_dirty = True

    def setPeriodicBoxVectors(self, a, b, c):
        self._box = np.array([a[0], b[1], c[2]], float)

    def getState(self, getEnergy=True, getForces=True, groups=None):
        if self._h is None:
            self._build()
        lib = _capi.load()
        box = None if self._box is None else as_c(self._box, np.float64)
        check(lib.mbpol_set_positions(self._h, ptr(self._pos), ptr(box)))
        mask = 0
        for f in self.system.forces:
            if getattr(f, "_no_kernel", False):
                continue
            g = f.getForceGroup()
            if groups is None or (int(groups) >> g) & 1:
                mask |= 1 << TERM_OF[type(f)]
        e = np.zeros(_capi.NUM_TERMS)
        forces = np.zeros((self.system.getNumParticles(), 3))
        check(lib.mbpol_compute(self._h, mask, ptr(e), ptr(forces)))
        return State(float(e.sum()), forces, e)

    def getInducedDipoles(self):
        lib = _capi.load()
        d = np.zeros((self.system.getNumParticles(), 3))
        it = ctypes.c_int()
        eps = ctypes.c_double()
        check(lib.mbpol_get_induced_dipoles(self._h, ptr(d), ctypes.byref(it), ctypes.byref(eps)))
        return d, it.value, eps.value

    def getCounts(self):
        c = np.zeros(4, dtype=np.int64)
        check(_capi.load().mbpol_get_counts(self._h, ptr(c)))
        return c

    # ---- launch shapes of the polynomial kernels (this library's addition)
    def setAutotune(self, evaluations_per_shape=3):
        """Time the candidate launch shapes over the next 12 x n force
        evaluations (MD steps included) and keep the fastest
        (mbpol_set_autotune); 0 stops tuning."""
        if self._h is None:
            self._build()
        check(_capi.load().mbpol_set_autotune(self._h, int(evaluations_per_shape)))

    def setLaunchShape(self, tc_reserve_sms=-1, walk_reserve_blocks=-1):
        if self._h is None:
            self._build()
        check(_capi.load().mbpol_set_launch_shape(self._h, int(tc_reserve_sms), int(walk_reserve_blocks)))

    def getLaunchShape(self):
        """(SMs the three-body tensor kernel leaves free, blocks the walks
        leave out, whether the autotuner has finished)."""
        if self._h is None:
            self._build()
        a, b, t = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        check(_capi.load().mbpol_get_launch_shape(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(t)))
        return a.value, b.value, bool(t.value)

    # ---- batched independent clusters (this library's addition): one
    # context evaluates many water clusters that do not interact
    def setClusters(self, cluster_of_particle):
        """cluster_of_particle: (N,) cluster index of every particle, or None
        to end batching.  All forces must be non-periodic."""
        if self._h is None:
            self._build()
        if cluster_of_particle is None:
            check(_capi.load().mbpol_set_clusters(self._h, None, 0))
            self._ncl = 0
            return
        c = np.ascontiguousarray(cluster_of_particle, np.int32)
        if c.size != self.system.getNumParticles():
            raise ValueError("one cluster index per particle")
        self._ncl = int(c.max()) + 1 if c.size else 0
        check(_capi.load().mbpol_set_clusters(self._h, ptr(c), self._ncl))

    def getClusterResults(self):
        """(energies (nclusters, 5) kJ/mol in term order 1B, 2B, 3B,
        electrostatics, dispersion; solver iterations (nclusters,)) of the
        last evaluation."""
        n = getattr(self, "_ncl", 0)
        e = np.zeros((n, _capi.NUM_TERMS))
        it = np.zeros(n, np.int32)
        check(_capi.load().mbpol_get_cluster_results(self._h, ptr(e), ptr(it)))
        return e, it

    # ---- learned initial guess for the induced dipoles (guess = 2); this
    # library's addition, no reference counterpart
    ColdStartNetwork, CorrectionNetwork = 0, 1

    def selectDipoleGuessNetwork(self, which):
        """The network the calls below act on: ColdStartNetwork (default) or
        CorrectionNetwork (added to the history predictor's dipoles at every
        solve once it has parameters; mbpol_guess_select_network)."""
        if self._h is None:
            self._build()
        check(_capi.load().mbpol_guess_select_network(self._h, int(which)))

    def collectDipoleGuessSample(self):
        """Append the last evaluation's descriptors and converged dipoles
        (one sample per water) to the device-resident training set."""
        check(_capi.load().mbpol_guess_collect(self._h))

    def getNumDipoleGuessSamples(self):
        n = ctypes.c_long()
        check(_capi.load().mbpol_guess_num_samples(self._h, ctypes.byref(n)))
        return n.value

    def trainDipoleGuess(self, steps, batch=4096, learning_rate=2e-3, seed=1):
        """Train the network on the GPU; returns the mean loss of the last
        10% of the steps."""
        loss = ctypes.c_double()
        check(_capi.load().mbpol_guess_train(self._h, int(steps), int(batch), float(learning_rate), int(seed),
                                             ctypes.byref(loss)))
        return loss.value

    def getDipoleGuessParameters(self):
        b = np.zeros(_capi.GUESS_BLOCK_FLOATS, np.float32)
        check(_capi.load().mbpol_guess_get_params(self._h, ptr(b)))
        return b

    def setDipoleGuessParameters(self, block):
        b = np.ascontiguousarray(block, np.float32)
        if b.size != _capi.GUESS_BLOCK_FLOATS:
            raise ValueError("a parameter block has %d floats" % _capi.GUESS_BLOCK_FLOATS)
        if self._h is None:
            self._build()
        check(_capi.load().mbpol_guess_set_params(self._h, ptr(b)))

    def getDipoleGuessDescriptors(self):
        nw = self.system.getNumParticles() // 4
        d = np.zeros((nw, _capi.GUESS_INPUTS), np.float32)
        check(_capi.load().mbpol_guess_descriptors(self._h, ptr(d)))
        return d

    def dipoleGuessLossGrad(self, X, T):
        """Loss, gradient (8905) and outputs (n, 9) of the current network on
        raw inputs X (n, 64) and targets T (n, 9); no update."""
        X = np.ascontiguousarray(X, np.float32)
        T = np.ascontiguousarray(T, np.float32)
        n = X.shape[0]
        g = np.zeros(_capi.GUESS_PARAMS, np.float32)
        Y = np.zeros((n, 9), np.float32)
        loss = ctypes.c_double()
        check(_capi.load().mbpol_guess_loss_grad(self._h, ptr(X), ptr(T), n, ctypes.byref(loss), ptr(g), ptr(Y)))
        return loss.value, g, Y


def create_mbpol_system(ws, nonbonded_method="auto", terms=("onebody", "twobody", "threebody", "electrostatics",
                                                            "dispersion"), nonbonded_cutoff=0.9,
                        ewald_alpha=0.0, pme_grid=None, ewald_tol=1e-5, target_epsilon=1e-8, max_iterations=200,
                        trimer_rule=0, guess=0, pme_fixed_field=0):
    """Build the MB-pol System for a WaterSystem as ForceField('mbpol.xml')
    does (python/mbpol.py:65-76, 138-150, 211-223, 288-326 and the <Script>
    of python/mbpol.xml): per water O, H1, H2, M with the M virtual site."""
    periodic = ws.box is not None if nonbonded_method == "auto" else nonbonded_method == "PME"
    sys_ = System()
    nw = ws.num_waters
    for _ in range(nw):
        for t in (0, 1, 1, 2):
            sys_.addParticle(MBPOL_MASS[t])
    for w in range(nw):
        sys_.setVirtualSite(4 * w + 3, ThreeParticleAverageSite(4 * w, 4 * w + 1, 4 * w + 2, 0.573293118,
                                                                0.213353441, 0.213353441))
    if periodic:
        sys_.setDefaultPeriodicBoxVectors((ws.box[0], 0, 0), (0, ws.box[1], 0), (0, 0, ws.box[2]))
    waters = ws.water_indices()
    if "onebody" in terms:
        f = MBPolOneBodyForce()
        f.setNonbondedMethod(MBPolOneBodyForce.Periodic if periodic else MBPolOneBodyForce.NonPeriodic)
        for w in waters:
            f.addOneBody(w)
        sys_.addForce(f)
    if "twobody" in terms:
        f = MBPolTwoBodyForce()
        f.setCutoff(MBPOL_2B_CUTOFF)
        f.setNonbondedMethod(MBPolTwoBodyForce.CutoffPeriodic if periodic else MBPolTwoBodyForce.CutoffNonPeriodic)
        for w in waters:
            f.addParticle(w)
        sys_.addForce(f)
    if "threebody" in terms:
        f = MBPolThreeBodyForce()
        f.setCutoff(MBPOL_3B_CUTOFF)
        f.setTrimerRule(trimer_rule)
        f.setNonbondedMethod(MBPolThreeBodyForce.CutoffPeriodic if periodic else MBPolThreeBodyForce.CutoffNonPeriodic)
        for w in waters:
            f.addParticle(w)
        sys_.addForce(f)
    if "electrostatics" in terms:
        f = MBPolElectrostaticsForce()
        f.setNonbondedMethod(MBPolElectrostaticsForce.PME if periodic else MBPolElectrostaticsForce.NoCutoff)
        f.setCutoffDistance(nonbonded_cutoff)
        f.setTholeParameters(MBPOL_THOLE)
        f.setMutualInducedTargetEpsilon(target_epsilon)
        f.setMutualInducedMaxIterations(max_iterations)
        f.setInducedDipoleGuess(guess)
        f.setPmeFixedField(pme_fixed_field)
        if periodic:
            f.setEwaldErrorTolerance(ewald_tol)
            if ewald_alpha:
                f.setAEwald(ewald_alpha)
            if pme_grid is not None:
                f.setPmeGridDimensions(pme_grid)
        for w in range(nw):
            for t in (0, 1, 1, 2):
                f.addElectrostatics(MBPOL_CHARGE[t], w, t, MBPOL_DAMPING[t], MBPOL_POLARITY[t])
        sys_.addForce(f)
    if "dispersion" in terms:
        f = MBPolDispersionForce()
        f.setCutoff(nonbonded_cutoff)
        f.setNonbondedMethod(MBPolDispersionForce.CutoffPeriodic if periodic else MBPolDispersionForce.NoCutoff)
        for w in waters:
            f.addParticle(w)
        sys_.addForce(f)
    return sys_


def pme_parameters(box_nm, cutoff, tol):
    """Ewald alpha and grid by OpenMM's documented rule:
    alpha = sqrt(-ln(2 tol))/rc, n = ceil(2 alpha L / (3 tol^(1/5))) rounded up
    to a 2,3,5,7-smooth size."""
    alpha = np.sqrt(-np.log(2 * tol)) / cutoff
    grid = []
    for L in box_nm:
        n = int(np.ceil(2 * alpha * L / (3 * tol ** 0.2)))
        while True:
            m = n
            for p in (2, 3, 5, 7):
                while m % p == 0:
                    m //= p
            if m == 1:
                break
            n += 1
        grid.append(max(n, 6))
    return float(alpha), grid
