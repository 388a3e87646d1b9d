/*
 * mbpol_gb300.h -- C ABI of the GB300-native MB-pol force/energy library.
 *
 * This is the drop-in boundary for the MB-pol OpenMM plugin's compute path.
 * In the reference, each force's computation sits behind an OpenMM kernel
 * (openmmapi/include/openmm/mbpolKernels.h:49-207):
 *     CalcMBPol{OneBody,TwoBody,ThreeBody,Electrostatics}ForceKernel
 *         ::initialize(const System&, const MBPol*Force&)
 *         ::execute(ContextImpl&, bool includeForces, bool includeEnergy)
 *         ::copyParametersToContext(ContextImpl&, const MBPol*Force&)
 * plus dispersion, which python/mbpol.xml:37-108 builds as an OpenMM
 * CustomNonbondedForce, and the M-site virtual site (python/mbpol.xml:14).
 * OpenMM is not part of this library, so the context (positions, box,
 * forces, virtual sites) is owned by an mbpol_context; the Force-class
 * layers (include/mbpol_gb300.hpp for C++, the mbpol_openmm_plugin_gb300
 * Python package) sit on top of these calls.
 *
 * Conventions (same as the reference): nm, kJ/mol, kJ/mol/nm; forces are
 * ACCUMULATED (+=) into caller-owned arrays; energies are doubles.  Host
 * pointers are borrowed for the duration of a call.  No C++ exception crosses
 * this boundary: every call returns an mbpol_status; mbpol_last_error() gives
 * the message for the calling thread.  One CUDA stream per context.  There is
 * no CPU fallback: without a usable CUDA device mbpol_context_create fails.
 */
#ifndef MBPOL_GB300_H
#define MBPOL_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

typedef int mbpol_status;
enum {
    MBPOL_OK = 0,
    MBPOL_ERR_INVALID_ARGUMENT = 1,  /* bad index, size or parameter        */
    MBPOL_ERR_CUDA = 2,              /* a CUDA runtime / cuFFT call failed   */
    MBPOL_ERR_NOT_CONVERGED = 3,     /* induced dipoles did not converge     */
    MBPOL_ERR_BOX_TOO_SMALL = 4,     /* box < 2 * cutoff                     */
    MBPOL_ERR_CAPACITY = 5,          /* neighbour capacity could not be met  */
    MBPOL_ERR_STATE = 6,             /* call order (e.g. no positions yet)   */
    MBPOL_ERR_NO_DEVICE = 7          /* no CUDA device                       */
};

/* Nonbonded methods, numbered as in the reference's Force classes. */
enum { MBPOL_ONEBODY_NONPERIODIC = 0, MBPOL_ONEBODY_PERIODIC = 1 };              /* MBPolOneBodyForce.h */
enum { MBPOL_NOCUTOFF = 0, MBPOL_CUTOFF_NONPERIODIC = 1, MBPOL_CUTOFF_PERIODIC = 2 }; /* MBPolTwoBodyForce.h, MBPolThreeBodyForce.h */
enum { MBPOL_ELEC_NOCUTOFF = 0, MBPOL_ELEC_PME = 1 };                             /* MBPolElectrostaticsForce.h */
/* Trimer enumeration: the reference's rule, or every trimer with a nonzero switch. */
enum { MBPOL_TRIMER_REFERENCE = 0, MBPOL_TRIMER_COMPLETE = 1 };

/* Energy slots returned by mbpol_compute (kJ/mol). */
enum {
    MBPOL_TERM_ONEBODY = 0,
    MBPOL_TERM_TWOBODY = 1,
    MBPOL_TERM_THREEBODY = 2,
    MBPOL_TERM_ELECTROSTATICS = 3,
    MBPOL_TERM_DISPERSION = 4,
    MBPOL_NUM_TERMS = 5
};
#define MBPOL_TERM_BIT(t) (1u << (t))
#define MBPOL_ALL_TERMS 0x1Fu

typedef struct mbpol_context mbpol_context;

/* Parameters of MBPolElectrostaticsForce (openmmapi/include/openmm/MBPolElectrostaticsForce.h:66-260;
 * defaults at openmmapi/src/MBPolElectrostaticsForce.cpp:43-48). */
typedef struct {
    int nonbonded_method;        /* MBPOL_ELEC_NOCUTOFF or MBPOL_ELEC_PME                      */
    double cutoff;               /* real-space cutoff (nm), PME only; default 0.9               */
    double ewald_alpha;          /* nm^-1; 0 = choose from ewald_error_tolerance               */
    int pme_grid[3];             /* 0 = choose from ewald_error_tolerance                       */
    double ewald_error_tolerance;/* default 1e-4                                                */
    int max_iterations;          /* mutual induced max iterations; default 200                  */
    double target_epsilon;       /* Debye; default 1e-7                                         */
    double thole[5];             /* TCC, TCD, TDD, TDDOH, TDDHH; default {0.4,0.4,0.055,0.626,0.055} */
    int include_charge_redistribution; /* default 1                                              */
    int guess;                   /* initial dipole guess: 0 direct (alpha*E_fixed, as the reference),
                                    1 previous call's dipoles, 2 learned (the network on a cold start,
                                    then polynomial extrapolation, then the learned linear predictor
                                    once MBPOL_GUESS_HISTORY solves exist), 3 polynomial extrapolation
                                    of the last (up to) four solves */
    int pme_fixed_field;         /* MBPOL_PME_FIELD_REFERENCE (default) or MBPOL_PME_FIELD_CONSISTENT;
                                    no reference counterpart, see the enum below */
} mbpol_electrostatics_params;

/* Real-space Thole term of the PME permanent field.  The reference adds the
 * damping correction (s3 - 1)/r^3 with the sign opposite to its energy
 * expression (MBPolReferenceElectrostaticsForce.cpp:1377-1391 against
 * :2609-2626), so under PME its forces are not the gradient of its energy
 * (the induced dipoles are not stationary for that energy).  CONSISTENT
 * takes bn1 - (1 - s3)/r^3, which makes forces and energy consistent;
 * REFERENCE reproduces the reference's numbers.  NoCutoff is unaffected. */
enum { MBPOL_PME_FIELD_REFERENCE = 0, MBPOL_PME_FIELD_CONSISTENT = 1 };

/* Fill p with the reference's defaults. */
void mbpol_electrostatics_params_default(mbpol_electrostatics_params* p);

/* Create / destroy a context for num_particles particles on CUDA device `device`.
 * Replaces the OpenMM Context + Platform::createKernel plumbing
 * (openmmapi/src/MBPolTwoBodyForceImpl.cpp:55-76). */
mbpol_status mbpol_context_create(int num_particles, int device, mbpol_context** out);
mbpol_status mbpol_context_destroy(mbpol_context* ctx);

/* Virtual site: particle `site` = w1*p1 + w2*p2 + w3*p3; its force is spread
 * back with the same weights (OpenMM ThreeParticleAverageSite, used for the
 * M site at python/mbpol.xml:14). */
mbpol_status mbpol_add_average3_site(mbpol_context* ctx, int site, int p1, int p2, int p3, double w1, double w2,
                                     double w3);

/* Force set-up.  `waters` holds num_waters x {O, H1, H2} particle indices
 * (the vector<int> passed to addOneBody/addParticle, python/mbpol.py:65-76).
 *   one-body:   CalcMBPolOneBodyForceKernel::initialize   (platforms/reference/src/MBPolReferenceKernels.cpp:77-101)
 *   two-body:   CalcMBPolTwoBodyForceKernel::initialize   (MBPolReferenceKernels.cpp:330-360)
 *   three-body: CalcMBPolThreeBodyForceKernel::initialize (MBPolReferenceKernels.cpp:420-449) */
mbpol_status mbpol_add_onebody_force(mbpol_context* ctx, int num_waters, const int* waters, int method);
mbpol_status mbpol_add_twobody_force(mbpol_context* ctx, int num_waters, const int* waters, int method,
                                     double cutoff);
mbpol_status mbpol_add_threebody_force(mbpol_context* ctx, int num_waters, const int* waters, int method,
                                       double cutoff, int trimer_rule);

/* Electrostatics over all num_particles particles (the reference requires one
 * entry per particle, openmmapi/src/MBPolElectrostaticsForceImpl.cpp:53-54),
 * with per-particle charge, molecule index, atom type (O=0, H=1, M=2),
 * damping factor and polarizability as in addElectrostatics
 * (MBPolElectrostaticsForce.h:153).  Waters must be laid out as consecutive
 * O, H1, H2, M particles, as the reference assumes
 * (platforms/reference/src/MBPolReferenceElectrostaticsForce.cpp:879-884).
 * Replaces CalcMBPolElectrostaticsForceKernel::initialize (MBPolReferenceKernels.cpp:127-207). */
mbpol_status mbpol_add_electrostatics_force(mbpol_context* ctx, const mbpol_electrostatics_params* params,
                                            const double* charge, const int* molecule, const int* atom_type,
                                            const double* damping, const double* polarity);

/* Dispersion over the O/H sites of `num_waters` waters ({O,H1,H2} each);
 * c6 and d6 are 4x4 class tables (O=0, H=1, M=2, Cl=3) as in python/mbpol.xml:52-83.
 * method: MBPOL_NOCUTOFF or MBPOL_CUTOFF_PERIODIC / MBPOL_CUTOFF_NONPERIODIC. */
mbpol_status mbpol_add_dispersion_force(mbpol_context* ctx, int num_waters, const int* waters, int method,
                                        double cutoff, const double* c6, const double* d6);

/* Chloride ions (class Cl of the tables) in the dispersion term, after
 * mbpol_add_dispersion_force: each ion interacts with the O and H sites of
 * every water and with the other ions, site distances within the cutoff, as
 * the CustomNonbondedForce of python/mbpol.xml:37-108 does for a Cl residue
 * (its exclusions: same residue, M sites).  Not available with batched
 * clusters. */
mbpol_status mbpol_add_dispersion_ions(mbpol_context* ctx, int num_ions, const int* particles);

/* Positions (3*num_particles, nm) and the rectangular box (3 lengths, nm),
 * or box = NULL for a non-periodic system.  Virtual sites are placed from
 * their parents on the device before each evaluation. */
mbpol_status mbpol_set_positions(mbpol_context* ctx, const double* xyz, const double* box);
/* updateParametersInContext / copyParametersToContext
 * (openmmapi/include/openmm/mbpolKernels.h:83,128,167,206;
 * MBPolReferenceKernels.cpp:116-126, 306-322, 401-411, 485-495): new
 * parameters of one term of a live context, which keeps its neighbour
 * lists, the dipoles of its last solves and its history predictor.
 * term MBPOL_TERM_ONEBODY / TWOBODY / THREEBODY / DISPERSION: count waters
 * with their particle indices [count][3] (O, H1, H2), count as at creation;
 * term MBPOL_TERM_ELECTROSTATICS: count = the particle count, with the
 * per-particle charge, molecule, atom type, damping and polarity of
 * mbpol_add_electrostatics_force (the molecule layout may not change).
 * Unused pointers may be NULL.  A changed count is MBPOL_ERR_INVALID_ARGUMENT
 * with the reference's message. */
mbpol_status mbpol_update_parameters(mbpol_context* ctx, unsigned term, int count, const int* waters,
                                     const double* charge, const int* molecule, const int* atom_type,
                                     const double* damping, const double* polarity);

/* Evaluate the terms in term_mask (MBPOL_TERM_BIT(...)), i.e. ::execute of each
 * kernel (MBPolReferenceKernels.cpp:120-125, 246-259, 362-399, 451-483).
 * energies (optional, MBPOL_NUM_TERMS doubles) receives each term's energy;
 * forces (optional, 3*num_particles) is ACCUMULATED into.  Returns
 * MBPOL_ERR_NOT_CONVERGED if the induced dipoles did not reach the target, as
 * the reference throws (MBPolReferenceElectrostaticsForce.cpp:888-894). */
mbpol_status mbpol_compute(mbpol_context* ctx, unsigned term_mask, double* energies, double* forces);

/* Molecular dynamics on the device (the integrator OpenMM provides for the
 * reference, python/example_nvt_nve.py): masses (amu; 0 = virtual/massless),
 * velocities (nm/ps).  mbpol_md_run advances nsteps of velocity Verlet with
 * time step dt (ps); collision_rate > 0 (1/ps) adds an Andersen thermostat at
 * `temperature` (K).  gpu_ms receives the CUDA-event time of the run on the
 * context's stream; energies (optional, MBPOL_NUM_TERMS + 1 doubles) the
 * last step's potential terms and kinetic energy; solver_iterations the
 * induced-dipole iterations summed over the run. */
mbpol_status mbpol_set_masses(mbpol_context* ctx, const double* masses);
mbpol_status mbpol_set_velocities(mbpol_context* ctx, const double* velocities);
mbpol_status mbpol_md_run(mbpol_context* ctx, int nsteps, double dt, double temperature, double collision_rate,
                          unsigned long long seed, double* gpu_ms, double* energies, long* solver_iterations);
/* Copy the device state (any pointer may be NULL). */
mbpol_status mbpol_get_state(mbpol_context* ctx, double* positions, double* velocities, double* forces);

/* Induced dipoles (3*num_particles, e*nm) of the last electrostatics
 * evaluation, with its solver iteration count and final epsilon (Debye). */
mbpol_status mbpol_get_induced_dipoles(mbpol_context* ctx, double* dipoles, int* iterations, double* epsilon);

/* Counts from the last evaluation: [0] two-body pairs, [1] trimers,
 * [2] electrostatics site pairs within the cutoff, [3] solver iterations. */
mbpol_status mbpol_get_counts(mbpol_context* ctx, long* counts4);

/* Electrostatic potential (kJ/mol/e) at num_points points (xyz, nm):
 * MBPolElectrostaticsForce::getElectrostaticPotential
 * (openmmapi/include/openmm/MBPolElectrostaticsForce.h:267;
 * MBPolReferenceKernels.cpp:261-283).  Evaluates the electrostatics at the
 * current positions (charges, converged induced dipoles), then sums
 * q/r - mu.(r_i - g)/r^3 over all particles, minimum-imaged under PME and
 * unscreened, as the reference.  Fails with MBPOL_ERR_NOT_CONVERGED as the
 * reference throws; not available with batched clusters. */
mbpol_status mbpol_get_electrostatic_potential(mbpol_context* ctx, int num_points, const double* points,
                                               double* potential);

/* System multipole moments: the reference's getSystemElectrostaticsMoments
 * (openmmapi/include/openmm/mbpolKernels.h:121; MBPolReferenceKernels.cpp:
 * 285-303, MBPolReferenceElectrostaticsForce.cpp:923-1021).  Evaluates the
 * electrostatics at the current positions, then, about the centre of mass
 * of masses[num_particles] (none when they sum to 0), moments[13] = net
 * charge (e), dipole x y z (Debye), the traceless quadrupole
 * xx xy xz yx yy yz zx zy zz (the reference's units: e nm^2 x 300 x 4.80321
 * / 2).  Positions as stored, not wrapped.  Fails with
 * MBPOL_ERR_NOT_CONVERGED as the reference throws; not available with
 * batched clusters. */
mbpol_status mbpol_get_system_multipole_moments(mbpol_context* ctx, const double* masses, double* moments);

/* Kernel timing with CUDA events on the launching stream (process-wide).
 * Kernel ids: 0 two-body polynomial, 1 three-body polynomial, 2 fixed field,
 * 3 induced field + solver update, 4 PME dipole pass (spread, FFT,
 * convolution, inverse FFT, gather), 5 electrostatic energy/forces.
 * Enabling clears previous records; read returns the summed time and count. */
mbpol_status mbpol_profile_enable(int on);
/* Kernels launched by this library so far (cuFFT's internal launches excluded). */
unsigned long long mbpol_launch_count(void);
mbpol_status mbpol_profile_read(int kernel, double* total_ms, long* launches);

const char* mbpol_status_string(mbpol_status s);
const char* mbpol_last_error(void);

/* ---- Three-body polynomial evaluator ------------------------------------
 * No reference counterpart (the reference runs the generated FP64 code of
 * platforms/reference/src/poly-3b-v2x.cpp).  MBPOL_POLY3B_TENSOR: the
 * polynomial re-expanded about a fixed point and evaluated as a quadratic
 * form on the tcgen05 tensor cores (fp16 operand pieces, FP32 sums; ~1e-5
 * kcal/mol per compact trimer).  MBPOL_POLY3B_TENSOR_SYNC: the same with
 * mma.sync (the legacy tensor-core path; kept for comparison).
 * MBPOL_POLY3B_WALK: the double-float trie walk on the FP32 pipe (~1e-12
 * relative).  MBPOL_POLY3B_AUTO (default): MBPOL_POLY3B_TENSOR from one full
 * wave of trimer tiles up (64 trimers per SM), the walk below, where a few
 * trimers' errors would be a larger share of the total energy and the
 * tensor kernel would not fill the GPU anyway.  A tcgen05 launch whose
 * bounded waits give up makes the evaluation return MBPOL_ERR_CUDA. */
enum { MBPOL_POLY3B_TENSOR = 0, MBPOL_POLY3B_WALK = 1, MBPOL_POLY3B_AUTO = 2, MBPOL_POLY3B_TENSOR_SYNC = 3 };
mbpol_status mbpol_set_threebody_evaluator(mbpol_context* ctx, int kind);

/* ---- Launch shapes and the autotuner -------------------------------------
 * No reference counterpart.  The persistent polynomial kernels leave part of
 * the GPU to the other streams (the electrostatics run beside them): the
 * three-body tensor kernel `tc_reserve_sms` SMs (default 52), the
 * double-float walks `walk_reserve_blocks` blocks of their grids (default
 * 24).  Results do not depend on these shapes (each unit's arithmetic is the
 * same on any grid); timing does, with the workload.
 * mbpol_set_autotune(ctx, n): the next 12 n force evaluations (MD steps
 *   included) time the candidate shapes (reserves 0/26/52/76 SMs x 0/48/96
 *   blocks), n evaluations each, with CUDA events on the context's stream,
 *   and keep the shape of the smallest median time; 0 turns tuning off.
 * mbpol_set_launch_shape: a fixed shape (negative values: the defaults);
 *   stops tuning.
 * mbpol_get_launch_shape: the shape in use; *tuned = 1 once tuning ended. */
mbpol_status mbpol_set_autotune(mbpol_context* ctx, int evaluations_per_shape);
mbpol_status mbpol_set_launch_shape(mbpol_context* ctx, int tc_reserve_sms, int walk_reserve_blocks);
mbpol_status mbpol_get_launch_shape(mbpol_context* ctx, int* tc_reserve_sms, int* walk_reserve_blocks, int* tuned);

/* ---- White-box probes ------------------------------------------------------
 * The reference tests two protected functions of its electrostatics directly
 * (platforms/reference/tests/TestReferenceMBPolElectrostaticsForce.cpp):
 * getAndScaleInverseRs (:80-131, src/MBPolReferenceElectrostaticsForce.cpp:261-333)
 * and computeWaterCharge (:326-417, src/...:2793-3096).  These run the device
 * functions the field kernels use, one thread on the current device, no
 * context needed.
 * mbpol_probe_thole_inverse_rs: rr[0..3] = Thole-scaled 1/r, 1/r^3, 3/r^5,
 *   15/r^7 (nm^-k) for site damping factors damp_i, damp_j and Thole
 *   parameter `thole` (FP32 as in the kernels).
 * mbpol_probe_water_charges: positions_nm = O, H1, H2 (9 doubles);
 *   charges[4] = O, H1, H2, M (e); derivatives[27] = [particle O, H1, H2]
 *   [charge of H1, H2, M][xyz] (e/nm), i.e. the reference's
 *   particle.chargeDerivatives[vsH1f | vsH2f | vsMf]. */
mbpol_status mbpol_probe_thole_inverse_rs(double r_nm, double damp_i, double damp_j, double thole, double rr[4]);
mbpol_status mbpol_probe_water_charges(const double positions_nm[9], double charges[4], double derivatives[27]);

/* ---- Batched independent clusters ---------------------------------------
 * No reference counterpart as one call: the reference evaluates each water
 * cluster in its own OpenMM Context.  Here one context holds many clusters
 * and every kernel runs over all of them at once: particle i belongs to
 * cluster cluster_of_particle[i] (0 .. num_clusters-1) and no term couples
 * two clusters (neighbour lists, dispersion and electrostatics are
 * restricted to the cluster; each cluster's induced dipoles converge on their
 * own epsilon with the reference's stopping rules).  All forces must use
 * non-periodic methods (NoCutoff electrostatics).  num_clusters = 0 ends
 * batching.  mbpol_compute's energies are then the sums over clusters. */
mbpol_status mbpol_set_clusters(mbpol_context* ctx, const int* cluster_of_particle, int num_clusters);
/* Per-cluster energies [num_clusters][MBPOL_NUM_TERMS] (kJ/mol, term order
 * of MBPOL_TERM_*) and solver iterations [num_clusters] of the last
 * evaluation (either pointer may be NULL). */
mbpol_status mbpol_get_cluster_results(mbpol_context* ctx, double* energies, int* iterations);

/* ---- Learned initial guess for the induced dipoles ----------------------
 * No reference counterpart: the reference starts every solve from
 * alpha * E_fixed (MBPolReferenceElectrostaticsForce.cpp:557-616).  The
 * network (64-64-64-9, SiLU, BF16 weights on the tensor cores) predicts the
 * O, H1, H2 dipoles in the water's own frame from 48 descriptors of the
 * water's neighbourhood within 0.6 nm and the permanent field at its three
 * sites.  With mbpol_electrostatics_params.guess = 2 and a trained network
 * the solver starts from the prediction (cold start, or mu_prev + m - m_prev
 * after one solve) and, once two solves exist, from the polynomial
 * extrapolation of the last solves (guess 3), which in a smooth trajectory
 * is more precise than a BF16 network.  The solver, its threshold and its
 * stopping rules are unchanged, so the results agree with the plain path
 * within the solver tolerance.
 * A parameter block is MBPOL_GUESS_BLOCK_FLOATS floats: W1[64][64], b1[64],
 * W2[64][64], b2[64], W3[9][64], b3[9], then the input means[64] and
 * inverse standard deviations[64]. */
#define MBPOL_GUESS_BLOCK_FLOATS 9033
/* Append the last evaluation's descriptors and converged dipoles (one sample
 * per water) to the context's training set on the device. */
mbpol_status mbpol_guess_collect(mbpol_context* ctx);
mbpol_status mbpol_guess_num_samples(mbpol_context* ctx, long* n);
/* Train on the collected samples on the GPU (Adam, cosine step decay,
 * batches drawn uniformly); final_loss = mean batch loss of the last 10% of
 * the steps (units: (1e-3 e nm)^2 / 2 per output). */
mbpol_status mbpol_guess_train(mbpol_context* ctx, int steps, int batch, double learning_rate,
                               unsigned long long seed, double* final_loss);
mbpol_status mbpol_guess_get_params(mbpol_context* ctx, float* block);
mbpol_status mbpol_guess_set_params(mbpol_context* ctx, const float* block);
/* Network inputs [n_waters][64] of the last evaluation (48 descriptors,
 * 9 field components, 7 zeros; for the correction network: 48 descriptors,
 * the water's unpredicted field change (9), its neighbours' (6), 1 zero). */
mbpol_status mbpol_guess_descriptors(mbpol_context* ctx, float* out);
/* Which network the mbpol_guess_* calls act on: 0 the cold-start network
 * above (default), 1 the correction network.  No reference counterpart.
 * The correction network has the same shape and parameter block; once it
 * has parameters, every solve that starts from the history predictor below
 * adds its output to the predictor's dipoles: mu = P(X) + g dF + N(D), where
 * dF = F_new - P(F) is the unpredicted change of alpha E0 and D the water's
 * 48 descriptors, its own dF at O, H1, H2 and the sums of fc(r) dF over the
 * waters within 0.6 nm (O and H sites), all in the water's frame; N outputs
 * the O, H1, H2 dipole corrections in units of 1e-7 e nm.  Its training
 * samples (mbpol_guess_collect with network 1 selected) are the last
 * solve's inputs with targets mu_converged - (P(X) + g dF); while network 1
 * is selected the inputs are computed at every predictor start. */
mbpol_status mbpol_guess_select_network(mbpol_context* ctx, int which);
/* Loss, gradient [8905] (the training kernel) and outputs [n][9] (the
 * prediction kernel the solves use) of the current network on host data
 * X [n][64] (raw inputs), T [n][9] (targets), without an update. */
mbpol_status mbpol_guess_loss_grad(mbpol_context* ctx, const float* X, const float* T, int n, double* loss,
                                   float* grad, float* Y);
/* The learned linear predictor used by guess 2 once MBPOL_GUESS_HISTORY
 * solves exist: mu = P(X) + g (F_new - P(F)), P(Y) = Y0 + sum_j a_j nabla^j Y0
 * over backward differences of orders 1..MBPOL_GUESS_PREDICTOR_ORDER, F =
 * alpha E0 (polarisability times permanent field) of each step, g =
 * MBPOL_GUESS_FIELD_GAIN; the a are refitted on the dipoles by least squares
 * over the last MBPOL_GUESS_PREDICTOR_WINDOW steps before every solve.  On
 * host history [MBPOL_GUESS_HISTORY][n3] of dipoles and of alpha E0 (newest
 * first) and alpha E0 of the new geometry [n3]: the coefficients
 * [MBPOL_GUESS_PREDICTOR_ORDER] and the prediction [n3]. */
#define MBPOL_GUESS_FIELD_GAIN 2.4
#define MBPOL_GUESS_PREDICTOR_ORDER 7
#define MBPOL_GUESS_PREDICTOR_WINDOW 4
#define MBPOL_GUESS_HISTORY 12
mbpol_status mbpol_guess_fit_predictor(mbpol_context* ctx, const double* history, const double* field,
                                       const double* field_now, int n3, double* coef, double* prediction);

/* ---- Two-body term without device allocation ---------------------------
 * No reference counterpart: the reference evaluates the two-body term only
 * inside MBPolReferenceTwoBodyForce::calculateForceAndEnergy
 * (platforms/reference/src/MBPolReferenceTwoBodyForce.cpp) over the
 * neighbour list it builds itself.  This entry point is for callers that own
 * all device memory and cannot let the library allocate (their own pool, no
 * cudaMalloc/cudaFree inside a step loop): it evaluates the two-body energy
 * and forces for a caller-built dimer list on caller-owned DEVICE buffers,
 * using per-device scratch held in static device arrays, and never calls
 * cudaMalloc, cudaFree or an allocating library.
 *   positions  device, 3*num_particles doubles (nm)
 *   waters     device, 4 ints per water {O, H1, H2, unused}, 16-byte aligned
 *   dimers     device, 2 ints per dimer (water indices), 8-byte aligned;
 *              indices are NOT checked and must be in range
 *   box_nm     HOST, 3 doubles (rectangular, each >= 1.3 nm), or NULL
 *   forces     device, 3*num_particles doubles, accumulated (+=), kJ/mol/nm
 *   energy     device, one double, accumulated (+=), kJ/mol
 *   stream     cudaStream_t (NULL: the default stream)
 * More than MBPOL_NOALLOC_MAX_DIMERS dimers is MBPOL_ERR_CAPACITY (split the
 * list into ordered calls).  The first call on a device does a synchronous
 * set-up (symbol addresses, tables, constants) and should precede any stream
 * capture.  The scratch is shared by all calls on a device: calls whose
 * kernels could overlap (other streams or threads) must be ordered. */
#define MBPOL_NOALLOC_MAX_DIMERS 65536
mbpol_status mbpol_twobody_dimers_noalloc(const double* positions, const int* waters, const int* dimers,
                                         int num_dimers, const double* box_nm, double* forces, double* energy,
                                         void* stream);

#ifdef __cplusplus
}
#endif
#endif /* MBPOL_GB300_H */
