/* Oracle harness (test infrastructure only).
 *
 * Exposes C entry points that drive the MB-pol Reference-platform force
 * classes, compiled unmodified from the reference's sources against the
 * project-written shim in oracle/shim.  The glue mirrors what the
 * reference's kernels do before calling the force classes:
 *   - one-body:  platforms/reference/src/MBPolReferenceKernels.cpp:77-118
 *   - two-body:  platforms/reference/src/MBPolReferenceKernels.cpp:362-399
 *                (O-O pair list with d <= cutoff; brute force here, in
 *                place of OpenMM's computeNeighborListVoxelHash)
 *   - three-body: platforms/reference/src/MBPolReferenceKernels.cpp:451-483
 *                (the reference's own computeThreeNeighborListVoxelHash)
 *   - electrostatics: platforms/reference/src/MBPolReferenceKernels.cpp:209-259
 * Dispersion has no plugin code in the reference (it is an OpenMM
 * CustomNonbondedForce built by python/mbpol.xml:37-108); it is restated
 * in oracle/mbpol_oracle.c, not here.
 *
 * Units: nm, kJ/mol, kJ/mol/nm.  Forces are accumulated (+=).
 * Never linked into the product library.
 */
#include <cstring>
#include <string>
#include <vector>
#include <set>
#include "MBPolReferenceOneBodyForce.h"
#include "MBPolReferenceTwoBodyForce.h"
#include "MBPolReferenceThreeBodyForce.h"
#include "MBPolReferenceElectrostaticsForce.h"
#include "ReferenceThreeNeighborList.h"

using OpenMM::RealVec;

namespace {

std::vector<RealVec> load_positions(int np, const double* pos) {
    std::vector<RealVec> v((size_t)np);
    for (int i = 0; i < np; ++i) v[(size_t)i] = RealVec(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    return v;
}

std::vector<std::vector<int> > load_waters(int nw, const int* idx) {
    std::vector<std::vector<int> > w((size_t)nw);
    for (int i = 0; i < nw; ++i) w[(size_t)i] = {idx[3 * i], idx[3 * i + 1], idx[3 * i + 2]};
    return w;
}

void store_forces(int np, const std::vector<RealVec>& f, double* out) {
    for (int i = 0; i < np; ++i)
        for (int k = 0; k < 3; ++k) out[3 * i + k] += f[(size_t)i][k];
}

double min_image(double d, double L) { return d - L * std::floor(d / L + 0.5); }

/* Subclasses give the harness read access to the converged dipoles
 * (protected members), as the reference's own white-box tests do. */
class NonPmeProbe : public MBPolReferenceElectrostaticsForce {
public:
    NonPmeProbe() : MBPolReferenceElectrostaticsForce(MBPolReferenceElectrostaticsForce::NoCutoff) {}
    const std::vector<RealVec>& dipoles() const { return _inducedDipole; }
};
class PmeProbe : public MBPolReferencePmeElectrostaticsForce {
public:
    const std::vector<RealVec>& dipoles() const { return _inducedDipole; }
};

void set_err(char* err, int errlen, const std::string& m) {
    if (err && errlen > 0) {
        std::strncpy(err, m.c_str(), (size_t)errlen - 1);
        err[errlen - 1] = 0;
    }
}

}  // namespace

extern "C" {

/* box: NULL for non-periodic, else 3 box lengths (nm). */
double ref_onebody(int nw, const int* idx, int np, const double* pos, const double* box, double* forces) {
    std::vector<RealVec> p = load_positions(np, pos), f((size_t)np);
    MBPolReferenceOneBodyForce force;
    if (box) {
        force.setNonbondedMethod(MBPolReferenceOneBodyForce::Periodic);
        force.setPeriodicBox(RealVec(box[0], box[1], box[2]));
    }
    double e = force.calculateForceAndEnergy(nw, p, load_waters(nw, idx), f);
    store_forces(np, f, forces);
    return e;
}

double ref_twobody(int nw, const int* idx, int np, const double* pos, const double* box, double cutoff,
                   double* forces, long* npairs) {
    std::vector<RealVec> p = load_positions(np, pos), f((size_t)np);
    OpenMM::NeighborList list;
    for (int i = 0; i < nw; ++i)
        for (int j = i + 1; j < nw; ++j) {
            double d2 = 0;
            for (int k = 0; k < 3; ++k) {
                double d = pos[3 * idx[3 * j] + k] - pos[3 * idx[3 * i] + k];
                if (box) d = min_image(d, box[k]);
                d2 += d * d;
            }
            if (d2 <= cutoff * cutoff) list.push_back(OpenMM::AtomPair(j, i));
        }
    MBPolReferenceTwoBodyForce force;
    force.setCutoff(cutoff);
    if (box) {
        force.setNonbondedMethod(MBPolReferenceTwoBodyForce::CutoffPeriodic);
        force.setPeriodicBox(RealVec(box[0], box[1], box[2]));
    } else {
        force.setNonbondedMethod(MBPolReferenceTwoBodyForce::CutoffNonPeriodic);
    }
    double e = force.calculateForceAndEnergy(nw, p, load_waters(nw, idx), list, f);
    store_forces(np, f, forces);
    if (npairs) *npairs = (long)list.size();
    return e;
}

double ref_threebody(int nw, const int* idx, int np, const double* pos, const double* box, double cutoff,
                     double* forces, long* ntriplets, int* triplets_out, long triplets_cap) {
    std::vector<RealVec> p = load_positions(np, pos), f((size_t)np);
    std::vector<RealVec> oxy((size_t)nw);
    for (int i = 0; i < nw; ++i) oxy[(size_t)i] = p[(size_t)idx[3 * i]];
    MBPolPlugin::ThreeNeighborList list;
    RealVec b = box ? RealVec(box[0], box[1], box[2]) : RealVec(0, 0, 0);
    MBPolPlugin::computeThreeNeighborListVoxelHash(list, nw, oxy, b, box != NULL, cutoff, 0.0);
    MBPolReferenceThreeBodyForce force;
    force.setCutoff(cutoff);
    if (box) {
        force.setNonbondedMethod(MBPolReferenceThreeBodyForce::CutoffPeriodic);
        force.setPeriodicBox(b);
    } else {
        force.setNonbondedMethod(MBPolReferenceThreeBodyForce::CutoffNonPeriodic);
    }
    double e = force.calculateForceAndEnergy(nw, p, load_waters(nw, idx), list, f);
    store_forces(np, f, forces);
    if (ntriplets) *ntriplets = (long)list.size();
    if (triplets_out)
        for (long t = 0; t < (long)list.size() && t < triplets_cap; ++t) {
            triplets_out[3 * t] = (int)list[(size_t)t].first;
            triplets_out[3 * t + 1] = (int)list[(size_t)t].second;
            triplets_out[3 * t + 2] = (int)list[(size_t)t].third;
        }
    return e;
}

/* Electrostatics over ns sites (waters laid out O,H1,H2,M per molecule when
 * charge redistribution is on).  pme=0: NoCutoff; pme=1: PME with explicit
 * alpha (nm^-1) and grid.  Returns 0 on success, 1 on an exception (message
 * in err). */
int ref_electrostatics(int ns, const double* pos, const double* charge, const int* mol, const int* type,
                       const double* damp, const double* pol, const double* thole5, int pme, double cutoff,
                       double alpha, const int* grid, const double* box, double target_eps, int maxiter,
                       int charge_redist, double* forces, double* energy, double* dipoles_out, int* iters,
                       char* err, int errlen) {
    std::vector<RealVec> p = load_positions(ns, pos), f((size_t)ns);
    std::vector<double> q(charge, charge + ns), d(damp, damp + ns), a(pol, pol + ns), th((size_t)ns, 0.0);
    std::vector<int> m(mol, mol + ns), t(type, type + ns);
    std::vector<double> thole(thole5, thole5 + 5);
    try {
        MBPolReferenceElectrostaticsForce* force = nullptr;
        NonPmeProbe* np_probe = nullptr;
        PmeProbe* pme_probe = nullptr;
        if (pme) {
            pme_probe = new PmeProbe();
            pme_probe->setAlphaEwald(alpha);
            pme_probe->setCutoffDistance(cutoff);
            std::vector<int> g(grid, grid + 3);
            pme_probe->setPmeGridDimensions(g);
            RealVec b(box[0], box[1], box[2]);
            pme_probe->setPeriodicBoxSize(b);
            force = pme_probe;
        } else {
            np_probe = new NonPmeProbe();
            force = np_probe;
        }
        force->setMutualInducedDipoleTargetEpsilon(target_eps);
        force->setMaximumMutualInducedDipoleIterations(maxiter);
        force->setIncludeChargeRedistribution(charge_redist != 0);
        force->setTholeParameters(thole);
        double e = force->calculateForceAndEnergy(p, q, m, t, th, d, a, f);
        store_forces(ns, f, forces);
        *energy = e;
        if (iters) *iters = force->getMutualInducedDipoleIterations();
        if (dipoles_out) {
            const std::vector<RealVec>& mu = pme ? pme_probe->dipoles() : np_probe->dipoles();
            for (int i = 0; i < ns; ++i)
                for (int k = 0; k < 3; ++k) dipoles_out[3 * i + k] = mu[(size_t)i][k];
        }
        delete force;
    } catch (const std::exception& ex) {
        set_err(err, errlen, ex.what());
        return 1;
    }
    return 0;
}

/* MBPolElectrostaticsForce::getElectrostaticPotential: the reference kernel
 * (MBPolReferenceKernels.cpp:261-283) calls calculateElectrostaticPotential
 * (MBPolReferenceElectrostaticsForce.cpp:1048-1085): setup (charges with
 * redistribution, converged induced dipoles), then for every grid point the
 * sum over all particles of q/r - mu.(r_i - g)/r^3 (minimum image under PME),
 * times 138.9354558456. */
int ref_electrostatic_potential(int ns, const double* pos, const double* charge, const int* mol, const int* type,
                                const double* damp, const double* pol, const double* thole5, int pme, double cutoff,
                                double alpha, const int* grid, const double* box, double target_eps, int maxiter,
                                int charge_redist, int npts, const double* points, double* potential, char* err,
                                int errlen) {
    std::vector<RealVec> p = load_positions(ns, pos), g = load_positions(npts, points);
    std::vector<double> q(charge, charge + ns), d(damp, damp + ns), a(pol, pol + ns), th((size_t)ns, 0.0);
    std::vector<int> m(mol, mol + ns), t(type, type + ns);
    std::vector<double> thole(thole5, thole5 + 5), out;
    try {
        MBPolReferenceElectrostaticsForce* force = nullptr;
        if (pme) {
            PmeProbe* pp = new PmeProbe();
            pp->setAlphaEwald(alpha);
            pp->setCutoffDistance(cutoff);
            std::vector<int> gd(grid, grid + 3);
            pp->setPmeGridDimensions(gd);
            RealVec b(box[0], box[1], box[2]);
            pp->setPeriodicBoxSize(b);
            force = pp;
        } else {
            force = new NonPmeProbe();
        }
        force->setMutualInducedDipoleTargetEpsilon(target_eps);
        force->setMaximumMutualInducedDipoleIterations(maxiter);
        force->setIncludeChargeRedistribution(charge_redist != 0);
        force->setTholeParameters(thole);
        force->calculateElectrostaticPotential(p, q, m, t, th, d, a, g, out);
        for (int i = 0; i < npts; ++i) potential[i] = out[(size_t)i];
        delete force;
    } catch (const std::exception& ex) {
        set_err(err, errlen, ex.what());
        return 1;
    }
    return 0;
}

/* System multipole moments (calculateMBPolSystemElectrostaticsMoments,
 * MBPolReferenceElectrostaticsForce.cpp:923-1021): the same setup as the
 * potential (charges with redistribution, converged induced dipoles), then
 * charge, dipole (Debye) and traceless quadrupole about the centre of mass
 * of `mass`, 13 values. */
int ref_system_moments(int ns, const double* pos, const double* charge, const int* mol, const int* type,
                       const double* damp, const double* pol, const double* thole5, int pme, double cutoff,
                       double alpha, const int* grid, const double* box, double target_eps, int maxiter,
                       int charge_redist, const double* mass, double* moments, char* err, int errlen) {
    std::vector<RealVec> p = load_positions(ns, pos);
    std::vector<double> q(charge, charge + ns), d(damp, damp + ns), a(pol, pol + ns), th((size_t)ns, 0.0);
    std::vector<double> m8(mass, mass + ns);
    std::vector<int> m(mol, mol + ns), t(type, type + ns);
    std::vector<double> thole(thole5, thole5 + 5), out;
    try {
        MBPolReferenceElectrostaticsForce* force = nullptr;
        if (pme) {
            PmeProbe* pp = new PmeProbe();
            pp->setAlphaEwald(alpha);
            pp->setCutoffDistance(cutoff);
            std::vector<int> gd(grid, grid + 3);
            pp->setPmeGridDimensions(gd);
            RealVec b(box[0], box[1], box[2]);
            pp->setPeriodicBoxSize(b);
            force = pp;
        } else {
            force = new NonPmeProbe();
        }
        force->setMutualInducedDipoleTargetEpsilon(target_eps);
        force->setMaximumMutualInducedDipoleIterations(maxiter);
        force->setIncludeChargeRedistribution(charge_redist != 0);
        force->setTholeParameters(thole);
        force->calculateMBPolSystemElectrostaticsMoments(m8, p, q, m, t, th, d, a, out);
        for (int i = 0; i < 13; ++i) moments[i] = out[(size_t)i];
        delete force;
    } catch (const std::exception& ex) {
        set_err(err, errlen, ex.what());
        return 1;
    }
    return 0;
}

}  // extern "C"
