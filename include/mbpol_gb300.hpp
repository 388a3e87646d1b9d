/*
 * mbpol_gb300.hpp -- C++ Force-class layer over the C ABI (mbpol_gb300.h),
 * mirroring the MB-pol plugin's public API
 * (openmmapi/include/openmm/MBPol{OneBody,TwoBody,ThreeBody,Electrostatics}Force.h)
 * plus MBPolDispersionForce (the dispersion term python/mbpol.xml:37-108
 * builds) and minimal System / Context stand-ins, since OpenMM itself is not
 * part of this library.  Same names, argument meanings and units (nm, kJ/mol);
 * errors throw MBPolException where the reference throws OpenMMException.
 * Header-only; link with libmbpol_gb300.so.
 */
#ifndef MBPOL_GB300_HPP
#define MBPOL_GB300_HPP

#include <array>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "mbpol_gb300.h"

namespace MBPolPlugin {

class MBPolException : public std::runtime_error {
public:
    MBPolException(mbpol_status s, const std::string& m) : std::runtime_error(m), status(s) {}
    mbpol_status status;
};

inline void mbpol_check(mbpol_status s) {
    if (s != MBPOL_OK) throw MBPolException(s, std::string(mbpol_status_string(s)) + ": " + mbpol_last_error());
}

typedef std::array<double, 3> Vec3;

class Context;

class Force {
public:
    virtual ~Force() {}
    void setForceGroup(int g) { group_ = g; }
    int getForceGroup() const { return group_; }
    virtual int term() const = 0;
    /* MBPol*Force::updateParametersInContext (copyParametersToContext,
     * MBPolReferenceKernels.cpp:116-126, 306-322, 401-411, 485-495): this
     * force's parameters into a live context (mbpol_update_parameters). */
    void updateParametersInContext(Context& context) const;

protected:
    int group_ = 0;
};

/* Waters given as {O, H1, H2} particle indices. */
class WaterForce : public Force {
public:
    int getNumMolecules() const { return (int)waters_.size(); }
    std::vector<int> flatWaters() const {
        std::vector<int> flat;
        for (const auto& t : waters_) flat.insert(flat.end(), t.begin(), t.end());
        return flat;
    }
    const std::vector<std::array<int, 3>>& waters() const { return waters_; }

protected:
    int add(const std::vector<int>& idx) {
        if (idx.size() != 3) throw MBPolException(MBPOL_ERR_INVALID_ARGUMENT, "a water needs 3 particle indices");
        waters_.push_back({idx[0], idx[1], idx[2]});
        return (int)waters_.size() - 1;
    }
    std::vector<std::array<int, 3>> waters_;
};

class MBPolOneBodyForce : public WaterForce {
public:
    enum NonbondedMethod { NonPeriodic = 0, Periodic = 1 };
    int addOneBody(const std::vector<int>& particleIndices) { return add(particleIndices); }
    int getNumOneBodys() const { return getNumMolecules(); }
    void setNonbondedMethod(NonbondedMethod m) { method_ = m; }
    NonbondedMethod getNonbondedMethod() const { return method_; }
    int term() const override { return MBPOL_TERM_ONEBODY; }

private:
    NonbondedMethod method_ = NonPeriodic;
};

class CutoffWaterForce : public WaterForce {
public:
    enum NonbondedMethod { NoCutoff = 0, CutoffNonPeriodic = 1, CutoffPeriodic = 2 };
    int addParticle(const std::vector<int>& particleIndices) { return add(particleIndices); }
    int getNumParticles() const { return getNumMolecules(); }
    void setCutoff(double c) { cutoff_ = c; }
    double getCutoff() const { return cutoff_; }
    void setNonbondedMethod(NonbondedMethod m) { method_ = m; }
    NonbondedMethod getNonbondedMethod() const { return method_; }

protected:
    double cutoff_ = 1.0;
    NonbondedMethod method_ = NoCutoff;
};

class MBPolTwoBodyForce : public CutoffWaterForce {
public:
    int term() const override { return MBPOL_TERM_TWOBODY; }
};

class MBPolThreeBodyForce : public CutoffWaterForce {
public:
    void setTrimerRule(int r) { rule_ = r; }
    int getTrimerRule() const { return rule_; }
    /* tensor cores (tcgen05; MBPOL_POLY3B_TENSOR_SYNC: mma.sync), the
     * double-float walk, or the automatic choice by size (default); no
     * reference counterpart (mbpol_set_threebody_evaluator) */
    enum Evaluator { TensorCores = MBPOL_POLY3B_TENSOR, DoubleFloatWalk = MBPOL_POLY3B_WALK,
                     AutomaticEvaluator = MBPOL_POLY3B_AUTO, TensorCoresMmaSync = MBPOL_POLY3B_TENSOR_SYNC };
    void setPolynomialEvaluator(int kind) { evaluator_ = kind; }
    int getPolynomialEvaluator() const { return evaluator_; }
    int term() const override { return MBPOL_TERM_THREEBODY; }

private:
    int rule_ = MBPOL_TRIMER_REFERENCE;
    int evaluator_ = MBPOL_POLY3B_AUTO;
};

class MBPolDispersionForce : public CutoffWaterForce {
public:
    MBPolDispersionForce() {
        cutoff_ = 0.9;
        // python/mbpol.xml:52-83 (classes O, H, M, Cl)
        c6_ = {9.92951990e-4, 3.49345451e-4, 0, 0.00456078851, 3.49345451e-4, 8.40715638e-5, 0, 0.00085979832,
               0, 0, 0, 0, 0.00456078851, 0.00085979832, 0, 0};
        d6_ = {9.29548582e+01, 9.77520243e+01, 0, 1.638868407461115e+02, 9.77520243e+01, 9.40647517e+01, 0,
               5.778854012725382e+01, 0, 0, 0, 0, 1.638868407461115e+02, 5.778854012725382e+01, 0, 0};
    }
    int term() const override { return MBPOL_TERM_DISPERSION; }
    std::array<double, 16> c6_, d6_;
};

class MBPolElectrostaticsForce : public Force {
public:
    enum NonbondedMethod { NoCutoff = 0, PME = 1 };
    MBPolElectrostaticsForce() { mbpol_electrostatics_params_default(&p_); }
    int addElectrostatics(double charge, int moleculeIndex, int atomType, double dampingFactor, double polarity) {
        q_.push_back(charge);
        mol_.push_back(moleculeIndex);
        type_.push_back(atomType);
        damp_.push_back(dampingFactor);
        pol_.push_back(polarity);
        return (int)q_.size() - 1;
    }
    int getNumElectrostatics() const { return (int)q_.size(); }
    void setNonbondedMethod(NonbondedMethod m) { p_.nonbonded_method = m; }
    NonbondedMethod getNonbondedMethod() const { return (NonbondedMethod)p_.nonbonded_method; }
    void setCutoffDistance(double d) { p_.cutoff = d; }
    double getCutoffDistance() const { return p_.cutoff; }
    void setAEwald(double a) { p_.ewald_alpha = a; }
    double getAEwald() const { return p_.ewald_alpha; }
    int getPmeBSplineOrder() const { return 5; }
    void setPmeGridDimensions(const std::vector<int>& g) {
        for (int k = 0; k < 3; ++k) p_.pme_grid[k] = g.size() > (size_t)k ? g[k] : 0;
    }
    void setEwaldErrorTolerance(double t) { p_.ewald_error_tolerance = t; }
    void setMutualInducedMaxIterations(int n) { p_.max_iterations = n; }
    int getMutualInducedMaxIterations() const { return p_.max_iterations; }
    void setMutualInducedTargetEpsilon(double e) { p_.target_epsilon = e; }
    double getMutualInducedTargetEpsilon() const { return p_.target_epsilon; }
    void setTholeParameters(const std::vector<double>& t) {
        for (int k = 0; k < 5 && k < (int)t.size(); ++k) p_.thole[k] = t[k];
    }
    void setIncludeChargeRedistribution(bool b) { p_.include_charge_redistribution = b ? 1 : 0; }
    bool getIncludeChargeRedistribution() const { return p_.include_charge_redistribution != 0; }
    void setInducedDipoleGuess(int g) { p_.guess = g; }
    /* MBPOL_PME_FIELD_REFERENCE (default) or MBPOL_PME_FIELD_CONSISTENT; no
     * reference counterpart (see mbpol_gb300.h) */
    void setPmeFixedField(int m) { p_.pme_fixed_field = m; }
    int getPmeFixedField() const { return p_.pme_fixed_field; }
    /* MBPolElectrostaticsForce.h:267: potential (kJ/mol/e) at the points of
     * inputGrid (nm) from the context's current positions (defined after
     * Context below) */
    void getElectrostaticPotential(const std::vector<Vec3>& inputGrid, class Context& context,
                                   std::vector<double>& outputElectrostaticPotential) const;
    /* mbpolKernels.h:121 getSystemElectrostaticsMoments: charge, dipole
     * (Debye) and traceless quadrupole about the System's centre of mass,
     * 13 values (defined after Context below) */
    void getSystemElectrostaticsMoments(class Context& context, std::vector<double>& outputMoments) const;
    int term() const override { return MBPOL_TERM_ELECTROSTATICS; }

    mbpol_electrostatics_params p_;
    std::vector<double> q_, damp_, pol_;
    std::vector<int> mol_, type_;
};

class System {
public:
    int addParticle(double mass) {
        masses_.push_back(mass);
        return (int)masses_.size() - 1;
    }
    int getNumParticles() const { return (int)masses_.size(); }
    double getParticleMass(int i) const { return masses_.at((size_t)i); }
    /* ThreeParticleAverageSite */
    void setVirtualSite(int index, int p1, int p2, int p3, double w1, double w2, double w3) {
        vs_.push_back({index, p1, p2, p3, w1, w2, w3});
    }
    /* The System owns its forces, as in OpenMM. */
    int addForce(Force* f) {
        forces_.emplace_back(f);
        return (int)forces_.size() - 1;
    }
    void setDefaultPeriodicBoxVectors(const Vec3& a, const Vec3& b, const Vec3& c) {
        box_ = {a[0], b[1], c[2]};
        periodic_ = true;
    }
    struct VSite {
        int index, p1, p2, p3;
        double w1, w2, w3;
    };
    std::vector<double> masses_;
    std::vector<VSite> vs_;
    std::vector<std::unique_ptr<Force>> forces_;
    Vec3 box_{0, 0, 0};
    bool periodic_ = false;
};

struct State {
    double potentialEnergy = 0.0;
    std::array<double, MBPOL_NUM_TERMS> termEnergies{};
    std::vector<Vec3> forces;
};

class Context {
public:
    explicit Context(const System& sys, int device = 0) : sys_(sys) {
        mbpol_check(mbpol_context_create(sys.getNumParticles(), device, &h_));
        for (const auto& v : sys.vs_) mbpol_check(mbpol_add_average3_site(h_, v.index, v.p1, v.p2, v.p3, v.w1, v.w2, v.w3));
        for (const auto& f : sys.forces_) add(*f);
        box_ = sys.box_;
        periodic_ = sys.periodic_;
    }
    ~Context() { mbpol_context_destroy(h_); }
    Context(const Context&) = delete;
    Context& operator=(const Context&) = delete;

    void setPositions(const std::vector<Vec3>& pos) {
        if ((int)pos.size() != sys_.getNumParticles())
            throw MBPolException(MBPOL_ERR_INVALID_ARGUMENT, "wrong number of positions");
        std::vector<double> flat(3 * pos.size());
        for (size_t i = 0; i < pos.size(); ++i)
            for (int k = 0; k < 3; ++k) flat[3 * i + k] = pos[i][k];
        mbpol_check(mbpol_set_positions(h_, flat.data(), periodic_ ? box_.data() : nullptr));
    }
    void setPeriodicBoxVectors(const Vec3& a, const Vec3& b, const Vec3& c) {
        box_ = {a[0], b[1], c[2]};
        periodic_ = true;
    }
    /* Energy and forces of the forces in `groups` (bit mask), as
     * Context::getState(State::Forces | State::Energy, groups). */
    State getState(int groups = 0xFFFFFFFF) {
        unsigned mask = 0;
        for (const auto& f : sys_.forces_)
            if ((groups >> f->getForceGroup()) & 1) mask |= MBPOL_TERM_BIT(f->term());
        State st;
        std::vector<double> flat(3 * (size_t)sys_.getNumParticles(), 0.0);
        mbpol_check(mbpol_compute(h_, mask, st.termEnergies.data(), flat.data()));
        st.forces.resize((size_t)sys_.getNumParticles());
        for (size_t i = 0; i < st.forces.size(); ++i) st.forces[i] = {flat[3 * i], flat[3 * i + 1], flat[3 * i + 2]};
        for (double e : st.termEnergies) st.potentialEnergy += e;
        return st;
    }
    mbpol_context* handle() { return h_; }
    const System& getSystem() const { return sys_; }
    /* launch shapes of the polynomial kernels: tune over the next 12 n
     * evaluations, or read the shape in use (no reference counterpart) */
    void setAutotune(int evaluationsPerShape) { mbpol_check(mbpol_set_autotune(h_, evaluationsPerShape)); }
    void getLaunchShape(int& tcReserveSms, int& walkReserveBlocks, bool& tuned) {
        int t = 0;
        mbpol_check(mbpol_get_launch_shape(h_, &tcReserveSms, &walkReserveBlocks, &t));
        tuned = t != 0;
    }

private:
    void add(const Force& f) {
        if (auto* e = dynamic_cast<const MBPolElectrostaticsForce*>(&f)) {
            if (e->getNumElectrostatics() != sys_.getNumParticles())
                throw MBPolException(MBPOL_ERR_INVALID_ARGUMENT,
                                     "MBPolElectrostaticsForce must have exactly as many particles as the System");
            mbpol_check(mbpol_add_electrostatics_force(h_, &e->p_, e->q_.data(), e->mol_.data(), e->type_.data(),
                                                       e->damp_.data(), e->pol_.data()));
            return;
        }
        const auto* w = dynamic_cast<const WaterForce*>(&f);
        std::vector<int> flat;
        for (const auto& t : w->waters()) flat.insert(flat.end(), t.begin(), t.end());
        const int nw = w->getNumMolecules();
        if (auto* o = dynamic_cast<const MBPolOneBodyForce*>(&f))
            mbpol_check(mbpol_add_onebody_force(h_, nw, flat.data(), o->getNonbondedMethod()));
        else if (auto* t2 = dynamic_cast<const MBPolTwoBodyForce*>(&f))
            mbpol_check(mbpol_add_twobody_force(h_, nw, flat.data(), t2->getNonbondedMethod(), t2->getCutoff()));
        else if (auto* t3 = dynamic_cast<const MBPolThreeBodyForce*>(&f)) {
            mbpol_check(mbpol_add_threebody_force(h_, nw, flat.data(), t3->getNonbondedMethod(), t3->getCutoff(),
                                                  t3->getTrimerRule()));
            mbpol_check(mbpol_set_threebody_evaluator(h_, t3->getPolynomialEvaluator()));
        }
        else if (auto* d = dynamic_cast<const MBPolDispersionForce*>(&f))
            mbpol_check(mbpol_add_dispersion_force(h_, nw, flat.data(), d->getNonbondedMethod(), d->getCutoff(),
                                                   d->c6_.data(), d->d6_.data()));
    }
    const System& sys_;
    mbpol_context* h_ = nullptr;
    Vec3 box_{0, 0, 0};
    bool periodic_ = false;
};

inline void Force::updateParametersInContext(Context& context) const {
    if (auto* e = dynamic_cast<const MBPolElectrostaticsForce*>(this)) {
        mbpol_check(mbpol_update_parameters(context.handle(), MBPOL_TERM_ELECTROSTATICS, e->getNumElectrostatics(),
                                            nullptr, e->q_.data(), e->mol_.data(), e->type_.data(), e->damp_.data(),
                                            e->pol_.data()));
        return;
    }
    const auto* w = dynamic_cast<const WaterForce*>(this);
    const std::vector<int> flat = w->flatWaters();
    mbpol_check(mbpol_update_parameters(context.handle(), (unsigned)term(), w->getNumMolecules(), flat.data(),
                                        nullptr, nullptr, nullptr, nullptr, nullptr));
}

inline void MBPolElectrostaticsForce::getElectrostaticPotential(const std::vector<Vec3>& inputGrid, Context& context,
                                                                std::vector<double>& outputElectrostaticPotential) const {
    std::vector<double> flat(3 * inputGrid.size());
    for (size_t i = 0; i < inputGrid.size(); ++i)
        for (int k = 0; k < 3; ++k) flat[3 * i + k] = inputGrid[i][k];
    outputElectrostaticPotential.assign(inputGrid.size(), 0.0);
    mbpol_check(mbpol_get_electrostatic_potential(context.handle(), (int)inputGrid.size(), flat.data(),
                                                  outputElectrostaticPotential.data()));
}

inline void MBPolElectrostaticsForce::getSystemElectrostaticsMoments(Context& context,
                                                                     std::vector<double>& outputMoments) const {
    const System& sys = context.getSystem();
    std::vector<double> m((size_t)sys.getNumParticles());
    for (int i = 0; i < sys.getNumParticles(); ++i) m[(size_t)i] = sys.getParticleMass(i);
    outputMoments.assign(13, 0.0);
    mbpol_check(mbpol_get_system_multipole_moments(context.handle(), m.data(), outputMoments.data()));
}

}  // namespace MBPolPlugin

#endif  // MBPOL_GB300_HPP
