// Electrostatics engine (charges with redistribution, Thole-damped
// permanent and induced fields, induced-dipole solver, PME, energy/forces).
#pragma once
#include <string>
#include <cuda_runtime.h>
#include "../../include/mbpol_gb300.h"
#include "mbpol_internal.cuh"

mbpol_status mbpol_fail(mbpol_status s, const std::string& msg);
mbpol_status mbpol_fail_cuda(cudaError_t e, const char* what);

namespace mbpol {

struct ElecImpl;

class ElecEngine {
public:
    ElecEngine();
    ~ElecEngine();
    mbpol_status init(int n, const mbpol_electrostatics_params& p, const double* charge, const int* molecule,
                      const int* atom_type, const double* damping, const double* polarity);
    // Adds forces (kJ/mol/nm) into force and the energy (kJ/mol) into *energy (device pointers).
    mbpol_status compute(cudaStream_t st, const double* pos, const Box& box, double* force, double* energy);
    mbpol_status get_dipoles(cudaStream_t st, double* dipoles, int* iterations, double* epsilon);
    bool converged() const;
    int iterations() const;
    long num_site_pairs() const;
    std::string convergence_message() const;

private:
    ElecImpl* impl_;
};

}  // namespace mbpol
