// Electrostatics engine (charges with redistribution, Thole-damped
// permanent and induced fields, induced-dipole solver, PME, energy/forces).
#pragma once
#include <string>
#include <vector>
#include <cuda_runtime.h>
#include "../../include/mbpol_gb300.h"
#include "mbpol_internal.cuh"

mbpol_status mbpol_fail(mbpol_status s, const std::string& msg);
mbpol_status mbpol_fail_cuda(cudaError_t e, const char* what);

namespace mbpol {

struct ElecImpl;

// white-box probes (one thread on the current device): the Thole-scaled
// inverse distances of orders 1, 3, 5, 7 as the field kernels evaluate them
// (FP32), and one water's charges and charge derivatives (FP64)
mbpol_status probe_thole(double r, double damp_i, double damp_j, double gamma, double* rr4);
mbpol_status probe_water_charges(const double* pos9, double* out31);

class ElecEngine {
public:
    ElecEngine();
    ~ElecEngine();
    mbpol_status init(int n, const mbpol_electrostatics_params& p, const double* charge, const int* molecule,
                      const int* atom_type, const double* damping, const double* polarity);
    // Adds forces (kJ/mol/nm) into force and the energy (kJ/mol) into *energy (device pointers).
    mbpol_status compute(cudaStream_t st, const double* pos, const Box& box, double* force, double* energy);
    mbpol_status get_dipoles(cudaStream_t st, double* dipoles, int* iterations, double* epsilon);
    // electrostatic potential (kJ/mol/e) at npts host points (nm) from the
    // last evaluation's charges and induced dipoles; pos: device positions
    mbpol_status potential(cudaStream_t st, const double* pos, int npts, const double* points, double* potential);
    // system multipole moments (13 values) of the last evaluation's charges
    // and induced dipoles about the centre of mass of the host masses
    mbpol_status moments(cudaStream_t st, const double* pos, const double* masses, double* out13);
    bool converged() const;
    int iterations() const;
    long num_site_pairs() const;
    std::string convergence_message() const;
    // learned initial guess (guess = 2); descriptors and collection refer to
    // the last evaluation's geometry and converged dipoles
    // updateParametersInContext: new per-particle parameters, same molecules
    mbpol_status update_parameters(const double* charge, const int* molecule, const int* atom_type,
                                   const double* damping, const double* polarity);
    mbpol_status guess_select(int which);
    mbpol_status guess_descriptors(cudaStream_t st, float* host_out);
    mbpol_status guess_collect(cudaStream_t st);
    mbpol_status guess_train(cudaStream_t st, int steps, int batch, double lr, unsigned long long seed,
                             double* loss);
    mbpol_status guess_get_params(float* block);
    mbpol_status guess_set_params(const float* block);
    mbpol_status guess_loss_grad(cudaStream_t st, const float* X, const float* T, int n, double* loss, float* grad,
                                 float* Y);
    long guess_num_samples() const;
    // the learned linear predictor on host history [kPredHistory][n3]
    // (newest first) of dipoles and of alpha E0, with alpha E0 of the new
    // geometry: its coefficients [kPredRegressors] and prediction [n3]
    mbpol_status guess_fit_predictor(cudaStream_t st, const double* history, const double* field,
                                     const double* field_now, int n3, double* coef, double* prediction);
    // batched independent clusters (NoCutoff only): cluster of every
    // particle; per-cluster electrostatic energies go to
    // cluster_energy[c * stride] (device).  ncl = 0 turns batching off.
    mbpol_status set_clusters(const int* cluster_of_particle, int ncl, double* cluster_energy, int stride);
    const std::vector<int>& cluster_iterations() const;

private:
    ElecImpl* impl_;
};

}  // namespace mbpol
