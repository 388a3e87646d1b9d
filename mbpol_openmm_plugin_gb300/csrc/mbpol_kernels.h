// Host-side launchers of the MB-pol kernels (internal to the library).
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "../../include/mbpol_gb300.h"
#include "mbpol_internal.cuh"
#include "poly_tables.h"

mbpol_status mbpol_fail_cuda(cudaError_t e, const char* what);

namespace mbpol {

// polyterms.cu
void upload_polyterm_constants(const double* c5z, const unsigned char* idx3x245);
void launch_onebody(cudaStream_t st, int nw, const int4* waters, const double* pos, Box box, double* force,
                    double* energy, ClusterSink cs = ClusterSink());
void launch_twobody_vars(cudaStream_t st, int npairs, const int2* pairs, const int4* waters, const double* pos,
                         Box box, float* X, int stride);
void launch_twobody_forces(cudaStream_t st, int npairs, const int2* pairs, const int4* waters, const double* pos,
                           Box box, const float* G, const float* E, int stride, double* force, double* energy,
                           ClusterSink cs = ClusterSink());
void launch_threebody_vars(cudaStream_t st, int ntrip, const int4* trips, const int4* waters, const double* pos,
                           Box box, float* X, int stride);
void launch_threebody_forces(cudaStream_t st, int ntrip, const int4* trips, const int4* waters,
                             const double* pos, Box box, const float* G, const float* E, int stride,
                             double* force, double* energy, ClusterSink cs = ClusterSink());

// poly_df.cu: the double-float trie walks; tables per device (upload with
// `device` current, once per process; thread-safe)
struct PolyWalkTables;
cudaError_t poly_tables_upload(int device, const PolyWalkTables** out);
// reserve_blocks: blocks left out of the persistent grid for the other
// streams (negative: the default, walk_default_reserve())
int walk_default_reserve();
void launch_poly2b(cudaStream_t st, const PolyWalkTables* t, const float* X, float* G, float* E, int n, int stride,
                   int num_sms, int reserve_blocks = -1);
void launch_poly3b(cudaStream_t st, const PolyWalkTables* t, const float* X, float* G, float* E, int n, int stride,
                   int num_sms, int reserve_blocks = -1);
// the two-body kernel on caller-supplied device tables (raise its dynamic
// shared-memory limit once per device with poly2b_kernel_setup first)
cudaError_t poly2b_kernel_setup();
void launch_poly2b_with(cudaStream_t st, const PolyNode* l1, const PolyNode* l2, const PolyNode* l3,
                        const PolyNode* lv, const float* X, float* G, float* E, int n, int stride, int num_sms,
                        int reserve_blocks = -1);

// neighbor.cu
// opos: scratch of nw float4 (FP32 O positions for the distance prefilter)
// clusters: mode-1 candidate set of batched clusters, or null; cell_scratch:
// cell_scratch_ints(nw, box, max radius) device ints (may be null: no cells)
mbpol_status launch_mol_neighbors(cudaStream_t st, int nw, const int4* waters, const double* pos, float4* opos,
                                  Box box, double r_full, double r_3b, double r_2b, int cap_full, int cap_lower,
                                  int* full, int* nfull, int* lower, int* nlower, int2* pairs, int cap_pairs,
                                  int* npairs, int* overflow, const CandidateSet* clusters, int* cell_scratch);
mbpol_status launch_cell_binning(cudaStream_t st, int n, const float4* opos, const Box& box, double r, int* scratch,
                                 CandidateSet* out);
// members of each cluster, ascending, and their offsets (host: molecule
// cluster indices in [0, ncl)); the mode-1 candidate set's arrays
void cluster_members(const int* cluster_of, int n, int ncl, std::vector<int>& members, std::vector<int>& start);
void launch_trimer_count(cudaStream_t st, int nw, const int* lower, const int* nlower, int cap_lower, int* count,
                         int* offs);
void launch_trimer_fill(cudaStream_t st, int nw, const int* lower, const int* nlower, int cap_lower,
                        const int* offs, int cap_trip, int4* trips);
void launch_trimer_complete(cudaStream_t st, int nw, const int4* waters, const double* pos, Box box, double rc,
                            const int* full, const int* nfull, int cap_full, int* count, int* offs, int cap_trip,
                            int4* trips, bool fill);

// dispersion.cu
void upload_dispersion_tables(const double* c6_4x4, const double* d6_4x4);
void launch_dispersion(cudaStream_t st, int nw, const int4* waters, const double* pos, Box box, const int* full,
                       const int* nfull, int cap_full, double rc, double* force, double* energy,
                       ClusterSink cs = ClusterSink());
// chloride ions (particle indices) against the water sites and each other
void launch_dispersion_ions(cudaStream_t st, int nion, const int* ions, int nw, const int4* waters,
                            const double* pos, Box box, double rc, double* force, double* energy);

// md.cu
void launch_kick_drift(cudaStream_t st, int n, const double* invm, double* vel, double* pos, const double* force,
                       double dt);
void launch_kick(cudaStream_t st, int n, const double* invm, double* vel, const double* force, double dt, double kT,
                 double nu, unsigned long long seed, unsigned long long step, double* ekin);

// vsites.cu
void launch_place_vsites(cudaStream_t st, int n, const int4* idx, const double* w, double* pos);
void launch_spread_vsites(cudaStream_t st, int n, const int4* idx, const double* w, double* force);

}  // namespace mbpol
