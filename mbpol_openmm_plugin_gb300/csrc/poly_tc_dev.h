// Device copy of the tensor-core polynomial tables (poly_tc.cu).
#pragma once
#include <cuda_runtime.h>

#include <cstddef>

namespace mbpol {

struct PolyTCDev {
    int nv = 0, ny = 0, npad = 0;
    const float* x0h = nullptr;
    const float* x0l = nullptr;
    const float* inv_bound = nullptr;
    const unsigned* ymeta = nullptr;
    const float* rowscale = nullptr;
    const int* warp_begin = nullptr;
    const int* rt_id = nullptr;
    const int* rt_entry = nullptr;
    const unsigned short* ent_kt = nullptr;
    const unsigned* frag = nullptr;
    int parts5 = 0, rows5 = 0, nblk5 = 0;
    const unsigned short* sblk = nullptr;
    const unsigned char* blk_kt = nullptr;
    const int* blk_begin = nullptr;
};

// Uploads the three-body tables to `device` (current) once per process and
// sets the kernel's shared-memory limit there; thread-safe.
cudaError_t poly_tc_setup(int device, const PolyTCDev** out);
// scratch of the three-body launch (floats): one slice of z per block
size_t poly3b_tc_scratch_floats(int num_sms);
// reserve_sms: SMs left out of the persistent grid for the other streams
// (negative: the default of each kernel)
void launch_poly3b_tc(cudaStream_t st, const PolyTCDev* tab, const float* X, float* G, float* E, int n, int stride,
                      int num_sms, float* zscratch, int reserve_sms = -1);
// The same evaluation with tcgen05.mma (poly_tc5.cu): Y' of 128 trimers in
// tensor memory as the A operand, S streamed through shared memory as B.
// `status` (device int, zero before the launch) receives a nonzero code if
// one of the kernel's bounded waits gave up; the outputs are then invalid.
cudaError_t poly_tc5_prepare();
size_t poly3b_tc5_scratch_floats(int num_sms);
int tc5_default_reserve();
void launch_poly3b_tc5(cudaStream_t st, const PolyTCDev* tab, const float* X, float* G, float* E, int n, int stride,
                       int num_sms, float* zscratch, int* status, int reserve_sms = -1);

}  // namespace mbpol
