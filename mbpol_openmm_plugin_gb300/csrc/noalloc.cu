// Two-body (dimer) term for a caller-built dimer list without any device
// allocation: mbpol_twobody_dimers_noalloc.
//
// Who needs it: callers that own the device memory and cannot let a library
// allocate behind them -- a host engine with its own pool allocator, a code
// that must not call cudaMalloc/cudaFree inside its step loop because those
// calls synchronise the device, or a step loop that is being prepared for
// stream capture, where an allocation in the middle would fail.  The context
// API (mbpol_compute) grows its buffers on demand and so cannot serve them.
//
// How: the per-dimer scratch of the existing two-body path -- the 31 FP64
// variables as FP32 hi/lo planes, the 31 gradient planes and the per-dimer
// energies -- lives in file-scope __device__ arrays sized for
// MBPOL_NOALLOC_MAX_DIMERS dimers, and so do this path's copies of the
// two-body trie tables.  The arrays belong to the library's device code, so
// a device holds them (24.6 MB) from the moment that code is loaded on it:
// with lazy module loading (CUDA_MODULE_LOADING=LAZY, the default) only once
// this entry point is first called there; with eager loading as soon as the
// library initialises the device, context API or not.
// The kernels are the ones mbpol_compute launches (twobody_vars, the
// double-float polynomial walk, twobody_forces), with the planes strided by
// the fixed capacity instead of the context's pair capacity.
//
// Set-up, once per device and under a mutex: cudaGetSymbolAddress of every
// array with that device current, one cudaMemcpyToSymbol of the tables, the
// kernel attribute for its dynamic shared memory and the model constants
// (cudaMemcpyToSymbol).  None of these allocate, but they are synchronous,
// so the first call on a device should come before any stream capture.  The
// model constants are the process-wide ones the context path uploads too
// (identical values; they must stay identical between the two paths).  The
// set-up is remembered for the life of the process: after cudaDeviceReset
// the symbol addresses, tables and constants are gone, and this entry point
// must not be called on that device again.
//
// Every scratch element a call reads is written earlier in the same call
// (variables by twobody_vars, gradients and energies by the walk, for each
// dimer below num_dimers), so nothing has to be cleared; the caller's energy
// and forces are accumulated into (+=), as mbpol_compute does.
//
// Race: the scratch is one per device and per process.  Two calls whose
// kernels overlap on the same device -- different streams, or different host
// threads without ordering -- overwrite each other's planes and both results
// are wrong.  Calls must be ordered (same stream, or events between them).
#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/mbpol_gb300.h"
#include "mbpol_kernels.h"
#include "poly_tables.h"

mbpol_status mbpol_fail(mbpol_status s, const std::string& msg);
mbpol_status mbpol_fail_cuda(cudaError_t e, const char* what);

namespace mbpol {

#include "gen/model_tables.inc"
#include "gen/poly2b_tables.inc"

namespace {

constexpr int kCap = MBPOL_NOALLOC_MAX_DIMERS;
constexpr int kVars = POLY2B_NVARS;

static __device__ __align__(256) float s_x[2 * kVars * (size_t)kCap];  // variables, hi then lo planes
static __device__ __align__(256) float s_g[kVars * (size_t)kCap];      // gradient planes
static __device__ __align__(256) float s_e[kCap];                      // per-dimer energies
static __device__ __align__(256) PolyNode s_l1[POLY2B_N1];
static __device__ __align__(256) PolyNode s_l2[POLY2B_N2];
static __device__ __align__(256) PolyNode s_l3[POLY2B_N3];
static __device__ __align__(256) PolyNode s_lv[POLY2B_NL];

struct NoAllocDevice {
    bool ready = false;
    float *x = nullptr, *g = nullptr, *e = nullptr;
    PolyNode *l1 = nullptr, *l2 = nullptr, *l3 = nullptr, *lv = nullptr;
    int num_sms = 0;
};

constexpr int kMaxDevices = 64;
NoAllocDevice g_dev[kMaxDevices];
std::mutex g_mu;

mbpol_status setup(int dev, const NoAllocDevice** out) {
    std::lock_guard<std::mutex> lock(g_mu);
    NoAllocDevice& d = g_dev[dev];
    if (!d.ready) {
        MBPOL_CUDA_OK(cudaGetSymbolAddress((void**)&d.x, s_x));
        MBPOL_CUDA_OK(cudaGetSymbolAddress((void**)&d.g, s_g));
        MBPOL_CUDA_OK(cudaGetSymbolAddress((void**)&d.e, s_e));
        MBPOL_CUDA_OK(cudaGetSymbolAddress((void**)&d.l1, s_l1));
        MBPOL_CUDA_OK(cudaGetSymbolAddress((void**)&d.l2, s_l2));
        MBPOL_CUDA_OK(cudaGetSymbolAddress((void**)&d.l3, s_l3));
        MBPOL_CUDA_OK(cudaGetSymbolAddress((void**)&d.lv, s_lv));
        MBPOL_CUDA_OK(cudaMemcpyToSymbol(s_l1, poly2b_l1, sizeof(poly2b_l1)));
        MBPOL_CUDA_OK(cudaMemcpyToSymbol(s_l2, poly2b_l2, sizeof(poly2b_l2)));
        MBPOL_CUDA_OK(cudaMemcpyToSymbol(s_l3, poly2b_l3, sizeof(poly2b_l3)));
        MBPOL_CUDA_OK(cudaMemcpyToSymbol(s_lv, poly2b_leaf, sizeof(poly2b_leaf)));
        MBPOL_CUDA_OK(cudaDeviceGetAttribute(&d.num_sms, cudaDevAttrMultiProcessorCount, dev));
        MBPOL_CUDA_OK(poly2b_kernel_setup());
        upload_polyterm_constants(kOneBodyCoef, &kOneBodyIdx[0][0]);
        MBPOL_CUDA_OK(cudaGetLastError());
        d.ready = true;
    }
    *out = &d;
    return MBPOL_OK;
}

}  // namespace
}  // namespace mbpol

using namespace mbpol;

extern "C" mbpol_status mbpol_twobody_dimers_noalloc(const double* positions, const int* waters, const int* dimers,
                                                    int num_dimers, const double* box_nm, double* forces,
                                                    double* energy, void* stream) {
    if (num_dimers < 0) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "negative dimer count");
    if (num_dimers > kCap)
        return mbpol_fail(MBPOL_ERR_CAPACITY, "more dimers than MBPOL_NOALLOC_MAX_DIMERS; split the list");
    if (num_dimers == 0) return MBPOL_OK;
    if (!positions || !waters || !dimers || !forces || !energy)
        return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null device pointer");
    if ((uintptr_t)waters % 16 || (uintptr_t)dimers % 8 || (uintptr_t)positions % 8 || (uintptr_t)forces % 8 ||
        (uintptr_t)energy % 8)
        return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "misaligned device pointer (waters 16 B, others 8 B)");
    Box box{};
    if (box_nm) {
        for (int k = 0; k < 3; ++k) {
            if (!(box_nm[k] > 0.0) || !std::isfinite(box_nm[k]))
                return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "bad box");
            // the two-body switch reaches 0.65 nm: one image per dimer
            if (box_nm[k] < 1.3) return mbpol_fail(MBPOL_ERR_BOX_TOO_SMALL, "box edge below 2 x 0.65 nm");
            box.L[k] = box_nm[k];
            box.inv[k] = 1.0 / box_nm[k];
        }
        box.periodic = 1;
    }
    int dev = 0;
    MBPOL_CUDA_OK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "device index out of range");
    const NoAllocDevice* d = nullptr;
    mbpol_status s = setup(dev, &d);
    if (s) return s;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int2* pairs = reinterpret_cast<const int2*>(dimers);
    const int4* w4 = reinterpret_cast<const int4*>(waters);
    launch_twobody_vars(st, num_dimers, pairs, w4, positions, box, d->x, kCap);
    launch_poly2b_with(st, d->l1, d->l2, d->l3, d->lv, d->x, d->g, d->e, num_dimers, kCap, d->num_sms);
    launch_twobody_forces(st, num_dimers, pairs, w4, positions, box, d->g, d->e, kCap, forces, energy);
    MBPOL_CUDA_OK(cudaGetLastError());
    return MBPOL_OK;
}
