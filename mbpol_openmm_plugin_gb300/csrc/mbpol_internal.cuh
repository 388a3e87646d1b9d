// Internal definitions shared by the MB-pol GB300 kernels and the C-ABI layer.
//
// Data layout in HBM (one context = one system):
//   pos      double[3*N]       particle positions (nm), as passed by the caller
//   force    double[3*N]       FP64 force accumulator (kJ/mol/nm), atomics
//   waters   int4[W]           particle indices (O, H1, H2, M or -1)
//   energy   double[MBPOL_NUM_TERMS]  FP64 energy accumulators (kJ/mol)
// Units: nm, kJ/mol.  The polynomial terms work in Angstrom and kcal/mol
// internally, as the MB-pol fits are expressed in those units.
#pragma once
#include <cuda_runtime.h>
#include <cstdint>

#define MBPOL_CUDA_OK(expr)                                   \
    do {                                                      \
        cudaError_t e_ = (expr);                              \
        if (e_ != cudaSuccess) return mbpol_fail_cuda(e_, #expr); \
    } while (0)

namespace mbpol {

// Per-kernel CUDA-event timing (enabled with mbpol_profile_enable): ids of
// the timed kernels.
enum KernelId { K_POLY2B = 0, K_POLY3B, K_ELEC_FIXED, K_ELEC_INDUCED, K_ELEC_PME, K_ELEC_FORCES, K_ELEC_FIELD, K_NUM };
void prof_begin(cudaStream_t st, int id);
// Whether the per-kernel timers are on (the solver then keeps its host loop,
// whose iterations the timers can bracket).
bool prof_on();
// Number of kernels this library has launched (cuFFT's own launches excluded).
void count_launch();
void prof_end(cudaStream_t st, int id);

constexpr double kNmToA = 10.0;
constexpr double kCalToJ = 4.184;
constexpr float kPiF = 3.14159265358979323846f;

struct Box {
    double L[3];     // box lengths (nm); ignored when !periodic
    double inv[3];
    int periodic;
};

__device__ __forceinline__ double min_image(double d, double L, double invL) {
    return d - L * floor(d * invL + 0.5);
}

// Image particle b next to reference a (component-wise floor(d/L+0.5)),
// as imageParticles() in platforms/reference/src/MBPolReferenceTwoBodyForce.cpp:66-75.
__device__ __forceinline__ double3 image_to(const double3 a, double3 b, const Box& box) {
    if (box.periodic) {
        b.x += box.L[0] * floor((a.x - b.x) * box.inv[0] + 0.5);
        b.y += box.L[1] * floor((a.y - b.y) * box.inv[1] + 0.5);
        b.z += box.L[2] * floor((a.z - b.z) * box.inv[2] + 0.5);
    }
    return b;
}

__device__ __forceinline__ double3 load_pos(const double* __restrict__ pos, int i) {
    return make_double3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
}

__device__ __forceinline__ void add_force(double* __restrict__ f, int i, double fx, double fy, double fz) {
    atomicAdd(f + 3 * i, fx);
    atomicAdd(f + 3 * i + 1, fy);
    atomicAdd(f + 3 * i + 2, fz);
}

// Neighbour candidates of molecule i when a warp builds i's list: all
// molecules (mode 0), the members of i's cluster (mode 1; batched
// independent clusters), or the molecules of the 27 cells around i's cell
// (mode 2; periodic boxes with at least 3 cells per dimension whose edges
// are at least the largest list radius).  Members are ascending within a
// cluster and within a cell, and cells are visited in a fixed order, so the
// lists are the same from run to run.
struct CandidateSet {
    int mode = 0;
    const int* members = nullptr;  // molecules grouped by cluster / cell
    const int* start = nullptr;    // offset of each group in members, and the end
    const int* group = nullptr;    // cluster / cell of each molecule
    int nc[3] = {0, 0, 0};         // cells per dimension (mode 2)
};

// body(j) is called by all 32 lanes of the warp together for each chunk of
// candidates; j = -1 on lanes without one (and j may equal i).
template <class F>
__device__ __forceinline__ void for_candidates(const CandidateSet& cs, int n, int i, int lane, F&& body) {
    if (cs.mode == 0) {
        for (int base = 0; base < n; base += 32) body(base + lane < n ? base + lane : -1);
        return;
    }
    if (cs.mode == 1) {
        const int g = cs.group[i];
        const int s0 = cs.start[g], s1 = cs.start[g + 1];
        for (int k = s0; k < s1; k += 32) body(k + lane < s1 ? cs.members[k + lane] : -1);
        return;
    }
    const int c = cs.group[i];
    const int cz = c % cs.nc[2], cy = (c / cs.nc[2]) % cs.nc[1], cx = c / (cs.nc[1] * cs.nc[2]);
    for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy)
            for (int dz = -1; dz <= 1; ++dz) {
                const int x = (cx + dx + cs.nc[0]) % cs.nc[0];
                const int y = (cy + dy + cs.nc[1]) % cs.nc[1];
                const int z = (cz + dz + cs.nc[2]) % cs.nc[2];
                const int cc = (x * cs.nc[1] + y) * cs.nc[2] + z;
                const int s0 = cs.start[cc], s1 = cs.start[cc + 1];
                for (int k = s0; k < s1; k += 32) body(k + lane < s1 ? cs.members[k + lane] : -1);
            }
}

// Cells per dimension of a periodic box for list radius r (edges >= r plus a
// margin for the FP32 positions the cells are assigned from); false when a
// dimension would have fewer than 3 cells (or the box is not periodic).
bool cell_grid_dims(const Box& box, double r, int nc[3]);
// Device ints the cell binning of n molecules needs (0 when no grid).
size_t cell_scratch_ints(int n, const Box& box, double r);
// launch_cell_binning (mbpol_kernels.h) bins n molecules by their FP32 O
// positions (wrapped into the box) into that grid, in scratch of
// cell_scratch_ints ints, and gives the mode-2 candidate set over it (mode 0
// when there is no grid).

// Block-wide FP64 sum, then one atomic per block into *out.
// Per-cluster energies for batched independent clusters: a unit's energy is
// also added to e[cluster_of_water[w] * stride] (e offset by the term).
// Empty (wcl null) for a single system.
struct ClusterSink {
    const int* wcl = nullptr;
    double* e = nullptr;
    int stride = 0;
};
__device__ __forceinline__ void cluster_energy(const ClusterSink& cs, int water, double e) {
    if (cs.wcl && e != 0.0) atomicAdd(cs.e + (size_t)cs.wcl[water] * cs.stride, e);
}

template <int BLOCK>
__device__ __forceinline__ void block_sum_atomic(double v, double* out) {
    __shared__ double red[BLOCK / 32];
    #pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = lane < BLOCK / 32 ? red[lane] : 0.0;
        #pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0 && v != 0.0) atomicAdd(out, v);
    }
}

struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mk(float x, float y, float z) { return f3{x, y, z}; }
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return f3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return f3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return f3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ f3& operator+=(f3& a, f3 b) { a.x += b.x; a.y += b.y; a.z += b.z; return a; }
__device__ __forceinline__ f3& operator-=(f3& a, f3 b) { a.x -= b.x; a.y -= b.y; a.z -= b.z; return a; }
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ f3 cross(f3 a, f3 b) {
    return f3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
// (b - a) in Angstrom, computed in FP64 then rounded once to FP32.
__device__ __forceinline__ f3 rel_A(double3 a, double3 b) {
    return f3{(float)((b.x - a.x) * kNmToA), (float)((b.y - a.y) * kNmToA), (float)((b.z - a.z) * kNmToA)};
}

}  // namespace mbpol
