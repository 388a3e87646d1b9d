// O-O neighbour structures for the many-body terms.
//
//  * mol_neighbors_kernel: one warp per water i scans the candidate waters j
//    (tiles of 32, ballot-compacted appends; distances prefiltered in FP32
//    and settled in FP64 near each threshold): the 27 cells around i's cell
//    in periodic boxes with at least 3 cells per dimension (cell binning by
//    counting sort, members ascending within a cell), the waters of i's
//    cluster for batched clusters, else all waters.  It records
//      - full[i][*]   j != i with d(i,j) <= r_full   (electrostatics, dispersion)
//      - lower[i][*]  j <  i with d(i,j) <= r_3b     (three-body chain rule)
//      - pairs        (i,j), j > i, d <= r_2b        (two-body half list)
//    Distances use the minimum image in periodic boxes.  Replaces OpenMM's
//    computeNeighborListVoxelHash (called at
//    platforms/reference/src/MBPolReferenceKernels.cpp:379-383) and the
//    voxel hash of platforms/reference/src/ReferenceThreeNeighborList.cpp:60-177.
//  * Trimers follow the reference's rule
//    (ReferenceThreeNeighborList.cpp:202-225): (I,J,K) with J in lower[I] and
//    K in lower[J], i.e. I > J > K, d(I,J) <= rc, d(J,K) <= rc; d(I,K) is not
//    tested.  MBPOL_TRIMER_COMPLETE instead takes every triple {a<b<c} with at
//    least two of its three O-O distances <= rc (all trimers with a nonzero
//    switch).
// Capacity overflows set an error flag instead of writing out of bounds.
#include "mbpol_internal.cuh"
#include "mbpol_kernels.h"

namespace mbpol {

__device__ __forceinline__ double oo_dist2(double3 a, double3 b, const Box& box) {
    double dx = b.x - a.x, dy = b.y - a.y, dz = b.z - a.z;
    if (box.periodic) {
        dx = min_image(dx, box.L[0], box.inv[0]);
        dy = min_image(dy, box.L[1], box.inv[1]);
        dz = min_image(dz, box.L[2], box.inv[2]);
    }
    return dx * dx + dy * dy + dz * dz;
}

// FP32 copy of each water's O position (wrapped into the box when periodic,
// so FP32 keeps its absolute precision) for the distance prefilter.
__global__ void o_positions_kernel(int nw, const int4* __restrict__ waters, const double* __restrict__ pos, Box box,
                                   float4* __restrict__ opos) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nw) return;
    double3 o = load_pos(pos, waters[i].x);
    if (box.periodic) {
        o.x -= box.L[0] * floor(o.x * box.inv[0]);
        o.y -= box.L[1] * floor(o.y * box.inv[1]);
        o.z -= box.L[2] * floor(o.z * box.inv[2]);
    }
    opos[i] = make_float4((float)o.x, (float)o.y, (float)o.z, 0.f);
}

// d^2 <= r^2 decided in FP32 when d^2 is farther than the FP32 error bound
// from r^2, else in FP64 (d2 is computed at most once per pair, lazily), so
// list membership is exactly the FP64 test.  Bound: each FP32 coordinate is
// off by <= 2^-24 |x|, so d^2 is off by <= ~2 |d| 2^-23 (|x_i| + |x_j|);
// the margin is 8x that, plus 1e-6 nm^2.
struct PairTest {
    const double3& oi;
    double d2 = -1.0;
    __device__ bool le(float d2f, float r, float slack, double r2, const int4* __restrict__ waters,
                       const double* __restrict__ pos, int j, const Box& box) {
        const float r2f = r * r;
        const float m = 1e-6f + slack * r;
        if (d2f < r2f - m) return true;
        if (d2f > r2f + m) return false;
        if (d2 < 0.0) {
            const double3 o = load_pos(pos, waters[j].x);
            double dx = o.x - oi.x, dy = o.y - oi.y, dz = o.z - oi.z;
            if (box.periodic) {
                dx = min_image(dx, box.L[0], box.inv[0]);
                dy = min_image(dy, box.L[1], box.inv[1]);
                dz = min_image(dz, box.L[2], box.inv[2]);
            }
            d2 = dx * dx + dy * dy + dz * dz;
        }
        return d2 <= r2;
    }
};

__global__ void mol_neighbors_kernel(int nw, const int4* __restrict__ waters, const double* __restrict__ pos,
                                     const float4* __restrict__ opos, Box box, double r_full2, double r_3b2,
                                     double r_2b2, int cap_full, int cap_lower, int* __restrict__ full,
                                     int* __restrict__ nfull, int* __restrict__ lower, int* __restrict__ nlower,
                                     int2* __restrict__ pairs, int cap_pairs, int* __restrict__ npairs,
                                     int* __restrict__ overflow, const CandidateSet cs) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= nw) return;
    const int i = warp;
    const double3 oi = load_pos(pos, waters[i].x);
    const float4 fi = opos[i];
    const float ai = fmaxf(fabsf(fi.x), fmaxf(fabsf(fi.y), fabsf(fi.z)));
    const float Lx = (float)box.L[0], Ly = (float)box.L[1], Lz = (float)box.L[2];
    const float ix = (float)box.inv[0], iy = (float)box.inv[1], iz = (float)box.inv[2];
    const float rf = full ? (float)sqrt(r_full2) : 0.f, r3 = lower ? (float)sqrt(r_3b2) : 0.f,
                r2 = pairs ? (float)sqrt(r_2b2) : 0.f;
    int nf = 0, nl = 0;
    for_candidates(cs, nw, i, lane, [&](const int j) {
        bool in_full = false, in_lower = false, in_pair = false;
        if (j >= 0 && j != i) {
            const float4 fj = opos[j];
            float dx = fj.x - fi.x, dy = fj.y - fi.y, dz = fj.z - fi.z;
            if (box.periodic) {
                dx -= Lx * rintf(dx * ix);
                dy -= Ly * rintf(dy * iy);
                dz -= Lz * rintf(dz * iz);
            }
            const float d2f = dx * dx + dy * dy + dz * dz;
            const float aj = fmaxf(fabsf(fj.x), fmaxf(fabsf(fj.y), fabsf(fj.z)));
            const float slack = 16.f * 1.2e-7f * 3.f * (ai + aj);
            PairTest pt{oi};
            in_full = full && pt.le(d2f, rf, slack, r_full2, waters, pos, j, box);
            in_lower = lower && j < i && pt.le(d2f, r3, slack, r_3b2, waters, pos, j, box);
            in_pair = pairs && j > i && pt.le(d2f, r2, slack, r_2b2, waters, pos, j, box);
        }
        unsigned m = __ballot_sync(0xffffffffu, in_full);
        if (in_full) {
            int slot = nf + __popc(m & ((1u << lane) - 1u));
            if (slot < cap_full) full[(size_t)i * cap_full + slot] = j;
        }
        nf += __popc(m);
        m = __ballot_sync(0xffffffffu, in_lower);
        if (in_lower) {
            int slot = nl + __popc(m & ((1u << lane) - 1u));
            if (slot < cap_lower) lower[(size_t)i * cap_lower + slot] = j;
        }
        nl += __popc(m);
        m = __ballot_sync(0xffffffffu, in_pair);
        if (m) {
            int base_slot = 0;
            if (lane == 0) base_slot = atomicAdd(npairs, __popc(m));
            base_slot = __shfl_sync(0xffffffffu, base_slot, 0);
            if (in_pair) {
                int slot = base_slot + __popc(m & ((1u << lane) - 1u));
                if (slot < cap_pairs) pairs[slot] = make_int2(i, j);
            }
        }
    });
    if (lane == 0) {
        if (nfull) nfull[i] = nf;
        if (nlower) nlower[i] = nl;
        if ((full && nf > cap_full) || (lower && nl > cap_lower)) atomicOr(overflow, 1);
    }
}

// Number of chain-rule trimers whose first index is i.
__global__ void trimer_count_kernel(int nw, const int* __restrict__ lower, const int* __restrict__ nlower,
                                    int cap_lower, int* __restrict__ count) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nw) return;
    int c = 0;
    const int n = min(nlower[i], cap_lower);
    for (int a = 0; a < n; ++a) c += min(nlower[lower[(size_t)i * cap_lower + a]], cap_lower);
    count[i] = c;
}

// Exclusive scan of count[0..n) into offs[0..n], offs[n] = total; one block.
__global__ void scan_kernel(int n, const int* __restrict__ count, int* __restrict__ offs) {
    __shared__ int part[1024];
    const int t = threadIdx.x;
    const int per = (n + blockDim.x - 1) / blockDim.x;
    const int lo = min(n, t * per), hi = min(n, lo + per);
    int s = 0;
    for (int k = lo; k < hi; ++k) s += count[k];
    part[t] = s;
    __syncthreads();
    for (int o = 1; o < (int)blockDim.x; o <<= 1) {
        int v = t >= o ? part[t - o] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    int run = t > 0 ? part[t - 1] : 0;
    for (int k = lo; k < hi; ++k) {
        offs[k] = run;
        run += count[k];
    }
    if (t == (int)blockDim.x - 1) offs[n] = part[t];
}

__global__ void trimer_fill_kernel(int nw, const int* __restrict__ lower, const int* __restrict__ nlower,
                                   int cap_lower, const int* __restrict__ offs, int cap_trip,
                                   int4* __restrict__ trips) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nw) return;
    int o = offs[i];
    const int n = min(nlower[i], cap_lower);
    for (int a = 0; a < n; ++a) {
        const int j = lower[(size_t)i * cap_lower + a];
        const int m = min(nlower[j], cap_lower);
        for (int b = 0; b < m; ++b) {
            if (o < cap_trip) trips[o] = make_int4(i, j, lower[(size_t)j * cap_lower + b], 0);
            ++o;
        }
    }
}

// Complete rule: triples {a,b,c} with >= 2 of the 3 O-O distances <= rc.
// Each such triple is enumerated once, at its designated centre v: the
// vertex adjacent (<= rc) to both others; for a closed triangle, the largest
// index.  Output order is (v, larger neighbour, smaller neighbour).
__global__ void trimer_complete_kernel(int nw, const int4* __restrict__ waters, const double* __restrict__ pos,
                                       Box box, double rc2, const int* __restrict__ full,
                                       const int* __restrict__ nfull, int cap_full, int* __restrict__ count,
                                       const int* __restrict__ offs, int cap_trip, int4* __restrict__ trips) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nw) return;
    const int n = min(nfull[v], cap_full);
    const int* nb = full + (size_t)v * cap_full;
    const double3 ov = load_pos(pos, waters[v].x);
    int o = offs ? offs[v] : 0;
    int cnt = 0;
    for (int p = 0; p < n; ++p) {
        const int w = nb[p];
        const double3 ow = load_pos(pos, waters[w].x);
        if (oo_dist2(ov, ow, box) > rc2) continue;
        for (int q = 0; q < n; ++q) {
            const int u = nb[q];
            if (u >= w) continue;
            const double3 ou = load_pos(pos, waters[u].x);
            if (oo_dist2(ov, ou, box) > rc2) continue;
            const bool closed = oo_dist2(ou, ow, box) <= rc2;
            if (closed && v < w) continue;  // triangle: counted at its largest vertex
            if (trips && o < cap_trip) trips[o] = make_int4(v, w, u, 0);
            ++o;
            ++cnt;
        }
    }
    if (count) count[v] = cnt;
}

// ---------------------------------------------------------------- cells
bool cell_grid_dims(const Box& box, double r, int nc[3]) {
    if (!box.periodic || !(r > 0.0)) return false;
    const double edge = r * (1.0 + 1e-5) + 1e-4;
    long total = 1;
    for (int d = 0; d < 3; ++d) {
        nc[d] = (int)floor(box.L[d] / edge);
        if (nc[d] < 3) return false;
        if (nc[d] > 1024) nc[d] = 1024;  // larger cells stay correct
        total *= nc[d];
    }
    return total <= (1L << 27);
}

size_t cell_scratch_ints(int n, const Box& box, double r) {
    int nc[3];
    if (n <= 0 || !cell_grid_dims(box, r, nc)) return 0;
    return 3 * (size_t)n + 3 * ((size_t)nc[0] * nc[1] * nc[2] + 1);
}

__global__ void cell_assign_kernel(int n, const float4* __restrict__ opos, float sx, float sy, float sz, int ncx,
                                   int ncy, int ncz, int* __restrict__ cell_of, int* __restrict__ count) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = opos[i];
    const int x = min(max((int)(p.x * sx), 0), ncx - 1);
    const int y = min(max((int)(p.y * sy), 0), ncy - 1);
    const int z = min(max((int)(p.z * sz), 0), ncz - 1);
    const int c = (x * ncy + y) * ncz + z;
    cell_of[i] = c;
    atomicAdd(count + c, 1);
}

__global__ void cell_scatter_kernel(int n, const int* __restrict__ cell_of, const int* __restrict__ start,
                                    int* __restrict__ fill, int* __restrict__ unsorted) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = cell_of[i];
    unsorted[start[c] + atomicAdd(fill + c, 1)] = i;
}

// each molecule's place in its cell is its rank among the cell's members,
// so members are ascending whatever order the scatter's atomics took
__global__ void cell_rank_kernel(int n, const int* __restrict__ cell_of, const int* __restrict__ start,
                                 const int* __restrict__ unsorted, int* __restrict__ sorted) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int c = cell_of[i];
    int r = 0;
    for (int k = start[c]; k < start[c + 1]; ++k) r += unsorted[k] < i;
    sorted[start[c] + r] = i;
}

mbpol_status launch_cell_binning(cudaStream_t st, int n, const float4* opos, const Box& box, double r, int* scratch,
                                 CandidateSet* out) {
    *out = CandidateSet();
    int nc[3];
    if (n <= 0 || !scratch || !cell_grid_dims(box, r, nc)) return MBPOL_OK;
    const int ncell = nc[0] * nc[1] * nc[2];
    int* cell_of = scratch;
    int* unsorted = cell_of + n;
    int* sorted = unsorted + n;
    int* count = sorted + n;
    int* start = count + (ncell + 1);
    int* fill = start + (ncell + 1);
    MBPOL_CUDA_OK(cudaMemsetAsync(count, 0, sizeof(int) * (size_t)(ncell + 1), st));
    MBPOL_CUDA_OK(cudaMemsetAsync(fill, 0, sizeof(int) * (size_t)(ncell + 1), st));
    const int blocks = (n + 255) / 256;
    count_launch();
    cell_assign_kernel<<<blocks, 256, 0, st>>>(n, opos, (float)(nc[0] * box.inv[0]), (float)(nc[1] * box.inv[1]),
                                               (float)(nc[2] * box.inv[2]), nc[0], nc[1], nc[2], cell_of, count);
    count_launch();
    scan_kernel<<<1, 1024, 0, st>>>(ncell, count, start);
    count_launch();
    cell_scatter_kernel<<<blocks, 256, 0, st>>>(n, cell_of, start, fill, unsorted);
    count_launch();
    cell_rank_kernel<<<blocks, 256, 0, st>>>(n, cell_of, start, unsorted, sorted);
    out->mode = 2;
    out->members = sorted;
    out->start = start;
    out->group = cell_of;
    for (int d = 0; d < 3; ++d) out->nc[d] = nc[d];
    return MBPOL_OK;
}

void cluster_members(const int* cluster_of, int n, int ncl, std::vector<int>& members, std::vector<int>& start) {
    start.assign((size_t)ncl + 1, 0);
    for (int i = 0; i < n; ++i) ++start[(size_t)cluster_of[i] + 1];
    for (int c = 0; c < ncl; ++c) start[(size_t)c + 1] += start[(size_t)c];
    members.assign((size_t)n, 0);
    std::vector<int> fill(start.begin(), start.end() - 1);
    for (int i = 0; i < n; ++i) members[(size_t)fill[(size_t)cluster_of[i]]++] = i;
}

mbpol_status launch_mol_neighbors(cudaStream_t st, int nw, const int4* waters, const double* pos, float4* opos,
                                  Box box, double r_full, double r_3b, double r_2b, int cap_full, int cap_lower,
                                  int* full, int* nfull, int* lower, int* nlower, int2* pairs, int cap_pairs,
                                  int* npairs, int* overflow, const CandidateSet* clusters, int* cell_scratch) {
    if (nw <= 0) return MBPOL_OK;
    count_launch();
    o_positions_kernel<<<(nw + 127) / 128, 128, 0, st>>>(nw, waters, pos, box, opos);
    CandidateSet cs;
    if (clusters) {
        cs = *clusters;
    } else {
        const double r = fmax(r_full, fmax(r_3b, r_2b));
        mbpol_status s = launch_cell_binning(st, nw, opos, box, r, cell_scratch, &cs);
        if (s) return s;
    }
    const int threads = 256;
    const int blocks = (nw * 32 + threads - 1) / threads;
    count_launch();
    mol_neighbors_kernel<<<blocks, threads, 0, st>>>(nw, waters, pos, opos, box, r_full * r_full, r_3b * r_3b,
                                                     r_2b * r_2b, cap_full, cap_lower, full, nfull, lower, nlower,
                                                     pairs, cap_pairs, npairs, overflow, cs);
    return MBPOL_OK;
}

void launch_trimer_count(cudaStream_t st, int nw, const int* lower, const int* nlower, int cap_lower, int* count,
                         int* offs) {
    if (nw <= 0) return;
    count_launch();
    trimer_count_kernel<<<(nw + 127) / 128, 128, 0, st>>>(nw, lower, nlower, cap_lower, count);
    count_launch();
    scan_kernel<<<1, 1024, 0, st>>>(nw, count, offs);
}

void launch_trimer_fill(cudaStream_t st, int nw, const int* lower, const int* nlower, int cap_lower,
                        const int* offs, int cap_trip, int4* trips) {
    if (nw <= 0) return;
    count_launch();
    trimer_fill_kernel<<<(nw + 127) / 128, 128, 0, st>>>(nw, lower, nlower, cap_lower, offs, cap_trip, trips);
}

void launch_trimer_complete(cudaStream_t st, int nw, const int4* waters, const double* pos, Box box, double rc,
                            const int* full, const int* nfull, int cap_full, int* count, int* offs, int cap_trip,
                            int4* trips, bool fill) {
    if (nw <= 0) return;
    if (!fill) {
        count_launch();
        trimer_complete_kernel<<<(nw + 127) / 128, 128, 0, st>>>(nw, waters, pos, box, rc * rc, full, nfull,
                                                                 cap_full, count, nullptr, 0, nullptr);
        count_launch();
        scan_kernel<<<1, 1024, 0, st>>>(nw, count, offs);
    } else {
        count_launch();
        trimer_complete_kernel<<<(nw + 127) / 128, 128, 0, st>>>(nw, waters, pos, box, rc * rc, full, nfull,
                                                                 cap_full, nullptr, offs, cap_trip, trips);
    }
}

}  // namespace mbpol
