// Three-body MB-pol polynomial (value and gradient) on the tcgen05 tensor
// cores.  Same formulation and tables as poly_tc.cu (mma.sync): with
// d = x - x0 and y the 703 monomials of degree <= 2 of d, E = y^T S y,
// z = S y, E = y . z, dE/dd_i = 2 sum_m z_m dy_m/dd_i (the reference's
// polynomial: platforms/reference/src/poly-3b-v2x.cpp:3-28378).  Here the
// product is taken transposed, Z^T [128 trimers x 704] = Y'^T . S^T:
//   - A operand: Y'^T of a tile of 128 trimers (one per tensor-memory
//     lane), two fp16 pieces, written to tensor memory by the trimers' own
//     threads.  Tensor memory holds a third of K at a time (besides four
//     accumulator buffers), so a tile runs in three K parts of 15, 15 and
//     14 k-tiles.
//   - B operand: S in blocks of 64 rows x 16 columns (three fp16 pieces,
//     6 KB), only blocks with a nonzero entry, streamed from global memory
//     (L2) by bulk copies through a 28-stage shared-memory ring.
//   - D: per block, Y0.S0 + Y1.S0 + Y0.S1 + Y0.S2 started from zero
//     (M = 128, N = 64, K = 16), so the tensor cores' own accumulation
//     rounding stays relative to one k-tile.  The blocks of a part go in
//     pairs, each block into its own buffer of 64 columns; two pair slots
//     (four buffers) alternate, so that one wait, one tensor-memory fence
//     and one commit serve two blocks.
// A persistent block (one per SM) runs four roles at once, linked by
// mbarriers:
//   warp 0      producer: bulk copies of the block stream, tile after tile,
//               as ring stages free up;
//   warp 1      MMA issue (one thread) once a part's Y' is in tensor memory;
//               owns the tensor-memory allocation;
//   warps 2-5   flush: add each block's D to FP32 sums in registers (thread
//               = trimer, 64 rows of S) and, when a row chunk's blocks are
//               done, add its partial z to the tile's scratch slice
//               (double-buffered by tile parity);
//   warps 6-9   Y' of each part into tensor memory (thread = trimer), and,
//               while the MMAs of a tile's last part run, the epilogue of
//               the previous tile from its scratch slice: E = y . z and the
//               gradient, double-float sums in a fixed order.
// A warp reaches the tensor-memory lanes 32 (warp % 4) .. + 31, so warps
// 2-5 and 6-9 each cover the 128 lanes once.
//
// Every wait is bounded (umma.cuh): a wait that gives up raises the block's
// abort flag and writes a code to `status`; every role then leaves its
// loops, the block waits (bounded) for its bulk copies and MMAs in flight,
// frees its tensor memory and returns.
#include <cuda_fp16.h>

#include "mbpol_internal.cuh"
#include "poly_tc.h"
#include "poly_tc_common.cuh"
#include "poly_tc_dev.h"
#include "umma.cuh"

namespace mbpol {

namespace {

using namespace umma;

constexpr int kNv = 36, kNpad = 704;
constexpr int kNy = 1 + kNv + kNv * (kNv + 1) / 2;  // 703 monomials (row 703 is padding)
constexpr int kU = 128;                   // trimers per tile (M; one tensor-memory lane each)
constexpr int kRows = 64;                 // rows of S per chunk (N)
constexpr int kKt = kNpad / 16;           // 44 k-tiles
constexpr int kParts = 3;                 // K parts
// first k-tile of part p (0, 15, 30, 44; codegen/gen_poly_tc.py tc5_part_bounds)
__host__ __device__ constexpr int part_kt0(int p) { return (p * kKt + kParts - 1) / kParts; }
constexpr int kKtPart = part_kt0(1);      // largest part: 15 k-tiles
constexpr int kChunks = kNpad / kRows;    // 11
constexpr int kYCols = 8 * kKtPart;       // tensor-memory columns of one piece of Y' (two fp16 per column)
constexpr int kAccCol = 2 * kYCols;       // first accumulator column (240)
constexpr int kBufs = 4;                  // accumulator buffers of kRows columns (two pair slots)
constexpr int kMaxBlk = 256;              // blocks in the stream (shared-memory copy of their k-tiles)
constexpr int kTmemCols = 512;
constexpr int kBlkBytes = 3 * kRows * 16 * 2;  // one block of S: three pieces
constexpr int kStages = 28;
constexpr int kWarps = 10, kThreads = 32 * kWarps;
constexpr int kYWarp0 = 6;                // warps 2-5 flush, 6-9 Y' and epilogue
constexpr int DS = kNv + 3;               // d row stride (odd: conflict-free); d_nv = 1, d_{nv+1} = 0
static_assert(kAccCol + kBufs * kRows <= kTmemCols, "tensor memory");
static_assert(part_kt0(2) - part_kt0(1) <= kKtPart && kKt - part_kt0(2) <= kKtPart, "part sizes");

// shared memory
constexpr size_t kOffD = (size_t)kStages * kBlkBytes;                   // d [2][kU][DS]
constexpr size_t kOffYmeta = kOffD + sizeof(float) * 2 * kU * DS;        // ymeta [kNpad]
constexpr size_t kOffRs = kOffYmeta + sizeof(unsigned) * kNpad;         // rowscale [kNpad]
constexpr size_t kOffBars = kOffRs + sizeof(float) * kNpad;
// barriers: full, empty [kStages]; tfull, tempty [2 pair slots + 2 unused];
// yready; mmadone; zdone [2]; edone [2]; done
constexpr int kNumBars = 2 * kStages + 2 * kBufs + 7;
constexpr size_t kOffMeta = kOffBars + 8 * kNumBars;   // blk_begin [kParts * kChunks + 1], blk_kt [kMaxBlk]
constexpr size_t kOffMisc = kOffMeta + sizeof(int) * (kParts * kChunks + 1) + kMaxBlk;
constexpr size_t kSmem = kOffMisc + 16;
static_assert(kSmem <= 232448, "shared memory per block");

// abort-path waits: ignore the abort flag, give up after kWaitCycles
__device__ __forceinline__ void drain_wait(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - t0 > kWaitCycles) return;
}

__device__ __forceinline__ uint32_t pack_h2(float a, float b) {
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

__global__ void __launch_bounds__(kThreads, 1)
    poly_tc5_kernel(const PolyTCDev tab, const float* __restrict__ X, float* __restrict__ G, float* __restrict__ E,
                    int n, int stride, float* __restrict__ zscratch, int* status) {
    extern __shared__ __align__(1024) unsigned char smem[];
    float* dsm = reinterpret_cast<float*>(smem + kOffD);
    unsigned* ymeta = reinterpret_cast<unsigned*>(smem + kOffYmeta);
    float* rowscale = reinterpret_cast<float*>(smem + kOffRs);
    int* s_begin = reinterpret_cast<int*>(smem + kOffMeta);
    unsigned char* s_kt = smem + kOffMeta + sizeof(int) * (kParts * kChunks + 1);
    uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(smem + kOffMisc);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(smem + kOffMisc + 4);
    const uint32_t s_stage = smem_addr(smem);
    const uint32_t b_full = smem_addr(smem + kOffBars);  // [kStages]: block landed
    const uint32_t b_empty = b_full + 8 * kStages;       // [kStages]: its MMAs are done
    const uint32_t b_tfull = b_empty + 8 * kStages;      // [2]: a pair's D ready
    const uint32_t b_tempty = b_tfull + 8 * kBufs;       // [2]: a pair's D read
    const uint32_t b_yready = b_tempty + 8 * kBufs;      // a part's Y' is in tensor memory
    const uint32_t b_mmadone = b_yready + 8;             // a part's MMAs are done (Y' may be replaced)
    const uint32_t b_zdone = b_mmadone + 8;              // [2]: a tile's z is complete in its slice
    const uint32_t b_edone = b_zdone + 16;               // [2]: a tile's epilogue has read its slice
    const uint32_t b_done = b_edone + 16;                // every MMA done (teardown)
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    if (tid == 0) {
        for (int i = 0; i < kStages; ++i) {
            mbar_init(b_full + 8 * i, 1);
            mbar_init(b_empty + 8 * i, 1);
        }
        for (int i = 0; i < kBufs; ++i) {
            mbar_init(b_tfull + 8 * i, 1);
            mbar_init(b_tempty + 8 * i, 4);
        }
        mbar_init(b_yready, 4);
        mbar_init(b_mmadone, 1);
        for (int i = 0; i < 2; ++i) {
            mbar_init(b_zdone + 8 * i, 4);
            mbar_init(b_edone + 8 * i, 4);
        }
        mbar_init(b_done, 1);
        *abort_flag = 0;
        fence_barrier_init();
    }
    for (int i = tid; i <= kParts * kChunks; i += kThreads) s_begin[i] = tab.blk_begin[i];
    for (int i = tid; i < tab.nblk5 && i < kMaxBlk; i += kThreads) s_kt[i] = tab.blk_kt[i];
    for (int i = tid; i < kNpad; i += kThreads) {
        ymeta[i] = tab.ymeta[i];
        rowscale[i] = tab.rowscale[i];
    }
    if (warp == 1) {
        tmem_alloc(smem_addr(tmem_slot), kTmemCols);
        tmem_relinquish();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tb = *tmem_slot;

    const int ntiles = (n + kU - 1) / kU;
    const int nt = (int)blockIdx.x < ntiles ? (ntiles - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
    const int nblk = tab.nblk5;
    float* zbase = zscratch + (size_t)blockIdx.x * 2 * kNpad * kU;  // [2][kNpad][kU]
    uint32_t n_copy = 0;                                             // teardown bookkeeping

    if (warp == 0) {
        // ---------------------------------------------------------- producer
        if (lane == 0) {
            const unsigned total = (unsigned)nt * (unsigned)nblk;
            for (unsigned g = 0; g < total; ++g) {
                const uint32_t st = g % kStages, ph = (g / kStages) & 1;
                if (!mbar_wait(b_empty + 8 * st, ph ^ 1, abort_flag, status, 1)) break;
                mbar_arrive_expect_tx(b_full + 8 * st, kBlkBytes);
                bulk_g2s(s_stage + st * kBlkBytes, tab.sblk + (size_t)(g % nblk) * (kBlkBytes / 2), kBlkBytes,
                         b_full + 8 * st);
                n_copy = g + 1;
            }
        }
    } else if (warp == 1) {
        // ---------------------------------------------------------- MMA issue
        if (lane == 0) {
            const uint32_t idesc = idesc_f16(kU, kRows);
            uint32_t g = 0, pr = 0;  // blocks, pairs
            bool ok = true;
            for (int i = 0; i < nt && ok; ++i) {
                for (int part = 0; part < kParts && ok; ++part) {
                    const uint32_t k = 3 * i + part;
                    if (!mbar_wait(b_yready, k & 1, abort_flag, status, 5)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const int blk0 = s_begin[part * kChunks], blk1 = s_begin[(part + 1) * kChunks];
                    for (int b = blk0; b < blk1 && ok; b += 2, ++pr) {
                        const uint32_t slot = pr & 1, sph = (pr >> 1) & 1;
                        if (!mbar_wait(b_tempty + 8 * slot, sph ^ 1, abort_flag, status, 3)) {
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        for (int q = 0; q < 2 && b + q < blk1; ++q, ++g) {
                            const uint32_t st = g % kStages, ph = (g / kStages) & 1;
                            if (!mbar_wait(b_full + 8 * st, ph, abort_flag, status, 2)) {
                                ok = false;
                                break;
                            }
                            const uint32_t j = s_kt[b + q];
                            const uint32_t sa = s_stage + st * kBlkBytes;
                            const uint32_t dt = tb + kAccCol + (2 * slot + q) * kRows;
                            const uint32_t y0 = tb + 8 * j, y1 = y0 + kYCols;
                            // S0 twice in a row: its operand fetch is shared
                            mma_ts(dt, y0, sdesc(sa, 1024, 128), idesc, 0);
                            mma_ts(dt, y1, sdesc(sa, 1024, 128), idesc, 1);
                            mma_ts(dt, y0, sdesc(sa + 2048, 1024, 128), idesc, 1);
                            mma_ts(dt, y0, sdesc(sa + 4096, 1024, 128), idesc, 1);
                            mma_commit(b_empty + 8 * st);
                        }
                        if (ok) mma_commit(b_tfull + 8 * slot);
                    }
                    if (ok) mma_commit(b_mmadone);
                }
            }
        }
    } else if (warp < kYWarp0) {
        // ---------------------------------------------------------- flush
        const int qd = warp & 3, t = 32 * qd + lane;
        const uint32_t lb = tb + ((uint32_t)(32 * qd) << 16) + kAccCol;
        uint32_t pr = 0;  // pairs
        bool ok = true;
        for (int i = 0; i < nt && ok; ++i) {
            float* zs = zbase + (size_t)(i & 1) * kNpad * kU + t;   // this trimer's column
            // the slice's previous tile (i - 2) must have been read by its epilogue
            if (i >= 2 && !mbar_wait(b_edone + 8 * (i & 1), ((i - 2) >> 1) & 1, abort_flag, status, 8)) break;
            for (int part = 0; part < kParts && ok; ++part) {
                const int blk0 = s_begin[part * kChunks], blk1 = s_begin[(part + 1) * kChunks];
                for (int c = 0; c < kChunks; ++c) {
                    const int c0 = s_begin[part * kChunks + c], c1 = s_begin[part * kChunks + c + 1];
                    if (c0 == c1 && part > 0) continue;  // nothing to add to these rows
                    float a[kRows];
                    #pragma unroll
                    for (int j = 0; j < kRows; ++j) a[j] = 0.f;
                    for (int b = c0; b < c1; ++b) {
                        // pairs of the part's blocks: (blk0, blk0 + 1), ...
                        const int q = (b - blk0) & 1;
                        const uint32_t slot = pr & 1, sph = (pr >> 1) & 1;
                        if (q == 0) {
                            if (!mbar_wait(b_tfull + 8 * slot, sph, abort_flag, status, 4)) {
                                ok = false;
                                break;
                            }
                            tc_fence_after();
                        }
                        const uint32_t buf = 2 * slot + q;
                        float v[32];
                        tmem_ld32(lb + buf * kRows, v);
                        tmem_wait_ld();
                        #pragma unroll
                        for (int j = 0; j < 32; ++j) a[j] = __fadd_rn(a[j], v[j]);
                        tmem_ld32(lb + buf * kRows + 32, v);
                        tmem_wait_ld();
                        #pragma unroll
                        for (int j = 0; j < 32; ++j) a[32 + j] = __fadd_rn(a[32 + j], v[j]);
                        if (q == 1 || b + 1 == blk1) {
                            tc_fence_before();
                            __syncwarp();
                            if (lane == 0) mbar_arrive(b_tempty + 8 * slot);
                            ++pr;
                        }
                    }
                    if (!ok) break;
                    // the chunk's rows of z (scaled by 2^-r_m) added to the
                    // earlier parts' sums; old values loaded 16 at a time
                    float* zc = zs + (size_t)c * kRows * kU;
                    #pragma unroll
                    for (int h = 0; h < kRows; h += 16) {
                        float old[16];
                        #pragma unroll
                        for (int j = 0; j < 16; ++j) old[j] = part == 0 ? 0.f : zc[(size_t)(h + j) * kU];
                        #pragma unroll
                        for (int j = 0; j < 16; ++j)
                            zc[(size_t)(h + j) * kU] =
                                __fadd_rn(old[j], __fmul_rn(a[h + j], rowscale[c * kRows + h + j]));
                    }
                }
            }
            if (!ok) break;
            __threadfence_block();
            __syncwarp();
            if (lane == 0) mbar_arrive(b_zdone + 8 * (i & 1));
        }
    } else {
        // ---------------------------------------------------------- Y' and epilogue
        const int qd = warp & 3, t = 32 * qd + lane;
        const uint32_t lb = tb + ((uint32_t)(32 * qd) << 16);
        bool ok = true;
        int e_cur = 0, e_prev = 0;
        // d = x - x0 of tile i's trimer t into its row of buffer (i & 1);
        // returns the trimer's exponent e (unit_exp of max |d_v| / bound_v)
        auto load_d = [&](int i) -> int {
            const int u = ((int)blockIdx.x + i * (int)gridDim.x) * kU + t;
            float* dt = dsm + ((size_t)(i & 1) * kU + t) * DS;
            float m = 0.f;
            float xh[kNv], xl[kNv];
            #pragma unroll
            for (int v = 0; v < kNv; ++v) {
                xh[v] = u < n ? X[(size_t)v * stride + u] : 0.f;
                xl[v] = u < n ? X[(size_t)(kNv + v) * stride + u] : 0.f;
            }
            #pragma unroll
            for (int v = 0; v < kNv; ++v) {
                const float d = u < n ? __fadd_rn(__fsub_rn(xh[v], __ldg(tab.x0h + v)), __fsub_rn(xl[v], __ldg(tab.x0l + v)))
                                      : 0.f;
                dt[v] = d;
                m = fmaxf(m, fabsf(d) * __ldg(tab.inv_bound + v));
            }
            dt[kNv] = 1.f;
            dt[kNv + 1] = 0.f;
            return unit_exp(m);
        };
        // E and the gradient of tile i's trimer t from its scratch slice.
        // Each sum runs as four double-float partial sums (terms j % 4),
        // added in a fixed order at the end; in E the loads of the next 16
        // rows are issued before the current 16 are summed.
        auto epilogue = [&](int i, int e) -> bool {
            if (!mbar_wait(b_zdone + 8 * (i & 1), (i >> 1) & 1, abort_flag, status, 7)) return false;
            const int u = ((int)blockIdx.x + i * (int)gridDim.x) * kU + t;
            const float* zs = zbase + (size_t)(i & 1) * kNpad * kU + t;
            const float* dt = dsm + ((size_t)(i & 1) * kU + t) * DS;
            const float ze = exp2i(e);
            // E = sum_m y_m z_m over the 704 rows (row 703: y = 0, z = 0)
            float2 es[4];
            #pragma unroll
            for (int q = 0; q < 4; ++q) es[q] = make_float2(0.f, 0.f);
            auto eload = [&](float (&z)[16], int r0) {
                #pragma unroll
                for (int j = 0; j < 16; ++j) z[j] = zs[(size_t)(r0 + j) * kU];
            };
            auto esum = [&](const float (&z)[16], int r0) {
                #pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const unsigned meta = ymeta[r0 + j];
                    df_fma(es[j & 3], __fmul_rn(dt[meta & 255], dt[(meta >> 8) & 255]), z[j]);
                }
            };
            {
                float zA[16], zB[16];
                eload(zA, 0);
                for (int r0 = 0; r0 < kNpad; r0 += 32) {
                    eload(zB, r0 + 16);
                    esum(zA, r0);
                    if (r0 + 32 < kNpad) eload(zA, r0 + 32);
                    esum(zB, r0 + 16);
                }
            }
            df_add(es[0], es[1]);
            df_add(es[0], es[2]);
            df_add(es[0], es[3]);
            if (u < n) E[u] = __fmul_rn(__fadd_rn(es[0].x, es[0].y), ze);
            // dE/dd_v = 2 z_(v) + sum_j (2 or 4) d_j z_(min(v,j), max(v,j))
            auto gload = [&](float (&z)[kNv + 1], int v) {
                z[kNv] = zs[(size_t)(1 + v) * kU];
                #pragma unroll
                for (int j = 0; j < kNv; ++j) {
                    const int a = min(v, j), b = max(v, j);
                    z[j] = zs[(size_t)(1 + kNv + a * kNv - (a * (a - 1)) / 2 + (b - a)) * kU];
                }
            };
            auto gsum = [&](const float (&z)[kNv + 1], int v) {
                float2 gq[4];
                #pragma unroll
                for (int q = 0; q < 4; ++q) gq[q] = make_float2(0.f, 0.f);
                df_fma(gq[3], 2.f, z[kNv]);
                #pragma unroll
                for (int j = 0; j < kNv; ++j) df_fma(gq[j & 3], (j == v ? 4.f : 2.f) * dt[j], z[j]);
                df_add(gq[0], gq[1]);
                df_add(gq[0], gq[2]);
                df_add(gq[0], gq[3]);
                if (u < n) G[(size_t)v * stride + u] = __fmul_rn(__fadd_rn(gq[0].x, gq[0].y), ze);
            };
            {
                float zA[kNv + 1];
                for (int v = 0; v < kNv; ++v) {
                    gload(zA, v);
                    gsum(zA, v);
                }
            }
            __threadfence_block();
            __syncwarp();
            if (lane == 0) mbar_arrive(b_edone + 8 * (i & 1));
            return true;
        };
        if (nt > 0) e_cur = load_d(0);
        for (int i = 0; i < nt && ok; ++i) {
            const float* dt = dsm + ((size_t)(i & 1) * kU + t) * DS;
            for (int part = 0; part < kParts; ++part) {
                const uint32_t k = 3 * i + part;
                // the previous part's MMAs must be done before its Y' is replaced
                if (k > 0 && !mbar_wait(b_mmadone, (k - 1) & 1, abort_flag, status, 6)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                // Y' = Y 2^(s_k - e) as two fp16 pieces: lane t, column 8 j + c
                // = monomials 16 j + 2c, 2c + 1 of the part's k-tile j
                const int kt0 = part_kt0(part), nkt = part_kt0(part + 1) - kt0;
                for (int j = 0; j < nkt; ++j) {
                    const int k0 = (kt0 + j) * 16;
                    uint32_t hi[8], lo[8];
                    #pragma unroll
                    for (int c = 0; c < 8; ++c) {
                        float y[2];
                        #pragma unroll
                        for (int h = 0; h < 2; ++h) {
                            const unsigned meta = ymeta[k0 + 2 * c + h];
                            const int a = meta & 255, b = (meta >> 8) & 255, s = (int)((meta >> 16) & 255) - 128;
                            y[h] = __fmul_rn(__fmul_rn(dt[a], dt[b]), exp2i(s - e_cur));
                        }
                        const __half2 hh = __floats2half2_rn(y[0], y[1]);
                        hi[c] = *reinterpret_cast<const uint32_t*>(&hh);
                        lo[c] = pack_h2(__fsub_rn(y[0], __low2float(hh)), __fsub_rn(y[1], __high2float(hh)));
                    }
                    tmem_st8(lb + 8 * j, hi);
                    tmem_st8(lb + kYCols + 8 * j, lo);
                }
                tmem_wait_st();
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(b_yready);
                if (part == kParts - 1) {
                    // while the last part's MMAs run: the previous tile's
                    // epilogue, then the next tile's d (into the buffer the
                    // epilogue has just finished with)
                    if (i > 0 && !epilogue(i - 1, e_prev)) {
                        ok = false;
                        break;
                    }
                    e_prev = e_cur;
                    if (i + 1 < nt) e_cur = load_d(i + 1);
                }
            }
        }
        if (ok && nt > 0) epilogue(nt - 1, e_prev);
    }

    // ---- teardown: no bulk copy or MMA may be in flight when the tensor
    // memory is freed and the block exits
    if (warp == 0 && lane == 0) {
        for (uint32_t g = n_copy > (uint32_t)kStages ? n_copy - kStages : 0u; g < n_copy; ++g)
            drain_wait(b_full + 8 * (g % kStages), (g / kStages) & 1);
    }
    if (warp == 1 && lane == 0) {
        mma_commit(b_done);
        drain_wait(b_done, 0);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tb, kTmemCols);
    }
}

}  // namespace

cudaError_t poly_tc5_prepare() {
    if (k_poly3b.parts5 != kParts || k_poly3b.rows5 != kRows || k_poly3b.npad != kNpad || k_poly3b.nblk5 > kMaxBlk)
        return cudaErrorInvalidValue;
    return cudaFuncSetAttribute(poly_tc5_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSmem);
}

// two z slices per block (tile parity)
size_t poly3b_tc5_scratch_floats(int num_sms) { return (size_t)num_sms * 2 * kNpad * kU; }

// SMs left out of the persistent grid for the electrostatics stream (a block
// takes a whole SM's shared memory and tensor memory).
#ifndef MBPOL_TC5_RESERVE_SMS
#define MBPOL_TC5_RESERVE_SMS 52
#endif

int tc5_default_reserve() { return MBPOL_TC5_RESERVE_SMS; }

void launch_poly3b_tc5(cudaStream_t st, const PolyTCDev* tab, const float* X, float* G, float* E, int n, int stride,
                       int num_sms, float* zscratch, int* status, int reserve_sms) {
    if (n <= 0) return;
    count_launch();
    const int ntiles = (n + kU - 1) / kU;
    int blocks = num_sms - (reserve_sms < 0 ? MBPOL_TC5_RESERVE_SMS : reserve_sms);
    if (blocks < num_sms / 2) blocks = num_sms / 2;
    if (blocks > ntiles) blocks = ntiles;
    poly_tc5_kernel<<<blocks, kThreads, kSmem, st>>>(*tab, X, G, E, n, stride, zscratch, status);
}

}  // namespace mbpol
