// C-ABI implementation: context, buffers, orchestration of the MB-pol
// kernels on one CUDA stream.  See include/mbpol_gb300.h for the contract.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/mbpol_gb300.h"
#include "elec.h"
#include "mbpol_kernels.h"
#include "poly_tc_dev.h"

// Generated at build time: one-body tables.
#include "gen/model_tables.inc"

namespace {
thread_local std::string g_last_error;
}

mbpol_status mbpol_fail(mbpol_status s, const std::string& msg) {
    g_last_error = msg;
    return s;
}
mbpol_status mbpol_fail_cuda(cudaError_t e, const char* what) {
    g_last_error = std::string(what) + ": " + cudaGetErrorString(e);
    return MBPOL_ERR_CUDA;
}

namespace mbpol {

// Event-pair timing of selected kernels, one global profile per process
// (the library drives one device per context and the bench uses one).
struct Profiler {
    bool on = false;
    std::vector<cudaEvent_t> pool;
    size_t used = 0;
    std::vector<std::pair<size_t, size_t>> rec[K_NUM];
    cudaEvent_t get() {
        if (used == pool.size()) {
            cudaEvent_t e;
            cudaEventCreate(&e);
            pool.push_back(e);
        }
        return pool[used++];
    }
};
Profiler g_prof;
unsigned long long g_launches = 0;
void count_launch() { ++g_launches; }
size_t g_open[K_NUM];

bool prof_on() { return g_prof.on; }

void prof_begin(cudaStream_t st, int id) {
    if (!g_prof.on) return;
    cudaEvent_t e = g_prof.get();
    cudaEventRecord(e, st);
    g_open[id] = g_prof.used - 1;
}
void prof_end(cudaStream_t st, int id) {
    if (!g_prof.on) return;
    cudaEvent_t e = g_prof.get();
    cudaEventRecord(e, st);
    g_prof.rec[id].push_back({g_open[id], g_prof.used - 1});
}

// Grow-only device buffer.
struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    cudaError_t ensure(size_t n) {
        if (n <= bytes) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        bytes = 0;
        size_t nb = n + n / 4 + 256;
        cudaError_t e = cudaMalloc(&p, nb);
        if (e == cudaSuccess) bytes = nb;
        return e;
    }
    template <class T>
    T* as() const {
        return static_cast<T*>(p);
    }
};

struct WaterTerm {
    bool on = false;
    int method = 0;
    double cutoff = 0.0;
    int rule = 0;
    std::vector<int4> waters;
    DevBuf d_waters;
    // batched clusters: cluster of each water of this term's list, the
    // waters of each cluster (ascending) and their offsets
    DevBuf d_cluster, d_cl_members, d_cl_start;
    CandidateSet cl_candidates;
    int max_cluster = 0;
};

}  // namespace mbpol

using namespace mbpol;

// Launch shape of the persistent polynomial kernels: SMs the three-body
// tensor kernel leaves to the other streams, blocks the double-float walks
// leave out of their grids.  Every unit's arithmetic is independent of the
// grid, so the shape changes timing only.
struct LaunchShape {
    int tc_reserve = -1;    // negative: the kernel's default (52 SMs)
    int walk_reserve = -1;  // negative: the walk's default (24 blocks)
};

// Project-written autotuner: over the next evaluations (each force
// evaluation, inside MD steps too) it cycles through candidate launch
// shapes, `reps` evaluations each, times each evaluation with CUDA events on
// the context's stream (which joins every other stream), and keeps the
// shape with the smallest median time.
struct Autotuner {
    int reps = 0;                        // 0: off
    bool done = false;
    size_t cand = 0;
    std::vector<LaunchShape> cands;
    std::vector<std::vector<float>> ms;  // [candidate][repetition]
    cudaEvent_t t0 = nullptr, t1 = nullptr;
    bool timing = false;
};

struct mbpol_context {
    int N = 0;
    int device = 0;
    cudaStream_t st = nullptr;
    DevBuf d_pos, d_force, d_energy, d_counters;
    std::vector<double> h_force;
    bool have_pos = false;
    Box box{};
    // virtual sites
    std::vector<int4> vs_idx;
    std::vector<double> vs_w;
    DevBuf d_vs_idx, d_vs_w;
    bool vs_dirty = false;
    WaterTerm t1, t2, t3, tdisp;
    // two-body buffers
    DevBuf p2, x2, g2, e2;
    int cap2 = 0;
    // three-body buffers
    DevBuf lower3, nlower3, count3, offs3, trips3, x3, g3, e3, full3, nfull3;
    int cap_lower3 = 48, cap3 = 0, cap_full3 = 96;
    // polynomial tables of this device; the three-body evaluator (tensor
    // cores by default) and its per-block scratch
    const PolyWalkTables* walk = nullptr;
    const PolyTCDev* tc3 = nullptr;
    int poly3b_kind = MBPOL_POLY3B_AUTO;
    DevBuf ztc;
    DevBuf kstatus;  // int: nonzero when a bounded wait of the tcgen05 kernel gave up
    // launch shapes of the persistent polynomial kernels (results do not
    // depend on them) and the autotuner that picks them
    LaunchShape shape;
    Autotuner tuner;
    // dispersion buffers
    DevBuf full_d, nfull_d, lower_d, nlower_d;
    int cap_full_d = 0;
    // FP32 O positions for the neighbour prefilter; lists built by one
    // shared pass for the two-body, three-body and dispersion terms
    DevBuf opos;
    DevBuf cells;  // cell binning scratch of the O-O lists
    bool shared_lists = false;
    // batched independent clusters (cluster of every particle)
    int ncl = 0;
    std::vector<int> cl_of_particle;
    bool cl_dirty = false;
    DevBuf d_cl_energy;  // [ncl][MBPOL_NUM_TERMS]
    double disp_c6[16], disp_d6[16];
    std::vector<int> disp_ions;  // chloride ions of the dispersion term
    DevBuf d_disp_ions;
    // electrostatics
    std::unique_ptr<ElecEngine> elec;
    int num_sms = 0;
    long counts[4] = {0, 0, 0, 0};
    // molecular dynamics state (device resident)
    DevBuf d_vel, d_invm, d_ekin;
    bool have_masses = false, have_vel = false, forces_valid = false;
    unsigned long long md_step = 0;
    long solver_iterations_total = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    // electrostatics run on their own stream, concurrently with the
    // polynomial terms (independent work; both latency-bound)
    cudaStream_t st_e = nullptr;
    cudaEvent_t ev_pos = nullptr, ev_elec = nullptr;
    // the one-body term (FP64, few threads) and the dispersion (latency
    // bound) run on a third stream beside the lists and the walks
    cudaStream_t st_a = nullptr;
    cudaEvent_t ev_lists = nullptr, ev_aux = nullptr;
};

namespace {

mbpol_status check_waters(mbpol_context* ctx, int nw, const int* w) {
    if (nw < 0 || (nw > 0 && !w)) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "bad water list");
    for (int i = 0; i < 3 * nw; ++i)
        if (w[i] < 0 || w[i] >= ctx->N) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "particle index out of range");
    return MBPOL_OK;
}

mbpol_status set_term(mbpol_context* ctx, WaterTerm& t, int nw, const int* w, int method, double cutoff, int rule) {
    mbpol_status s = check_waters(ctx, nw, w);
    if (s) return s;
    t.on = true;
    t.method = method;
    t.cutoff = cutoff;
    t.rule = rule;
    t.waters.resize((size_t)nw);
    for (int i = 0; i < nw; ++i) t.waters[(size_t)i] = make_int4(w[3 * i], w[3 * i + 1], w[3 * i + 2], -1);
    MBPOL_CUDA_OK(t.d_waters.ensure(sizeof(int4) * (size_t)(nw > 0 ? nw : 1)));
    if (nw > 0)
        MBPOL_CUDA_OK(cudaMemcpy(t.d_waters.p, t.waters.data(), sizeof(int4) * (size_t)nw, cudaMemcpyHostToDevice));
    return MBPOL_OK;
}

Box term_box(const mbpol_context* ctx, bool periodic) {
    Box b = ctx->box;
    b.periodic = periodic && ctx->box.periodic;
    return b;
}

mbpol_status check_box(const mbpol_context* ctx, double cutoff) {
    if (!ctx->box.periodic) return mbpol_fail(MBPOL_ERR_STATE, "periodic method requires a box");
    for (int k = 0; k < 3; ++k)
        if (ctx->box.L[k] < 1.999999 * cutoff)
            return mbpol_fail(MBPOL_ERR_BOX_TOO_SMALL, "The periodic box size has decreased to less than twice the cutoff.");
    return MBPOL_OK;
}

const CandidateSet* term_clusters(const mbpol_context* ctx, const WaterTerm& t) {
    return ctx->ncl > 0 ? &t.cl_candidates : nullptr;
}

// Device scratch for the cell binning of n waters at list radius r (null
// when the box has no cell grid, or on allocation failure: then all pairs
// are scanned).
int* cell_scratch(mbpol_context* ctx, int n, const Box& box, double r) {
    const size_t ints = cell_scratch_ints(n, box, r);
    if (ints == 0 || ctx->cells.ensure(sizeof(int) * ints) != cudaSuccess) return nullptr;
    return ctx->cells.as<int>();
}

ClusterSink term_sink(mbpol_context* ctx, const WaterTerm& t, int term) {
    ClusterSink cs;
    if (ctx->ncl > 0) {
        cs.wcl = t.d_cluster.as<int>();
        cs.e = ctx->d_cl_energy.as<double>() + term;
        cs.stride = MBPOL_NUM_TERMS;
    }
    return cs;
}

// Per-term cluster arrays and the electrostatics engine's clusters, built at
// the first evaluation after mbpol_set_clusters.
mbpol_status apply_clusters(mbpol_context* ctx) {
    ctx->cl_dirty = false;
    const int ncl = ctx->ncl;
    if (ncl > 0) {
        MBPOL_CUDA_OK(ctx->d_cl_energy.ensure(sizeof(double) * MBPOL_NUM_TERMS * (size_t)ncl));
        for (WaterTerm* t : {&ctx->t1, &ctx->t2, &ctx->t3, &ctx->tdisp}) {
            const int nw = (int)t->waters.size();
            if (nw == 0) continue;
            std::vector<int> wc(nw), count(ncl, 0);
            for (int w = 0; w < nw; ++w) {
                const int4 wi = t->waters[w];
                const int c = ctx->cl_of_particle[wi.x];
                if (ctx->cl_of_particle[wi.y] != c || ctx->cl_of_particle[wi.z] != c)
                    return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "the atoms of one water are in different clusters");
                wc[w] = c;
                ++count[c];
            }
            t->max_cluster = 0;
            for (int c = 0; c < ncl; ++c) t->max_cluster = std::max(t->max_cluster, count[c]);
            MBPOL_CUDA_OK(t->d_cluster.ensure(sizeof(int) * (size_t)nw));
            MBPOL_CUDA_OK(cudaMemcpy(t->d_cluster.p, wc.data(), sizeof(int) * nw, cudaMemcpyHostToDevice));
            std::vector<int> members, start;
            cluster_members(wc.data(), nw, ncl, members, start);
            MBPOL_CUDA_OK(t->d_cl_members.ensure(sizeof(int) * members.size()));
            MBPOL_CUDA_OK(t->d_cl_start.ensure(sizeof(int) * start.size()));
            MBPOL_CUDA_OK(cudaMemcpy(t->d_cl_members.p, members.data(), sizeof(int) * members.size(),
                                     cudaMemcpyHostToDevice));
            MBPOL_CUDA_OK(cudaMemcpy(t->d_cl_start.p, start.data(), sizeof(int) * start.size(), cudaMemcpyHostToDevice));
            t->cl_candidates = CandidateSet();
            t->cl_candidates.mode = 1;
            t->cl_candidates.members = t->d_cl_members.as<int>();
            t->cl_candidates.start = t->d_cl_start.as<int>();
            t->cl_candidates.group = t->d_cluster.as<int>();
        }
    }
    ctx->cap_full_d = 0;
    if (ctx->elec) {
        mbpol_status s = ctx->elec->set_clusters(
            ncl > 0 ? ctx->cl_of_particle.data() : nullptr, ncl,
            ncl > 0 ? ctx->d_cl_energy.as<double>() + MBPOL_TERM_ELECTROSTATICS : nullptr, MBPOL_NUM_TERMS);
        if (s) return s;
    }
    return MBPOL_OK;
}

// Two-body pair list on its own (one neighbour pass, one host sync).
mbpol_status twobody_list(mbpol_context* ctx, const Box& box, double rc, int* np_out) {
    WaterTerm& t = ctx->t2;
    const int nw = (int)t.waters.size();
    int* cnt = ctx->d_counters.as<int>();
    MBPOL_CUDA_OK(ctx->opos.ensure(sizeof(float4) * (size_t)nw));
    for (int attempt = 0; attempt < 2; ++attempt) {
        if (ctx->cap2 == 0) ctx->cap2 = nw * 24 + 64;
        MBPOL_CUDA_OK(ctx->p2.ensure(sizeof(int2) * (size_t)ctx->cap2));
        MBPOL_CUDA_OK(cudaMemsetAsync(cnt, 0, 2 * sizeof(int), ctx->st));
        mbpol_status ns = launch_mol_neighbors(
            ctx->st, nw, t.d_waters.as<int4>(), ctx->d_pos.as<double>(), ctx->opos.as<float4>(), box, -1.0, -1.0, rc,
            0, 0, nullptr, nullptr, nullptr, nullptr, ctx->p2.as<int2>(), ctx->cap2, cnt, cnt + 1,
            term_clusters(ctx, t), cell_scratch(ctx, nw, box, rc));
        if (ns) return ns;
        int h[2];
        MBPOL_CUDA_OK(cudaMemcpyAsync(h, cnt, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
        MBPOL_CUDA_OK(cudaStreamSynchronize(ctx->st));
        if (h[0] > ctx->cap2) {
            ctx->cap2 = h[0] + h[0] / 4 + 64;
            continue;
        }
        *np_out = h[0];
        return MBPOL_OK;
    }
    return mbpol_fail(MBPOL_ERR_CAPACITY, "two-body pair list capacity");
}

// Each term runs in two phases: the list phase builds its neighbour list on
// ctx->st (host synchronisations for the list sizes), the launch phase
// queues its kernels on `ls` without synchronising.  All list phases run
// before any launch phase, so no host wait queues behind a walk and the
// electrostatics stream starts while the walks run.
mbpol_status run_twobody(mbpol_context* ctx, double* energy, cudaStream_t ls, bool list_phase) {
    WaterTerm& t = ctx->t2;
    const int nw = (int)t.waters.size();
    if (nw < 2) return MBPOL_OK;
    const bool periodic = t.method == MBPOL_CUTOFF_PERIODIC;
    if (periodic) {
        mbpol_status s = check_box(ctx, t.cutoff);
        if (s) return s;
    }
    const Box box = term_box(ctx, periodic);
    const double rc = t.method == MBPOL_NOCUTOFF ? 1e30 : t.cutoff;
    if (list_phase) {
        if (!ctx->shared_lists) {
            int np = 0;
            mbpol_status s = twobody_list(ctx, box, rc, &np);
            if (s) return s;
            ctx->counts[0] = np;
        }
        return MBPOL_OK;
    }
    const int np = (int)ctx->counts[0];
    const int stride = ctx->cap2;
    MBPOL_CUDA_OK(ctx->x2.ensure(sizeof(float) * 2 * 31 * (size_t)stride));
    MBPOL_CUDA_OK(ctx->g2.ensure(sizeof(float) * 31 * (size_t)stride));
    MBPOL_CUDA_OK(ctx->e2.ensure(sizeof(float) * (size_t)stride));
    launch_twobody_vars(ls, np, ctx->p2.as<int2>(), t.d_waters.as<int4>(), ctx->d_pos.as<double>(), box,
                        ctx->x2.as<float>(), stride);
    prof_begin(ls, K_POLY2B);
    launch_poly2b(ls, ctx->walk, ctx->x2.as<float>(), ctx->g2.as<float>(), ctx->e2.as<float>(), np, stride,
                  ctx->num_sms, ctx->shape.walk_reserve);
    prof_end(ls, K_POLY2B);
    launch_twobody_forces(ls, np, ctx->p2.as<int2>(), t.d_waters.as<int4>(), ctx->d_pos.as<double>(), box,
                          ctx->g2.as<float>(), ctx->e2.as<float>(), stride, ctx->d_force.as<double>(), energy,
                          term_sink(ctx, t, MBPOL_TERM_TWOBODY));
    return MBPOL_OK;
}

// Three-body neighbour lists and trimer count on their own (one host sync).
mbpol_status threebody_list(mbpol_context* ctx, const Box& box, double rc, int* ntrip_out) {
    WaterTerm& t = ctx->t3;
    const int nw = (int)t.waters.size();
    int* cnt = ctx->d_counters.as<int>();
    const bool complete = t.rule == MBPOL_TRIMER_COMPLETE;
    MBPOL_CUDA_OK(ctx->opos.ensure(sizeof(float4) * (size_t)nw));
    for (int attempt = 0; attempt < 4; ++attempt) {
        MBPOL_CUDA_OK(ctx->nlower3.ensure(sizeof(int) * (size_t)nw));
        MBPOL_CUDA_OK(ctx->count3.ensure(sizeof(int) * (size_t)nw));
        MBPOL_CUDA_OK(ctx->offs3.ensure(sizeof(int) * (size_t)(nw + 1)));
        MBPOL_CUDA_OK(cudaMemsetAsync(cnt, 0, 2 * sizeof(int), ctx->st));
        if (!complete) {
            MBPOL_CUDA_OK(ctx->lower3.ensure(sizeof(int) * (size_t)nw * ctx->cap_lower3));
            mbpol_status ns = launch_mol_neighbors(
                ctx->st, nw, t.d_waters.as<int4>(), ctx->d_pos.as<double>(), ctx->opos.as<float4>(), box, -1.0, rc,
                -1.0, 0, ctx->cap_lower3, nullptr, nullptr, ctx->lower3.as<int>(), ctx->nlower3.as<int>(), nullptr, 0,
                cnt, cnt + 1, term_clusters(ctx, t), cell_scratch(ctx, nw, box, rc));
            if (ns) return ns;
            launch_trimer_count(ctx->st, nw, ctx->lower3.as<int>(), ctx->nlower3.as<int>(), ctx->cap_lower3,
                                ctx->count3.as<int>(), ctx->offs3.as<int>());
        } else {
            MBPOL_CUDA_OK(ctx->full3.ensure(sizeof(int) * (size_t)nw * ctx->cap_full3));
            MBPOL_CUDA_OK(ctx->nfull3.ensure(sizeof(int) * (size_t)nw));
            mbpol_status ns = launch_mol_neighbors(
                ctx->st, nw, t.d_waters.as<int4>(), ctx->d_pos.as<double>(), ctx->opos.as<float4>(), box, rc, -1.0,
                -1.0, ctx->cap_full3, 0, ctx->full3.as<int>(), ctx->nfull3.as<int>(), nullptr, nullptr, nullptr, 0, cnt,
                cnt + 1, term_clusters(ctx, t), cell_scratch(ctx, nw, box, rc));
            if (ns) return ns;
            launch_trimer_complete(ctx->st, nw, t.d_waters.as<int4>(), ctx->d_pos.as<double>(), box, rc,
                                   ctx->full3.as<int>(), ctx->nfull3.as<int>(), ctx->cap_full3,
                                   ctx->count3.as<int>(), ctx->offs3.as<int>(), 0, nullptr, false);
        }
        int h[3];
        MBPOL_CUDA_OK(cudaMemcpyAsync(h, cnt, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
        MBPOL_CUDA_OK(cudaMemcpyAsync(h + 2, ctx->offs3.as<int>() + nw, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
        MBPOL_CUDA_OK(cudaStreamSynchronize(ctx->st));
        if (h[1]) {  // neighbour capacity overflow: grow and redo
            if (complete) ctx->cap_full3 *= 2;
            else ctx->cap_lower3 *= 2;
            continue;
        }
        *ntrip_out = h[2];
        return MBPOL_OK;
    }
    return mbpol_fail(MBPOL_ERR_CAPACITY, "three-body neighbour capacity");
}

mbpol_status run_threebody(mbpol_context* ctx, double* energy, cudaStream_t ls, bool list_phase) {
    WaterTerm& t = ctx->t3;
    const int nw = (int)t.waters.size();
    if (nw < 3) return MBPOL_OK;
    const bool periodic = t.method == MBPOL_CUTOFF_PERIODIC;
    if (periodic) {
        mbpol_status s = check_box(ctx, t.cutoff);
        if (s) return s;
    }
    const Box box = term_box(ctx, periodic);
    const double rc = t.method == MBPOL_NOCUTOFF ? 1e30 : t.cutoff;
    const bool complete = t.rule == MBPOL_TRIMER_COMPLETE;
    if (list_phase) {
        if (!ctx->shared_lists) {
            int ntrip = 0;
            mbpol_status s = threebody_list(ctx, box, rc, &ntrip);
            if (s) return s;
            ctx->counts[1] = ntrip;
        }
        return MBPOL_OK;
    }
    const int ntrip = (int)ctx->counts[1];
    if (ntrip > ctx->cap3) ctx->cap3 = ntrip + ntrip / 4 + 64;
    const int stride = ctx->cap3;
    MBPOL_CUDA_OK(ctx->trips3.ensure(sizeof(int4) * (size_t)stride));
    MBPOL_CUDA_OK(ctx->x3.ensure(sizeof(float) * 2 * 36 * (size_t)stride));
    MBPOL_CUDA_OK(ctx->g3.ensure(sizeof(float) * 36 * (size_t)stride));
    MBPOL_CUDA_OK(ctx->e3.ensure(sizeof(float) * (size_t)stride));
    if (!complete)
        launch_trimer_fill(ls, nw, ctx->lower3.as<int>(), ctx->nlower3.as<int>(), ctx->cap_lower3,
                           ctx->offs3.as<int>(), stride, ctx->trips3.as<int4>());
    else
        launch_trimer_complete(ls, nw, t.d_waters.as<int4>(), ctx->d_pos.as<double>(), box, rc,
                               ctx->full3.as<int>(), ctx->nfull3.as<int>(), ctx->cap_full3, nullptr,
                               ctx->offs3.as<int>(), stride, ctx->trips3.as<int4>(), true);
    launch_threebody_vars(ls, ntrip, ctx->trips3.as<int4>(), t.d_waters.as<int4>(), ctx->d_pos.as<double>(),
                          box, ctx->x3.as<float>(), stride);
    const int kind = ctx->poly3b_kind == MBPOL_POLY3B_AUTO
                         ? (ntrip >= 64 * ctx->num_sms ? MBPOL_POLY3B_TENSOR : MBPOL_POLY3B_WALK)
                         : ctx->poly3b_kind;
    if (kind == MBPOL_POLY3B_TENSOR)
        MBPOL_CUDA_OK(ctx->ztc.ensure(sizeof(float) * poly3b_tc5_scratch_floats(ctx->num_sms)));
    if (kind == MBPOL_POLY3B_TENSOR_SYNC)
        MBPOL_CUDA_OK(ctx->ztc.ensure(sizeof(float) * poly3b_tc_scratch_floats(ctx->num_sms)));
    prof_begin(ls, K_POLY3B);
    if (kind == MBPOL_POLY3B_TENSOR)
        launch_poly3b_tc5(ls, ctx->tc3, ctx->x3.as<float>(), ctx->g3.as<float>(), ctx->e3.as<float>(), ntrip,
                          stride, ctx->num_sms, ctx->ztc.as<float>(), ctx->kstatus.as<int>(), ctx->shape.tc_reserve);
    else if (kind == MBPOL_POLY3B_TENSOR_SYNC)
        launch_poly3b_tc(ls, ctx->tc3, ctx->x3.as<float>(), ctx->g3.as<float>(), ctx->e3.as<float>(), ntrip, stride,
                         ctx->num_sms, ctx->ztc.as<float>(), ctx->shape.tc_reserve);
    else
        launch_poly3b(ls, ctx->walk, ctx->x3.as<float>(), ctx->g3.as<float>(), ctx->e3.as<float>(), ntrip, stride,
                      ctx->num_sms, ctx->shape.walk_reserve);
    prof_end(ls, K_POLY3B);
    launch_threebody_forces(ls, ntrip, ctx->trips3.as<int4>(), t.d_waters.as<int4>(), ctx->d_pos.as<double>(),
                            box, ctx->g3.as<float>(), ctx->e3.as<float>(), stride, ctx->d_force.as<double>(), energy,
                            term_sink(ctx, t, MBPOL_TERM_THREEBODY));
    return MBPOL_OK;
}

// Dispersion molecule list radius: site cutoff plus twice the largest O-H
// extent (every H-H, O-H pair within the cutoff has its waters listed).
double dispersion_list_radius(const WaterTerm& t) {
    return t.method == MBPOL_NOCUTOFF ? 1e30 : t.cutoff + 0.25;
}

// Dispersion molecule list on its own (one host sync).
mbpol_status dispersion_list(mbpol_context* ctx, const Box& box) {
    WaterTerm& t = ctx->tdisp;
    const int nw = (int)t.waters.size();
    const double rlist = dispersion_list_radius(t);
    int* cnt = ctx->d_counters.as<int>();
    MBPOL_CUDA_OK(ctx->opos.ensure(sizeof(float4) * (size_t)nw));
    for (int attempt = 0; attempt < 4; ++attempt) {
        MBPOL_CUDA_OK(ctx->full_d.ensure(sizeof(int) * (size_t)nw * ctx->cap_full_d));
        MBPOL_CUDA_OK(ctx->nfull_d.ensure(sizeof(int) * (size_t)nw));
        MBPOL_CUDA_OK(cudaMemsetAsync(cnt, 0, 2 * sizeof(int), ctx->st));
        mbpol_status ns = launch_mol_neighbors(
            ctx->st, nw, t.d_waters.as<int4>(), ctx->d_pos.as<double>(), ctx->opos.as<float4>(), box, rlist, -1.0,
            -1.0, ctx->cap_full_d, 0, ctx->full_d.as<int>(), ctx->nfull_d.as<int>(), nullptr, nullptr, nullptr, 0, cnt,
            cnt + 1, term_clusters(ctx, t), cell_scratch(ctx, nw, box, rlist));
        if (ns) return ns;
        int h[2];
        MBPOL_CUDA_OK(cudaMemcpyAsync(h, cnt, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
        MBPOL_CUDA_OK(cudaStreamSynchronize(ctx->st));
        if (h[1]) {
            ctx->cap_full_d *= 2;
            continue;
        }
        return MBPOL_OK;
    }
    return mbpol_fail(MBPOL_ERR_CAPACITY, "dispersion neighbour capacity");
}

mbpol_status run_dispersion(mbpol_context* ctx, double* energy, cudaStream_t ls, bool list_phase) {
    WaterTerm& t = ctx->tdisp;
    const int nw = (int)t.waters.size();
    const int nion = (int)ctx->disp_ions.size();
    if (nw < 2 && nion == 0) return MBPOL_OK;
    const bool periodic = t.method == MBPOL_CUTOFF_PERIODIC;
    if (periodic) {
        mbpol_status s = check_box(ctx, t.cutoff);
        if (s) return s;
    }
    const Box box = term_box(ctx, periodic);
    const double rc = t.method == MBPOL_NOCUTOFF ? 1e30 : t.cutoff;
    if (nw >= 2) {
        if (ctx->cap_full_d == 0)
            ctx->cap_full_d = t.method == MBPOL_NOCUTOFF ? (((ctx->ncl > 0 ? t.max_cluster : nw) + 31) / 32) * 32 : 256;
        if (list_phase) {
            if (!ctx->shared_lists) {
                mbpol_status s = dispersion_list(ctx, box);
                if (s) return s;
            }
            return MBPOL_OK;
        }
        launch_dispersion(ls, nw, t.d_waters.as<int4>(), ctx->d_pos.as<double>(), box, ctx->full_d.as<int>(),
                          ctx->nfull_d.as<int>(), ctx->cap_full_d, rc, ctx->d_force.as<double>(), energy,
                          term_sink(ctx, t, MBPOL_TERM_DISPERSION));
    }
    if (list_phase) return MBPOL_OK;
    launch_dispersion_ions(ls, nion, ctx->d_disp_ions.as<int>(), nw, t.d_waters.as<int4>(),
                           ctx->d_pos.as<double>(), box, rc, ctx->d_force.as<double>(), energy);
    return MBPOL_OK;
}

bool same_waters(const WaterTerm& a, const WaterTerm& b) {
    if (a.waters.size() != b.waters.size()) return false;
    for (size_t i = 0; i < a.waters.size(); ++i)
        if (a.waters[i].x != b.waters[i].x || a.waters[i].y != b.waters[i].y || a.waters[i].z != b.waters[i].z)
            return false;
    return true;
}

// One neighbour pass for the two-body pairs, the three-body chain-rule
// lists (and trimer count) and the dispersion list, when the three terms
// share the water list and are all periodic with cutoffs: one launch and one
// host synchronisation per evaluation instead of three of each.  Returns
// false (and builds nothing) when the terms cannot share.
mbpol_status build_shared_lists(mbpol_context* ctx, unsigned mask, bool* built) {
    *built = false;
    const unsigned need = MBPOL_TERM_BIT(MBPOL_TERM_TWOBODY) | MBPOL_TERM_BIT(MBPOL_TERM_THREEBODY) |
                          MBPOL_TERM_BIT(MBPOL_TERM_DISPERSION);
    const WaterTerm &t2 = ctx->t2, &t3 = ctx->t3, &td = ctx->tdisp;
    if ((mask & need) != need || !t2.on || !t3.on || !td.on || ctx->ncl > 0) return MBPOL_OK;
    if (t2.method != MBPOL_CUTOFF_PERIODIC || t3.method != MBPOL_CUTOFF_PERIODIC ||
        td.method != MBPOL_CUTOFF_PERIODIC || t3.rule == MBPOL_TRIMER_COMPLETE)
        return MBPOL_OK;
    if (!same_waters(t2, t3) || !same_waters(t2, td)) return MBPOL_OK;
    const int nw = (int)t2.waters.size();
    if (nw < 3) return MBPOL_OK;
    for (const WaterTerm* t : {&t2, &t3, &td}) {
        mbpol_status s = check_box(ctx, t->cutoff);
        if (s) return s;
    }
    const Box box = term_box(ctx, true);
    int* cnt = ctx->d_counters.as<int>();
    if (ctx->cap2 == 0) ctx->cap2 = nw * 24 + 64;
    if (ctx->cap_full_d == 0) ctx->cap_full_d = 256;
    MBPOL_CUDA_OK(ctx->opos.ensure(sizeof(float4) * (size_t)nw));
    MBPOL_CUDA_OK(ctx->nlower3.ensure(sizeof(int) * (size_t)nw));
    MBPOL_CUDA_OK(ctx->count3.ensure(sizeof(int) * (size_t)nw));
    MBPOL_CUDA_OK(ctx->offs3.ensure(sizeof(int) * (size_t)(nw + 1)));
    MBPOL_CUDA_OK(ctx->nfull_d.ensure(sizeof(int) * (size_t)nw));
    for (int attempt = 0; attempt < 6; ++attempt) {
        MBPOL_CUDA_OK(ctx->p2.ensure(sizeof(int2) * (size_t)ctx->cap2));
        MBPOL_CUDA_OK(ctx->lower3.ensure(sizeof(int) * (size_t)nw * ctx->cap_lower3));
        MBPOL_CUDA_OK(ctx->full_d.ensure(sizeof(int) * (size_t)nw * ctx->cap_full_d));
        MBPOL_CUDA_OK(cudaMemsetAsync(cnt, 0, 2 * sizeof(int), ctx->st));
        const double rmax = std::max(dispersion_list_radius(td), std::max(t3.cutoff, t2.cutoff));
        mbpol_status ns = launch_mol_neighbors(
            ctx->st, nw, t2.d_waters.as<int4>(), ctx->d_pos.as<double>(), ctx->opos.as<float4>(), box,
            dispersion_list_radius(td), t3.cutoff, t2.cutoff, ctx->cap_full_d, ctx->cap_lower3, ctx->full_d.as<int>(),
            ctx->nfull_d.as<int>(), ctx->lower3.as<int>(), ctx->nlower3.as<int>(), ctx->p2.as<int2>(), ctx->cap2, cnt,
            cnt + 1, nullptr, cell_scratch(ctx, nw, box, rmax));
        if (ns) return ns;
        launch_trimer_count(ctx->st, nw, ctx->lower3.as<int>(), ctx->nlower3.as<int>(), ctx->cap_lower3,
                            ctx->count3.as<int>(), ctx->offs3.as<int>());
        int h[3];
        MBPOL_CUDA_OK(cudaMemcpyAsync(h, cnt, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
        MBPOL_CUDA_OK(cudaMemcpyAsync(h + 2, ctx->offs3.as<int>() + nw, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
        MBPOL_CUDA_OK(cudaStreamSynchronize(ctx->st));
        bool again = false;
        if (h[1]) {  // a per-water list overflowed (which one is not recorded): grow both
            ctx->cap_lower3 *= 2;
            ctx->cap_full_d *= 2;
            again = true;
        }
        if (h[0] > ctx->cap2) {
            ctx->cap2 = h[0] + h[0] / 4 + 64;
            again = true;
        }
        if (again) continue;
        ctx->counts[0] = h[0];
        ctx->counts[1] = h[2];
        *built = true;
        return MBPOL_OK;
    }
    return mbpol_fail(MBPOL_ERR_CAPACITY, "neighbour list capacity");
}

}  // namespace

extern "C" {

void mbpol_electrostatics_params_default(mbpol_electrostatics_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->nonbonded_method = MBPOL_ELEC_NOCUTOFF;
    p->cutoff = 0.9;
    p->ewald_alpha = 0.0;
    p->ewald_error_tolerance = 1e-4;
    p->max_iterations = 200;
    p->target_epsilon = 1e-7;
    const double th[5] = {0.4, 0.4, 0.055, 0.626, 0.055};
    for (int k = 0; k < 5; ++k) p->thole[k] = th[k];
    p->include_charge_redistribution = 1;
    p->guess = 0;
}

mbpol_status mbpol_context_create(int num_particles, int device, mbpol_context** out) {
    if (!out || num_particles <= 0) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "bad context arguments");
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return mbpol_fail(MBPOL_ERR_NO_DEVICE, "no CUDA device is available; this library has no CPU fallback");
    if (device < 0 || device >= ndev) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "bad device index");
    MBPOL_CUDA_OK(cudaSetDevice(device));
    std::unique_ptr<mbpol_context> ctx(new mbpol_context());
    ctx->N = num_particles;
    ctx->device = device;
    MBPOL_CUDA_OK(cudaStreamCreateWithFlags(&ctx->st, cudaStreamNonBlocking));
    MBPOL_CUDA_OK(cudaStreamCreateWithFlags(&ctx->st_e, cudaStreamNonBlocking));
    MBPOL_CUDA_OK(cudaStreamCreateWithFlags(&ctx->st_a, cudaStreamNonBlocking));
    MBPOL_CUDA_OK(cudaEventCreate(&ctx->tuner.t0));
    MBPOL_CUDA_OK(cudaEventCreate(&ctx->tuner.t1));
    MBPOL_CUDA_OK(cudaEventCreateWithFlags(&ctx->ev_pos, cudaEventDisableTiming));
    MBPOL_CUDA_OK(cudaEventCreateWithFlags(&ctx->ev_elec, cudaEventDisableTiming));
    MBPOL_CUDA_OK(cudaEventCreateWithFlags(&ctx->ev_lists, cudaEventDisableTiming));
    MBPOL_CUDA_OK(cudaEventCreateWithFlags(&ctx->ev_aux, cudaEventDisableTiming));
    MBPOL_CUDA_OK(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device));
    MBPOL_CUDA_OK(ctx->d_pos.ensure(sizeof(double) * 3 * (size_t)num_particles));
    MBPOL_CUDA_OK(ctx->d_force.ensure(sizeof(double) * 3 * (size_t)num_particles));
    MBPOL_CUDA_OK(ctx->d_energy.ensure(sizeof(double) * MBPOL_NUM_TERMS));
    MBPOL_CUDA_OK(ctx->d_counters.ensure(sizeof(int) * 16));
    ctx->h_force.resize(3 * (size_t)num_particles);
    upload_polyterm_constants(kOneBodyCoef, &kOneBodyIdx[0][0]);
    MBPOL_CUDA_OK(cudaGetLastError());
    MBPOL_CUDA_OK(poly_tables_upload(device, &ctx->walk));
    MBPOL_CUDA_OK(poly_tc_setup(device, &ctx->tc3));
    MBPOL_CUDA_OK(ctx->kstatus.ensure(sizeof(int)));
    MBPOL_CUDA_OK(cudaMemset(ctx->kstatus.p, 0, sizeof(int)));
    *out = ctx.release();
    return MBPOL_OK;
}

mbpol_status mbpol_context_destroy(mbpol_context* ctx) {
    if (!ctx) return MBPOL_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->st);
    if (ctx->st_e) cudaStreamSynchronize(ctx->st_e);
    if (ctx->st_a) cudaStreamSynchronize(ctx->st_a);
    ctx->elec.reset();
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    if (ctx->ev_pos) cudaEventDestroy(ctx->ev_pos);
    if (ctx->tuner.t0) cudaEventDestroy(ctx->tuner.t0);
    if (ctx->tuner.t1) cudaEventDestroy(ctx->tuner.t1);
    if (ctx->ev_elec) cudaEventDestroy(ctx->ev_elec);
    if (ctx->ev_lists) cudaEventDestroy(ctx->ev_lists);
    if (ctx->ev_aux) cudaEventDestroy(ctx->ev_aux);
    if (ctx->st_e) cudaStreamDestroy(ctx->st_e);
    if (ctx->st_a) cudaStreamDestroy(ctx->st_a);
    cudaStreamDestroy(ctx->st);
    delete ctx;
    return MBPOL_OK;
}

mbpol_status mbpol_add_average3_site(mbpol_context* ctx, int site, int p1, int p2, int p3, double w1, double w2,
                                     double w3) {
    if (!ctx) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null context");
    const int idx[4] = {site, p1, p2, p3};
    for (int k = 0; k < 4; ++k)
        if (idx[k] < 0 || idx[k] >= ctx->N) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "virtual site index out of range");
    ctx->vs_idx.push_back(make_int4(site, p1, p2, p3));
    ctx->vs_w.push_back(w1);
    ctx->vs_w.push_back(w2);
    ctx->vs_w.push_back(w3);
    ctx->vs_dirty = true;
    return MBPOL_OK;
}

mbpol_status mbpol_add_onebody_force(mbpol_context* ctx, int nw, const int* w, int method) {
    if (!ctx) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null context");
    return set_term(ctx, ctx->t1, nw, w, method, 0.0, 0);
}

mbpol_status mbpol_add_twobody_force(mbpol_context* ctx, int nw, const int* w, int method, double cutoff) {
    if (!ctx) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null context");
    if (method != MBPOL_NOCUTOFF && !(cutoff > 0)) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "bad cutoff");
    return set_term(ctx, ctx->t2, nw, w, method, cutoff, 0);
}

mbpol_status mbpol_add_threebody_force(mbpol_context* ctx, int nw, const int* w, int method, double cutoff,
                                       int rule) {
    if (!ctx) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null context");
    if (method != MBPOL_NOCUTOFF && !(cutoff > 0)) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "bad cutoff");
    return set_term(ctx, ctx->t3, nw, w, method, cutoff, rule);
}

mbpol_status mbpol_add_dispersion_force(mbpol_context* ctx, int nw, const int* w, int method, double cutoff,
                                        const double* c6, const double* d6) {
    if (!ctx || !c6 || !d6) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null argument");
    if (method != MBPOL_NOCUTOFF && !(cutoff > 0)) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "bad cutoff");
    std::memcpy(ctx->disp_c6, c6, sizeof(ctx->disp_c6));
    std::memcpy(ctx->disp_d6, d6, sizeof(ctx->disp_d6));
    upload_dispersion_tables(c6, d6);
    return set_term(ctx, ctx->tdisp, nw, w, method, cutoff, 0);
}

mbpol_status mbpol_update_parameters(mbpol_context* ctx, unsigned term, int count, const int* waters,
                                     const double* charge, const int* molecule, const int* atom_type,
                                     const double* damping, const double* polarity) {
    if (!ctx) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null context");
    MBPOL_CUDA_OK(cudaSetDevice(ctx->device));
    // nothing of an earlier evaluation may still read the old parameters
    MBPOL_CUDA_OK(cudaStreamSynchronize(ctx->st));
    if (ctx->st_e) MBPOL_CUDA_OK(cudaStreamSynchronize(ctx->st_e));
    if (ctx->st_a) MBPOL_CUDA_OK(cudaStreamSynchronize(ctx->st_a));
    if (term == MBPOL_TERM_ELECTROSTATICS) {
        if (!ctx->elec) return mbpol_fail(MBPOL_ERR_STATE, "no electrostatics force in this context");
        if (count != ctx->N)
            return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "updateParametersInContext: The number of multipoles has changed");
        if (!charge || !molecule || !atom_type || !damping || !polarity)
            return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null argument");
        ctx->forces_valid = false;
        return ctx->elec->update_parameters(charge, molecule, atom_type, damping, polarity);
    }
    WaterTerm* t = term == MBPOL_TERM_ONEBODY ? &ctx->t1 : term == MBPOL_TERM_TWOBODY ? &ctx->t2
                 : term == MBPOL_TERM_THREEBODY ? &ctx->t3 : term == MBPOL_TERM_DISPERSION ? &ctx->tdisp : nullptr;
    if (!t) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "unknown term");
    if (!t->on) return mbpol_fail(MBPOL_ERR_STATE, "the term has no force in this context");
    if (count != (int)t->waters.size())
        return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, term == MBPOL_TERM_ONEBODY
                          ? "updateParametersInContext: The number of one-body molecules has changed"
                          : "updateParametersInContext: The number of particles has changed");
    mbpol_status s = set_term(ctx, *t, count, waters, t->method, t->cutoff, t->rule);
    if (s) return s;
    if (ctx->ncl > 0) ctx->cl_dirty = true;
    ctx->forces_valid = false;
    return MBPOL_OK;
}

mbpol_status mbpol_add_dispersion_ions(mbpol_context* ctx, int num_ions, const int* particles) {
    if (!ctx || num_ions < 0 || (num_ions > 0 && !particles))
        return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "bad ion list");
    if (!ctx->tdisp.on) return mbpol_fail(MBPOL_ERR_STATE, "add the dispersion force first");
    std::vector<int> ions(particles, particles + num_ions);
    for (int p : ions)
        if (p < 0 || p >= ctx->N) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "ion particle index out of range");
    for (const int4& w : ctx->tdisp.waters)
        for (int p : ions)
            if (p == w.x || p == w.y || p == w.z)
                return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "an ion particle is also a water atom");
    MBPOL_CUDA_OK(cudaSetDevice(ctx->device));
    ctx->disp_ions.insert(ctx->disp_ions.end(), ions.begin(), ions.end());
    MBPOL_CUDA_OK(ctx->d_disp_ions.ensure(sizeof(int) * std::max<size_t>(ctx->disp_ions.size(), 1)));
    if (!ctx->disp_ions.empty())
        MBPOL_CUDA_OK(cudaMemcpy(ctx->d_disp_ions.p, ctx->disp_ions.data(), sizeof(int) * ctx->disp_ions.size(),
                                 cudaMemcpyHostToDevice));
    return MBPOL_OK;
}

mbpol_status mbpol_add_electrostatics_force(mbpol_context* ctx, const mbpol_electrostatics_params* p,
                                            const double* charge, const int* molecule, const int* atom_type,
                                            const double* damping, const double* polarity) {
    if (!ctx || !p || !charge || !molecule || !atom_type || !damping || !polarity)
        return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null argument");
    ctx->elec.reset(new ElecEngine());
    return ctx->elec->init(ctx->N, *p, charge, molecule, atom_type, damping, polarity);
}

mbpol_status mbpol_set_positions(mbpol_context* ctx, const double* xyz, const double* box) {
    if (!ctx || !xyz) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null argument");
    MBPOL_CUDA_OK(cudaSetDevice(ctx->device));
    for (size_t i = 0; i < 3 * (size_t)ctx->N; ++i)
        if (!std::isfinite(xyz[i])) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "non-finite position");
    if (box) {
        for (int k = 0; k < 3; ++k) {
            if (!(box[k] > 0) || !std::isfinite(box[k]))
                return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "Box size of zero is invalid.");
            ctx->box.L[k] = box[k];
            ctx->box.inv[k] = 1.0 / box[k];
        }
        ctx->box.periodic = 1;
    } else {
        ctx->box.periodic = 0;
    }
    MBPOL_CUDA_OK(cudaMemcpyAsync(ctx->d_pos.p, xyz, sizeof(double) * 3 * ctx->N, cudaMemcpyHostToDevice, ctx->st));
    ctx->have_pos = true;
    ctx->forces_valid = false;
    return MBPOL_OK;
}

}  // extern "C"

namespace {

// Reads (and clears) the tcgen05 kernel's status word after the stream's
// work; nonzero means one of its bounded waits gave up and the three-body
// results of that evaluation are invalid.
mbpol_status check_kernel_status(mbpol_context* ctx) {
    int h = 0;
    MBPOL_CUDA_OK(cudaMemcpyAsync(&h, ctx->kstatus.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->st));
    MBPOL_CUDA_OK(cudaStreamSynchronize(ctx->st));
    if (!h) return MBPOL_OK;
    MBPOL_CUDA_OK(cudaMemsetAsync(ctx->kstatus.p, 0, sizeof(int), ctx->st));
    return mbpol_fail(MBPOL_ERR_CUDA, "three-body tensor kernel: a bounded wait gave up (site " +
                                          std::to_string(h) + "); results discarded");
}

// Evaluate the requested terms; forces and energies stay on the device
// (d_force, d_energy).  Host synchronisation happens only for list sizes and
// the solver's convergence test.
mbpol_status compute_device_inner(mbpol_context* ctx, unsigned mask);

// One evaluation, with the autotuner's bookkeeping while it measures.
mbpol_status compute_device(mbpol_context* ctx, unsigned mask) {
    Autotuner& T = ctx->tuner;
    const bool tune = T.reps > 0 && !T.done && !T.cands.empty();
    if (tune) {
        ctx->shape = T.cands[T.cand];
        MBPOL_CUDA_OK(cudaEventRecord(T.t0, ctx->st));
    }
    const mbpol_status s = compute_device_inner(ctx, mask);
    if (tune && s == MBPOL_OK) {
        MBPOL_CUDA_OK(cudaEventRecord(T.t1, ctx->st));
        MBPOL_CUDA_OK(cudaEventSynchronize(T.t1));
        float ms = 0.f;
        MBPOL_CUDA_OK(cudaEventElapsedTime(&ms, T.t0, T.t1));
        T.ms[T.cand].push_back(ms);
        if ((int)T.ms[T.cand].size() >= T.reps && ++T.cand == T.cands.size()) {
            size_t best = 0;
            float best_ms = 0.f;
            for (size_t c = 0; c < T.cands.size(); ++c) {
                std::vector<float> v = T.ms[c];
                std::sort(v.begin(), v.end());
                const float med = v[v.size() / 2];
                if (c == 0 || med < best_ms) {
                    best = c;
                    best_ms = med;
                }
            }
            ctx->shape = T.cands[best];
            T.done = true;
        }
    }
    return s;
}

mbpol_status compute_device_inner(mbpol_context* ctx, unsigned mask) {
    if (ctx->vs_dirty) {
        MBPOL_CUDA_OK(ctx->d_vs_idx.ensure(sizeof(int4) * ctx->vs_idx.size()));
        MBPOL_CUDA_OK(ctx->d_vs_w.ensure(sizeof(double) * ctx->vs_w.size()));
        MBPOL_CUDA_OK(cudaMemcpy(ctx->d_vs_idx.p, ctx->vs_idx.data(), sizeof(int4) * ctx->vs_idx.size(), cudaMemcpyHostToDevice));
        MBPOL_CUDA_OK(cudaMemcpy(ctx->d_vs_w.p, ctx->vs_w.data(), sizeof(double) * ctx->vs_w.size(), cudaMemcpyHostToDevice));
        ctx->vs_dirty = false;
    }
    const int nvs = (int)ctx->vs_idx.size();
    launch_place_vsites(ctx->st, nvs, ctx->d_vs_idx.as<int4>(), ctx->d_vs_w.as<double>(), ctx->d_pos.as<double>());
    MBPOL_CUDA_OK(cudaMemsetAsync(ctx->d_force.p, 0, sizeof(double) * 3 * ctx->N, ctx->st));
    MBPOL_CUDA_OK(cudaMemsetAsync(ctx->d_energy.p, 0, sizeof(double) * MBPOL_NUM_TERMS, ctx->st));
    double* e = ctx->d_energy.as<double>();
    mbpol_status s = MBPOL_OK;
    if (ctx->cl_dirty) {
        s = apply_clusters(ctx);
        if (s) return s;
    }
    if (ctx->ncl > 0) {
        for (const WaterTerm* t : {&ctx->t1, &ctx->t2, &ctx->t3, &ctx->tdisp})
            if (t->on && (t->method == MBPOL_CUTOFF_PERIODIC || (t == &ctx->t1 && t->method == MBPOL_ONEBODY_PERIODIC)))
                return mbpol_fail(MBPOL_ERR_STATE, "batched clusters need non-periodic methods");
        if (!ctx->disp_ions.empty()) return mbpol_fail(MBPOL_ERR_STATE, "batched clusters of waters only (no ions)");
        MBPOL_CUDA_OK(cudaMemsetAsync(ctx->d_cl_energy.p, 0, sizeof(double) * MBPOL_NUM_TERMS * (size_t)ctx->ncl,
                                      ctx->st));
    }
    // positions (with M sites) and zeroed outputs are ready here: the
    // electrostatics stream starts from this point, not after the terms below
    MBPOL_CUDA_OK(cudaEventRecord(ctx->ev_pos, ctx->st));
    MBPOL_CUDA_OK(cudaStreamWaitEvent(ctx->st_a, ctx->ev_pos, 0));
    if ((mask & MBPOL_TERM_BIT(MBPOL_TERM_ONEBODY)) && ctx->t1.on) {
        const bool periodic = ctx->t1.method == MBPOL_ONEBODY_PERIODIC && ctx->box.periodic;
        launch_onebody(ctx->st_a, (int)ctx->t1.waters.size(), ctx->t1.d_waters.as<int4>(), ctx->d_pos.as<double>(),
                       term_box(ctx, periodic), ctx->d_force.as<double>(), e + MBPOL_TERM_ONEBODY,
                       term_sink(ctx, ctx->t1, MBPOL_TERM_ONEBODY));
    }
    const bool do2 = (mask & MBPOL_TERM_BIT(MBPOL_TERM_TWOBODY)) && ctx->t2.on;
    const bool do3 = (mask & MBPOL_TERM_BIT(MBPOL_TERM_THREEBODY)) && ctx->t3.on;
    const bool dod = (mask & MBPOL_TERM_BIT(MBPOL_TERM_DISPERSION)) && ctx->tdisp.on;
    ctx->shared_lists = false;
    if (!s) s = build_shared_lists(ctx, mask, &ctx->shared_lists);
    if (!s && do2) s = run_twobody(ctx, e + MBPOL_TERM_TWOBODY, ctx->st, true);
    if (!s && do3) s = run_threebody(ctx, e + MBPOL_TERM_THREEBODY, ctx->st, true);
    if (!s && dod) s = run_dispersion(ctx, e + MBPOL_TERM_DISPERSION, ctx->st, true);
    if (!s) {
        MBPOL_CUDA_OK(cudaEventRecord(ctx->ev_lists, ctx->st));
        MBPOL_CUDA_OK(cudaStreamWaitEvent(ctx->st_a, ctx->ev_lists, 0));
    }
    if (!s && dod) s = run_dispersion(ctx, e + MBPOL_TERM_DISPERSION, ctx->st_a, false);
    // the three-body term first: its tensor kernel holds one block on each of
    // a fixed number of SMs and leaves whole SMs to the electrostatics, whose
    // charges, neighbour list and fixed field then run beside it and reach
    // the solver early; the two-body walk (blocks on every SM, minus the
    // tuned reserve) follows and shares the GPU with the solver iterations
    if (!s && do3) s = run_threebody(ctx, e + MBPOL_TERM_THREEBODY, ctx->st, false);
    if (!s && do2) s = run_twobody(ctx, e + MBPOL_TERM_TWOBODY, ctx->st, false);
    ctx->shared_lists = false;
    MBPOL_CUDA_OK(cudaEventRecord(ctx->ev_aux, ctx->st_a));
    if (!s && (mask & MBPOL_TERM_BIT(MBPOL_TERM_ELECTROSTATICS)) && ctx->elec) {
        // the polynomial kernels are queued on st, the one-body term and
        // the dispersion on st_a; the electrostatics (whose solver loop
        // waits on the host every iteration) run on st_e meanwhile, joined
        // before the M-site projection.  All accumulate forces with atomics.
        MBPOL_CUDA_OK(cudaStreamWaitEvent(ctx->st_e, ctx->ev_pos, 0));
        s = ctx->elec->compute(ctx->st_e, ctx->d_pos.as<double>(), ctx->box, ctx->d_force.as<double>(),
                               e + MBPOL_TERM_ELECTROSTATICS);
        MBPOL_CUDA_OK(cudaEventRecord(ctx->ev_elec, ctx->st_e));
        MBPOL_CUDA_OK(cudaStreamWaitEvent(ctx->st, ctx->ev_elec, 0));
        ctx->counts[2] = ctx->elec->num_site_pairs();
        ctx->counts[3] = ctx->elec->iterations();
        ctx->solver_iterations_total += ctx->elec->iterations();
    }
    MBPOL_CUDA_OK(cudaStreamWaitEvent(ctx->st, ctx->ev_aux, 0));
    if (s) {
        cudaStreamSynchronize(ctx->st);
        cudaStreamSynchronize(ctx->st_e);
        cudaStreamSynchronize(ctx->st_a);
        return s;
    }
    launch_spread_vsites(ctx->st, nvs, ctx->d_vs_idx.as<int4>(), ctx->d_vs_w.as<double>(), ctx->d_force.as<double>());
    MBPOL_CUDA_OK(cudaGetLastError());
    if (ctx->elec && (mask & MBPOL_TERM_BIT(MBPOL_TERM_ELECTROSTATICS)) && !ctx->elec->converged())
        return mbpol_fail(MBPOL_ERR_NOT_CONVERGED, ctx->elec->convergence_message());
    return MBPOL_OK;
}

}  // namespace

extern "C" {

mbpol_status mbpol_compute(mbpol_context* ctx, unsigned mask, double* energies, double* forces) {
    if (!ctx) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null context");
    if (!ctx->have_pos) return mbpol_fail(MBPOL_ERR_STATE, "positions have not been set");
    MBPOL_CUDA_OK(cudaSetDevice(ctx->device));
    ctx->forces_valid = false;
    mbpol_status s = compute_device(ctx, mask);
    if (s && s != MBPOL_ERR_NOT_CONVERGED) return s;
    double h_e[MBPOL_NUM_TERMS];
    MBPOL_CUDA_OK(cudaMemcpyAsync(h_e, ctx->d_energy.p, sizeof(h_e), cudaMemcpyDeviceToHost, ctx->st));
    if (forces)
        MBPOL_CUDA_OK(cudaMemcpyAsync(ctx->h_force.data(), ctx->d_force.p, sizeof(double) * 3 * ctx->N,
                                      cudaMemcpyDeviceToHost, ctx->st));
    MBPOL_CUDA_OK(cudaStreamSynchronize(ctx->st));
    {
        const mbpol_status ks = check_kernel_status(ctx);
        if (ks) return ks;
    }
    if (energies)
        for (int k = 0; k < MBPOL_NUM_TERMS; ++k) energies[k] = h_e[k];
    if (forces)
        for (size_t i = 0; i < 3 * (size_t)ctx->N; ++i) forces[i] += ctx->h_force[i];
    if (s) return s;
    ctx->forces_valid = mask == MBPOL_ALL_TERMS;
    return MBPOL_OK;
}

mbpol_status mbpol_set_masses(mbpol_context* ctx, const double* masses) {
    if (!ctx || !masses) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null argument");
    std::vector<double> im((size_t)ctx->N);
    for (int i = 0; i < ctx->N; ++i) {
        if (!(masses[i] >= 0)) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "negative mass");
        im[(size_t)i] = masses[i] > 0 ? 1.0 / masses[i] : 0.0;
    }
    MBPOL_CUDA_OK(cudaSetDevice(ctx->device));
    MBPOL_CUDA_OK(ctx->d_invm.ensure(sizeof(double) * ctx->N));
    MBPOL_CUDA_OK(cudaMemcpy(ctx->d_invm.p, im.data(), sizeof(double) * ctx->N, cudaMemcpyHostToDevice));
    ctx->have_masses = true;
    return MBPOL_OK;
}

mbpol_status mbpol_set_velocities(mbpol_context* ctx, const double* v) {
    if (!ctx || !v) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null argument");
    MBPOL_CUDA_OK(cudaSetDevice(ctx->device));
    MBPOL_CUDA_OK(ctx->d_vel.ensure(sizeof(double) * 3 * ctx->N));
    MBPOL_CUDA_OK(cudaMemcpy(ctx->d_vel.p, v, sizeof(double) * 3 * ctx->N, cudaMemcpyHostToDevice));
    ctx->have_vel = true;
    return MBPOL_OK;
}

mbpol_status mbpol_md_run(mbpol_context* ctx, int nsteps, double dt, double temperature, double collision_rate,
                          unsigned long long seed, double* gpu_ms, double* energies, long* solver_iterations) {
    if (!ctx || nsteps < 0 || !(dt > 0)) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "bad MD arguments");
    if (!ctx->have_pos || !ctx->have_masses || !ctx->have_vel)
        return mbpol_fail(MBPOL_ERR_STATE, "MD needs positions, masses and velocities");
    MBPOL_CUDA_OK(cudaSetDevice(ctx->device));
    if (!ctx->ev0) {
        MBPOL_CUDA_OK(cudaEventCreate(&ctx->ev0));
        MBPOL_CUDA_OK(cudaEventCreate(&ctx->ev1));
    }
    MBPOL_CUDA_OK(ctx->d_ekin.ensure(sizeof(double)));
    const double kT = 0.00831446261815324 * temperature;  // kJ/mol
    ctx->solver_iterations_total = 0;
    MBPOL_CUDA_OK(cudaEventRecord(ctx->ev0, ctx->st));
    if (!ctx->forces_valid) {
        mbpol_status s = compute_device(ctx, MBPOL_ALL_TERMS);
        if (s) return s;
        ctx->forces_valid = true;
    }
    for (int step = 0; step < nsteps; ++step) {
        launch_kick_drift(ctx->st, ctx->N, ctx->d_invm.as<double>(), ctx->d_vel.as<double>(), ctx->d_pos.as<double>(),
                          ctx->d_force.as<double>(), dt);
        ctx->forces_valid = false;
        mbpol_status s = compute_device(ctx, MBPOL_ALL_TERMS);
        if (s) return s;
        ctx->forces_valid = true;
        MBPOL_CUDA_OK(cudaMemsetAsync(ctx->d_ekin.p, 0, sizeof(double), ctx->st));
        launch_kick(ctx->st, ctx->N, ctx->d_invm.as<double>(), ctx->d_vel.as<double>(), ctx->d_force.as<double>(),
                    dt, kT, collision_rate, seed, ctx->md_step++, ctx->d_ekin.as<double>());
    }
    MBPOL_CUDA_OK(cudaEventRecord(ctx->ev1, ctx->st));
    double h[MBPOL_NUM_TERMS + 1];
    MBPOL_CUDA_OK(cudaMemcpyAsync(h, ctx->d_energy.p, sizeof(double) * MBPOL_NUM_TERMS, cudaMemcpyDeviceToHost, ctx->st));
    MBPOL_CUDA_OK(cudaMemcpyAsync(h + MBPOL_NUM_TERMS, ctx->d_ekin.p, sizeof(double), cudaMemcpyDeviceToHost, ctx->st));
    MBPOL_CUDA_OK(cudaStreamSynchronize(ctx->st));
    {
        const mbpol_status ks = check_kernel_status(ctx);
        if (ks) return ks;
    }
    float ms = 0.f;
    MBPOL_CUDA_OK(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
    if (gpu_ms) *gpu_ms = ms;
    if (energies)
        for (int k = 0; k <= MBPOL_NUM_TERMS; ++k) energies[k] = nsteps > 0 || k < MBPOL_NUM_TERMS ? h[k] : 0.0;
    if (solver_iterations) *solver_iterations = ctx->solver_iterations_total;
    return MBPOL_OK;
}

mbpol_status mbpol_get_state(mbpol_context* ctx, double* positions, double* velocities, double* forces) {
    if (!ctx) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null context");
    MBPOL_CUDA_OK(cudaSetDevice(ctx->device));
    const size_t nb = sizeof(double) * 3 * ctx->N;
    if (positions) MBPOL_CUDA_OK(cudaMemcpyAsync(positions, ctx->d_pos.p, nb, cudaMemcpyDeviceToHost, ctx->st));
    if (velocities && ctx->have_vel) MBPOL_CUDA_OK(cudaMemcpyAsync(velocities, ctx->d_vel.p, nb, cudaMemcpyDeviceToHost, ctx->st));
    if (forces) MBPOL_CUDA_OK(cudaMemcpyAsync(forces, ctx->d_force.p, nb, cudaMemcpyDeviceToHost, ctx->st));
    MBPOL_CUDA_OK(cudaStreamSynchronize(ctx->st));
    return MBPOL_OK;
}

mbpol_status mbpol_get_induced_dipoles(mbpol_context* ctx, double* dipoles, int* iterations, double* epsilon) {
    if (!ctx || !ctx->elec) return mbpol_fail(MBPOL_ERR_STATE, "no electrostatics force");
    return ctx->elec->get_dipoles(ctx->st, dipoles, iterations, epsilon);
}

mbpol_status mbpol_get_electrostatic_potential(mbpol_context* ctx, int num_points, const double* points,
                                               double* potential) {
    if (!ctx || num_points < 0 || (num_points > 0 && (!points || !potential)))
        return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "bad argument");
    if (!ctx->elec) return mbpol_fail(MBPOL_ERR_STATE, "no electrostatics force");
    if (!ctx->have_pos) return mbpol_fail(MBPOL_ERR_STATE, "positions have not been set");
    if (ctx->ncl > 0) return mbpol_fail(MBPOL_ERR_STATE, "the potential is not defined for batched clusters");
    MBPOL_CUDA_OK(cudaSetDevice(ctx->device));
    // the reference's setup: charges and converged induced dipoles at the
    // current positions (MBPolReferenceElectrostaticsForce.cpp:857-892)
    ctx->forces_valid = false;
    mbpol_status s = compute_device(ctx, MBPOL_TERM_BIT(MBPOL_TERM_ELECTROSTATICS));
    if (s) return s;
    return ctx->elec->potential(ctx->st, ctx->d_pos.as<double>(), num_points, points, potential);
}

mbpol_status mbpol_get_system_multipole_moments(mbpol_context* ctx, const double* masses, double* moments) {
    if (!ctx || !masses || !moments) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null argument");
    if (!ctx->elec) return mbpol_fail(MBPOL_ERR_STATE, "no electrostatics force");
    if (!ctx->have_pos) return mbpol_fail(MBPOL_ERR_STATE, "positions have not been set");
    if (ctx->ncl > 0) return mbpol_fail(MBPOL_ERR_STATE, "the moments are not defined for batched clusters");
    MBPOL_CUDA_OK(cudaSetDevice(ctx->device));
    // the reference's setup: charges and converged induced dipoles at the
    // current positions (MBPolReferenceElectrostaticsForce.cpp:936-941)
    ctx->forces_valid = false;
    mbpol_status s = compute_device(ctx, MBPOL_TERM_BIT(MBPOL_TERM_ELECTROSTATICS));
    if (s) return s;
    return ctx->elec->moments(ctx->st, ctx->d_pos.as<double>(), masses, moments);
}

mbpol_status mbpol_get_counts(mbpol_context* ctx, long* c) {
    if (!ctx || !c) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null argument");
    for (int k = 0; k < 4; ++k) c[k] = ctx->counts[k];
    return MBPOL_OK;
}

const char* mbpol_status_string(mbpol_status s) {
    switch (s) {
        case MBPOL_OK: return "ok";
        case MBPOL_ERR_INVALID_ARGUMENT: return "invalid argument";
        case MBPOL_ERR_CUDA: return "CUDA error";
        case MBPOL_ERR_NOT_CONVERGED: return "induced dipoles did not converge";
        case MBPOL_ERR_BOX_TOO_SMALL: return "periodic box smaller than twice the cutoff";
        case MBPOL_ERR_CAPACITY: return "neighbour capacity exceeded";
        case MBPOL_ERR_STATE: return "invalid call order";
        case MBPOL_ERR_NO_DEVICE: return "no CUDA device";
        default: return "unknown status";
    }
}

const char* mbpol_last_error(void) { return g_last_error.c_str(); }

unsigned long long mbpol_launch_count(void) { return g_launches; }

mbpol_status mbpol_profile_enable(int on) {
    g_prof.on = on != 0;
    for (auto& r : g_prof.rec) r.clear();
    g_prof.used = 0;
    return MBPOL_OK;
}

mbpol_status mbpol_profile_read(int kernel, double* total_ms, long* launches) {
    if (kernel < 0 || kernel >= K_NUM) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "bad kernel id");
    double t = 0.0;
    for (auto& pr : g_prof.rec[kernel]) {
        MBPOL_CUDA_OK(cudaEventSynchronize(g_prof.pool[pr.second]));
        float ms = 0.f;
        MBPOL_CUDA_OK(cudaEventElapsedTime(&ms, g_prof.pool[pr.first], g_prof.pool[pr.second]));
        t += ms;
    }
    if (total_ms) *total_ms = t;
    if (launches) *launches = (long)g_prof.rec[kernel].size();
    return MBPOL_OK;
}


// ---- learned initial guess for the induced dipoles (no reference counterpart)
static mbpol_status need_elec(mbpol_context* ctx) {
    if (!ctx) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null context");
    if (!ctx->elec) return mbpol_fail(MBPOL_ERR_STATE, "the context has no electrostatics force");
    return MBPOL_OK;
}

mbpol_status mbpol_guess_select_network(mbpol_context* ctx, int which) {
    mbpol_status s = need_elec(ctx);
    return s ? s : ctx->elec->guess_select(which);
}

mbpol_status mbpol_guess_collect(mbpol_context* ctx) {
    mbpol_status s = need_elec(ctx);
    return s ? s : ctx->elec->guess_collect(ctx->st);
}

mbpol_status mbpol_guess_num_samples(mbpol_context* ctx, long* n) {
    mbpol_status s = need_elec(ctx);
    if (s) return s;
    if (!n) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null argument");
    *n = ctx->elec->guess_num_samples();
    return MBPOL_OK;
}

mbpol_status mbpol_guess_train(mbpol_context* ctx, int steps, int batch, double learning_rate,
                               unsigned long long seed, double* final_loss) {
    mbpol_status s = need_elec(ctx);
    return s ? s : ctx->elec->guess_train(ctx->st, steps, batch, learning_rate, seed, final_loss);
}

mbpol_status mbpol_guess_get_params(mbpol_context* ctx, float* block) {
    mbpol_status s = need_elec(ctx);
    return s ? s : ctx->elec->guess_get_params(block);
}

mbpol_status mbpol_guess_set_params(mbpol_context* ctx, const float* block) {
    mbpol_status s = need_elec(ctx);
    return s ? s : ctx->elec->guess_set_params(block);
}

mbpol_status mbpol_guess_descriptors(mbpol_context* ctx, float* out) {
    mbpol_status s = need_elec(ctx);
    if (s) return s;
    if (!out) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null argument");
    return ctx->elec->guess_descriptors(ctx->st, out);
}

mbpol_status mbpol_guess_loss_grad(mbpol_context* ctx, const float* X, const float* T, int n, double* loss,
                                   float* grad, float* Y) {
    mbpol_status s = need_elec(ctx);
    return s ? s : ctx->elec->guess_loss_grad(ctx->st, X, T, n, loss, grad, Y);
}

mbpol_status mbpol_guess_fit_predictor(mbpol_context* ctx, const double* history, const double* field,
                                       const double* field_now, int n3, double* coef, double* prediction) {
    mbpol_status s = need_elec(ctx);
    return s ? s : ctx->elec->guess_fit_predictor(ctx->st, history, field, field_now, n3, coef, prediction);
}

// ---- batched independent clusters (no reference counterpart as one call)
mbpol_status mbpol_set_threebody_evaluator(mbpol_context* ctx, int kind) {
    if (!ctx) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null context");
    if (kind != MBPOL_POLY3B_TENSOR && kind != MBPOL_POLY3B_WALK && kind != MBPOL_POLY3B_AUTO &&
        kind != MBPOL_POLY3B_TENSOR_SYNC)
        return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "unknown three-body evaluator");
    ctx->poly3b_kind = kind;
    return MBPOL_OK;
}

mbpol_status mbpol_set_autotune(mbpol_context* ctx, int evaluations_per_shape) {
    if (!ctx || evaluations_per_shape < 0) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "bad autotune arguments");
    Autotuner& T = ctx->tuner;
    T.reps = evaluations_per_shape;
    T.done = false;
    T.cand = 0;
    T.cands.clear();
    T.ms.clear();
    if (T.reps > 0) {
        for (int tc : {0, 26, 52, 76})
            for (int walk : {0, 48, 96}) {
                LaunchShape sh;
                sh.tc_reserve = tc;
                sh.walk_reserve = walk;
                T.cands.push_back(sh);
            }
        T.ms.resize(T.cands.size());
    }
    return MBPOL_OK;
}

mbpol_status mbpol_set_launch_shape(mbpol_context* ctx, int tc_reserve_sms, int walk_reserve_blocks) {
    if (!ctx) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null context");
    if (tc_reserve_sms >= ctx->num_sms || walk_reserve_blocks >= 3 * ctx->num_sms)
        return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "reserve larger than the device");
    ctx->tuner.reps = 0;
    ctx->tuner.done = false;
    ctx->shape.tc_reserve = tc_reserve_sms;
    ctx->shape.walk_reserve = walk_reserve_blocks;
    return MBPOL_OK;
}

mbpol_status mbpol_get_launch_shape(mbpol_context* ctx, int* tc_reserve_sms, int* walk_reserve_blocks, int* tuned) {
    if (!ctx) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null context");
    if (tc_reserve_sms) *tc_reserve_sms = ctx->shape.tc_reserve < 0 ? tc5_default_reserve() : ctx->shape.tc_reserve;
    if (walk_reserve_blocks)
        *walk_reserve_blocks = ctx->shape.walk_reserve < 0 ? walk_default_reserve() : ctx->shape.walk_reserve;
    if (tuned) *tuned = ctx->tuner.done ? 1 : 0;
    return MBPOL_OK;
}

mbpol_status mbpol_probe_thole_inverse_rs(double r_nm, double damp_i, double damp_j, double thole, double rr[4]) {
    if (!rr || !(r_nm > 0) || damp_i < 0 || damp_j < 0 || thole < 0)
        return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "bad probe arguments");
    return probe_thole(r_nm, damp_i, damp_j, thole, rr);
}

mbpol_status mbpol_probe_water_charges(const double positions_nm[9], double charges[4], double derivatives[27]) {
    if (!positions_nm || !charges || !derivatives) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null probe buffer");
    double out[31];
    const mbpol_status s = probe_water_charges(positions_nm, out);
    if (s) return s;
    for (int k = 0; k < 4; ++k) charges[k] = out[k];
    for (int k = 0; k < 27; ++k) derivatives[k] = out[4 + k];
    return MBPOL_OK;
}

mbpol_status mbpol_set_clusters(mbpol_context* ctx, const int* cluster_of_particle, int num_clusters) {
    if (!ctx) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null context");
    if (num_clusters < 0 || (num_clusters > 0 && !cluster_of_particle))
        return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "bad cluster arguments");
    if (num_clusters > 0)
        for (int i = 0; i < ctx->N; ++i)
            if (cluster_of_particle[i] < 0 || cluster_of_particle[i] >= num_clusters)
                return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "cluster index out of range");
    ctx->ncl = num_clusters;
    ctx->cl_of_particle.assign(cluster_of_particle, cluster_of_particle + (num_clusters > 0 ? ctx->N : 0));
    ctx->cl_dirty = true;
    ctx->forces_valid = false;
    return MBPOL_OK;
}

mbpol_status mbpol_get_cluster_results(mbpol_context* ctx, double* energies, int* iterations) {
    if (!ctx) return mbpol_fail(MBPOL_ERR_INVALID_ARGUMENT, "null context");
    if (ctx->ncl <= 0 || ctx->cl_dirty) return mbpol_fail(MBPOL_ERR_STATE, "no batched-cluster evaluation yet");
    if (energies) {
        MBPOL_CUDA_OK(cudaMemcpy(energies, ctx->d_cl_energy.p, sizeof(double) * MBPOL_NUM_TERMS * (size_t)ctx->ncl,
                                 cudaMemcpyDeviceToHost));
    }
    if (iterations) {
        const std::vector<int>* it = ctx->elec ? &ctx->elec->cluster_iterations() : nullptr;
        for (int c = 0; c < ctx->ncl; ++c) iterations[c] = it && (int)it->size() == ctx->ncl ? (*it)[c] : 0;
    }
    return MBPOL_OK;
}

}  // extern "C"
