// engine.cu - host driver of the GB300 Louvain engine and the Louvain entry
// points of the C ABI (include/gala.h).
//
// A gala_context owns one CUDA stream and all device workspace for graphs up
// to its capacity; nothing is allocated while a run is in progress.  Per
// phase-1 iteration the host reads back one small counter block (sum of In,
// sum of Tot^2, error bits) to decide convergence, which is the only
// device->host traffic of the iteration.
#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <thread>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "internal.h"

using namespace gala;

namespace {
struct BatchRun;
}

struct gala_context {
    int device = 0;
    cudaStream_t stream = nullptr;      // stream all work is ordered on
    cudaStream_t own_stream = nullptr;  // the context's own stream
    int32_t n_cap = 0;
    int64_t e_cap = 0;
    int64_t *offs[2] = {nullptr, nullptr};
    int32_t *nbr[2] = {nullptr, nullptr};
    int32_t *w[2] = {nullptr, nullptr};
    int32_t *orig = nullptr;
    Phase1Buffers p1{};
    ContractBuffers cb{};
    RefineBuffers ref{};  // allocated on the first run with gala_options.refine
    DevStats *d_stats = nullptr;
    DevStats *h_stats = nullptr;
    int32_t *scratch = nullptr;
    long long scratch_ints = 0;
    // per table chunk of the hub bin: best candidate of the chunk
    long long *hub_px = nullptr;
    int32_t *hub_pc = nullptr, *hub_pw = nullptr, *hub_pt = nullptr, *hub_pwc = nullptr;
    double *hub_pdq = nullptr;
    int32_t *hub_pfc = nullptr;
    cudaEvent_t ev[8] = {};
    // slots of the largest hub table (gala_context_set_hub_table_cap; 0 = by degree)
    long long hub_table_cap = 0;
    // weight update of the sweeps (gala_context_set_update_mode): 0 = the
    // incremental update when the movers' rows are few, 1 = always the full
    // update, 2 = incremental whenever allowed
    int update_mode = 0;
    // symmetry of the current run's graph: -1 = not known yet, 0 / 1
    int sym_state = -1;
    // gala_louvain of a pinned unweighted graph copies the neighbours in
    // row-range chunks on copy_stream while level 0 starts on the rows that
    // arrived (gala_context_set_copy_overlap)
    int copy_overlap = 8;            // row chunks (0: one copy up front)
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t copy_ev[2] = {};     // start and end of a chunked copy (timing)
    cudaEvent_t offs_ev = nullptr;   // the offsets have been copied
    PendingRows pend_store;
    PendingRows *pending = nullptr;  // set by gala_louvain, consumed by the first phase 1
    int32_t *d_chunk = nullptr;      // vstart[kMax + 1], lo[(kMax + 1) x 8], cnt[kMax x 8]
    int32_t *h_chunk = nullptr;      // page-locked copy of vstart and lo
    DevStats *d_stats2 = nullptr;    // level-init sums of a level whose rows were still in flight
    DevStats *h_stats2 = nullptr;
    // per-graph state of gala_louvain_batch, kept between calls (reallocated
    // only for a larger batch)
    BatchRun *batch = nullptr;
    // the degree bins of one sweep are independent: they run concurrently on
    // auxiliary streams, forked from and joined back into `stream`
    static constexpr int kAux = 4;
    cudaStream_t aux[kAux] = {};
    cudaEvent_t fork_ev = nullptr;
    cudaEvent_t join_ev[kAux] = {};
    std::vector<void *> allocs;
};

namespace {

// Q from exact integer sums (the same expression as the oracle's
// orc_q_from_sums); the host is compiled with -ffp-contract=off.
// The sum of Tot^2 is (hi, lo): 128 bits for fixed-point weights, hi = 0
// otherwise; hi * 2^64 + lo is the oracle's orc_q_from_sums128 expression.
double q_from_sums(unsigned long long sum_in, unsigned long long sum_tot2, long long m2,
                   unsigned long long sum_tot2_hi = 0)
{
    double c = 1.0 / (double)m2;
    double t2 = (double)sum_tot2_hi * 18446744073709551616.0 + (double)sum_tot2;
    return (double)(long long)sum_in * c - t2 * c * c;
}

template <typename T>
bool dalloc(gala_context *ctx, T **p, size_t count)
{
    if (count == 0) count = 1;
    void *q = nullptr;
    if (cudaMalloc(&q, count * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    ctx->allocs.push_back(q);
    *p = (T *)q;
    return true;
}

// Float weights -> 64-bit fixed point round(w * 2^shift) (w * 2^shift is exact
// in FP64, so the rounding is the host's llrint).
__global__ void k_fixed_from_f32(const float *__restrict__ in, long long *out, long long E, double scale)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < E; i += (long long)gridDim.x * blockDim.x)
        out[i] = __double2ll_rn((double)in[i] * scale);
}
void fixed_from_f32(const float *in, long long *out, long long E, int shift, cudaStream_t st)
{
    if (E <= 0) return;
    long long grid = (E + 255) / 256;
    if (grid > 4096) grid = 4096;
    k_fixed_from_f32<<<(int)grid, 256, 0, st>>>(in, out, E, ldexp(1.0, shift));
    note_launch(1);
}

// Arrays that hold int32 values, or int64 values for fixed-point weights:
// 8 bytes per element.
bool dalloc8(gala_context *ctx, int32_t **p, size_t count)
{
    long long *q = nullptr;
    if (!dalloc(ctx, &q, count)) return false;
    *p = (int32_t *)q;
    return true;
}

__global__ void k_iota(int32_t *a, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = i;
}

struct Counts8 {
    int c[kNumBins];
};
__global__ void k_set_act_counts(DevStats *st, int slot, Counts8 c, int nv, unsigned long long ne)
{
    for (int i = 0; i < kNumBins; ++i) st->act_count[slot][i] = c.c[i];
    st->act_vertices[slot] = nv;
    st->act_edges[slot] = ne;
}

gala_status check(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return GALA_OK;
    return cuda_fail(e, what);
}

// Waits for the stream; a kernel launch that failed since the last check (an
// invalid configuration or missing resources, which the synchronize alone
// would not report) fails the call too.
gala_status sync_check(cudaStream_t st, const char *what)
{
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) return cuda_fail(le, what);
    return check(cudaStreamSynchronize(st), what);
}

float ev_ms(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    return ms;
}

// Fork the auxiliary streams off the context stream and join them back.
void fork(gala_context *ctx)
{
    cudaEventRecord(ctx->fork_ev, ctx->stream);
    for (int i = 0; i < gala_context::kAux; ++i) cudaStreamWaitEvent(ctx->aux[i], ctx->fork_ev, 0);
}
void join(gala_context *ctx)
{
    for (int i = 0; i < gala_context::kAux; ++i) {
        cudaEventRecord(ctx->join_ev[i], ctx->aux[i]);
        cudaStreamWaitEvent(ctx->stream, ctx->join_ev[i], 0);
    }
}
// Heaviest bins first, spread over the auxiliary streams.
constexpr int kBinLaunchOrder[kNumBins] = {7, 6, 5, 4, 3, 2, 1, 0};
cudaStream_t aux_for(gala_context *ctx, int k) { return ctx->aux[k % gala_context::kAux]; }

struct Phase1Out {
    double q = 0;
    int iterations = 0;
    double decide_ms = 0, update_ms = 0, total_ms = 0;
    long long decide_bytes = 0, update_bytes = 0, sweeps = 0;
    long long decisions = 0;      // vertices decided (active, or proposed)
    long long skipped = 0;        // active vertices the network let stay
    long long verify_sweeps = 0;  // full plain sweeps run to judge convergence
    long long movers = 0;         // moves applied (kept or dropped)
    long long nv = 0;             // vertices with edges (the degree-bin order)
    long long active_entries = 0; // row entries decided
    long long incr_sweeps = 0;    // sweeps with the incremental weight update
};

// Move-proposal settings of one run (mode GALA_PROPOSAL_OFF / TRACE / SKIP).
struct PropRun {
    int mode = GALA_PROPOSAL_OFF;
    ProposalView pv{};
    float threshold = 0.5f;
    int sample_shift = 0;
    int level = 0;
    int from = 2;  // SKIP: first sweep of a level that may skip vertices
};

// State of a batch of graphs run as one union graph (gala_louvain_batch).
struct BatchRun {
    int G = 0;
    // device arrays
    int32_t *gid = nullptr, *gid2 = nullptr;  // graph of each vertex (this / next level)
    long long *m2g = nullptr;
    double *cg = nullptr;
    uint8_t *stop = nullptr, *reject = nullptr;
    int32_t *min_tot = nullptr, *ncomm = nullptr;
    unsigned long long *sum_in = nullptr, *sum_tot2 = nullptr, *sum_k = nullptr;
    int64_t *goff = nullptr;  // G+1 vertex offsets of the current level
    // pinned host mirrors
    unsigned long long *h_sum_in = nullptr, *h_sum_tot2 = nullptr, *h_sum_k = nullptr;
    int32_t *h_ncomm = nullptr;
    uint8_t *h_stop = nullptr, *h_reject = nullptr;
    int64_t *h_goff = nullptr;
    // source table of the input graphs, 5G+2 words: device-mapped offsets,
    // neighbour and weight addresses (G each), then the first vertex and the
    // first entry of every graph in the union (G+1 each); pinned host copy
    // and device copy
    int64_t *h_tab = nullptr, *tab = nullptr;
    int cap = 0;       // graphs the per-graph arrays hold
    int n_cap = 0;     // vertices gid / gid2 hold
    // pinned staging of the raw graph arrays (graphs that are not
    // page-locked): the context's vertex and entry capacity
    int64_t *h_offs = nullptr;
    int32_t *h_nbr = nullptr, *h_w = nullptr;
    std::vector<void *> stage;
    // workspace of the one-CTA-per-graph path (allocated on its first use,
    // for the context's vertex and entry capacity)
    BatchCtaArgs cta{};
    int32_t *h_order = nullptr;   // pinned: graphs, largest first
    double *h_q = nullptr;
    int32_t *h_c = nullptr, *h_rounds = nullptr, *h_iters = nullptr;
    int cta_cap = 0;              // graphs the per-graph outputs hold
    std::vector<void *> cta_dev, cta_host;
    // per-graph host state
    std::vector<long long> m2;
    std::vector<double> prev_q;  // accepted Q of the current level
    std::vector<double> prev_mod, cur_mod;  // round rule per graph
    std::vector<char> finished;  // no further round
    std::vector<void *> dev, host;
    GraphSums sums() const { return GraphSums{sum_in, sum_tot2, sum_k, min_tot, ncomm}; }
    int64_t *h_vstart() const { return h_tab + 3LL * cap; }
    int64_t *h_estart() const { return h_tab + 4LL * cap + 1; }
    int64_t *vstart() const { return tab + 3LL * cap; }
    int64_t *estart() const { return tab + 4LL * cap + 1; }
    BatchSrc src() const
    {
        return BatchSrc{(const int64_t *const *)tab, (const int32_t *const *)(tab + cap),
                        (const int32_t *const *)(tab + 2LL * cap), tab + 3LL * cap, tab + 4LL * cap + 1};
    }
    void release()
    {
        for (void *p : dev) cudaFree(p);
        for (void *p : host) cudaFreeHost(p);
        dev.clear();
        host.clear();
        cap = n_cap = 0;
    }
    void release_cta()
    {
        for (void *p : cta_dev) cudaFree(p);
        for (void *p : cta_host) cudaFreeHost(p);
        cta_dev.clear();
        cta_host.clear();
        cta = BatchCtaArgs{};
        h_order = nullptr;
        h_q = nullptr;
        h_c = h_rounds = h_iters = nullptr;
        cta_cap = 0;
    }
    void release_stage()
    {
        for (void *p : stage) cudaFreeHost(p);
        stage.clear();
        h_offs = nullptr;
        h_nbr = h_w = nullptr;
    }
};

// Per-vertex and per-edge algorithmic bytes of a decide-and-move sweep:
// offsets (2 x 8 B), own label, K, Self, label write (4 B each); per edge the
// neighbour id, its label and (weighted) the weight.
long long decide_bytes_for(long long nv, long long ne, bool weighted)
{
    return nv * (2 * 8 + 4 * 4) + ne * (8 + (weighted ? 4 : 0));
}

// One phase-1 run on level graph g (louvain_main_process).  The accepted
// partition is left in ctx->p1.comm.
//
// With a proposal in SKIP mode, sweeps after the first decide only the
// vertices the network proposes (hub vertices are always decided).  The
// first proposal sweep that raises Q by less than min_mod is kept (one that
// lowers Q is reverted) and the level continues with plain sweeps; only a
// plain sweep can end the level, with the reference's rule.  So the
// partition a level returns has passed a plain sweep that found no further
// gain of min_mod.
//
// With a batch (bt), every graph of the union has its own m2, min Tot, Q and
// convergence: a graph whose Q did not grow by min_mod gets this iteration's
// moves reverted and stops, the others go on; the level ends when all graphs
// have stopped.
gala_status phase1(gala_context *ctx, const LevelGraph &g, long long &m2, double min_mod, bool verbose,
                   std::vector<double> *trace, Phase1Out *out, int fp64_only = 0, const PropRun *pr = nullptr,
                   BatchRun *bt = nullptr, bool use_graphs = false, const int32_t *init = nullptr)
{
    const int pmode = pr ? pr->mode : GALA_PROPOSAL_OFF;
    cudaStream_t st = ctx->stream;
    Phase1Buffers &b = ctx->p1;
    DevStats *h = ctx->h_stats;
    const bool weighted = g.w != nullptr;
    gala_status s;

    // Level-0 rows still being copied (gala_louvain of a pinned unweighted
    // graph): the level init needs only the offsets, K = Tot = degree, and
    // the first sweep initialises and decides each degree bin's vertices of a
    // row chunk as soon as that chunk has arrived.  Other runs wait for the
    // whole copy first.
    PendingRows *pend = ctx->pending;
    ctx->pending = nullptr;
    if (pend && (bt || pmode != GALA_PROPOSAL_OFF || init || g.w || g.wide || g.ks_ready)) {
        cudaStreamWaitEvent(st, pend->ev[pend->P - 1], 0);
        pend = nullptr;
    }
    int32_t *const d_vstart = ctx->d_chunk;
    int32_t *const d_lo = d_vstart + PendingRows::kMax + 1;
    int32_t *const d_cnt = d_lo + (PendingRows::kMax + 1) * kNumBins;
    const int32_t *const h_lo = ctx->h_chunk + PendingRows::kMax + 1;

    p1_reset_level_stats(b, st);
    p1_level_init(g, b, st);
    if (pend) {
        p1_init_degree(g, b, st);
        ChunkStarts vs{};
        static_assert(sizeof(vs.v) / sizeof(vs.v[0]) == PendingRows::kMax + 1, "chunk starts");
        memcpy(vs.v, pend->vstart, (size_t)(pend->P + 1) * sizeof(int32_t));
        p1_chunk_bounds(b, vs, pend->P, d_lo, d_cnt, st);
        cudaMemcpyAsync(ctx->h_chunk + PendingRows::kMax + 1, d_lo, (size_t)(pend->P + 1) * kNumBins * sizeof(int32_t),
                        cudaMemcpyDeviceToHost, st);
        cudaMemsetAsync(ctx->d_stats2, 0, sizeof(DevStats), st);
    }
    if ((s = check(cudaMemcpyAsync(h, b.stats, sizeof(DevStats), cudaMemcpyDeviceToHost, st), "level init")) ||
        (s = sync_check(st, "level init")))
        return s;
    int bin_start[kNumBinSlots + 1];
    memcpy(bin_start, h->bin_start, sizeof(bin_start));
    const int max_deg = h->max_deg;
    if (!g.ks_ready && !pend) {
        p1_level_init_rows(g, b, bin_start, st);
        if ((s = check(cudaMemcpyAsync(h, b.stats, sizeof(DevStats), cudaMemcpyDeviceToHost, st), "level rows")) ||
            (s = sync_check(st, "level rows")))
            return s;
    }
    if (m2 == 0) {  // first level: total weight m2 = sum of K (louvain.cu:165-167)
        // rows in flight: unweighted, so the sum of K is the entry count (the
        // row kernels' own sum is checked after the first sweep)
        m2 = pend ? (long long)g.E : (long long)h->sum_k;
        if (m2 <= 0) {
            set_error("graph has no edges (total weight 0)");
            return GALA_ERR_INVALID;
        }
        if (!g.wide && m2 > 0x7fffffffLL) {
            set_error("total weight %lld exceeds the int32 range of community totals", m2);
            return GALA_ERR_INVALID;
        }
    }
    if (!pend && (long long)h->sum_k != m2) {
        set_error("level weight %llu differs from total weight %lld", h->sum_k, m2);
        return GALA_ERR_INVALID;
    }
    const double constant = 1 / (double)m2;
    int level_cnt[kNumBins];
    long long nv_all = 0;
    for (int i = 0; i < kNumBins; ++i) {
        level_cnt[i] = bin_start[i + 1] - bin_start[i];
        nv_all += level_cnt[i];
    }
    (void)max_deg;
    // hub vertices (bin 7): per-hub global tables in the long-row pool of the
    // contraction, which is idle during phase 1
    HubPlan hp{};
    hp.H = level_cnt[7];
    if (hp.H > 0) {
        ContractBuffers &cb = ctx->cb;
        hp.hubs = b.order + bin_start[7];
        hp.T = cb.big_T;
        hp.chunks = cb.big_chunks;
        hp.tchunks = cb.big_tchunks;
        hp.toff = cb.big_toff;
        hp.coff = cb.big_coff;
        hp.tcoff = cb.big_tcoff;
        hp.work = cb.big_work;
        hp.twork = cb.big_twork;
        hp.pool = cb.big_pool;
        hp.px = ctx->hub_px;
        hp.pc = ctx->hub_pc;
        hp.pw = ctx->hub_pw;
        hp.pt = ctx->hub_pt;
        hp.pwc = ctx->hub_pwc;
        hp.pdq = ctx->hub_pdq;
        hp.pfc = ctx->hub_pfc;
        hp.t_cap = ctx->hub_table_cap;
        p1_hub_plan_launch(g, b, hp, st);
        if ((s = check(cudaMemcpyAsync(h, b.stats, sizeof(DevStats), cudaMemcpyDeviceToHost, st), "hub plan")) ||
            (s = sync_check(st, "hub plan")))
            return s;
        hp.half = h->total;
        hp.nwork = h->total2;
        hp.ntwork = h->total3;
        const long long vints = g.wide ? 2 : 1;  // int32 per table value
        if ((1 + vints) * hp.half > cb.big_pool_ints || hp.nwork > cb.big_work_cap ||
            hp.ntwork > cb.big_twork_cap) {
            set_error("hub tables need %lld slots / %lld + %lld chunks, pool holds %lld / %lld / %lld", hp.half,
                      hp.nwork, hp.ntwork, cb.big_pool_ints / 2, cb.big_work_cap, cb.big_twork_cap);
            return GALA_ERR_CAPACITY;
        }
        p1_hub_work_launch(hp, st);
    }
    cudaMemsetAsync(b.act_flag, 1, (size_t)g.n, st);
    // incremental weight updates: plain runs of one graph on a symmetric
    // graph (the symmetry hash of the run's first level, summed by its
    // level-init row kernels, is 0)
    const bool incr_level = !bt && pmode == GALA_PROPOSAL_OFF && ctx->update_mode != 1;
    if (incr_level) {
        cudaMemsetAsync(b.moved, 0, (size_t)g.n, st);
        if (ctx->sym_state < 0 && !pend) ctx->sym_state = (!g.ks_ready && h->sym_hash == 0) ? 1 : 0;
    }
    b.features_on = pmode != GALA_PROPOSAL_OFF;
    b.wide = g.wide;
    if (b.features_on) p1_features_init(b, g.n, st);
    const int G = bt ? bt->G : 0;
    if (bt) {
        // per-graph m2 (first level), singleton Q, graphs that take part
        batch_graph_sums(kSumIn | kSumTot2 | kSumK, G, bt->goff, nullptr, b, bt->sums(), st);
        cudaMemcpyAsync(bt->h_sum_in, bt->sum_in, G * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(bt->h_sum_tot2, bt->sum_tot2, G * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(bt->h_sum_k, bt->sum_k, G * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
        if ((s = sync_check(st, "batch level sums"))) return s;
        const bool first = bt->m2.empty();
        if (first) {
            bt->m2.resize(G);
            std::vector<double> c(G);
            for (int i = 0; i < G; ++i) {
                bt->m2[i] = (long long)bt->h_sum_k[i];
                c[i] = bt->m2[i] > 0 ? 1 / (double)bt->m2[i] : 0.0;
            }
            cudaMemcpyAsync(bt->m2g, bt->m2.data(), G * sizeof(long long), cudaMemcpyHostToDevice, st);
            cudaMemcpyAsync(bt->cg, c.data(), G * sizeof(double), cudaMemcpyHostToDevice, st);
            if ((s = sync_check(st, "batch m2"))) return s;
        }
        bt->prev_q.assign(G, 0.0);
        for (int i = 0; i < G; ++i) {
            if (!first && (long long)bt->h_sum_k[i] != bt->m2[i]) {
                set_error("graph %d: level weight %llu differs from total weight %lld", i, bt->h_sum_k[i],
                          bt->m2[i]);
                return GALA_ERR_INVALID;
            }
            bt->h_stop[i] = bt->finished[i] || bt->m2[i] <= 0;
            if (bt->m2[i] > 0) bt->prev_q[i] = q_from_sums(bt->h_sum_in[i], bt->h_sum_tot2[i], bt->m2[i]);
        }
        cudaMemcpyAsync(bt->stop, bt->h_stop, G, cudaMemcpyHostToDevice, st);
    }

    if (init) {
        // a refined level starts from its parent communities: Tot and size
        // follow them, the weight update gives In and the sums, and every
        // vertex starts active
        p1_iter_reset(b, 1, (!g.wide && m2 > 0x7fffffffLL) ? 0x7fffffffLL : m2, st);
        p1_start_partition(b, init, g.n, st);
        p1_tot_reduce(b, g.n, st);
        fork(ctx);
        for (int k = 0; k < kNumBins; ++k) {
            const int bin = kBinLaunchOrder[k];
            if (bin == 7)
                p1_hub_update(g, b, hp, 1, bin_start[bin], constant, m2, aux_for(ctx, k));
            else
                p1_update(g, b, bin, b.order + bin_start[bin], level_cnt[bin], 1, bin_start[bin], constant, m2,
                          aux_for(ctx, k));
        }
        join(ctx);
        if ((s = check(cudaMemcpyAsync(h, b.stats, sizeof(DevStats), cudaMemcpyDeviceToHost, st), "start partition")) ||
            (s = sync_check(st, "start partition")))
            return s;
    }
    // Q of the singleton partition (with rows in flight: after the first
    // sweep, from the sums of the row kernels)
    double q = pend ? 0.0 : q_from_sums(h->sum_in, h->sum_tot2, m2, h->sum_tot2_hi);
    if (!pend) {
        if (trace) trace->push_back(q);
        if (verbose) printf("Iteration:%d Q:%f\n", 0, q);
    }
    double prev_q = q;
    int iteration = 1;

    Counts8 c8;
    for (int i = 0; i < kNumBins; ++i) c8.c[i] = level_cnt[i];
    k_set_act_counts<<<1, 1, 0, st>>>(b.stats, 0, c8, (int)nv_all, (unsigned long long)g.E);
    note_launch(1);
    long long act_nv = nv_all, act_ne = g.E;
    out->nv = nv_all;
    int cur = 0;
    const long long min_tot_init = (!g.wide && m2 > 0x7fffffffLL) ? 0x7fffffffLL : m2;
    unsigned long long skipped0 = h->skipped, skipped_e0 = h->skipped_edges;
    bool verify = false;  // proposals stalled: the rest of the level runs plain sweeps
    // CUDA graphs of the repeated sweeps (plain runs): one per active-list slot
    const bool graphs = use_graphs && pmode == GALA_PROPOSAL_OFF;
    // (and per kind of weight update: with or without the incremental path)
    cudaGraphExec_t gexec[4] = {nullptr, nullptr, nullptr, nullptr};
    long long glaunch[4] = {0, 0, 0, 0};
    struct GraphGuard {
        cudaGraphExec_t *e;
        ~GraphGuard()
        {
            for (int i = 0; i < 4; ++i)
                if (e[i]) cudaGraphExecDestroy(e[i]);
        }
    } gguard{gexec};
    // row entries of the previous sweep's movers (the incremental update is
    // enqueued only after a sweep that moved under a third of them)
    unsigned long long prev_mv_edges = ~0ull;
    cudaEventRecord(ctx->ev[0], st);
    for (;;) {
        const int nxt = cur ^ 1;
        const int32_t *lists = iteration == 1 ? b.order : b.act[cur];
        const int *counts = &b.stats->act_count[cur][0];
        // sweep kind: the first sweep of a level and verification sweeps are plain
        const bool proposal_sweep = pmode == GALA_PROPOSAL_SKIP && iteration >= pr->from && !verify;
        ProposalStep ps{};
        if (pmode != GALA_PROPOSAL_OFF) {
            ps.mode = pmode;
            ps.pv = pr->pv;
            ps.threshold = pr->threshold;
            ps.sample_shift = pr->sample_shift;
            ps.iteration = iteration;
            ps.level = pr->level;
        }
        // incremental weight update of this sweep (its kernels decide on the
        // device whether it runs): from a level's second sweep on, on levels
        // of at least 2^23 entries (below, the full update takes tens of
        // microseconds), after a sweep whose movers held under a third of the
        // entries (otherwise its launches would mostly return at once)
        const bool incr = incr_level && ctx->sym_state == 1 && iteration > 1 &&
                          (ctx->update_mode == 2 ||
                           (g.E >= (1LL << 23) && prev_mv_edges * 3 < (unsigned long long)g.E));
        // the sweep: decide, apply, reductions, update, counters to the host
        auto enqueue = [&](bool capturing) {
            // timing events become event nodes of a captured graph
            auto rec = [&](cudaEvent_t e) {
                if (capturing)
                    cudaEventRecordWithFlags(e, st, cudaEventRecordExternal);
                else
                    cudaEventRecord(e, st);
            };
            p1_iter_reset(b, nxt, min_tot_init, st);
            rec(ctx->ev[2]);
            if ((pmode == GALA_PROPOSAL_TRACE && iteration > 1) || proposal_sweep) {
                p1_proposal_step(g, b, ps, lists, counts, bin_start, level_cnt, st);
                if (proposal_sweep) {
                    lists = b.prop_list;
                    counts = &b.stats->prop_count[0];
                }
            }
            fork(ctx);
            if (pend && iteration == 1) {
                // rows in flight: per chunk and bin, the init rows and the
                // first sweep of the bin's vertices in that chunk; hubs after
                // the last chunk
                const cudaEvent_t last = pend->ev[pend->P - 1];
                for (int c = 0; c < pend->P; ++c)
                    for (int k = 0; k < kNumBins; ++k) {
                        const int bin = kBinLaunchOrder[k];
                        if (bin == 7) continue;
                        const int lo = h_lo[c * kNumBins + bin], cnt = h_lo[(c + 1) * kNumBins + bin] - lo;
                        if (cnt <= 0) continue;
                        cudaStream_t sb = aux_for(ctx, k);
                        cudaStreamWaitEvent(sb, pend->ev[c], 0);
                        const int32_t *lst = b.order + bin_start[bin] + lo;
                        p1_init_rows_range(g, b, bin, lst, cnt, ctx->d_stats2, sb);
                        p1_decide(g, b, bin, lst, d_cnt + c * kNumBins + bin, cnt, constant, m2, fp64_only,
                                  g.distinct, sb);
                    }
                // hubs (few, long rows) once the chunk with the last of them
                // has arrived
                int hub_chunk = -1;
                for (int c = 0; c < pend->P; ++c)
                    if (h_lo[(c + 1) * kNumBins + 7] > h_lo[c * kNumBins + 7]) hub_chunk = c;
                for (int k = 0; k < kNumBins; ++k) {
                    if (kBinLaunchOrder[k] == 7 && hub_chunk >= 0) {
                        cudaStreamWaitEvent(aux_for(ctx, k), pend->ev[hub_chunk], 0);
                        p1_init_rows_range(g, b, 7, b.order + bin_start[7], level_cnt[7], ctx->d_stats2,
                                           aux_for(ctx, k));
                        p1_hub_decide(g, b, hp, constant, m2, fp64_only, aux_for(ctx, k));
                    }
                }
                for (int k = 0; k < kNumBins; ++k) cudaStreamWaitEvent(aux_for(ctx, k), last, 0);
            } else {
                for (int k = 0; k < kNumBins; ++k) {
                    const int bin = kBinLaunchOrder[k];
                    if (bin == 7)
                        p1_hub_decide(g, b, hp, constant, m2, fp64_only, aux_for(ctx, k));
                    else
                        p1_decide(g, b, bin, lists + bin_start[bin], counts + bin, level_cnt[bin], constant, m2,
                                  fp64_only, iteration == 1 && g.distinct && !init, aux_for(ctx, k));
                }
            }
            join(ctx);
            rec(ctx->ev[3]);
            p1_apply_movers(b, +1, g.n, st, iteration, g.offs, incr ? b.moved : nullptr);
            if (pmode == GALA_PROPOSAL_TRACE && iteration > 1) p1_trace_labels(b, ps, st);
            if (bt)
                batch_graph_sums(kMinTot | kSumTot2, G, bt->goff, bt->stop, b, bt->sums(), st);
            else
                p1_tot_reduce(b, g.n, st);
            rec(ctx->ev[4]);
            // the incremental update decides on the device whether it runs
            // (the per-bin updates below then return at once); In is exact
            // from the first sweep's update on
            if (incr) p1_push_update(g, b, bin_start, nxt, constant, m2, 1, ctx->update_mode == 2 ? 1 : 0, st);
            fork(ctx);
            for (int k = 0; k < kNumBins; ++k) {
                const int bin = kBinLaunchOrder[k];
                if (bin == 7)
                    p1_hub_update(g, b, hp, nxt, bin_start[bin], constant, m2, aux_for(ctx, k));
                else
                    p1_update(g, b, bin, b.order + bin_start[bin], level_cnt[bin], nxt, bin_start[bin], constant,
                              m2, aux_for(ctx, k));
            }
            join(ctx);
            if (bt) {
                batch_graph_sums(kSumIn, G, bt->goff, bt->stop, b, bt->sums(), st);
                cudaMemcpyAsync(bt->h_sum_in, bt->sum_in, G * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                st);
                cudaMemcpyAsync(bt->h_sum_tot2, bt->sum_tot2, G * sizeof(unsigned long long),
                                cudaMemcpyDeviceToHost, st);
            }
            rec(ctx->ev[5]);
            cudaMemcpyAsync(h, b.stats, sizeof(DevStats), cudaMemcpyDeviceToHost, st);
            if (pend && iteration == 1)
                cudaMemcpyAsync(ctx->h_stats2, ctx->d_stats2, sizeof(DevStats), cudaMemcpyDeviceToHost, st);
        };
        if (graphs && iteration > 1) {
            // sweeps after the first repeat the same launches with the active
            // lists of slot `cur`: captured once per level and slot, replayed
            const int gi = cur + (incr ? 2 : 0);
            if (!gexec[gi]) {
                const long long l0 = gala_kernel_launch_count();
                cudaGraph_t gr = nullptr;
                if ((s = check(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal), "graph capture")))
                    return s;
                enqueue(true);
                if ((s = check(cudaStreamEndCapture(st, &gr), "graph capture"))) return s;
                const cudaError_t ie = cudaGraphInstantiate(&gexec[gi], gr, 0);
                cudaGraphDestroy(gr);
                if ((s = check(ie, "graph instantiate"))) return s;
                glaunch[gi] = gala_kernel_launch_count() - l0;
                note_launch((int)-glaunch[gi]);  // counted when replayed
            }
            if ((s = check(cudaGraphLaunch(gexec[gi], st), "graph launch"))) return s;
            note_launch((int)glaunch[gi]);
        } else {
            enqueue(false);
        }
        if ((s = sync_check(st, "iteration"))) return s;
        if (h->err) {
            set_error("phase 1: device error bits %d", h->err);
            return GALA_ERR_OVERFLOW;
        }
        if (pend && iteration == 1) {  // the level init's sums, from the row kernels of the first sweep
            const DevStats *h2 = ctx->h_stats2;
            if ((long long)h2->sum_k != m2) {
                set_error("level weight %llu differs from total weight %lld", h2->sum_k, m2);
                return GALA_ERR_INVALID;
            }
            prev_q = q_from_sums(h2->sum_in, h2->sum_tot2, m2, h2->sum_tot2_hi);
            if (trace) trace->push_back(prev_q);
            if (verbose) printf("Iteration:%d Q:%f\n", 0, prev_q);
            if (incr_level && ctx->sym_state < 0) ctx->sym_state = h2->sym_hash == 0 ? 1 : 0;
        }
        long long dec_nv = act_nv, dec_ne = act_ne;
        if (proposal_sweep) {
            const long long sk = (long long)(h->skipped - skipped0), ske = (long long)(h->skipped_edges - skipped_e0);
            dec_nv -= sk;
            dec_ne -= ske;
            out->skipped += sk;
        }
        skipped0 = h->skipped;
        skipped_e0 = h->skipped_edges;
        out->decisions += dec_nv;
        out->movers += h->n_movers;
        out->active_entries += dec_ne;
        out->decide_ms += ev_ms(ctx->ev[2], ctx->ev[3]);
        out->update_ms += ev_ms(ctx->ev[4], ctx->ev[5]);
        out->decide_bytes += decide_bytes_for(dec_nv, dec_ne, weighted);
        prev_mv_edges = h->mv_edges;
        if (h->push_mode) {  // the movers' rows, then one pass over the vertices
            out->incr_sweeps += 1;
            out->update_bytes += h->push_total * (8 + (weighted ? 4 : 0)) + nv_all * (4 * 4 + 4 + 4 + 1 + 2 * 8);
        } else {
            out->update_bytes += nv_all * (2 * 8 + 4 * 4) + g.E * (8 + (weighted ? 4 : 0));
        }
        out->sweeps += 1;
        if (verify) out->verify_sweeps += 1;
        act_nv = h->act_vertices[nxt];
        act_ne = (long long)h->act_edges[nxt];
        if (bt) {
            // per-graph convergence (louvain_main_process.cu:1004-1007 for
            // every graph): a graph whose Q did not grow by min_mod drops
            // this iteration's moves and stops
            bool running = false, any_reject = false;
            for (int i = 0; i < G; ++i) {
                bt->h_reject[i] = 0;
                if (bt->h_stop[i]) continue;
                const double qg = q_from_sums(bt->h_sum_in[i], bt->h_sum_tot2[i], bt->m2[i]);
                if (qg - bt->prev_q[i] < min_mod) {
                    bt->h_reject[i] = 1;
                    bt->h_stop[i] = 1;
                    any_reject = true;
                } else {
                    bt->prev_q[i] = qg;
                    running = true;
                }
            }
            if (any_reject) {
                cudaMemcpyAsync(bt->reject, bt->h_reject, G, cudaMemcpyHostToDevice, st);
                cudaMemcpyAsync(bt->stop, bt->h_stop, G, cudaMemcpyHostToDevice, st);
                batch_revert(b, bt->gid, bt->reject, g.n, st);
                // the host arrays must stay unchanged until the copies ran
                if ((s = sync_check(st, "batch revert"))) return s;
            }
            if (!running) break;
            cur = nxt;
            iteration++;
            continue;
        }
        q = q_from_sums(h->sum_in, h->sum_tot2, m2, h->sum_tot2_hi);
        if (trace) trace->push_back(q);
        if (verbose) printf("Iteration:%d Q:%f\n", iteration, q);
        // convergence (louvain_main_process.cu:1004-1007): the partition of
        // this iteration is dropped when Q did not grow by min_mod
        if (q - prev_q < min_mod && proposal_sweep && q > prev_q) {
            // a proposal sweep that still raised Q: keep it and continue with
            // plain sweeps, which judge convergence
            verify = true;
            prev_q = q;
            cur = nxt;
            iteration++;
            continue;
        }
        if (q - prev_q < min_mod) {
            p1_apply_movers(b, -1, g.n, st);
            if (!proposal_sweep) break;
            // a proposal sweep that lowered Q: restore the partition, rebuild
            // In, the active set and the sums into slot nxt, then judge the
            // restored partition with a plain sweep
            p1_iter_reset(b, nxt, min_tot_init, st);
            p1_tot_reduce(b, g.n, st);
            fork(ctx);
            for (int k = 0; k < kNumBins; ++k) {
                const int bin = kBinLaunchOrder[k];
                if (bin == 7)
                    p1_hub_update(g, b, hp, nxt, bin_start[bin], constant, m2, aux_for(ctx, k));
                else
                    p1_update(g, b, bin, b.order + bin_start[bin], level_cnt[bin], nxt, bin_start[bin], constant,
                              m2, aux_for(ctx, k));
            }
            join(ctx);
            if ((s = check(cudaMemcpyAsync(h, b.stats, sizeof(DevStats), cudaMemcpyDeviceToHost, st), "restore")) ||
                (s = sync_check(st, "restore")))
                return s;
            act_nv = h->act_vertices[nxt];
            act_ne = (long long)h->act_edges[nxt];
            verify = true;
            cur = nxt;
            iteration++;
            continue;
        }
        prev_q = q;
        cur = nxt;
        iteration++;
    }
    cudaEventRecord(ctx->ev[1], st);
    if ((s = sync_check(st, "phase 1 end"))) return s;
    out->total_ms = ev_ms(ctx->ev[0], ctx->ev[1]);
    out->q = prev_q;
    out->iterations = iteration;
    if (verbose) {
        printf("time without data init = %fms\n", out->total_ms);
        printf("decideandmove time = %fms weight updating time = %fms remaining time = %fms\n", out->decide_ms,
               out->update_ms, out->total_ms - out->decide_ms - out->update_ms);
    }
    return GALA_OK;
}

void bind_contract_buffers(gala_context *ctx)
{
    ContractBuffers &cb = ctx->cb;
    cb.stats = ctx->d_stats;
    cb.scan_partial = ctx->p1.scan_partial;
    cb.big_bitmap = ctx->scratch;
    cb.big_bitmap_words = ctx->scratch_ints;
    static_assert(ContractBuffers::kAux == gala_context::kAux, "auxiliary streams");
    for (int i = 0; i < gala_context::kAux; ++i) {
        cb.aux[i] = ctx->aux[i];
        cb.join_ev[i] = ctx->join_ev[i];
    }
    cb.fork_ev = ctx->fork_ev;
}

struct RunOut {
    std::vector<double> trace;
};

// Checkpoint of the level graph reached after `round` rounds: the graph in
// the .bin layout (inclusive offsets, int32 weights) and the community of
// every input vertex in it.
gala_status write_level(gala_context *ctx, const LevelGraph &g, int32_t n0, const char *dir, int round)
{
    cudaStream_t st = ctx->stream;
    std::vector<int64_t> offs((size_t)g.n + 1);
    std::vector<int32_t> nbr((size_t)g.E), w((size_t)g.E), lab((size_t)n0);
    gala_status s;
    cudaMemcpyAsync(offs.data(), g.offs, offs.size() * sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (g.E) {
        cudaMemcpyAsync(nbr.data(), g.nbr, nbr.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
        cudaMemcpyAsync(w.data(), g.w, w.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    }
    cudaMemcpyAsync(lab.data(), ctx->orig, lab.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if ((s = sync_check(st, "level checkpoint"))) return s;
    char path[4096];
    snprintf(path, sizeof(path), "%s/level_%d.bin", dir, round);
    gala_graph *h = nullptr;
    if ((s = gala_graph_from_csr(g.n, offs.data() + 1, nbr.data(), w.data(), &h))) return s;
    s = gala_graph_store_bin(h, path);
    gala_graph_destroy(h);
    if (s) return s;
    snprintf(path, sizeof(path), "%s/labels_%d.bin", dir, round);
    FILE *f = fopen(path, "wb");
    const bool ok = f && fwrite(lab.data(), sizeof(int32_t), lab.size(), f) == lab.size();
    if (f) fclose(f);
    if (!ok) {
        set_error("cannot write %s", path);
        return GALA_ERR_IO;
    }
    return GALA_OK;
}

// Multi-round loop of louvain.cu:193-226 on a device graph.  Level 0 reads
// the caller's arrays; later levels live in the context's ping-pong buffers.
// ctx->orig receives the final community of every level-0 vertex.
//
// With a batch (bt), each graph follows the round rule on its own Q; the loop
// ends when every graph has finished.  bt->h_goff then holds the community
// id range of every graph in ctx->orig's numbering and bt->cur_mod the
// final modularity of every graph.
gala_status run_levels(gala_context *ctx, int32_t n0, int64_t E0, const int64_t *offs0, const int32_t *nbr0,
                       const void *w0, const gala_options *opt, gala_result *res, BatchRun *bt = nullptr,
                       bool wide = false, bool distinct0 = false)
{
    cudaStream_t st = ctx->stream;
    gala_status s;
    const bool verbose = opt && opt->verbose;
    const double min_mod = opt ? opt->min_modularity : 1e-6;
    const int max_levels = opt ? opt->max_levels : 0;
    if (n0 > ctx->n_cap || E0 > ctx->e_cap) {
        set_error("graph (%d vertices, %lld entries) exceeds context capacity (%d, %lld)", n0, (long long)E0,
                  ctx->n_cap, (long long)ctx->e_cap);
        return GALA_ERR_CAPACITY;
    }
    ctx->sym_state = -1;  // checked with the first level
    // degree-bin tuning
    {
        BinLimits lim;
        if (opt) {
            if (opt->bin_max[0] > 0) lim.m4 = opt->bin_max[0];
            if (opt->bin_max[1] > 0) lim.m5 = opt->bin_max[1];
            if (opt->bin_max[2] > 0) lim.m6 = opt->bin_max[2];
        }
        if (lim.m4 < 32 || lim.m4 > kMaxWarpDeg || lim.m5 < lim.m4 || lim.m5 > kMaxCta5Deg || lim.m6 < lim.m5 ||
            lim.m6 > kMaxCta6Deg) {
            set_error("bin limits %d / %d / %d outside 32 <= b4 <= 256, b4 <= b5 <= 2048, b5 <= b6 <= 8192", lim.m4,
                      lim.m5, lim.m6);
            return GALA_ERR_INVALID;
        }
        const int b5 = opt && opt->bin5_block ? opt->bin5_block : 256;
        if (b5 != 256 && b5 != 512) {
            set_error("bin5_block must be 256 or 512");
            return GALA_ERR_INVALID;
        }
        ctx->p1.lim = lim;
        ctx->p1.b5_block = b5;
    }
    PropRun pr;
    if (opt && opt->proposal_mode != GALA_PROPOSAL_OFF) {
        if (opt->proposal_mode != GALA_PROPOSAL_TRACE && opt->proposal_mode != GALA_PROPOSAL_SKIP) {
            set_error("unknown proposal mode %d", opt->proposal_mode);
            return GALA_ERR_INVALID;
        }
        if (!opt->proposal) {
            set_error("proposal mode %d needs a proposal network (options.proposal)", opt->proposal_mode);
            return GALA_ERR_INVALID;
        }
        pr.mode = opt->proposal_mode;
        pr.pv = proposal_view(opt->proposal);
        pr.threshold = opt->proposal_threshold;
        pr.sample_shift = opt->trace_sample_shift;
        if (opt->proposal_from < 0) {
            set_error("proposal_from must be >= 0");
            return GALA_ERR_INVALID;
        }
        pr.from = opt->proposal_from > 2 ? opt->proposal_from : 2;
        if (pr.mode == GALA_PROPOSAL_TRACE && pr.pv.cap <= 0) {
            set_error("trace mode needs a proposal with sample capacity");
            return GALA_ERR_INVALID;
        }
    }
    bind_contract_buffers(ctx);
    long long m2 = 0;  // set by the first phase-1 run
    cudaEvent_t t0 = ctx->ev[6], t1 = ctx->ev[7];
    cudaEventRecord(t0, st);
    k_iota<<<std::min(4096, (n0 + 255) / 256), 256, 0, st>>>(ctx->orig, n0);
    cudaMemsetAsync(&ctx->d_stats->fp64_decisions, 0, sizeof(unsigned long long), st);
    note_launch(1);

    const char *level_dir = opt ? opt->level_dir : nullptr;
    if (level_dir && (wide || bt)) {
        set_error("level checkpoints are not available for batches or float-weight graphs");
        return GALA_ERR_INVALID;
    }
    if (wide && pr.mode != GALA_PROPOSAL_OFF) {
        set_error("proposal modes are not available for float-weight graphs");
        return GALA_ERR_INVALID;
    }
    const bool refine = opt && opt->refine == 1;
    if (refine && (bt || pr.mode != GALA_PROPOSAL_OFF || level_dir)) {
        set_error("refinement is available for single graphs without proposals or checkpoints");
        return GALA_ERR_INVALID;
    }
    if (refine && !ctx->ref.R) {
        RefineBuffers &rb = ctx->ref;
        const size_t nc = (size_t)ctx->n_cap + 1;
        long long *wC = nullptr, *ext = nullptr, *Kr = nullptr;  // 8 bytes a vertex: either weight width
        if (!(dalloc(ctx, &rb.R, nc) && dalloc(ctx, &rb.target, nc) && dalloc(ctx, &rb.marks, nc) &&
              dalloc(ctx, &rb.sz, nc) && dalloc(ctx, &wC, nc) && dalloc(ctx, &ext, nc) && dalloc(ctx, &Kr, nc) &&
              dalloc(ctx, &rb.pmin, nc) && dalloc(ctx, &rb.init, nc) && dalloc(ctx, &rb.list, nc) &&
              dalloc(ctx, &rb.list2, nc) && dalloc(ctx, &rb.moved, 4))) {
            rb = RefineBuffers{};
            set_error("refinement: out of device memory");
            return GALA_ERR_CAPACITY;
        }
        rb.wC = wC;
        rb.ext = ext;
        rb.Kr = Kr;
    }
    bool have_init = false;  // this round starts from the previous round's communities
    LevelGraph g{n0, E0, offs0, nbr0, w0, wide, distinct0 || (opt && opt->distinct_rows == 1)};
    int buf = 0;
    double prev_mod = -1, cur_mod = -1;
    int round = 0;
    res->num_levels = 0;
    res->total_iterations = 0;
    res->iter_count = 0;
    std::vector<double> trace;
    double contract_ms = 0, p1_ms = 0, dec_ms = 0, upd_ms = 0;
    long long dec_bytes = 0, upd_bytes = 0, sweeps = 0;
    long long decisions = 0, skipped = 0, verify_sweeps = 0, incr_sweeps = 0;
    int C = n0;
    for (;;) {
        if (verbose) printf("===============round:%d===============\n", round);
        Phase1Out po;
        pr.level = round;
        const bool started_refined = have_init;
        if ((s = phase1(ctx, g, m2, min_mod, verbose, &trace, &po, opt ? opt->fp64_gains : 0, &pr, bt,
                        opt && opt->use_graphs, have_init ? ctx->ref.init : nullptr)))
            return s;
        if (bt)  // communities per graph, for the graphs' id ranges at the next level
            batch_graph_sums(kCountComm, bt->G, bt->goff, nullptr, ctx->p1, bt->sums(), st);
        decisions += po.decisions;
        skipped += po.skipped;
        verify_sweeps += po.verify_sweeps;
        incr_sweeps += po.incr_sweeps;
        p1_ms += po.total_ms;
        dec_ms += po.decide_ms;
        upd_ms += po.update_ms;
        dec_bytes += po.decide_bytes;
        upd_bytes += po.update_bytes;
        sweeps += po.sweeps;
        if (verbose && round == 0) printf("louvain time in the first round = %fms\n", po.total_ms);
        // contraction into the other ping-pong buffer; the last round (the
        // stop rule below decides it from this round's Q already) only needs
        // the labels, unless the level graph is checkpointed
        // (a round that started from refined communities and gained less
        // than min_mod is not the last: the next contracts the communities)
        const bool gained = po.q - cur_mod >= min_mod;
        const bool last = !bt && !level_dir &&
                          ((!gained && !started_refined) || (max_levels > 0 && round + 1 >= max_levels) ||
                           round + 1 >= GALA_MAX_LEVELS);
        const bool do_refine = refine && !last && gained;
        cudaEventRecord(ctx->ev[0], st);
        int64_t newE = 0;
        gala_status cs = GALA_OK;
        // the refinement (counted with the contraction) replaces the labels
        // the contraction groups by and the totals of the new vertices
        const int32_t *ccomm = ctx->p1.comm;
        NextLevelInit nli{ctx->p1.Tot, ctx->p1.K, ctx->p1.Self};
        if (do_refine) {
            if (refine_run(g, ctx->p1.comm, ctx->p1.K, ctx->p1.Tot, m2, ctx->p1.order, (int)po.nv, ctx->ref,
                           ctx->d_stats, st, &cs) < 0)
                return cs;
            ccomm = ctx->ref.R;
            nli.tot = ctx->ref.Kr;
        }
        C = contract_run(g, ccomm, ctx->cb, ctx->offs[buf], ctx->nbr[buf], ctx->w[buf], ctx->orig, n0, &newE, st,
                         &cs, false, opt && opt->sorted_levels == 1, nli, last);
        if (C < 0) return cs;
        if (do_refine) refine_next_init(ctx->p1.comm, ctx->cb.lab, g.n, ctx->ref, st);
        have_init = do_refine;
        cudaEventRecord(ctx->ev[1], st);
        if ((s = sync_check(st, "contraction"))) return s;
        float cms = ev_ms(ctx->ev[0], ctx->ev[1]);
        contract_ms += cms;
        if (verbose && round == 0) printf("build time in the first round = %fms\n", cms);
        if (verbose) printf("number of communities:%d modularity:%f\n", C, po.q);
        if (round < GALA_MAX_LEVELS) {
            res->level_modularity[round] = po.q;
            res->level_communities[round] = C;
            res->level_iterations[round] = po.iterations;
            res->level_vertices[round] = g.n;
            res->level_entries[round] = g.E;
            res->level_phase1_ms[round] = po.total_ms;
            res->level_decide_ms[round] = po.decide_ms;
            res->level_update_ms[round] = po.update_ms;
            res->level_contract_ms[round] = cms;
            res->level_movers[round] = po.movers;
            res->level_active_entries[round] = po.active_entries;
        }
        res->total_iterations += po.iterations;
        round++;
        prev_mod = cur_mod;
        cur_mod = po.q;
        g = LevelGraph{C, newE, ctx->offs[buf], ctx->nbr[buf], ctx->w[buf], wide, true, true};
        buf ^= 1;
        if (level_dir && (s = write_level(ctx, g, n0, level_dir, round))) return s;
        if (bt) {
            const int G = bt->G;
            if ((s = check(cudaMemcpyAsync(bt->h_ncomm, bt->ncomm, G * sizeof(int32_t), cudaMemcpyDeviceToHost, st),
                           "batch communities")) ||
                (s = sync_check(st, "batch communities")))
                return s;
            bt->h_goff[0] = 0;
            bool running = false;
            for (int i = 0; i < G; ++i) {
                bt->h_goff[i + 1] = bt->h_goff[i] + bt->h_ncomm[i];
                if (bt->finished[i]) continue;
                // louvain.cu:202 per graph
                bt->prev_mod[i] = bt->cur_mod[i];
                bt->cur_mod[i] = bt->prev_q[i];
                if (!(bt->cur_mod[i] - bt->prev_mod[i] >= min_mod)) bt->finished[i] = 1;
                else running = true;
            }
            if (bt->h_goff[G] != C) {
                set_error("batch: per-graph communities sum to %lld, contraction made %d", (long long)bt->h_goff[G],
                          C);
                return GALA_ERR_INVALID;
            }
            cudaMemcpyAsync(bt->goff, bt->h_goff, (G + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st);
            batch_gid_fill(G, bt->goff, bt->gid2, st);
            std::swap(bt->gid, bt->gid2);
            ctx->p1.gid = bt->gid;
            if ((s = sync_check(st, "batch ranges"))) return s;
            if (!running) break;
            if (max_levels > 0 && round >= max_levels) break;
            if (round >= GALA_MAX_LEVELS) break;
            continue;
        }
        // louvain.cu:202: continue while the round gained at least min_mod
        // (or, refining, while it started from refined communities)
        if (!(cur_mod - prev_mod >= min_mod) && !started_refined) break;
        if (max_levels > 0 && round >= max_levels) break;
        if (round >= GALA_MAX_LEVELS) break;
    }
    cudaEventRecord(t1, st);
    if ((s = sync_check(st, "run end"))) return s;
    double total_ms = ev_ms(t0, t1);
    if (verbose) {
        printf("=====================================\n");
        printf("final number of communities:%d -> %d final modularity:%f\n", n0, C, cur_mod);
        printf("execution time without data transfer = %fms\n", total_ms);
    }
    res->modularity = cur_mod;
    res->num_vertices = n0;
    res->num_communities = C;
    res->num_levels = round;
    res->time_total_ms = total_ms;
    res->time_phase1_ms = p1_ms;
    res->time_decide_ms = dec_ms;
    res->time_update_ms = upd_ms;
    res->time_contract_ms = contract_ms;
    res->decide_bytes = dec_bytes;
    res->update_bytes = upd_bytes;
    res->decide_sweeps = sweeps;
    res->decisions = decisions;
    res->skipped = skipped;
    res->verify_sweeps = verify_sweeps;
    res->incremental_sweeps = (int32_t)incr_sweeps;
    res->samples = 0;
    if (pr.mode == GALA_PROPOSAL_TRACE) {
        long long cnt = 0;
        if ((s = check(cudaMemcpyAsync(&cnt, pr.pv.count, sizeof(cnt), cudaMemcpyDeviceToHost, st), "samples")) ||
            (s = sync_check(st, "samples")))
            return s;
        res->samples = std::min<long long>(cnt, pr.pv.cap);
    }
    if (res->iter_modularity && res->iter_capacity > 0) {
        int k = (int)std::min<size_t>(trace.size(), (size_t)res->iter_capacity);
        memcpy(res->iter_modularity, trace.data(), (size_t)k * sizeof(double));
    }
    res->iter_count = (int)trace.size();
    unsigned long long nfp = 0;
    if ((s = check(cudaMemcpyAsync(&nfp, &ctx->d_stats->fp64_decisions, sizeof(nfp), cudaMemcpyDeviceToHost, st),
                   "fp64 count")) ||
        (s = sync_check(st, "fp64 count")))
        return s;
    res->fp64_decisions = (int64_t)nfp;
    return GALA_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
extern "C" {

void gala_default_options(gala_options *opt)
{
    if (!opt) return;
    memset(opt, 0, sizeof(*opt));
    opt->min_modularity = 1e-6;  // gala_main.cu:48
    opt->max_levels = 0;
    opt->verbose = 0;
    opt->use_graphs = 0;
}

void gala_context_destroy(gala_context *ctx)
{
    if (!ctx) return;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->batch) {
        ctx->batch->release();
        ctx->batch->release_stage();
        ctx->batch->release_cta();
        delete ctx->batch;
    }
    for (void *p : ctx->allocs) cudaFree(p);
    if (ctx->h_stats) cudaFreeHost(ctx->h_stats);
    for (auto &e : ctx->ev)
        if (e) cudaEventDestroy(e);
    for (int i = 0; i < gala_context::kAux; ++i) {
        if (ctx->aux[i]) cudaStreamDestroy(ctx->aux[i]);
        if (ctx->join_ev[i]) cudaEventDestroy(ctx->join_ev[i]);
    }
    if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
    for (auto &e : ctx->pend_store.ev)
        if (e) cudaEventDestroy(e);
    if (ctx->copy_stream) {
        cudaStreamSynchronize(ctx->copy_stream);
        cudaStreamDestroy(ctx->copy_stream);
    }
    for (auto &e : ctx->copy_ev)
        if (e) cudaEventDestroy(e);
    if (ctx->offs_ev) cudaEventDestroy(ctx->offs_ev);
    if (ctx->h_chunk) cudaFreeHost(ctx->h_chunk);
    if (ctx->h_stats2) cudaFreeHost(ctx->h_stats2);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    cudaSetDevice(prev);
    delete ctx;
}

gala_status gala_context_create(int32_t device, int32_t max_vertices, int64_t max_entries, gala_context **out)
{
    clear_error();
    if (!out || max_vertices <= 0 || max_entries < 0) {
        set_error("gala_context_create: bad arguments");
        return GALA_ERR_INVALID;
    }
    *out = nullptr;
    int ndev = 0;
    cudaError_t ce = cudaGetDeviceCount(&ndev);
    if (ce != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        set_error("no CUDA device visible");
        return GALA_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= ndev) {
        set_error("device %d out of range (%d devices)", device, ndev);
        return GALA_ERR_INVALID;
    }
    if ((ce = cudaSetDevice(device)) != cudaSuccess) return cuda_fail(ce, "cudaSetDevice");
    gala_context *ctx = new gala_context();
    ctx->device = device;
    ctx->n_cap = max_vertices;
    ctx->e_cap = max_entries;
    const size_t n = (size_t)max_vertices, E = (size_t)(max_entries > 0 ? max_entries : 1);
    const size_t nblk = (n + 1023) / 1024;
    // scans run over at most max(n, 9 * blocks, scratch words) items (the
    // scratch pool is at most 2^27 ints)
    const size_t scan_items = std::max(std::max(n + 2, (size_t)kNumBinSlots * nblk), (size_t)1 << 27);
    const size_t nparts = scan_items / 4096 + 4;
    bool ok = cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking) == cudaSuccess;
    ctx->stream = ctx->own_stream;
    for (auto &e : ctx->ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
    ok = ok && cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming) == cudaSuccess;
    for (int i = 0; i < gala_context::kAux; ++i) {
        ok = ok && cudaStreamCreateWithFlags(&ctx->aux[i], cudaStreamNonBlocking) == cudaSuccess;
        ok = ok && cudaEventCreateWithFlags(&ctx->join_ev[i], cudaEventDisableTiming) == cudaSuccess;
    }
    ok = ok && cudaMallocHost(&ctx->h_stats, sizeof(DevStats)) == cudaSuccess;
    ok = ok && cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) == cudaSuccess;
    for (auto &e : ctx->copy_ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
    ok = ok && cudaEventCreateWithFlags(&ctx->offs_ev, cudaEventDisableTiming) == cudaSuccess;
    for (auto &e : ctx->pend_store.ev) ok = ok && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess;
    constexpr int kChunkInts = (PendingRows::kMax + 1) + (PendingRows::kMax + 1) * kNumBins + PendingRows::kMax * kNumBins;
    ok = ok && cudaMallocHost(&ctx->h_chunk, kChunkInts * sizeof(int32_t)) == cudaSuccess;
    ok = ok && cudaMallocHost(&ctx->h_stats2, sizeof(DevStats)) == cudaSuccess;
    ok = ok && dalloc(ctx, &ctx->d_chunk, kChunkInts) && dalloc(ctx, &ctx->d_stats2, 1);
    for (int i = 0; i < 2 && ok; ++i)
        ok = dalloc(ctx, &ctx->offs[i], n + 1) && dalloc(ctx, &ctx->nbr[i], E) && dalloc8(ctx, &ctx->w[i], E);
    Phase1Buffers &b = ctx->p1;
    ok = ok && dalloc(ctx, &ctx->orig, n) && dalloc(ctx, &ctx->d_stats, 1) && dalloc(ctx, &b.comm, n) &&
         dalloc8(ctx, &b.K, n) && dalloc8(ctx, &b.Self, n) && dalloc8(ctx, &b.Tot, n) && dalloc(ctx, &b.size, n) &&
         dalloc8(ctx, &b.In, n) && dalloc(ctx, &b.order, n) && dalloc(ctx, &b.act[0], n) &&
         dalloc(ctx, &b.act[1], n) && dalloc(ctx, &b.mv_v, n) && dalloc(ctx, &b.mv_old, n) &&
         dalloc(ctx, &b.mv_new, n) && dalloc(ctx, &b.blockcnt, kNumBinSlots * nblk) &&
         dalloc(ctx, &b.blockoff, kNumBinSlots * nblk) && dalloc(ctx, &b.scan_partial, nparts) &&
         dalloc(ctx, &b.feat_gain, n) && dalloc(ctx, &b.feat_ndist, n) && dalloc(ctx, &b.last_move, n) &&
         dalloc(ctx, &b.prop_list, n);
    ContractBuffers &c = ctx->cb;
    ok = ok && dalloc(ctx, &c.cnt, n + 1) && dalloc(ctx, &c.newid, n + 1) && dalloc(ctx, &c.lab, n) &&
         dalloc(ctx, &c.csz, n + 1) && dalloc(ctx, &c.moff, n + 1) && dalloc(ctx, &c.cursor, n + 1) &&
         dalloc(ctx, &c.members, n) && dalloc(ctx, &c.mpos, n) && dalloc(ctx, &c.ec, n + 1) &&
         dalloc(ctx, &c.medge, n + 1) && dalloc(ctx, &c.stream_key, E) && dalloc8(ctx, &c.stream_w, E) &&
         dalloc(ctx, &c.tmp_off, n + 1) && dalloc(ctx, &c.tmp_nbr, E) && dalloc8(ctx, &c.tmp_w, E) &&
         dalloc(ctx, &c.kc, n + 1) && dalloc(ctx, &c.cls_list, 6 * n);
    // tables of the rows longer than 4096 entries: at most 4 slots per entry
    // (keys + values), chunk list of at most E / 4096 + n entries
    c.big_pool_ints = 8LL * (long long)E + 64;
    c.big_work_cap = (long long)E / 4096 + (long long)n + 1;
    c.big_twork_cap = (long long)E / 1024 + (long long)n + 1;  // table slots <= 4E, 4096 per chunk
    ok = ok && dalloc(ctx, &c.big_pool, (size_t)c.big_pool_ints) && dalloc(ctx, &c.big_T, n) &&
         dalloc(ctx, &c.big_chunks, n) && dalloc(ctx, &c.big_toff, n + 1) && dalloc(ctx, &c.big_coff, n + 1) &&
         dalloc(ctx, &c.big_mode, n) && dalloc(ctx, &c.big_work, (size_t)c.big_work_cap) &&
         dalloc(ctx, &c.big_tchunks, n) && dalloc(ctx, &c.big_tcoff, n + 1) &&
         dalloc(ctx, &c.big_twork, (size_t)c.big_twork_cap) && dalloc(ctx, &c.big_kdist, n) &&
         dalloc(ctx, &c.big_cursor, n) && dalloc(ctx, &c.big_gwords, n) && dalloc(ctx, &c.big_gofs, n + 1);
    ok = ok && dalloc(ctx, &b.moved, n) && dalloc(ctx, &b.mv_pre, (size_t)n + 1);
    ok = ok && dalloc(ctx, &b.act_flag, n) && dalloc(ctx, &ctx->hub_px, (size_t)c.big_twork_cap) &&
         dalloc(ctx, &ctx->hub_pc, (size_t)c.big_twork_cap) && dalloc8(ctx, &ctx->hub_pw, (size_t)c.big_twork_cap) &&
         dalloc(ctx, &ctx->hub_pt, (size_t)c.big_twork_cap) && dalloc8(ctx, &ctx->hub_pwc, (size_t)c.big_twork_cap) &&
         dalloc(ctx, &ctx->hub_pdq, (size_t)c.big_twork_cap) && dalloc(ctx, &ctx->hub_pfc, (size_t)c.big_twork_cap) &&
         dalloc(ctx, &c.nz_pos, n + 1) && dalloc(ctx, &c.nz_rows, n + 1) && dalloc(ctx, &c.nz_offs, n + 1) &&
         dalloc(ctx, &c.nz_shift, n + 1) && dalloc(ctx, &c.task_row, E / 1024 + 2);
    // scratch pool for hub tables (phase 1) and the emission bitmaps of the
    // contraction: 8 ints per entry+vertex, 16 MB .. 512 MB
    long long want = 8LL * ((long long)E + (long long)n);
    want = std::max(want, 4LL << 20);
    want = std::min(want, 128LL << 20);
    ok = ok && dalloc(ctx, &ctx->scratch, (size_t)want);
    ctx->scratch_ints = want;
    if (!ok) {
        cudaGetLastError();
        gala_context_destroy(ctx);
        set_error("gala_context_create: device allocation failed (%d vertices, %lld entries)", max_vertices,
                  (long long)max_entries);
        return GALA_ERR_OOM;
    }
    b.stats = ctx->d_stats;
    memset(ctx->h_stats, 0, sizeof(DevStats));
    cudaMemsetAsync(ctx->d_stats, 0, sizeof(DevStats), ctx->stream);
    p1_configure_kernels();
    contract_configure_kernels();
    batch_cta_configure();
    bind_contract_buffers(ctx);
    if ((ce = cudaStreamSynchronize(ctx->stream)) != cudaSuccess) {
        gala_context_destroy(ctx);
        return cuda_fail(ce, "gala_context_create");
    }
    *out = ctx;
    return GALA_OK;
}

gala_status gala_context_set_stream(gala_context *ctx, void *stream)
{
    clear_error();
    if (!ctx) {
        set_error("gala_context_set_stream: null context");
        return GALA_ERR_INVALID;
    }
    cudaSetDevice(ctx->device);
    gala_status s = sync_check(ctx->stream, "gala_context_set_stream");
    if (s) return s;
    ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    return GALA_OK;
}

gala_status gala_context_set_hub_table_cap(gala_context *ctx, int64_t slots)
{
    clear_error();
    if (!ctx || slots < 0 || (slots > 0 && (slots < 32 || (slots & (slots - 1)) != 0))) {
        set_error("gala_context_set_hub_table_cap: slots must be 0 or a power of two >= 32");
        return GALA_ERR_INVALID;
    }
    ctx->hub_table_cap = slots;
    return GALA_OK;
}

gala_status gala_context_set_copy_overlap(gala_context *ctx, int32_t chunks)
{
    clear_error();
    if (!ctx || chunks < 0 || chunks == 1 || chunks > PendingRows::kMax) {
        set_error("gala_context_set_copy_overlap: chunks must be 0 or 2..%d", PendingRows::kMax);
        return GALA_ERR_INVALID;
    }
    ctx->copy_overlap = chunks;
    return GALA_OK;
}

gala_status gala_context_set_long_rows(gala_context *ctx, int32_t mode)
{
    clear_error();
    if (!ctx || mode < 0 || mode > 1) {
        set_error("gala_context_set_long_rows: mode must be 0 or 1");
        return GALA_ERR_INVALID;
    }
    ctx->cb.long_rows_mode = mode;
    return GALA_OK;
}

gala_status gala_context_set_update_mode(gala_context *ctx, int32_t mode)
{
    clear_error();
    if (!ctx || mode < 0 || mode > 2) {
        set_error("gala_context_set_update_mode: mode must be 0, 1 or 2");
        return GALA_ERR_INVALID;
    }
    ctx->update_mode = mode;
    return GALA_OK;
}

gala_status gala_louvain_device(gala_context *ctx, int32_t n, const int64_t *d_offsets, const int32_t *d_neighbors,
                                const int32_t *d_weights, const gala_options *opt, int32_t *d_community_out,
                                gala_result *res)
{
    clear_error();
    if (!ctx || n <= 0 || !d_offsets || !d_neighbors || !d_community_out) {
        set_error("gala_louvain_device: bad arguments");
        return GALA_ERR_INVALID;
    }
    gala_result local{};
    if (!res) res = &local;
    cudaSetDevice(ctx->device);
    int64_t E = 0;
    gala_status s;
    if ((s = check(cudaMemcpyAsync(&E, d_offsets + n, sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream),
                   "read entry count")) ||
        (s = sync_check(ctx->stream, "read entry count")))
        return s;
    long long l0 = gala_kernel_launch_count();
    if ((s = run_levels(ctx, n, E, d_offsets, d_neighbors, d_weights, opt, res))) return s;
    if ((s = check(cudaMemcpyAsync(d_community_out, ctx->orig, (size_t)n * sizeof(int32_t),
                                   cudaMemcpyDeviceToDevice, ctx->stream),
                   "labels")) ||
        (s = sync_check(ctx->stream, "labels")))
        return s;
    res->kernel_launches = gala_kernel_launch_count() - l0;
    return GALA_OK;
}

gala_status gala_louvain(gala_context *ctx, const gala_graph *g, const gala_options *opt, int32_t *community_out,
                         gala_result *res)
{
    clear_error();
    if (!g || !community_out || g->n <= 0) {
        set_error("gala_louvain: bad arguments");
        return GALA_ERR_INVALID;
    }
    gala_context *own = nullptr;
    gala_status s;
    if (!ctx) {
        if ((s = gala_context_create(0, g->n, g->entries(), &own))) return s;
        ctx = own;
    }
    gala_result local{};
    if (!res) res = &local;
    cudaSetDevice(ctx->device);
    const int32_t n = g->n;
    const int64_t E = g->entries();
    if (n > ctx->n_cap || E > ctx->e_cap) {
        if (own) gala_context_destroy(own);
        set_error("graph (%d vertices, %lld entries) exceeds context capacity", n, (long long)E);
        return GALA_ERR_CAPACITY;
    }
    long long l0 = gala_kernel_launch_count();
    cudaStream_t st = ctx->stream;
    const auto host0 = std::chrono::steady_clock::now();
    auto host_ms = [&]() {
        return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - host0).count();
    };
    // a pinned unweighted graph: the neighbours go in row-range chunks of
    // about equal entries on the copy stream, and level 0 starts on the rows
    // that arrived (phase 1 consumes ctx->pending); otherwise one copy
    const bool chunked = ctx->copy_overlap >= 2 && g->pinned && !g->weighted && !g->float_w && E >= (1LL << 22);
    // host -> device: offsets with a leading 0, neighbours, weights
    cudaEventRecord(ctx->ev[6], st);
    if (chunked) cudaEventRecord(ctx->copy_ev[0], st);
    cudaMemsetAsync(ctx->offs[1], 0, sizeof(int64_t), st);
    cudaMemcpyAsync(ctx->offs[1] + 1, g->offs.data(), (size_t)n * sizeof(int64_t), cudaMemcpyHostToDevice, st);
    if (chunked) {
        PendingRows &pr = ctx->pend_store;
        pr.P = ctx->copy_overlap;
        pr.vstart[0] = 0;
        pr.vstart[pr.P] = n;
        for (int k = 1; k < pr.P; ++k) {  // rows that end at or before k E / P
            const int64_t target = E / pr.P * k;
            pr.vstart[k] = (int32_t)(std::upper_bound(g->offs.begin(), g->offs.end(), target) - g->offs.begin());
            if (pr.vstart[k] < pr.vstart[k - 1]) pr.vstart[k] = pr.vstart[k - 1];
        }
        // after the offsets (which the level init needs first: copies that
        // share the host link would otherwise finish together) and after
        // earlier work on the level buffers
        cudaEventRecord(ctx->offs_ev, st);
        cudaStreamWaitEvent(ctx->copy_stream, ctx->offs_ev, 0);
        for (int k = 0; k < pr.P; ++k) {
            const int64_t e0 = pr.vstart[k] ? g->offs[pr.vstart[k] - 1] : 0;
            const int64_t e1 = pr.vstart[k + 1] ? g->offs[pr.vstart[k + 1] - 1] : 0;
            if (e1 > e0)
                cudaMemcpyAsync(ctx->nbr[1] + e0, g->nbr.data() + e0, (size_t)(e1 - e0) * sizeof(int32_t),
                                cudaMemcpyHostToDevice, ctx->copy_stream);
            cudaEventRecord(pr.ev[k], ctx->copy_stream);
        }
        cudaEventRecord(ctx->copy_ev[1], ctx->copy_stream);
        ctx->pending = &pr;
    } else {
        cudaMemcpyAsync(ctx->nbr[1], g->nbr.data(), (size_t)E * sizeof(int32_t), cudaMemcpyHostToDevice, st);
    }
    const void *dw = nullptr;
    if (g->weighted) {
        cudaMemcpyAsync(ctx->w[1], g->w.data(), (size_t)E * sizeof(int32_t), cudaMemcpyHostToDevice, st);
        dw = ctx->w[1];
    } else if (g->float_w) {
        // float weights staged in the other level buffer, converted to fixed point
        cudaMemcpyAsync(ctx->w[0], g->wf.data(), (size_t)E * sizeof(float), cudaMemcpyHostToDevice, st);
        fixed_from_f32((const float *)ctx->w[0], (long long *)ctx->w[1], E, g->fixed_shift, st);
        dw = ctx->w[1];
    }
    float h2d = 0;
    if (!chunked) {
        cudaEventRecord(ctx->ev[7], st);
        if ((s = sync_check(st, "host to device copy"))) {
            if (own) gala_context_destroy(own);
            return s;
        }
        h2d = ev_ms(ctx->ev[6], ctx->ev[7]);
    }
    const double t_h2d = host_ms();
    // level 0 lives in buffer 1; the first contraction writes buffer 0
    s = run_levels(ctx, n, E, ctx->offs[1], ctx->nbr[1], dw, opt, res, nullptr, g->float_w, g->rows_distinct);
    if (chunked) {  // the copy has ended (phase 1 waited for it); also when a run stopped early
        ctx->pending = nullptr;
        cudaStreamWaitEvent(st, ctx->copy_ev[1], 0);
        gala_status s2 = sync_check(st, "host to device copy");
        if (s == GALA_OK) s = s2;
        h2d = ev_ms(ctx->copy_ev[0], ctx->copy_ev[1]);
    }
    const double t_run = host_ms();
    if (s == GALA_OK) {
        cudaEventRecord(ctx->ev[6], st);
        cudaMemcpyAsync(community_out, ctx->orig, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
        cudaEventRecord(ctx->ev[7], st);
        s = sync_check(st, "device to host copy");
        res->time_d2h_ms = ev_ms(ctx->ev[6], ctx->ev[7]);
    }
    const double t_end = host_ms();
    res->host_total_ms = t_end;
    res->host_h2d_ms = t_h2d;
    res->host_run_ms = t_run - t_h2d;
    res->host_d2h_ms = t_end - t_run;
    res->time_h2d_ms = h2d;
    res->h2d_bytes = (long long)n * 8 + E * 4 + ((g->weighted || g->float_w) ? E * 4 : 0);
    res->d2h_bytes = (long long)n * 4;
    res->kernel_launches = gala_kernel_launch_count() - l0;
    if (own) gala_context_destroy(own);
    return s;
}

gala_status gala_autotune(gala_context *ctx, const gala_graph *const *graphs, int32_t count,
                          const gala_options *opt, int32_t repeats, gala_tuning *out)
{
    clear_error();
    if (!ctx || !graphs || count <= 0 || !out) {
        set_error("gala_autotune: bad arguments");
        return GALA_ERR_INVALID;
    }
    if (repeats <= 0) repeats = 1;
    long long n_tot = 0;
    for (int i = 0; i < count; ++i) {
        if (!graphs[i]) {
            set_error("gala_autotune: graph %d is null", i);
            return GALA_ERR_INVALID;
        }
        n_tot += graphs[i]->n;
    }
    gala_options base;
    if (opt)
        base = *opt;
    else
        gala_default_options(&base);
    base.verbose = 0;
    std::vector<int32_t> labels((size_t)n_tot);
    struct Point {
        int m4, m5, m6, b5;
        bool operator<(const Point &o) const
        {
            return m4 != o.m4 ? m4 < o.m4 : m5 != o.m5 ? m5 < o.m5 : m6 != o.m6 ? m6 < o.m6 : b5 < o.b5;
        }
    };
    std::vector<std::pair<Point, double>> seen;
    gala_status s = GALA_OK;
    // device time of one configuration: minimum over the repeats
    auto time_of = [&](const Point &p) -> double {
        for (auto &e : seen)
            if (!(e.first < p) && !(p < e.first)) return e.second;
        gala_options o = base;
        o.bin_max[0] = p.m4;
        o.bin_max[1] = p.m5;
        o.bin_max[2] = p.m6;
        o.bin5_block = p.b5;
        double best = 1e300;
        for (int r = 0; r < repeats && s == GALA_OK; ++r) {
            double ms = 0;
            if (count == 1) {
                gala_result res{};
                s = gala_louvain(ctx, graphs[0], &o, labels.data(), &res);
                ms = res.time_total_ms;
            } else {
                gala_batch_result br{};
                s = gala_louvain_batch(ctx, graphs, count, &o, labels.data(), nullptr, nullptr, &br);
                ms = br.time_total_ms;
            }
            best = std::min(best, ms);
        }
        seen.push_back({p, best});
        return best;
    };
    Point cur{kMaxWarpDeg, kMaxCta5Deg, kMaxCta6Deg, 256};
    const double def_ms = time_of(cur);
    double cur_ms = def_ms;
    auto consider = [&](Point p) {
        const double t = time_of(p);
        if (s == GALA_OK && t < cur_ms) {
            cur_ms = t;
            cur = p;
        }
    };
    for (int m4 : {64, 128, 256}) consider(Point{m4, cur.m5, cur.m6, cur.b5});
    for (int m5 : {1024, 2048}) consider(Point{cur.m4, m5, cur.m6, cur.b5});
    for (int m6 : {4096, 8192}) consider(Point{cur.m4, cur.m5, m6, cur.b5});
    for (int b5 : {256, 512}) consider(Point{cur.m4, cur.m5, cur.m6, b5});
    if (s) return s;
    out->bin_max[0] = cur.m4;
    out->bin_max[1] = cur.m5;
    out->bin_max[2] = cur.m6;
    out->bin5_block = cur.b5;
    out->ms = cur_ms;
    out->default_ms = def_ms;
    out->candidates = (int32_t)seen.size();
    return GALA_OK;
}

namespace {

// One persistent launch over the batch's graphs (batch_cta.cu): each CTA runs
// whole graphs.  The union CSR is in ctx->offs[1] / nbr[1] / w[1].
gala_status batch_per_graph(gala_context *ctx, BatchRun &bt, const gala_graph *const *graphs, int G, int32_t n,
                            long long e_tot, int nmax, bool weighted, const gala_options *opt, int32_t *community_out,
                            double *modularity_out, int32_t *communities_out, gala_batch_result *res)
{
    cudaStream_t st = ctx->stream;
    gala_status s;
    if (!bt.cta.K || bt.cta_cap < G) {
        if ((s = sync_check(st, "batch workspace"))) return s;
        bt.release_cta();
        bool ok = true;
        auto dal = [&](auto **p, size_t cnt) {
            void *q = nullptr;
            if (ok && cudaMalloc(&q, (cnt ? cnt : 1) * sizeof(**p)) == cudaSuccess) {
                bt.cta_dev.push_back(q);
                *p = (std::remove_reference_t<decltype(*p)>)q;
            } else {
                ok = false;
            }
        };
        auto hal = [&](auto **p, size_t cnt) {
            void *q = nullptr;
            if (ok && cudaMallocHost(&q, (cnt ? cnt : 1) * sizeof(**p)) == cudaSuccess) {
                bt.cta_host.push_back(q);
                *p = (std::remove_reference_t<decltype(*p)>)q;
            } else {
                ok = false;
            }
        };
        BatchCtaArgs &a = bt.cta;
        const size_t nv = (size_t)ctx->n_cap, nvo = nv + (size_t)G + 1, ne = (size_t)std::max<int64_t>(ctx->e_cap, 1);
        int32_t **vert[] = {&a.K, &a.Self, &a.Tot, &a.In, &a.prev, &a.cur, &a.size, &a.cnt, &a.newid, &a.rl,
                            &a.cursor, &a.members, &a.kc};
        for (auto p : vert) dal(p, nv);
        dal(&a.moff, nvo);
        dal(&a.active, nv);
        for (int k = 0; k < 2; ++k) {
            dal(&a.loffs[k], nvo);
            dal(&a.lnbr[k], ne);
            dal(&a.lw[k], ne);
        }
        int32_t *order = nullptr;
        dal(&order, G);
        a.order = order;
        dal(&a.q_out, G);
        dal(&a.c_out, G);
        dal(&a.rounds_out, G);
        dal(&a.iters_out, G);
        dal(&a.queue, 2);
        // dense tables of long rows: one per warp of the largest grid
        dal(&a.gacc, batch_cta_gacc_ints(batch_cta_grid(1 << 30), kCtaMaxN));
        hal(&bt.h_order, G);
        hal(&bt.h_q, G);
        hal(&bt.h_c, G);
        hal(&bt.h_rounds, G);
        hal(&bt.h_iters, G);
        if (!ok) {
            cudaGetLastError();
            bt.release_cta();
            set_error("gala_louvain_batch: workspace of the per-graph run could not be allocated");
            return GALA_ERR_OOM;
        }
        a.err = a.queue + 1;
        bt.cta_cap = G;
    }
    BatchCtaArgs a = bt.cta;
    a.G = G;
    a.vstart = bt.vstart();
    a.estart = bt.estart();
    a.u_offs = ctx->offs[1];
    a.u_nbr = ctx->nbr[1];
    a.u_w = weighted ? ctx->w[1] : nullptr;
    a.labels = ctx->orig;
    a.min_mod = opt ? opt->min_modularity : 1e-6;
    a.max_levels = opt ? opt->max_levels : 0;
    a.nmax = nmax;
    // largest graphs first: the queue's tail holds the short ones
    for (int i = 0; i < G; ++i) bt.h_order[i] = i;
    std::sort(bt.h_order, bt.h_order + G, [&](int x, int y) {
        const int64_t ex = graphs[x]->entries(), ey = graphs[y]->entries();
        return ex != ey ? ex > ey : x < y;
    });
    const int grid = batch_cta_grid(G);
    cudaMemcpyAsync((void *)a.order, bt.h_order, (size_t)G * sizeof(int32_t), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(a.queue, 0, 2 * sizeof(int), st);
    cudaMemsetAsync(a.gacc, 0, batch_cta_gacc_ints(grid, nmax) * sizeof(int32_t), st);
    cudaEventRecord(ctx->ev[0], st);
    batch_cta_launch(a, grid, st);
    cudaEventRecord(ctx->ev[1], st);
    int herr = 0;
    cudaMemcpyAsync(bt.h_q, a.q_out, (size_t)G * sizeof(double), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(bt.h_c, a.c_out, (size_t)G * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(bt.h_rounds, a.rounds_out, (size_t)G * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(bt.h_iters, a.iters_out, (size_t)G * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(&herr, a.err, sizeof(int), cudaMemcpyDeviceToHost, st);
    cudaEventRecord(ctx->ev[6], st);
    cudaMemcpyAsync(community_out, ctx->orig, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    cudaEventRecord(ctx->ev[7], st);
    if ((s = sync_check(st, "per-graph batch run"))) return s;
    if (herr) {
        set_error("gala_louvain_batch: a graph's total weight exceeds the int32 range");
        return GALA_ERR_INVALID;
    }
    res->time_total_ms = ev_ms(ctx->ev[0], ctx->ev[1]);
    res->time_phase1_ms = res->time_total_ms;
    res->time_contract_ms = 0;
    res->time_d2h_ms = ev_ms(ctx->ev[6], ctx->ev[7]);
    int rounds = 0, iters = 0;
    for (int i = 0; i < G; ++i) {
        if (modularity_out) modularity_out[i] = bt.h_q[i];
        if (communities_out) communities_out[i] = bt.h_c[i];
        rounds = std::max(rounds, bt.h_rounds[i]);
        iters = std::max(iters, bt.h_iters[i]);
    }
    res->num_graphs = G;
    res->num_levels = rounds;
    res->total_iterations = iters;
    res->vertices = n;
    res->entries = e_tot;
    return GALA_OK;
}

}  // namespace

gala_status gala_louvain_batch(gala_context *ctx, const gala_graph *const *graphs, int32_t count,
                               const gala_options *opt, int32_t *community_out, double *modularity_out,
                               int32_t *communities_out, gala_batch_result *res)
{
    clear_error();
    if (!graphs || count <= 0 || !community_out) {
        set_error("gala_louvain_batch: bad arguments");
        return GALA_ERR_INVALID;
    }
    if (opt && opt->proposal_mode != GALA_PROPOSAL_OFF) {
        set_error("gala_louvain_batch: proposal modes are not available for a batch");
        return GALA_ERR_INVALID;
    }
    long long n_tot = 0, e_tot = 0;
    bool weighted = false;
    for (int i = 0; i < count; ++i) {
        if (!graphs[i] || graphs[i]->n <= 0) {
            set_error("gala_louvain_batch: graph %d is empty", i);
            return GALA_ERR_INVALID;
        }
        if (graphs[i]->float_w) {
            set_error("gala_louvain_batch: graph %d has float weights (batches take int32 weights)", i);
            return GALA_ERR_INVALID;
        }
        n_tot += graphs[i]->n;
        e_tot += graphs[i]->entries();
        weighted = weighted || graphs[i]->weighted;
    }
    if (n_tot > 0x7fffffffLL) {
        set_error("gala_louvain_batch: %lld vertices exceed the int32 id range", n_tot);
        return GALA_ERR_INVALID;
    }
    gala_context *own = nullptr;
    gala_status s;
    if (!ctx) {
        if ((s = gala_context_create(0, (int32_t)n_tot, e_tot, &own))) return s;
        ctx = own;
    }
    struct OwnGuard {
        gala_context *c;
        ~OwnGuard()
        {
            if (c) gala_context_destroy(c);
        }
    } guard{own};
    if (n_tot > ctx->n_cap || e_tot > ctx->e_cap) {
        set_error("batch (%lld vertices, %lld entries) exceeds context capacity (%d, %lld)", n_tot, e_tot, ctx->n_cap,
                  (long long)ctx->e_cap);
        return GALA_ERR_CAPACITY;
    }
    gala_batch_result local{};
    if (!res) res = &local;
    memset(res, 0, sizeof(*res));
    cudaSetDevice(ctx->device);
    cudaStream_t st = ctx->stream;
    const int G = count;
    const int32_t n = (int32_t)n_tot;
    // per-graph state, kept in the context between calls
    if (!ctx->batch) ctx->batch = new BatchRun();
    BatchRun &bt = *ctx->batch;
    if (bt.cap < G || bt.n_cap < ctx->n_cap) {
        if ((s = sync_check(st, "batch state"))) return s;
        bt.release();
        bool ok = true;
        auto dal = [&](auto **p, size_t cnt) {
            void *q = nullptr;
            if (ok && cudaMalloc(&q, (cnt ? cnt : 1) * sizeof(**p)) == cudaSuccess) {
                bt.dev.push_back(q);
                *p = (std::remove_reference_t<decltype(*p)>)q;
            } else {
                ok = false;
            }
        };
        auto hal = [&](auto **p, size_t cnt) {
            void *q = nullptr;
            if (ok && cudaMallocHost(&q, (cnt ? cnt : 1) * sizeof(**p)) == cudaSuccess) {
                bt.host.push_back(q);
                *p = (std::remove_reference_t<decltype(*p)>)q;
            } else {
                ok = false;
            }
        };
        const size_t nc = (size_t)ctx->n_cap;
        dal(&bt.gid, nc);
        dal(&bt.gid2, nc);
        dal(&bt.m2g, G);
        dal(&bt.cg, G);
        dal(&bt.stop, G);
        dal(&bt.reject, G);
        dal(&bt.min_tot, G);
        dal(&bt.ncomm, G);
        dal(&bt.sum_in, G);
        dal(&bt.sum_tot2, G);
        dal(&bt.sum_k, G);
        dal(&bt.goff, (size_t)G + 1);
        dal(&bt.tab, 5 * (size_t)G + 2);
        hal(&bt.h_sum_in, G);
        hal(&bt.h_sum_tot2, G);
        hal(&bt.h_sum_k, G);
        hal(&bt.h_ncomm, G);
        hal(&bt.h_stop, G);
        hal(&bt.h_reject, G);
        hal(&bt.h_goff, (size_t)G + 1);
        hal(&bt.h_tab, 5 * (size_t)G + 2);
        if (!ok) {
            cudaGetLastError();
            bt.release();
            set_error("gala_louvain_batch: allocation of the per-graph state failed (%d graphs)", G);
            return GALA_ERR_OOM;
        }
        bt.cap = G;
        bt.n_cap = ctx->n_cap;
    }
    bt.G = G;
    bt.m2.clear();
    bt.prev_q.clear();
    bt.finished.assign(G, 0);
    bt.prev_mod.assign(G, -1.0);
    bt.cur_mod.assign(G, -1.0);
    int64_t *vstart = bt.h_vstart(), *estart = bt.h_estart();
    vstart[0] = estart[0] = 0;
    bool mapped = true;  // every graph readable in place by the GPU (gala_graph_pin)
    for (int i = 0; i < G; ++i) {
        const gala_graph *gg = graphs[i];
        vstart[i + 1] = vstart[i] + gg->n;
        estart[i + 1] = estart[i] + gg->entries();
        mapped = mapped && gg->dev_offs && (gg->entries() == 0 || gg->dev_nbr) && (!gg->weighted || gg->dev_w);
    }
    memcpy(bt.h_goff, vstart, ((size_t)G + 1) * sizeof(int64_t));
    if (!mapped) {
        // raw copies of every graph into the context's pinned staging, one
        // transfer of it, ids and offsets shifted on the device
        if (!bt.h_offs || (weighted && !bt.h_w)) {
            if ((s = sync_check(st, "batch staging"))) return s;
            bt.release_stage();
            void *a = nullptr, *b2 = nullptr, *c = nullptr;
            const size_t nc = (size_t)ctx->n_cap + 1, ec = (size_t)std::max<int64_t>(ctx->e_cap, 1);
            if (cudaMallocHost(&a, nc * sizeof(int64_t)) != cudaSuccess ||
                (bt.stage.push_back(a), cudaMallocHost(&b2, ec * sizeof(int32_t)) != cudaSuccess) ||
                (bt.stage.push_back(b2), weighted && cudaMallocHost(&c, ec * sizeof(int32_t)) != cudaSuccess)) {
                cudaGetLastError();
                bt.release_stage();
                set_error("gala_louvain_batch: pinned staging of %lld entries failed", (long long)ctx->e_cap);
                return GALA_ERR_OOM;
            }
            if (c) bt.stage.push_back(c);
            bt.h_offs = (int64_t *)a;
            bt.h_nbr = (int32_t *)b2;
            bt.h_w = (int32_t *)c;
        }
        std::atomic<int> next{0};
        auto copy = [&] {
            for (int i = next++; i < G; i = next++) {
                const gala_graph *gg = graphs[i];
                const long long v0 = vstart[i], e0 = estart[i], E = gg->entries();
                memcpy(bt.h_offs + v0 + 1, gg->offs.data(), (size_t)gg->n * sizeof(int64_t));
                if (E) memcpy(bt.h_nbr + e0, gg->nbr.data(), (size_t)E * sizeof(int32_t));
                if (weighted) {
                    if (gg->weighted)
                        memcpy(bt.h_w + e0, gg->w.data(), (size_t)E * sizeof(int32_t));
                    else
                        std::fill(bt.h_w + e0, bt.h_w + e0 + E, 1);
                }
            }
        };
        const unsigned hw = std::thread::hardware_concurrency();
        const int nt = std::max(1, std::min<int>(G, hw ? (int)hw : 1));
        std::vector<std::thread> th;
        for (int t = 1; t < nt; ++t) th.emplace_back(copy);
        copy();
        for (auto &x : th) x.join();
        bt.h_offs[0] = 0;
    } else {
        for (int i = 0; i < G; ++i) {
            bt.h_tab[i] = (int64_t)(uintptr_t)graphs[i]->dev_offs;
            bt.h_tab[bt.cap + i] = (int64_t)(uintptr_t)graphs[i]->dev_nbr;
            bt.h_tab[2LL * bt.cap + i] = (int64_t)(uintptr_t)graphs[i]->dev_w;
        }
    }
    long long l0 = gala_kernel_launch_count();
    cudaEventRecord(ctx->ev[6], st);
    const int32_t *dw = weighted ? ctx->w[1] : nullptr;
    // the source table (or, staged, just the vertex and entry starts)
    // (laid out for bt.cap graphs; this batch fills the first G of each part)
    cudaMemcpyAsync(bt.vstart(), bt.h_vstart(), ((size_t)G + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(bt.estart(), bt.h_estart(), ((size_t)G + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st);
    if (mapped) {
        cudaMemcpyAsync(bt.tab, bt.h_tab, 3 * (size_t)bt.cap * sizeof(int64_t), cudaMemcpyHostToDevice, st);
        batch_gather(G, bt.src(), ctx->offs[1], ctx->nbr[1], weighted ? ctx->w[1] : nullptr, st);
    } else {
        cudaMemcpyAsync(ctx->offs[1], bt.h_offs, ((size_t)n + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(ctx->nbr[1], bt.h_nbr, (size_t)e_tot * sizeof(int32_t), cudaMemcpyHostToDevice, st);
        if (weighted)
            cudaMemcpyAsync(ctx->w[1], bt.h_w, (size_t)e_tot * sizeof(int32_t), cudaMemcpyHostToDevice, st);
        batch_shift(G, bt.vstart(), bt.estart(), ctx->offs[1], ctx->nbr[1], st);
    }
    cudaMemcpyAsync(bt.goff, bt.h_goff, ((size_t)G + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st);
    cudaEventRecord(ctx->ev[7], st);
    batch_gid_fill(G, bt.goff, bt.gid, st);
    if ((s = sync_check(st, "batch host to device copy"))) return s;
    res->time_h2d_ms = ev_ms(ctx->ev[6], ctx->ev[7]);
    int nmax = 0;
    for (int i = 0; i < G; ++i) nmax = std::max(nmax, graphs[i]->n);
    if (!(opt && opt->batch_mode == 1) && nmax <= kCtaMaxN) {
        s = batch_per_graph(ctx, bt, graphs, G, n, e_tot, nmax, weighted, opt, community_out, modularity_out,
                            communities_out, res);
        if (s) return s;
        res->h2d_bytes = ((long long)n + 1) * 8 + e_tot * 4 * (weighted ? 2 : 1) + ((long long)G + 1) * 8 +
                         (mapped ? 3LL * bt.cap + 2LL * G + 2 : 2LL * G + 2) * 8 + (long long)G * 4;
        res->d2h_bytes = (long long)n * 4 + (long long)G * (8 + 3 * 4);
        res->kernel_launches = gala_kernel_launch_count() - l0;
        return GALA_OK;
    }
    Phase1Buffers &b = ctx->p1;
    b.gid = bt.gid;
    b.m2g = bt.m2g;
    b.cg = bt.cg;
    b.gstop = bt.stop;
    b.min_tot_g = bt.min_tot;
    gala_result r{};
    bool distinct = true;
    for (int i = 0; i < G; ++i) distinct = distinct && graphs[i]->rows_distinct;
    s = run_levels(ctx, n, e_tot, ctx->offs[1], ctx->nbr[1], dw, opt, &r, &bt, false, distinct);
    b.gid = nullptr;
    b.m2g = nullptr;
    b.cg = nullptr;
    b.gstop = nullptr;
    b.min_tot_g = nullptr;
    if (s) return s;
    // union community ids -> ids local to each graph, on the device
    batch_local_labels(G, bt.vstart(), bt.goff, ctx->orig, st);
    cudaEventRecord(ctx->ev[6], st);
    cudaMemcpyAsync(community_out, ctx->orig, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    cudaEventRecord(ctx->ev[7], st);
    if ((s = sync_check(st, "batch device to host copy"))) return s;
    res->time_d2h_ms = ev_ms(ctx->ev[6], ctx->ev[7]);
    for (int i = 0; i < G; ++i) {
        if (modularity_out) modularity_out[i] = bt.m2[i] > 0 ? bt.cur_mod[i] : 0.0;
        if (communities_out) communities_out[i] = (int32_t)(bt.h_goff[i + 1] - bt.h_goff[i]);
    }
    res->num_graphs = G;
    res->num_levels = r.num_levels;
    res->total_iterations = r.total_iterations;
    res->vertices = n;
    res->entries = e_tot;
    res->time_total_ms = r.time_total_ms;
    res->time_phase1_ms = r.time_phase1_ms;
    res->time_contract_ms = r.time_contract_ms;
    res->h2d_bytes = ((long long)n + 1) * 8 + e_tot * 4 * (weighted ? 2 : 1) + ((long long)G + 1) * 8 +
                     (mapped ? 3LL * bt.cap + 2LL * G + 2 : 2LL * G + 2) * 8;
    res->d2h_bytes = (long long)n * 4;
    res->kernel_launches = gala_kernel_launch_count() - l0;
    return GALA_OK;
}

gala_status gala_phase1_device(gala_context *ctx, int32_t n, const int64_t *d_offsets, const int32_t *d_neighbors,
                               const int32_t *d_weights, double min_modularity, int32_t *d_community_out,
                               double *modularity, double *iter_q, int32_t iter_capacity, int32_t *iterations)
{
    clear_error();
    if (!ctx || n <= 0 || !d_offsets || !d_neighbors || !d_community_out) {
        set_error("gala_phase1_device: bad arguments");
        return GALA_ERR_INVALID;
    }
    cudaSetDevice(ctx->device);
    cudaStream_t st = ctx->stream;
    int64_t E = 0;
    gala_status s;
    if ((s = check(cudaMemcpyAsync(&E, d_offsets + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st), "entries")) ||
        (s = sync_check(st, "entries")))
        return s;
    if (n > ctx->n_cap || E > ctx->e_cap) {
        set_error("graph exceeds context capacity");
        return GALA_ERR_CAPACITY;
    }
    LevelGraph g{n, E, d_offsets, d_neighbors, d_weights};
    ctx->p1.lim = BinLimits();
    ctx->p1.b5_block = 256;
    long long m2 = 0;
    std::vector<double> trace;
    Phase1Out po;
    ctx->sym_state = -1;  // a new graph: checked with its first sweep
    if ((s = phase1(ctx, g, m2, min_modularity, false, &trace, &po))) return s;
    if ((s = check(cudaMemcpyAsync(d_community_out, ctx->p1.comm, (size_t)n * sizeof(int32_t),
                                   cudaMemcpyDeviceToDevice, st),
                   "labels")) ||
        (s = sync_check(st, "labels")))
        return s;
    if (modularity) *modularity = po.q;
    if (iterations) *iterations = po.iterations;
    if (iter_q)
        for (int i = 0; i < iter_capacity && i < (int)trace.size(); ++i) iter_q[i] = trace[i];
    return GALA_OK;
}

gala_status gala_contract_device(gala_context *ctx, int32_t n, const int64_t *d_offsets, const int32_t *d_neighbors,
                                 const int32_t *d_weights, int32_t *d_community, int64_t *d_new_offsets,
                                 int32_t *d_new_neighbors, int32_t *d_new_weights, int32_t *num_communities,
                                 int64_t *num_entries)
{
    clear_error();
    if (!ctx || n <= 0 || !d_offsets || !d_neighbors || !d_community || !d_new_offsets || !d_new_neighbors ||
        !d_new_weights) {
        set_error("gala_contract_device: bad arguments");
        return GALA_ERR_INVALID;
    }
    cudaSetDevice(ctx->device);
    cudaStream_t st = ctx->stream;
    int64_t E = 0;
    gala_status s;
    if ((s = check(cudaMemcpyAsync(&E, d_offsets + n, sizeof(int64_t), cudaMemcpyDeviceToHost, st), "entries")) ||
        (s = sync_check(st, "entries")))
        return s;
    if (n > ctx->n_cap || E > ctx->e_cap) {
        set_error("graph exceeds context capacity");
        return GALA_ERR_CAPACITY;
    }
    bind_contract_buffers(ctx);
    LevelGraph g{n, E, d_offsets, d_neighbors, d_weights};
    int64_t newE = 0;
    gala_status cs = GALA_OK;
    int C = contract_run(g, d_community, ctx->cb, d_new_offsets, d_new_neighbors, d_new_weights, nullptr, 0, &newE,
                         st, &cs, true);
    if (C < 0) return cs;
    // the reference rewrites the labels with the new ids (build_compressed_graph.cu:22-23)
    if ((s = check(cudaMemcpyAsync(d_community, ctx->cb.lab, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToDevice,
                                   st),
                   "relabel")) ||
        (s = sync_check(st, "relabel")))
        return s;
    if (num_communities) *num_communities = C;
    if (num_entries) *num_entries = newE;
    return GALA_OK;
}

}  // extern "C"
