// internal.h - host-side declarations shared by the translation units of
// libgala (not part of the public C ABI in include/gala.h).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/gala.h"
#include "binlimits.h"

// Host graph in the reference layout (src/graph/graph.h:7-19): inclusive
// offsets without a leading 0; weights optional.
struct gala_graph {
    int32_t n = 0;
    std::vector<int64_t> offs;  // n entries, inclusive prefix sums
    std::vector<int32_t> nbr;   // offs[n-1] entries
    std::vector<int32_t> w;     // empty when unweighted
    std::vector<float> wf;      // float weights (float graphs; w is then empty)
    bool weighted = false;      // int32 weights
    bool float_w = false;       // float32 weights, run as 64-bit fixed point
    int32_t fixed_shift = 0;    // float graphs: weights are round(w * 2^fixed_shift)
    bool rows_distinct = false; // every row lists a neighbour at most once (built here)
    bool pinned = false;  // arrays registered with cudaHostRegister
    // device-mapped addresses of the registered arrays (null when not pinned)
    const int64_t *dev_offs = nullptr;
    const int32_t *dev_nbr = nullptr;
    const int32_t *dev_w = nullptr;
    int64_t entries() const { return n ? offs[n - 1] : 0; }
    ~gala_graph();
};

namespace gala {
// Fixed-point shift of float weights (the same rule as the oracle's
// orc_fixed_shift); -1 when a weight is not positive and finite or rounds to 0.
int32_t fixed_shift_of(const float *w, int64_t E);
}

namespace gala {

// Move-proposal network: 8 features, 8 -> 32 -> 32 -> 1.
constexpr int kPropFeatures = 8;
constexpr int kPropParams = 32 * 8 + 32 + 32 * 32 + 32 + 32 + 1;

// Device view of a proposal's sample set and inference weights.
struct ProposalView {
    float *X;           // features, kPropFeatures per sample
    float *Y;           // labels (1 = moved)
    int32_t *V;         // vertex of each sample (labelled after the sweep)
    long long cap;
    long long *count;   // samples written (may exceed cap; clamp)
    const void *wb;     // BF16 inference weights
};
ProposalView proposal_view(gala_proposal *p);

// Error text of the last failure on this host thread.
void set_error(const char *fmt, ...);
void clear_error();
gala_status cuda_fail(cudaError_t e, const char *what);
void note_launch(int k);

struct DevStats;

// Device arrays of one phase-1 level (device layout CSR).
struct LevelGraph {
    int32_t n;
    int64_t E;
    const int64_t *offs;  // n+1, leading 0
    const int32_t *nbr;
    const void *w;        // nullptr = unweighted; int32, or int64 fixed point when wide
    bool wide = false;
    bool distinct = false;  // rows list each neighbour at most once (contracted levels always)
    bool ks_ready = false;  // K and Self of every vertex are already in the phase-1 buffers
};

// Phase-1 workspace (all device pointers, sized for the context capacity).
struct Phase1Buffers {
    int32_t *comm, *K, *Self, *Tot, *size, *In;
    int32_t *order;            // vertices grouped by degree bin
    int32_t *act[2];           // active lists (bin segments as in order)
    int32_t *mv_v, *mv_old, *mv_new;
    int32_t *blockcnt;         // counting-sort scratch (kNumBinSlots * blocks)
    int32_t *blockoff;
    long long *scan_partial;
    int32_t *hub_table;        // global hash tables of the largest bin
    long long hub_table_slots; // capacity in int32 pairs
    uint8_t *act_flag;         // 1 = vertex is in the current active set
    // incremental weight update: movers of the sweep flagged (cleared by the
    // prune pass) and the prefix of their row lengths
    uint8_t *moved;
    long long *mv_pre;
    // move-proposal features (written only when a proposal mode is on)
    float *feat_gain;          // best corrected gain at the last decision / (K m2)
    int32_t *feat_ndist;       // distinct neighbour communities at the last decision (-1 = unknown)
    int32_t *last_move;        // iteration of the vertex's last move
    int32_t *prop_list;        // proposed vertices (bin segments as in order)
    int features_on;           // 1 = decide kernels write the features above
    int wide;                  // 1 = K, Self, Tot, In and weights are 64-bit fixed point
    BinLimits lim;             // upper degrees of bins 4-6 (tuning)
    int b5_block;              // threads per vertex in bin 5: 512 or 256 (tuning)
    // batched graphs (all null for one graph): graph of each vertex, the
    // graph's m2 and 1/m2, stopped graphs, per-graph min Tot
    const int32_t *gid;
    const long long *m2g;
    const double *cg;
    const uint8_t *gstop;
    const int32_t *min_tot_g;
    DevStats *stats;
};

// Per-iteration proposal step: features of the active vertices, then either
// training samples (mode 1) or the proposed lists (mode 2).
struct ProposalStep {
    int mode;                  // GALA_PROPOSAL_TRACE or GALA_PROPOSAL_SKIP
    ProposalView pv;
    float threshold;
    int sample_shift;
    int iteration, level;
};
void p1_features_init(Phase1Buffers &b, int n, cudaStream_t st);
// Features of the active vertices of bins 0-6 (lists / counts of the current
// active set); mode TRACE appends sampled rows to the sample set, mode SKIP
// fills prop_list / prop_count with the vertices the network proposes.
void p1_proposal_step(const LevelGraph &g, Phase1Buffers &b, const ProposalStep &ps, const int32_t *lists,
                      const int *counts, const int *bin_start, const int *level_cnt, cudaStream_t st);
// Labels of the samples of the current sweep (moved in this iteration).
void p1_trace_labels(Phase1Buffers &b, const ProposalStep &ps, cudaStream_t st);

// Hub vertices (largest degree bin): per-hub global tables filled by many
// CTAs.  Arrays are borrowed from the contraction's long-row buffers, which
// are idle during phase 1.
struct HubPlan {
    const int32_t *hubs;  // the bin's vertices (order segment)
    int H;
    long long *T, *chunks, *tchunks, *toff, *coff, *tcoff;
    int32_t *work, *twork;
    int32_t *pool;
    long long half;       // keys at pool[0, half), values at pool[half, 2 half)
    long long t_cap;      // largest table (power of two; 0 = sized by degree only)
    long long nwork, ntwork;
    long long *px;        // per table chunk: best exact gain numerator
    int32_t *pc, *pw, *pt, *pwc;
    double *pdq;          // per table chunk: best FP64 gain (hubs decided in FP64)
    int32_t *pfc;
};

// ---- phase 1 kernels (phase1.cu) ----
void p1_level_init(const LevelGraph &g, Phase1Buffers &b, cudaStream_t st);
void p1_iter_reset(Phase1Buffers &b, int next, long long min_tot_init, cudaStream_t st);
// first = the level's first sweep (every vertex its own community).
void p1_decide(const LevelGraph &g, Phase1Buffers &b, int bin, const int32_t *list,
               const int *count_ptr, int level_count, double constant, long long m2,
               int fp64_only, bool first, cudaStream_t st);
// offs: the movers' row lengths are summed into stats->mv_edges (sign +1);
// moved: movers are flagged for the incremental weight update.
void p1_apply_movers(Phase1Buffers &b, int sign, int n, cudaStream_t st, int iteration = 0,
                     const int64_t *offs = nullptr, uint8_t *moved = nullptr);
// Incremental weight update of a sweep, enqueued after the movers are
// applied and before the per-bin updates: a device flag (stats->push_mode)
// picks it when `allow` (In exact from the previous sweep, symmetric graph)
// and the movers' rows hold under a third of the entries (always with
// `force`); the per-bin update kernels then return at once.  It sums In of
// every mover over its row, pushes +-w from every mover to its neighbours
// that did not move, then runs one pass over the vertices of bins 0-7 for the
// pruning bound, the next active lists and the sums.  bin_start: the level's
// order-list bin starts (host copy).
void p1_push_update(const LevelGraph &g, Phase1Buffers &b, const int *bin_start, int next, double constant,
                    long long m2, int allow, int force, cudaStream_t st);

void p1_tot_reduce(Phase1Buffers &b, int n, cudaStream_t st);
void p1_update(const LevelGraph &g, Phase1Buffers &b, int bin, const int32_t *list, int count, int next,
               int bin_start, double constant, long long m2, cudaStream_t st);
void p1_level_init_rows(const LevelGraph &g, Phase1Buffers &b, const int *bin_start, cudaStream_t st);
// Level-0 rows still in flight (unweighted graphs): K = Tot = degree from the
// offsets; per row chunk k and bin, the bin's sub-range of the order list
// (d_lo[(P + 1) x 8], d_cnt[P x 8]); init rows of one sub-range into `stats`.
// (The chunk starts go as a kernel argument: a small copy to the device would
// queue behind the chunks themselves.)
struct ChunkStarts {
    int32_t v[17];
};
void p1_init_degree(const LevelGraph &g, Phase1Buffers &b, cudaStream_t st);
void p1_chunk_bounds(Phase1Buffers &b, const ChunkStarts &vs, int P, int32_t *d_lo, int32_t *d_cnt, cudaStream_t st);
void p1_init_rows_range(const LevelGraph &g, Phase1Buffers &b, int bin, const int32_t *list, int cnt, DevStats *stats,
                        cudaStream_t st);
// Neighbour arrays of a level-0 graph still being copied: row-range chunks on
// another stream, one event per chunk (chunk k holds the rows of vertices
// [vstart[k], vstart[k + 1])).
struct PendingRows {
    static constexpr int kMax = 16;  // ChunkStarts holds kMax + 1 starts
    int P = 0;
    int32_t vstart[kMax + 1] = {};
    cudaEvent_t ev[kMax] = {};
};
void p1_configure_kernels();
void contract_configure_kernels();
void p1_reset_level_stats(Phase1Buffers &b, cudaStream_t st);
int hub_grid_size();
void p1_hub_plan_launch(const LevelGraph &g, Phase1Buffers &b, HubPlan &p, cudaStream_t st);
void p1_hub_work_launch(HubPlan &p, cudaStream_t st);
void p1_hub_decide(const LevelGraph &g, Phase1Buffers &b, const HubPlan &p, double constant, long long m2,
                   int fp64_only, cudaStream_t st);
// Weight update + pruning of the hub bin (bin 7), chunked over many CTAs.
void p1_hub_update(const LevelGraph &g, Phase1Buffers &b, const HubPlan &p, int next, int bin_start, double constant,
                   long long m2, cudaStream_t st);

// ---- batched graphs (batch.cu) ----
constexpr int kSumIn = 1, kSumTot2 = 2, kMinTot = 4, kSumK = 8, kCountComm = 16;
struct GraphSums {  // per-graph outputs (device arrays of G entries)
    unsigned long long *sum_in, *sum_tot2, *sum_k;
    int32_t *min_tot, *ncomm;
};
void batch_graph_sums(int what, int G, const int64_t *goff, const uint8_t *stop, const Phase1Buffers &b,
                      const GraphSums &out, cudaStream_t st);
void batch_revert(Phase1Buffers &b, const int32_t *gid, const uint8_t *reject, int n, cudaStream_t st);
void batch_gid_fill(int G, const int64_t *goff, int32_t *gid, cudaStream_t st);
// Source arrays of a batch of page-locked host graphs (device-mapped
// addresses, one per graph) and each graph's first vertex and entry in the
// union (G+1 entries each).
struct BatchSrc {
    const int64_t *const *offs;  // inclusive offsets, n_g entries
    const int32_t *const *nbr;
    const int32_t *const *w;     // null entries: unweighted graphs
    const int64_t *vstart;
    const int64_t *estart;
};
// Union CSR (device layout, ids shifted per graph) gathered from the host
// graphs by the GPU; w may be null (no graph weighted).
void batch_gather(int G, const BatchSrc &src, int64_t *offs, int32_t *nbr, int32_t *w, cudaStream_t st);
// Union CSR whose graphs were copied raw (inclusive offsets of graph g at
// offs[vstart[g]+1 ...], its entries at nbr[estart[g] ...]): shift them into
// union ids and offsets in place.
void batch_shift(int G, const int64_t *vstart, const int64_t *estart, int64_t *offs, int32_t *nbr, cudaStream_t st);
// A batch whose graphs all have at most kCtaMaxN vertices runs in one
// persistent launch, one CTA per graph at a time (batch_cta.cu).  All arrays
// are union-indexed: vertex arrays at the graph's first vertex, offsets
// arrays (one more entry per graph) at first vertex + graph index, entry
// arrays at the graph's first entry.
constexpr int kCtaMaxN = 4096;
struct BatchCtaArgs {
    int G;
    const int32_t *order;  // graphs, largest first
    const int64_t *vstart, *estart;
    const int64_t *u_offs;  // union CSR (device layout)
    const int32_t *u_nbr;
    const int32_t *u_w;     // null: unit weights
    int32_t *K, *Self, *Tot, *In, *prev, *cur, *size, *cnt, *newid, *rl, *cursor, *members, *kc, *moff;
    uint8_t *active;
    int32_t *loffs[2], *lnbr[2], *lw[2];  // contracted level graphs (ping-pong)
    int32_t *labels;  // out: every input vertex's community, local to its graph
    double *q_out;
    int32_t *c_out, *rounds_out, *iters_out;
    int *queue, *err;
    double min_mod;
    int max_levels;
    int nmax;       // largest graph (vertices)
    int32_t *gacc;  // per warp of the grid: nmax ints, zero (dense tables of long rows)
};
void batch_cta_configure();
int batch_cta_grid(int G);
size_t batch_cta_gacc_ints(int grid, int nmax);
void batch_cta_launch(const BatchCtaArgs &a, int grid, cudaStream_t st);
// labels[v] -= goff[g] for the input vertices v of every graph g.
void batch_local_labels(int G, const int64_t *vstart, const int64_t *goff, int32_t *labels, cudaStream_t st);

// ---- contraction (contract.cu) ----
struct ContractBuffers {
    int32_t *cnt;        // n+1
    int32_t *newid;      // n
    int32_t *lab;        // n
    int32_t *csz;        // n+1
    int32_t *moff;       // n+1 member offsets
    int32_t *cursor;     // n
    int32_t *members;    // n
    int32_t *mpos;       // n: member position of each vertex
    long long *ec;       // n+1 edges per community
    long long *medge;    // n+1 prefix of member degrees
    int32_t *stream_key; // E
    int32_t *stream_w;   // E weights (int32, or int64 when wide: allocated 8 bytes per entry)
    long long *tmp_off;  // n+1
    int32_t *tmp_nbr;    // E
    int32_t *tmp_w;      // E weights (as stream_w)
    int32_t *kc;         // n+1 distinct neighbours per community
    int32_t *nz_pos;     // n+1: rows with entries, compacted (walk list)
    int32_t *nz_rows;    // n+1
    long long *nz_offs;  // n+1
    long long *nz_shift; // n+1: per listed row, the value its walk adds to an entry index
    int32_t *task_row;   // E / 1024 + 2: first listed row of every 1024-entry walk task
    int32_t *cls_list;   // n: communities by size class
    // rows of more than 4096 entries: one global table per community, filled
    // by many CTAs (chunks of the stream), then emitted by one CTA each
    int32_t *big_pool;        // keys then values of all tables
    int long_rows_mode = 0;   // 0: by key range when it fits, 1: global tables only
    long long big_pool_ints;
    long long *big_T;         // n: table slots per community (list order)
    long long *big_chunks;    // n: stream chunks per community
    long long *big_toff;      // n+1: table offsets
    long long *big_coff;      // n+1: chunk offsets
    int32_t *big_mode;        // n: 1 = dense table indexed by community id
    int32_t *big_work;        // stream chunk -> list index
    long long big_work_cap;
    long long *big_tchunks;   // n: table chunks per community
    long long *big_tcoff;     // n+1: table chunk offsets
    int32_t *big_twork;       // table chunk -> list index
    long long big_twork_cap;
    int32_t *big_kdist;       // n: distinct neighbour communities
    int32_t *big_cursor;      // n: unsorted emission cursor
    long long *big_gwords;    // n: bitmap words of rows ranked by bitmap (0 = sorted in smem)
    long long *big_gofs;      // n+1: bitmap word offsets
    int32_t *big_bitmap;      // per-CTA bitmaps over communities (emission)
    long long big_bitmap_words;
    long long *scan_partial;
    DevStats *stats;
    // auxiliary streams (null: none): the size classes aggregate concurrently
    static constexpr int kAux = 4;
    cudaStream_t aux[kAux] = {};
    cudaEvent_t fork_ev = nullptr;
    cudaEvent_t join_ev[kAux] = {};
};
// sort_rows = false (the level-to-level contraction of a Louvain run) leaves
// every new row in hash-table order: phase 1 does not depend on the order of
// a row's entries (all weight sums are exact integers), and the sorts are
// skipped.  gala_contract_device sorts, as the oracle does.
// Leiden-style refinement (refine.cu).  All arrays hold one entry per level
// vertex (int32: integer-weight graphs only).
struct RefineBuffers {
    int32_t *R = nullptr;       // sub-community of every vertex (a vertex id)
    int32_t *target = nullptr;  // the sub-community a singleton joins this sweep, or -1
    int32_t *marks = nullptr;   // vertices that target a vertex's sub-community
    int32_t *sz = nullptr;      // members per sub-community
    // weights (WT per vertex: int32, or int64 for fixed-point float weights)
    void *wC = nullptr;         // weight from a vertex to the rest of its community
    void *ext = nullptr;        // weight from a sub-community to the rest of its community
    void *Kr = nullptr;         // weighted degree of a sub-community
    int32_t *pmin = nullptr;    // per community: its sub-community of lowest new id
    int32_t *init = nullptr;    // starting community of every vertex of the next level
    int32_t *moved = nullptr;   // 3 ints: moves of the sweep, long rows listed, candidates listed
    int32_t *list = nullptr;    // vertices with rows longer than 32 entries
    int32_t *list2 = nullptr;   // the singletons that may move
};
// Refines the partition P of level g into R (returns the sweeps run, or -1
// on a CUDA error with *status set); K and TotC are the level's weighted
// degrees and community totals (WT per vertex, as g.wide says).  Afterwards
// b.Kr holds the sub-community totals (the K of the next level's vertices).
// order[0, nv): the level's vertices with edges (the degree-bin order).
int refine_run(const LevelGraph &g, const int32_t *P, const void *K, const void *TotC, long long m2,
               const int32_t *order, int nv, RefineBuffers &b, DevStats *stats, cudaStream_t st,
               gala_status *status);
// The next level's starting partition: b.init[lab[v]] = the lowest new id of a
// sub-community in v's community P[v] (lab: the contraction's new id of every
// level vertex).
void refine_next_init(const int32_t *P, const int32_t *lab, int n, RefineBuffers &b, cudaStream_t st);
// Level start from a given partition: comm = init, Tot and size of its
// communities from K (32- or 64-bit weights, as b.wide says).
void p1_start_partition(Phase1Buffers &b, const int32_t *init, int n, cudaStream_t st);

// labels_only: the new labels (renumbering and orig_map composition) and the
// community count only, no rows (the last round of a run, whose graph nobody
// reads); *new_E is 0.
// Optional by-products for the next level's phase 1 (all null: none): the
// weighted degree of every new vertex (K_new[c'] = Tot[c], the community
// total of the level contracted) and its self-loop weight (the weight of the
// row entry c' -> c'), so that the next level needs no row scan for them.
struct NextLevelInit {
    const void *tot = nullptr;  // Tot of the contracted level (WT per vertex)
    void *k = nullptr;          // receives K_new (WT per new vertex)
    void *self = nullptr;       // receives Self_new (WT per new vertex)
};
int contract_run(const LevelGraph &g, const int32_t *comm, ContractBuffers &b, int64_t *new_offs,
                 int32_t *new_nbr, void *new_w, int32_t *orig_map, int32_t n_orig,
                 int64_t *new_E, cudaStream_t st, gala_status *status, bool validate_labels = false,
                 bool sort_rows = true, const NextLevelInit &nli = NextLevelInit(), bool labels_only = false);

}  // namespace gala
