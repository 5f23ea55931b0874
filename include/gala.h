/*
 * gala.h - C ABI of the GB300 Louvain engine (libgala.so).
 *
 * Plain C, plain pointers and sizes.  Every entry point returns a gala_status
 * and never aborts; gala_last_error() returns a text for the last failure on
 * the calling host thread.
 *
 * CSR conventions used at this boundary
 * -------------------------------------
 *  - "reference layout" (the on-disk .bin layout of the reference,
 *    src/graph/graph.cpp:153-219): int32 n, then int64 offsets[n] holding
 *    INCLUSIVE prefix sums of the row lengths (no leading 0), then int32
 *    neighbours[offsets[n-1]], then optionally int32 weights[offsets[n-1]].
 *  - "device layout" (used by the *_device entry points): int64
 *    offsets[n+1] with a leading 0, neighbours and weights as above.  A NULL
 *    weight pointer means every edge has weight 1.
 *
 * Types follow the reference (src/graph/graph_config.h:3-5): vertex ids and
 * weights are int32, edge offsets are int64.
 */
#ifndef GALA_H
#define GALA_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    GALA_OK = 0,
    GALA_ERR_INVALID = 1,   /* bad argument or malformed CSR */
    GALA_ERR_IO = 2,        /* file cannot be opened / read / written */
    GALA_ERR_FORMAT = 3,    /* .bin file is truncated or inconsistent */
    GALA_ERR_CUDA = 4,      /* a CUDA runtime call failed */
    GALA_ERR_NO_DEVICE = 5, /* no CUDA device is visible */
    GALA_ERR_OOM = 6,       /* device or host allocation failed */
    GALA_ERR_OVERFLOW = 7,  /* a device hash table or probe limit overflowed */
    GALA_ERR_CAPACITY = 8   /* graph larger than the context was created for */
} gala_status;

/* Host-resident graph (owned by the library). */
typedef struct gala_graph gala_graph;
/* Device context: one CUDA stream plus all device workspace for graphs of up
 * to a given size.  One context per host thread at a time. */
typedef struct gala_context gala_context;
/* Learned move-proposal network (8 features -> 32 -> 32 -> 1 MLP) and its
 * training samples, on one device.  No counterpart in the reference. */
typedef struct gala_proposal gala_proposal;

#define GALA_MAX_LEVELS 64

#define GALA_PROPOSAL_OFF 0
#define GALA_PROPOSAL_TRACE 1  /* plain run; sampled decisions become training samples */
#define GALA_PROPOSAL_SKIP 2   /* decide only vertices the network expects to move;
                                  every convergence is confirmed by a plain sweep */

typedef struct {
    double min_modularity; /* stop threshold on the Q gain; reference: 1e-6
                              (src/gala_main.cu:48) */
    int32_t max_levels;    /* 0 = run until the gain is below min_modularity */
    int32_t verbose;       /* 1 = print the reference's stdout lines
                              (README.md:59-89, louvain_main_process.cu:1003) */
    int32_t use_graphs;    /* 1 = the phase-1 sweeps after the first of a level are
                              captured once per level (per active-list slot)
                              as CUDA graphs and replayed (plain runs) */
    int32_t fp64_gains;    /* 1 = evaluate every gain with the reference's FP64
                              expressions (default 0: exact integer gains,
                              FP64 only where rounding could decide; both give
                              the same partition) */
    int32_t proposal_mode;      /* GALA_PROPOSAL_* (needs `proposal`) */
    float proposal_threshold;   /* SKIP: decide vertices with P(move) >= this */
    int32_t trace_sample_shift; /* TRACE: keep about one decision in 2^shift */
    int32_t sorted_levels;      /* 1 = contracted level graphs keep every row sorted
                                   by neighbour id (as gala_contract_device does);
                                   default 0: rows in hash-table order, which
                                   skips the sorts and gives the same partition */
    gala_proposal *proposal;
    int32_t distinct_rows;      /* 1 = the caller guarantees that no row lists a
                                   neighbour twice (lets the first sweep of
                                   level 0 skip aggregation; graphs built by
                                   this library are known to be distinct) */
    int32_t bin5_block;         /* threads per vertex of degree bin 5: 256
                                   (default, 0) or 512 */
    int32_t bin_max[3];         /* upper degrees of bins 4, 5, 6 (0 = default
                                   256 / 2048 / 8192; each at most its default,
                                   non-decreasing, bin 4 at least 32); larger
                                   rows go to the next bin, above bin 6 to the
                                   multi-CTA hub path.  Any values give the same
                                   partition; gala_autotune picks fast ones. */
    int32_t refine;             /* 1 = Leiden-style refinement (no counterpart in
                                   the reference): a round that gained at least
                                   min_modularity contracts the refinement of its
                                   communities into well-connected
                                   sub-communities, and the next round starts
                                   from the communities; single graphs only
                                   (integer or float weights; not with batches,
                                   proposals or level_dir).  0 = the
                                   reference's rounds. */
    /* Checkpoints (no counterpart in the reference, which never writes its
       partition, louvain.cu:226): when set, after every round r the
       contracted graph is written to <level_dir>/level_<r+1>.bin (the .bin
       layout with int32 weights) and the community of every input vertex in
       that graph to <level_dir>/labels_<r+1>.bin (int32 per input vertex).
       A run resumes from round r+1 on level_<r+1>.bin (weighted); its labels
       composed with labels_<r+1> are the full run's.  Not for batches or
       float-weight graphs. */
    const char *level_dir;
    int32_t proposal_from;      /* SKIP: the first sweep of a level that decides
                                   only proposed vertices (0 = 2, the sweep after
                                   the level's first; larger values keep more
                                   sweeps of every level plain) */
    int32_t batch_mode;         /* gala_louvain_batch: 0 = one persistent launch
                                   in which each CTA runs a whole graph (every
                                   round) when all graphs have at most 4096
                                   vertices, else the union run; 1 = always the
                                   union run (every sweep one set of launches
                                   for all graphs).  Both give the same
                                   partitions. */
} gala_options;

/* Tuning of the degree bins (the fields of gala_options they set). */
typedef struct {
    int32_t bin_max[3];
    int32_t bin5_block;
    double ms;                  /* device time of one run with this tuning */
    double default_ms;          /* device time of one run with the defaults */
    int32_t candidates;         /* configurations timed */
    int32_t reserved;
} gala_tuning;

typedef struct {
    double modularity;                 /* final Q */
    int32_t num_vertices;              /* input vertex count */
    int32_t num_communities;           /* final community count */
    int32_t num_levels;                /* rounds run */
    int32_t total_iterations;          /* phase-1 iterations over all rounds */
    double level_modularity[GALA_MAX_LEVELS];
    int32_t level_communities[GALA_MAX_LEVELS];
    int32_t level_iterations[GALA_MAX_LEVELS];
    /* optional per-iteration Q trace, caller-owned (may be NULL) */
    double *iter_modularity;
    int32_t iter_capacity;
    int32_t iter_count;
    /* timings (ms), measured with CUDA events on the context's stream */
    double time_total_ms;       /* all rounds, device-resident graph */
    double time_phase1_ms;      /* all phase-1 work */
    double time_decide_ms;      /* decide-and-move sweeps only */
    double time_update_ms;      /* weight update + prune sweeps */
    double time_contract_ms;    /* phase-2 contraction */
    double time_h2d_ms;         /* host->device copy (gala_louvain only) */
    double time_d2h_ms;         /* device->host copy of labels */
    /* roofline bookkeeping for the decide-and-move sweeps */
    int64_t decide_sweeps;
    int64_t decide_bytes;       /* algorithmic bytes over all sweeps */
    int64_t update_bytes;       /* algorithmic bytes of the update sweeps */
    int64_t kernel_launches;    /* kernels launched by this call */
    int64_t h2d_bytes;
    int64_t d2h_bytes;
    /* vertex decisions taken with the FP64 gain expressions (the others use
       exact integer gains; see gala_options.fp64_gains) */
    int64_t fp64_decisions;
    /* proposal modes */
    int64_t decisions;          /* vertices decided (all sweeps) */
    int64_t skipped;            /* active vertices the network skipped (SKIP) */
    int32_t verify_sweeps;      /* plain sweeps run because a proposal sweep
                                   gained less than min_modularity (SKIP) */
    int32_t incremental_sweeps; /* sweeps whose weight update was incremental
                                   (gala_context_set_update_mode) */
    int64_t samples;            /* training samples recorded (TRACE) */
    /* per round: the level graph it ran on, its times and its moves */
    int32_t level_vertices[GALA_MAX_LEVELS];
    int64_t level_entries[GALA_MAX_LEVELS];      /* CSR entries (2x edges) */
    double level_phase1_ms[GALA_MAX_LEVELS];
    double level_decide_ms[GALA_MAX_LEVELS];
    double level_update_ms[GALA_MAX_LEVELS];
    double level_contract_ms[GALA_MAX_LEVELS];
    int64_t level_movers[GALA_MAX_LEVELS];       /* moves applied, all sweeps */
    int64_t level_active_entries[GALA_MAX_LEVELS]; /* row entries decided, all sweeps */
    /* host wall time (ms) of gala_louvain: the whole call, up to the end of
       the host->device copy, the rounds, the device->host copy of labels */
    double host_total_ms;
    double host_h2d_ms;
    double host_run_ms;
    double host_d2h_ms;
} gala_result;

/* ---- errors / info --------------------------------------------------- */
const char *gala_last_error(void);
const char *gala_status_string(gala_status s);
/* Number of kernels the library launched in this process so far. */
int64_t gala_kernel_launch_count(void);
void gala_default_options(gala_options *opt);

/* ---- host graph I/O ---------------------------------------------------- */
/* Replaces Graph::load_bin_graph (src/graph/graph.cpp:177-219).  weighted=1
 * reads the weight block (the reference ignores its -w flag here, graph.cpp:200;
 * this loader honours it).  Rejects truncated or inconsistent files. */
gala_status gala_graph_load_bin(const char *path, int32_t weighted, gala_graph **out);
/* Replaces Graph::store_bin_graph (src/graph/graph.cpp:153-174). */
gala_status gala_graph_store_bin(const gala_graph *g, const char *path);
/* Replaces Graph::Graph(file, is_wt) (src/graph/graph.cpp:18-151): parse an
 * edge list "src dst [w]" ('#' lines skipped), symmetrise, deduplicate per
 * row (weights of duplicates summed when weighted), drop ids without edges
 * and renumber densely in id order.  nthreads <= 0 uses all cores. */
gala_status gala_graph_from_text(const char *path, int32_t weighted, int32_t nthreads,
                                 gala_graph **out);
/* Copy a caller-owned CSR in reference layout (inclusive offsets, no leading
 * 0).  weights may be NULL (all 1). */
gala_status gala_graph_from_csr(int32_t n, const int64_t *offsets_inclusive,
                                const int32_t *neighbors, const int32_t *weights,
                                gala_graph **out);
/* weighted: 0 = unweighted, 1 = int32 weights, 2 = float32 weights. */
gala_status gala_graph_info(const gala_graph *g, int32_t *n, int64_t *num_entries,
                            int32_t *weighted);
/* Float-weight graphs (no counterpart in the reference, whose weights are
 * int32): weights must be positive and finite.  The engine holds them as
 * exact 64-bit fixed-point integers round(w * 2^S) (S chosen from the total
 * weight so that it stays below 2^62), accumulates K, Tot, In and contracted
 * weights exactly in those integers and evaluates every gain and the pruning
 * bound with the FP64 expressions.  Results repeat bit-exactly; modularity is
 * reported from the fixed-point sums.  gala_graph_load_bin / store_bin with
 * weighted = 2 read / write the .bin layout with a float32 weight block. */
gala_status gala_graph_from_csr_f32(int32_t n, const int64_t *offsets_inclusive,
                                    const int32_t *neighbors, const float *weights,
                                    gala_graph **out);
/* Borrow the float weights (NULL for graphs without float weights). */
gala_status gala_graph_weights_f32(const gala_graph *g, const float **weights);
/* Borrow the host arrays (reference layout).  Valid until destroy. */
gala_status gala_graph_arrays(const gala_graph *g, const int64_t **offsets_inclusive,
                              const int32_t **neighbors, const int32_t **weights);
void gala_graph_destroy(gala_graph *g);

/* ---- synthetic graphs (seeded) ---------------------------------------- */
/* Planted-partition SBM: n vertices in k equal blocks, p_in / p_out. */
gala_status gala_generate_sbm(int32_t n, int32_t k, double p_in, double p_out,
                              uint64_t seed, gala_graph **out);
/* `count` planted-partition graphs of uneven sizes (no counterpart in the
 * reference): graph i has n log-uniform in [n_min, n_max], k uniform in
 * [k_min, k_max] equal blocks (fewer when the blocks could not hold the
 * degree), expected degree d uniform in [deg_min, deg_max] and mixing mu
 * uniform in [mix_min, mix_max] (p_in = d (1 - mu) / (n/k - 1),
 * p_out = d mu / (n - n/k)).  out receives count graphs; graph i depends only
 * on seed and i. */
gala_status gala_generate_sbm_batch(int32_t count, int32_t n_min, int32_t n_max, int32_t k_min,
                                    int32_t k_max, double deg_min, double deg_max, double mix_min,
                                    double mix_max, uint64_t seed, int32_t nthreads, gala_graph **out);
/* LFR-style planted graph (no counterpart in the reference): n vertices,
 * degrees power-law with exponent tau1 on [dmin, dmax], community sizes
 * power-law with exponent tau2 on [cmin, cmax], mixing mu (a fraction 1 - mu
 * of every vertex's edges inside its community), configuration-model
 * pairing, self-loops dropped, parallel edges merged.  float_weights = 1
 * gives lognormal(0, 1) float32 weights (parallel edges sum), 0 no weights.
 * Depends only on the arguments, not on nthreads. */
gala_status gala_generate_lfr(int32_t n, double tau1, int32_t dmin, int32_t dmax, double tau2,
                              int32_t cmin, int32_t cmax, double mu, int32_t float_weights,
                              uint64_t seed, int32_t nthreads, gala_graph **out);
/* R-MAT with 2^scale ids and `edges` raw undirected samples; duplicates and
 * self-loops removed, ids without edges dropped and renumbered in order.
 * noise > 0 perturbs a, b, c, d independently by a factor in
 * [1 - noise, 1 + noise] at every recursion level of every edge (then
 * renormalises), which smooths the degree staircase of plain R-MAT.
 * keep_isolated = 1 keeps all 2^scale ids (ids without edges become vertices
 * of degree 0) instead of dropping them.  The graph depends only on the
 * arguments, not on nthreads. */
gala_status gala_generate_rmat(int32_t scale, int64_t edges, double a, double b,
                               double c, double noise, int32_t keep_isolated, uint64_t seed,
                               int32_t nthreads, gala_graph **out);

/* ---- device context ---------------------------------------------------- */
gala_status gala_context_create(int32_t device, int32_t max_vertices, int64_t max_entries,
                                gala_context **out);
void gala_context_destroy(gala_context *ctx);
/* Run the context's work on a caller-owned CUDA stream (a cudaStream_t passed
 * as void*); NULL goes back to the context's own stream.  The reference runs
 * everything on the default stream with device-wide syncs
 * (louvain_main_process.cu:594-857); here all work of a context is ordered
 * on one stream and only that stream is synchronised. */
gala_status gala_context_set_stream(gala_context *ctx, void *stream);
/* Cap the global hash table of every hub (a vertex of degree > 8192 whose
 * neighbour communities are summed by many CTAs) at `slots` (a power of two
 * >= 32; 0 = sized by degree, at most 2/3 full, the default).  A cap below a
 * hub's count of distinct neighbour communities makes that table's bounded
 * probes run out: the run stops with GALA_ERR_OVERFLOW instead of dropping
 * weight (the reference drops it silently,
 * src/louvain_gpu/kernel_functions.cu:217), and the context stays usable.
 * For tests of that error path; no counterpart in the reference. */
gala_status gala_context_set_hub_table_cap(gala_context *ctx, int64_t slots);
/* Weight update of the phase-1 sweeps (compute_In / compute_In_blk,
 * src/louvain_gpu/kernel_functions.cu:890-1034, sums In over every row after
 * every sweep).  mode 0 (default): on levels of at least 2^23 entries, a
 * sweep whose movers' rows (like those of the sweep before it) hold under a
 * third of the level's entries updates In incrementally - each mover's In is
 * summed again over its row and +-w is pushed from each mover to its
 * neighbours that did not move - on graphs whose every entry (v, u, w) has a
 * mirror (u, v, w), checked once per run; mode 1: always the full update;
 * mode 2: incrementally whenever allowed (symmetric graph, from a level's
 * second sweep on).  Integer sums: every mode gives the same In, active sets
 * and results bit for bit.  Plain runs of one graph only; proposal runs and
 * batches always take the full update. */
gala_status gala_context_set_update_mode(gala_context *ctx, int32_t mode);

/* Aggregation of the contraction rows longer than 8192 entries inside a
 * Louvain run (rows in any order; the reference's contraction,
 * build_compressed_graph.cu:5-173 with kernel_functions.cu:1083-1694, builds
 * every row with a per-community hash table).  mode 0 (default): each
 * 4096-entry chunk of a
 * row is summed per neighbour community in shared memory, its distinct
 * communities are partitioned by id range (8192 ids per bucket) and every
 * (row, bucket) is summed in one shared-memory table, whenever the level has
 * at most 2^24 rows and the scratch holds the work lists; mode 1: every chunk
 * adds its sums into a global hash table of the row.  Both give the same rows
 * up to their order, and the same results.  Sorted rows
 * (gala_contract_device) always take the global tables. */
gala_status gala_context_set_long_rows(gala_context *ctx, int32_t mode);
/* Host -> device copy of gala_louvain: with chunks = 2..16 (8 by default) a
 * page-locked (gala_graph_pin) unweighted graph of at least 2^22 entries has
 * its neighbour array copied in that many row-range chunks on a second
 * stream, and the first sweep of level 0 initialises and decides the
 * vertices of each chunk as soon as it has arrived (a vertex's first decision
 * needs only its own row and the degrees), so the copy overlaps the first
 * sweep.  chunks = 0: one copy, then the run.  The results are the same bit
 * for bit. */
gala_status gala_context_set_copy_overlap(gala_context *ctx, int32_t chunks);
/* Page-lock the host arrays of g so host<->device copies run at full
 * bandwidth; gala_graph_destroy unpins them.  Needs a CUDA device. */
gala_status gala_graph_pin(gala_graph *g);

/* ---- Louvain ------------------------------------------------------------ */
/* Replaces louvain_gpu(Graph&, vertex_t*, double, int, int)
 * (src/louvain_gpu/louvain.cuh:8, louvain.cu:136-229) running the multi-round
 * loop of louvain.cu:193-226.  Copies the host graph to the device, runs all
 * rounds and writes the final community of every input vertex to
 * community_out (host, length n).  ctx may be NULL (a temporary context is
 * created on device 0). */
gala_status gala_louvain(gala_context *ctx, const gala_graph *g, const gala_options *opt,
                         int32_t *community_out, gala_result *res);

/* Same run on a device-resident CSR in device layout.  community_out is a
 * device pointer of length n.  The input arrays are not modified. */
gala_status gala_louvain_device(gala_context *ctx, int32_t n, const int64_t *d_offsets,
                                const int32_t *d_neighbors, const int32_t *d_weights,
                                const gala_options *opt, int32_t *d_community_out,
                                gala_result *res);

/* Batched graphs (no counterpart in the reference): `count` independent
 * graphs run together as one block-diagonal union graph, every sweep of
 * every level being one set of launches for all graphs.  Each graph keeps
 * its own total weight m2, minimum community weight, modularity, iteration
 * convergence and round rule, so its partition equals the one gala_louvain
 * gives for it alone.  community_out (host, sum of the graphs' vertex
 * counts, graph after graph) receives each vertex's community id local to
 * its graph (dense from 0); modularity_out / communities_out (host, count
 * entries, optional) the final Q and community count of each graph.  The
 * context must hold the union (sum of vertices and entries); ctx may be NULL.
 * Proposal modes are not available in a batch. */
typedef struct {
    int32_t num_graphs;
    int32_t num_levels;        /* rounds run (the longest graph's) */
    int32_t total_iterations;  /* phase-1 sweeps over all rounds */
    int32_t reserved;
    int64_t vertices;          /* union vertices */
    int64_t entries;           /* union CSR entries */
    double time_total_ms;      /* all rounds, device-resident union */
    double time_phase1_ms;
    double time_contract_ms;
    double time_h2d_ms;
    double time_d2h_ms;
    int64_t kernel_launches;
    int64_t h2d_bytes;
    int64_t d2h_bytes;
} gala_batch_result;
/* Autotuner of the degree bins (no counterpart in the reference): times full
 * runs (gala_louvain for one graph, gala_louvain_batch for count > 1) with
 * candidate bin limits and bin-5 block sizes - a coordinate search over the
 * bin-4 upper degree {64, 128, 256}, bin 5 {1024, 2048}, bin 6 {4096, 8192}
 * and the bin-5 block {256, 512}, each point the minimum of `repeats` runs -
 * and returns the fastest (every candidate gives the same partition).  The
 * other fields of opt apply to every run. */
gala_status gala_autotune(gala_context *ctx, const gala_graph *const *graphs, int32_t count,
                          const gala_options *opt, int32_t repeats, gala_tuning *out);

gala_status gala_louvain_batch(gala_context *ctx, const gala_graph *const *graphs, int32_t count,
                               const gala_options *opt, int32_t *community_out,
                               double *modularity_out, int32_t *communities_out,
                               gala_batch_result *res);

/* One phase-1 run (decide-and-move iterations until the Q gain is below
 * min_modularity) on a device CSR.  Replaces louvain_main_process
 * (src/louvain_gpu/louvain.cuh:10-16, louvain_main_process.cu:237-1060).
 * d_community_out (device, length n) receives the accepted partition;
 * *modularity receives its Q; iter_q (host, optional) the Q of every
 * iteration including iteration 0. */
gala_status gala_phase1_device(gala_context *ctx, int32_t n, const int64_t *d_offsets,
                               const int32_t *d_neighbors, const int32_t *d_weights,
                               double min_modularity, int32_t *d_community_out,
                               double *modularity, double *iter_q, int32_t iter_capacity,
                               int32_t *iterations);

/* Contract a partition into a community graph.  Replaces
 * build_compressed_graph (src/louvain_gpu/louvain.cuh:18-22,
 * build_compressed_graph.cu:5-173).  Communities are renumbered densely in
 * ascending order of their label; d_community (device, length n) is
 * rewritten in place with the new ids (as the reference does,
 * build_compressed_graph.cu:22-23).  The output CSR (device layout) goes to
 * caller buffers: d_new_offsets (n+1), d_new_neighbors / d_new_weights
 * (capacity >= number of input entries).  Rows are sorted by neighbour id. */
gala_status gala_contract_device(gala_context *ctx, int32_t n, const int64_t *d_offsets,
                                 const int32_t *d_neighbors, const int32_t *d_weights,
                                 int32_t *d_community, int64_t *d_new_offsets,
                                 int32_t *d_new_neighbors, int32_t *d_new_weights,
                                 int32_t *num_communities, int64_t *num_entries);

/* ---- learned move proposal (no counterpart in the reference) ---------- */
/* Create a network with seeded random weights and room for max_samples
 * training samples (8 features + label each) on `device`. */
gala_status gala_proposal_create(int32_t device, int64_t max_samples, uint64_t seed,
                                 gala_proposal **out);
void gala_proposal_destroy(gala_proposal *p);
/* FP32 master weights (count = 1377: W1[32][8], b1, W2[32][32], b2, w3, b3). */
gala_status gala_proposal_get_params(gala_proposal *p, float *params, int32_t capacity,
                                     int32_t *count);
gala_status gala_proposal_set_params(gala_proposal *p, const float *params, int32_t count);
/* Samples recorded so far by GALA_PROPOSAL_TRACE runs (and how many moved). */
gala_status gala_proposal_samples(gala_proposal *p, int64_t *count, int64_t *positives);
gala_status gala_proposal_clear_samples(gala_proposal *p);
gala_status gala_proposal_read_samples(gala_proposal *p, int64_t first, int64_t n, float *features,
                                       float *labels);
/* Weighted BCE loss and its gradient (summed over the n samples, FP32) of
 * caller samples under the master weights, computed by the GPU backward
 * kernel; n <= 65536. */
gala_status gala_proposal_gradient(gala_proposal *p, const float *features, const float *labels,
                                   int32_t n, float pos_weight, float *grad_out, float *loss_out);
/* Logits of caller samples with the BF16 inference weights; n <= 65536. */
gala_status gala_proposal_logits(gala_proposal *p, const float *features, int32_t n, float *logits);
/* Adam on the GPU over the recorded samples. */
gala_status gala_proposal_train(gala_proposal *p, int32_t epochs, int32_t batch_size, float lr,
                                float pos_weight, uint64_t seed, float *final_loss);

/* Host FP64 modularity of a partition of a host graph (the host check the
 * reference keeps at src/louvain_gpu/kernel_functions.cu:1037-1079). */
gala_status gala_modularity_host(const gala_graph *g, const int32_t *community, double *q);

/* Modularity of a partition of a device CSR (device layout) on the current
 * device, for callers that must not allocate device memory - e.g. a host
 * application whose device memory is all owned by its own pool allocator, or
 * a latency-bound path where cudaMalloc/cudaFree and the synchronisation they
 * can cause are not allowed.  No counterpart in the reference.
 * It calls no cudaMalloc, cudaFree or allocating library routine: its scratch
 * (per-community totals and three sums) is a file-scope device array that
 * every GPU loading the library holds until the process exits, sized for at
 * most 1,048,576 vertices (8 MB); larger n returns GALA_ERR_CAPACITY.
 * The first call on a device looks up the array's device address (make it
 * before any stream capture).  All calls on a device share the scratch and
 * clear it first; calls that overlap on the GPU (several host threads at
 * once on one device) race.  Runs on the legacy default stream and returns
 * after the result is on the host.  That stream is not ordered after
 * non-blocking streams (e.g. PyTorch's side streams): the caller must finish
 * the work that wrote d_offsets, d_neighbors, d_weights and d_community
 * (synchronise that stream, or make the default stream wait on an event
 * recorded on it) before the call.  Weights must be positive (as in every
 * graph of this library); sums are exact (Tot^2 in 128 bits), so any total
 * weight below 2^64 gives the right Q.  A label outside [0, n) or a weight
 * that is not positive returns GALA_ERR_INVALID. */
gala_status gala_modularity_device_static(int32_t n, const int64_t *d_offsets,
                                          const int32_t *d_neighbors, const int32_t *d_weights,
                                          const int32_t *d_community, double *modularity);

#ifdef __cplusplus
}
#endif
#endif /* GALA_H */
