/*
 * oracle.h - CPU restatement of the reference's Louvain path.
 *
 * TEST INFRASTRUCTURE ONLY.  This code is the checker for the CUDA engine in
 * gala-mg_gb300/ and the timed CPU baseline of bench.py; the engine never
 * calls it.  Only tests/, __graft_entry__.smoke() and bench.py load it.
 *
 * Every function restates the reference (LinXi-lx/GALA-mg, src/...) with the
 * same decision rules and the same FP64 operation order; see the comments in
 * louvain_oracle.c for the file:line each step follows.
 *
 * CSR layout: offs[n+1] with a leading 0, nbr[offs[n]], w[offs[n]] or NULL
 * (all weights 1).
 */
#ifndef GALA_ORACLE_H
#define GALA_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Q from exact integer sums: sum_in = sum over vertices of In[v],
 * sum_tot2 = sum over communities of Tot[c]^2, m2 = total weight. */
double orc_q_from_sums(int64_t sum_in, int64_t sum_tot2, int64_t m2);

/* One phase-1 run (louvain_main_process).  Returns the number of phase-1
 * iterations run (>= 1), or -1 on bad input.  labels_out[n] receives the
 * accepted partition, *q_out its modularity, iter_q[] the Q of iteration 0..k. */
int32_t orc_phase1(int32_t n, const int64_t *offs, const int32_t *nbr, const int32_t *w,
                   int64_t m2, double min_mod, int32_t *labels_out, double *q_out,
                   double *iter_q, int32_t iter_cap, int32_t *n_iter_q, int32_t nthreads);

/* Contraction (build_compressed_graph) with rows sorted by neighbour id.
 * relabel_out[n] receives the new id of every vertex.  new_offs needs n+1
 * slots, new_nbr/new_w offs[n] slots.  Returns the community count. */
int32_t orc_contract(int32_t n, const int64_t *offs, const int32_t *nbr, const int32_t *w,
                     const int32_t *labels, int32_t *relabel_out, int64_t *new_offs,
                     int32_t *new_nbr, int32_t *new_w, int64_t *new_entries);

/* Multi-round driver (the loop at louvain.cu:193-226).  comm_out[n] receives
 * the final community of every input vertex.  Returns the number of rounds. */
/* Leiden-style refinement of a partition P (see louvain_oracle.c) and the
 * multi-round driver that contracts refined partitions. */
void orc_refine(int32_t n, const int64_t *offs, const int32_t *nbr, const int32_t *w, const int32_t *P,
                int32_t *R);
int32_t orc_louvain_refine(int32_t n, const int64_t *offs, const int32_t *nbr, const int32_t *w,
                           double min_mod, int32_t max_levels, int32_t *comm_out, double *level_q,
                           int32_t *level_c, int32_t *level_iters, int32_t level_cap, double *iter_q,
                           int32_t iter_cap, int32_t *n_iter_q, int32_t nthreads);
int32_t orc_louvain(int32_t n, const int64_t *offs, const int32_t *nbr, const int32_t *w,
                    double min_mod, int32_t max_levels, int32_t *comm_out, double *level_q,
                    int32_t *level_c, int32_t *level_iters, int32_t level_cap, double *iter_q,
                    int32_t iter_cap, int32_t *n_iter_q, int32_t nthreads);

/* Host FP64 modularity, summed vertex by vertex as the reference's host check
 * (kernel_functions.cu:1037-1079). */
double orc_modularity(int32_t n, const int64_t *offs, const int32_t *nbr, const int32_t *w,
                      const int32_t *labels);

/* Float-weight graphs (no counterpart in the reference): weights held as
 * 64-bit fixed-point integers round(w * 2^shift).  orc_fixed_shift returns
 * the shift (-1 for a weight that is not positive and finite or rounds to
 * 0); orc_louvain_fixed runs the multi-round driver on int64 weights;
 * orc_modularity_f32 is the FP64 host modularity of the float weights. */
int32_t orc_fixed_shift(const float *w, int64_t E);
void orc_fixed_weights(const float *w, int64_t E, int32_t shift, int64_t *out);
int32_t orc_louvain_fixed(int32_t n, const int64_t *offs, const int32_t *nbr, const int64_t *w,
                          double min_mod, int32_t max_levels, int32_t *comm_out, double *level_q,
                          int32_t *level_c, int32_t *level_iters, int32_t level_cap, double *iter_q,
                          int32_t iter_cap, int32_t *n_iter_q, int32_t nthreads);
/* the same with the refinement of orc_louvain_refine */
int32_t orc_louvain_fixed_refine(int32_t n, const int64_t *offs, const int32_t *nbr, const int64_t *w,
                                 double min_mod, int32_t max_levels, int32_t *comm_out, double *level_q,
                                 int32_t *level_c, int32_t *level_iters, int32_t level_cap, double *iter_q,
                                 int32_t iter_cap, int32_t *n_iter_q, int32_t nthreads);
double orc_modularity_f32(int32_t n, const int64_t *offs, const int32_t *nbr, const float *w,
                          const int32_t *labels);
/* Q from a 128-bit sum of Tot^2 (hi, lo words): hi * 2^64 + lo in FP64. */
double orc_q_from_sums128(int64_t sum_in, uint64_t tot2_lo, uint64_t tot2_hi, int64_t m2);

/* Seeded R-MAT graph (generators.c), byte-identical to the engine library's
 * gala_generate_rmat: *offs_out (n+1, leading 0) and *nbr_out are malloc'd;
 * release them with orc_free.  Returns 0, or -1 on bad arguments. */
int32_t orc_generate_rmat(int32_t scale, int64_t nedges, double a, double b, double c, double noise,
                          int32_t keep_isolated, uint64_t seed, int32_t nthreads, int32_t *n_out,
                          int64_t **offs_out, int32_t **nbr_out);
void orc_free(void *p);

/* The classic sequential (asynchronous, Blondel et al. 2008) Louvain method
 * on one thread (seq_louvain.c): the timed sequential CPU baseline, not a
 * restatement of the reference.  comm_out[n] receives the final community of
 * every vertex; level_q/level_c the Q and community count of every level;
 * *moves_out the number of moves.  Returns the number of levels. */
int32_t orc_seq_louvain(int32_t n, const int64_t *offs, const int32_t *nbr, const int32_t *w, double min_mod,
                        int32_t max_levels, int32_t *comm_out, double *level_q, int32_t *level_c, int32_t level_cap,
                        int64_t *moves_out);

#ifdef __cplusplus
}
#endif
#endif
