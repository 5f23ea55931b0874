/*
 * louvain_oracle.c - CPU restatement of the reference's GPU Louvain path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA engine and the timed CPU
 * baseline.  The engine does not link or call this file.
 *
 * Reference: LinXi-lx/GALA-mg.  The reference runs each phase-1 iteration
 * with synchronous (Jacobi) semantics: every vertex decides from the labels
 * and community totals of the previous iteration (prev_community, Tot), the
 * moves are applied after the sweep (louvain_main_process.cu:571-1029).  The
 * restatement below therefore gives the same partition independent of the
 * order vertices are visited in, and parallelises over vertices.
 *
 * Compile with -ffp-contract=off: the FP64 expressions below must round
 * exactly as written (no fused multiply-add), like the engine's kernels.
 *
 * Weights are held as int64 internally: the reference's int32 weights
 * promote exactly, and float-weight graphs (no counterpart in the reference)
 * enter as 64-bit fixed-point integers (orc_fixed_shift / orc_fixed_weights),
 * the representation the engine uses for them.  Sums of Tot^2 are exact in
 * 128 bits.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128;
#ifdef _OPENMP
#include <omp.h>
#endif

double orc_q_from_sums(int64_t sum_in, int64_t sum_tot2, int64_t m2)
{
    /* Q = sum(In)/m2 - sum(Tot^2)/m2^2 (louvain_main_process.cu:990-999 with
     * modularity_op, kernel_functions.cuh:77-87), from exact integer sums. */
    double c = 1.0 / (double)m2;
    return (double)sum_in * c - (double)sum_tot2 * c * c;
}

/* The same with a 128-bit sum of Tot^2 given as (hi, lo) words, converted
 * as hi * 2^64 + lo (the engine's host code uses the same expression). */
double orc_q_from_sums128(int64_t sum_in, uint64_t tot2_lo, uint64_t tot2_hi, int64_t m2)
{
    double c = 1.0 / (double)m2;
    double t2 = (double)tot2_hi * 18446744073709551616.0 + (double)tot2_lo;
    return (double)sum_in * c - t2 * c * c;
}

static double q_of(int64_t sum_in, u128 sum_tot2, int64_t m2)
{
    return orc_q_from_sums128(sum_in, (uint64_t)sum_tot2, (uint64_t)(sum_tot2 >> 64), m2);
}

/* Fixed-point shift S of a float-weight graph: the weights are held as
 * round(w * 2^S) in int64 with S = 61 - e, 2^e >= sum(w) (frexp), capped to
 * [0, 40], so the total stays below 2^62.  The sum runs in entry order.
 * Returns -1 when a weight is not positive and finite or rounds to 0. */
int32_t orc_fixed_shift(const float *w, int64_t E)
{
    double sum = 0, mn = INFINITY;
    for (int64_t e = 0; e < E; ++e) {
        const double x = (double)w[e];
        if (!(x > 0) || !isfinite(x)) return -1;
        sum += x;
        if (x < mn) mn = x;
    }
    int ex = 0;
    frexp(sum > 0 ? sum : 1.0, &ex);
    int s = 61 - ex;
    if (s > 40) s = 40;
    if (s < 0) s = 0;
    if (E > 0 && llrint(mn * ldexp(1.0, s)) <= 0) return -1;
    return s;
}

void orc_fixed_weights(const float *w, int64_t E, int32_t shift, int64_t *out)
{
    const double scale = ldexp(1.0, shift);
    for (int64_t e = 0; e < E; ++e) out[e] = llrint((double)w[e] * scale);
}

/* Gain of moving a vertex into community cn before the correction for the
 * vertex's own community: kernel_functions.cu:136 / :362 (same order of the
 * FP64 operations). */
static inline double dq_of(int64_t w_to_c, int64_t ki, int64_t tot_c, int64_t tot_cur,
                           double constant)
{
    return 2.0 * (double)w_to_c - 2.0 * (double)ki * ((double)tot_c - (double)tot_cur + (double)ki) * constant;
}

typedef struct {
    int64_t *acc;     /* dense per-community weight accumulator, zero between uses */
    int32_t *touched; /* communities with acc != 0 */
} scratch_t;

/* Decide one vertex: kernel_functions.cu:289-441 (degree < 32),
 * :473-593 (degree 32-128), :640-813 (degree >= 129).  Returns the new label. */
static int32_t decide_vertex(int32_t v, const int64_t *offs, const int32_t *nbr, const int64_t *w,
                             const int32_t *prev, const int64_t *K, const int64_t *Self,
                             const int64_t *Tot, const int32_t *size, double constant,
                             scratch_t *s)
{
    int32_t cur = prev[v];
    int64_t ki = K[v];
    int32_t nt = 0;
    /* aggregate w(v, c) over neighbour communities (the hash tables of
     * insert_neighbor_com_info, kernel_functions.cu:102-221, or the shuffle
     * sum of :321-335) */
    for (int64_t e = offs[v]; e < offs[v + 1]; ++e) {
        int32_t c = prev[nbr[e]];
        int64_t wt = w ? w[e] : 1;
        if (s->acc[c] == 0) s->touched[nt++] = c;
        s->acc[c] += wt;
    }
    int64_t w_cur = s->acc[cur]; /* find_neighbor_com_info(cur_com), :513 / :684 */
    /* argmax with ties to the lowest id; only gains > 0 compete with the
     * initial state (0, cur): :136-142 and :366-379 */
    double maxdq = 0.0;
    int32_t best = cur;
    for (int32_t i = 0; i < nt; ++i) {
        int32_t c = s->touched[i];
        if (c != cur) {
            double dq = dq_of(s->acc[c], ki, Tot[c], Tot[cur], constant);
            if (dq > 0.0 && (dq > maxdq || (dq == maxdq && c < best))) {
                maxdq = dq;
                best = c;
            }
        }
        s->acc[c] = 0;
    }
    /* correction for leaving the own community: :381 / :532 / :748 */
    maxdq = maxdq - 2 * w_cur + 2 * Self[v];
    if (best >= 0 && best != cur && maxdq > 0) {
        /* singleton swap guard: :386-390 */
        if (size[best] == 1 && size[cur] == 1 && best > cur) return cur;
        return best;
    }
    return cur;
}

/* init (NULL: singletons) is the starting partition of a refined level (no
 * counterpart in the reference): Tot and size follow it, In is the weight
 * update of compute_In on it, and every vertex starts active. */
static int32_t phase1_w64(int32_t n, const int64_t *offs, const int32_t *nbr, const int64_t *w,
                          int64_t m2, double min_mod, int32_t *labels_out, double *q_out,
                          double *iter_q, int32_t iter_cap, int32_t *n_iter_q, int32_t nthreads,
                          const int32_t *init)
{
    if (n <= 0 || m2 <= 0) return -1;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    nthreads = 1;
#endif
    const double constant = 1 / (double)m2; /* louvain_main_process.cu:273 */
    int64_t *K = (int64_t *)calloc((size_t)n, sizeof(int64_t));
    int64_t *Self = (int64_t *)calloc((size_t)n, sizeof(int64_t));
    int64_t *Tot = (int64_t *)calloc((size_t)n, sizeof(int64_t));
    int32_t *size = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    int64_t *In = (int64_t *)calloc((size_t)n, sizeof(int64_t));
    int32_t *prev = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    int32_t *cur = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    unsigned char *active = (unsigned char *)calloc((size_t)n, 1);
    scratch_t *scr = (scratch_t *)calloc((size_t)nthreads, sizeof(scratch_t));
    for (int t = 0; t < nthreads; ++t) {
        scr[t].acc = (int64_t *)calloc((size_t)n, sizeof(int64_t));
        scr[t].touched = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    }

    /* init_communities (kernel_functions.cu:34-73): K = Tot = row weight sum,
     * Self = self-loop weight, label = own id, community size 1
     * (louvain_main_process.cu:337). */
    int64_t sum_in = 0;
    u128 sum_tot2 = 0;
    /* (the 128-bit square sum is accumulated outside the parallel loop) */
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 4096) reduction(+ : sum_in)
    for (int32_t v = 0; v < n; ++v) {
        int64_t k = 0, sf = 0;
        for (int64_t e = offs[v]; e < offs[v + 1]; ++e) {
            int64_t wt = w ? w[e] : 1;
            k += wt;
            if (nbr[e] == v) sf = wt;
        }
        K[v] = k;
        Tot[v] = k;
        Self[v] = sf;
        size[v] = 1;
        prev[v] = v;
        cur[v] = v;
        /* the first efficient_weight_updating (louvain_main_process.cu:538)
         * gives In = Self for the singleton partition */
        In[v] = sf;
        sum_in += sf;
        active[v] = 1;
    }
    if (init) {
        for (int32_t v = 0; v < n; ++v) {
            Tot[v] = 0;
            size[v] = 0;
        }
        for (int32_t v = 0; v < n; ++v) {
            prev[v] = cur[v] = init[v];
            Tot[init[v]] += K[v];
            size[init[v]] += 1;
        }
        sum_in = 0;
        for (int32_t v = 0; v < n; ++v) {
            int64_t s = 0;
            for (int64_t e = offs[v]; e < offs[v + 1]; ++e)
                if (init[nbr[e]] == init[v]) s += w ? w[e] : 1;
            In[v] = s;
            sum_in += s;
        }
        for (int32_t c = 0; c < n; ++c) sum_tot2 += (u128)(uint64_t)Tot[c] * (uint64_t)Tot[c];
    } else {
        for (int32_t v = 0; v < n; ++v) sum_tot2 += (u128)(uint64_t)K[v] * (uint64_t)K[v];
    }
    double q = q_of(sum_in, sum_tot2, m2);
    int32_t nq = 0;
    if (iter_q && nq < iter_cap) iter_q[nq] = q;
    nq++;
    double prev_q = q;

    for (;;) {
        /* decide-and-move over the active set (louvain_main_process.cu:594-857):
         * every decision reads prev / Tot / size of the previous iteration. */
#pragma omp parallel num_threads(nthreads)
        {
            int tid = 0;
#ifdef _OPENMP
            tid = omp_get_thread_num();
#endif
#pragma omp for schedule(dynamic, 1024)
            for (int32_t v = 0; v < n; ++v) {
                int32_t nv = prev[v];
                if (active[v] && offs[v + 1] > offs[v])
                    nv = decide_vertex(v, offs, nbr, w, prev, K, Self, Tot, size, constant, &scr[tid]);
                cur[v] = nv;
            }
        }
        /* Tot += Tot_update, size += size_update (louvain_main_process.cu:949-953) */
        for (int32_t v = 0; v < n; ++v) {
            if (cur[v] != prev[v]) {
                Tot[cur[v]] += K[v];
                Tot[prev[v]] -= K[v];
                size[cur[v]] += 1;
                size[prev[v]] -= 1;
            }
        }
        /* min_Tot over non-empty communities, m2 when none (Tot_op,
         * kernel_functions.cuh:112-121, louvain_main_process.cu:955) */
        int64_t min_tot = m2;
        sum_tot2 = 0;
#pragma omp parallel for num_threads(nthreads) reduction(min : min_tot)
        for (int32_t c = 0; c < n; ++c) {
            int64_t t = Tot[c];
            if (t != 0 && t < min_tot) min_tot = t;
        }
        for (int32_t c = 0; c < n; ++c) sum_tot2 += (u128)(uint64_t)Tot[c] * (uint64_t)Tot[c];
        /* (the reference holds minTot in the int32 weight type) */
        const int64_t min_tot_i = min_tot;
        /* weight update + pruning (compute_In, kernel_functions.cu:890-955,
         * compute_In_blk :958-1034): In = weight to the own community, and
         * the vertex leaves the active set when the bound at :944 holds. */
        sum_in = 0;
#pragma omp parallel for num_threads(nthreads) schedule(dynamic, 4096) reduction(+ : sum_in)
        for (int32_t v = 0; v < n; ++v) {
            if (offs[v + 1] == offs[v]) { /* in no degree bin: never touched */
                active[v] = 1;
                continue;
            }
            int32_t c = cur[v];
            int64_t s = 0;
            for (int64_t e = offs[v]; e < offs[v + 1]; ++e)
                if (cur[nbr[e]] == c) s += w ? w[e] : 1;
            In[v] = s;
            sum_in += s;
            int64_t ki = K[v];
            active[v] = !(2 * (s - Self[v]) - (ki - Self[v]) +
                              (double)(min_tot_i - (Tot[c] - ki)) * constant * ki >
                          0);
        }
        q = q_of(sum_in, sum_tot2, m2);
        if (iter_q && nq < iter_cap) iter_q[nq] = q;
        nq++;
        /* convergence: louvain_main_process.cu:1004-1007; the partition of the
         * rejected iteration is dropped (prev_community is returned). */
        if (q - prev_q < min_mod) break;
        prev_q = q;
        memcpy(prev, cur, (size_t)n * sizeof(int32_t));
    }

    memcpy(labels_out, prev, (size_t)n * sizeof(int32_t));
    if (q_out) *q_out = prev_q;
    if (n_iter_q) *n_iter_q = nq;

    for (int t = 0; t < nthreads; ++t) {
        free(scr[t].acc);
        free(scr[t].touched);
    }
    free(scr);
    free(K); free(Self); free(Tot); free(size); free(In); free(prev); free(cur); free(active);
    return nq - 1;
}

static int64_t *promote(const int32_t *w, int64_t E)
{
    if (!w) return NULL;
    int64_t *o = (int64_t *)malloc((size_t)(E > 0 ? E : 1) * sizeof(int64_t));
    for (int64_t e = 0; e < E; ++e) o[e] = w[e];
    return o;
}

int32_t orc_phase1(int32_t n, const int64_t *offs, const int32_t *nbr, const int32_t *w,
                   int64_t m2, double min_mod, int32_t *labels_out, double *q_out,
                   double *iter_q, int32_t iter_cap, int32_t *n_iter_q, int32_t nthreads)
{
    if (n <= 0) return -1;
    int64_t *w64 = promote(w, offs[n]);
    int32_t r = phase1_w64(n, offs, nbr, w64, m2, min_mod, labels_out, q_out, iter_q, iter_cap, n_iter_q,
                           nthreads, NULL);
    free(w64);
    return r;
}

static int cmp_i32(const void *a, const void *b)
{
    int32_t x = *(const int32_t *)a, y = *(const int32_t *)b;
    return (x > y) - (x < y);
}

static int32_t contract_w64(int32_t n, const int64_t *offs, const int32_t *nbr, const int64_t *w,
                            const int32_t *labels, int32_t *relabel_out, int64_t *new_offs,
                            int32_t *new_nbr, int64_t *new_w, int64_t *new_entries)
{
    /* community sizes and dense renumbering in ascending label order
     * (build_compressed_graph.cu:11-24) */
    int32_t *newid = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    int32_t *cnt = (int32_t *)calloc((size_t)n + 1, sizeof(int32_t));
    for (int32_t v = 0; v < n; ++v) cnt[labels[v]]++;
    int32_t C = 0;
    for (int32_t c = 0; c < n; ++c) newid[c] = cnt[c] > 0 ? C++ : -1;
    for (int32_t v = 0; v < n; ++v) relabel_out[v] = newid[labels[v]];
    /* members of each community (gather_vertex_by_community, :32-37) */
    int64_t *moff = (int64_t *)calloc((size_t)C + 1, sizeof(int64_t));
    for (int32_t v = 0; v < n; ++v) moff[relabel_out[v] + 1]++;
    for (int32_t c = 0; c < C; ++c) moff[c + 1] += moff[c];
    int32_t *members = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    int64_t *pos = (int64_t *)malloc((size_t)C * sizeof(int64_t));
    for (int32_t c = 0; c < C; ++c) pos[c] = moff[c];
    for (int32_t v = 0; v < n; ++v) members[pos[relabel_out[v]]++] = v;
    /* new row of community c: (c', sum of w over member edges into c')
     * (compute_neighbors_weights*, kernel_functions.cu:1239-1561), listed in
     * ascending c' */
    int64_t *acc = (int64_t *)calloc((size_t)C, sizeof(int64_t));
    int32_t *touched = (int32_t *)malloc((size_t)C * sizeof(int32_t));
    int64_t out = 0;
    new_offs[0] = 0;
    for (int32_t c = 0; c < C; ++c) {
        int32_t nt = 0;
        for (int64_t i = moff[c]; i < moff[c + 1]; ++i) {
            int32_t v = members[i];
            for (int64_t e = offs[v]; e < offs[v + 1]; ++e) {
                int32_t cc = relabel_out[nbr[e]];
                if (acc[cc] == 0) touched[nt++] = cc;
                acc[cc] += w ? w[e] : 1;
            }
        }
        qsort(touched, (size_t)nt, sizeof(int32_t), cmp_i32);
        for (int32_t i = 0; i < nt; ++i) {
            new_nbr[out] = touched[i];
            new_w[out] = acc[touched[i]];
            acc[touched[i]] = 0;
            out++;
        }
        new_offs[c + 1] = out;
    }
    if (new_entries) *new_entries = out;
    free(newid); free(cnt); free(moff); free(members); free(pos); free(acc); free(touched);
    return C;
}

int32_t orc_contract(int32_t n, const int64_t *offs, const int32_t *nbr, const int32_t *w,
                     const int32_t *labels, int32_t *relabel_out, int64_t *new_offs,
                     int32_t *new_nbr, int32_t *new_w, int64_t *new_entries)
{
    const int64_t E = offs[n];
    int64_t *w64 = promote(w, E);
    int64_t *nw64 = (int64_t *)malloc((size_t)(E > 0 ? E : 1) * sizeof(int64_t));
    int64_t ne = 0;
    int32_t C = contract_w64(n, offs, nbr, w64, labels, relabel_out, new_offs, new_nbr, nw64, &ne);
    for (int64_t e = 0; e < ne; ++e) new_w[e] = (int32_t)nw64[e];
    if (new_entries) *new_entries = ne;
    free(w64);
    free(nw64);
    return C;
}

/* Leiden-style refinement of a level's phase-1 partition P (no counterpart in
 * the reference; the deterministic synchronous rule the engine implements):
 * every vertex starts as its own sub-community of its P-community C.  Per
 * sweep, a singleton v of degree 1..kRefineMaxDeg that is well connected,
 * w(v, C - v) m2 >= K_v (Tot_C - K_v), picks among the well connected
 * sub-communities r of C next to it, ext(r) m2 >= K_r (Tot_C - K_r) with ext(r)
 * the weight from r to the rest of C, the one of largest
 * X = w(v, r) m2 - K_v K_r (lowest id on ties) and targets it when X > 0.
 * A vertex moves to its target unless another vertex targets it, except when
 * exactly one does and that is its own target with a lower id (a mutual pair
 * joins the lower id).  Sweeps repeat while vertices move, at most
 * kRefineSweeps times.  R receives the sub-community labels (vertex ids). */
enum { kRefineMaxDeg = 256, kRefineSweeps = 8 };
typedef __int128 i128;
static void refine_w64(int32_t n, const int64_t *offs, const int32_t *nbr, const int64_t *w, int64_t m2,
                       const int32_t *P, int32_t *R)
{
    int64_t *K = (int64_t *)calloc((size_t)n, sizeof(int64_t));
    int64_t *totC = (int64_t *)calloc((size_t)n, sizeof(int64_t));
    int64_t *wC = (int64_t *)calloc((size_t)n, sizeof(int64_t));
    int64_t *ext = (int64_t *)calloc((size_t)n, sizeof(int64_t));
    int64_t *Kr = (int64_t *)calloc((size_t)n, sizeof(int64_t));
    int32_t *sz = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    int32_t *target = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    int32_t *marks = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    int64_t *acc = (int64_t *)calloc((size_t)n, sizeof(int64_t));
    int32_t *touched = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    for (int32_t v = 0; v < n; ++v) {
        int64_t k = 0, s = 0;
        for (int64_t e = offs[v]; e < offs[v + 1]; ++e) {
            const int64_t wt = w ? w[e] : 1;
            k += wt;
            if (nbr[e] != v && P[nbr[e]] == P[v]) s += wt;
        }
        K[v] = k;
        wC[v] = s;
        R[v] = v;
    }
    for (int32_t v = 0; v < n; ++v) totC[P[v]] += K[v];
    for (int sweep = 0; sweep < kRefineSweeps; ++sweep) {
        memset(Kr, 0, (size_t)n * sizeof(int64_t));
        memset(sz, 0, (size_t)n * sizeof(int32_t));
        memset(ext, 0, (size_t)n * sizeof(int64_t));
        for (int32_t v = 0; v < n; ++v) {
            Kr[R[v]] += K[v];
            sz[R[v]] += 1;
            for (int64_t e = offs[v]; e < offs[v + 1]; ++e) {
                const int32_t u = nbr[e];
                if (u != v && P[u] == P[v] && R[u] != R[v]) ext[R[v]] += w ? w[e] : 1;
            }
        }
        for (int32_t v = 0; v < n; ++v) {
            target[v] = -1;
            const int64_t deg = offs[v + 1] - offs[v];
            if (R[v] != v || sz[v] != 1 || deg < 1 || deg > kRefineMaxDeg) continue;
            const int32_t p = P[v];
            if (!((i128)wC[v] * m2 >= (i128)K[v] * (totC[p] - K[v]))) continue;
            int32_t nt = 0;
            for (int64_t e = offs[v]; e < offs[v + 1]; ++e) {
                const int32_t u = nbr[e];
                if (u == v || P[u] != p || R[u] == v) continue;
                if (acc[R[u]] == 0) touched[nt++] = R[u];
                acc[R[u]] += w ? w[e] : 1;
            }
            i128 bx = 0;
            int32_t best = -1;
            for (int32_t i = 0; i < nt; ++i) {
                const int32_t r = touched[i];
                if ((i128)ext[r] * m2 >= (i128)Kr[r] * (totC[p] - Kr[r])) {
                    const i128 x = (i128)acc[r] * m2 - (i128)K[v] * Kr[r];
                    if (x > 0 && (best < 0 || x > bx || (x == bx && r < best))) {
                        bx = x;
                        best = r;
                    }
                }
                acc[r] = 0;
            }
            target[v] = best;
        }
        memset(marks, 0, (size_t)n * sizeof(int32_t));
        for (int32_t v = 0; v < n; ++v)
            if (target[v] >= 0) marks[target[v]]++;
        int64_t moved = 0;
        for (int32_t v = 0; v < n; ++v) {
            const int32_t t = target[v];
            if (t < 0) continue;
            if (marks[v] == 0 || (marks[v] == 1 && target[t] == v && t < v)) {
                R[v] = t;
                moved++;
            }
        }
        if (!moved) break;
    }
    free(K); free(totC); free(wC); free(ext); free(Kr); free(sz); free(target); free(marks); free(acc); free(touched);
}

void orc_refine(int32_t n, const int64_t *offs, const int32_t *nbr, const int32_t *w, const int32_t *P,
                int32_t *R)
{
    const int64_t E = offs[n];
    int64_t *w64 = promote(w, E);
    int64_t m2 = 0;
    for (int64_t e = 0; e < E; ++e) m2 += w ? w[e] : 1;
    refine_w64(n, offs, nbr, w64, m2, P, R);
    free(w64);
}

/* Multi-round driver on int64 weights (NULL = all 1). */
/* refine: a round that gained at least min_mod contracts the refined
 * partition (see refine_w64), and the next round starts from the phase-1
 * communities, each labelled by its sub-community of lowest new id.  A round
 * that started so and gained less contracts its phase-1 communities instead
 * and the rounds go on (merging whole communities needs the plain
 * aggregation); a round that started from singletons and gained less is the
 * last, as without refinement. */
static int32_t louvain_w64(int32_t n, const int64_t *offs, const int32_t *nbr, const int64_t *w,
                           double min_mod, int32_t max_levels, int32_t *comm_out, double *level_q,
                           int32_t *level_c, int32_t *level_iters, int32_t level_cap, double *iter_q,
                           int32_t iter_cap, int32_t *n_iter_q, int32_t nthreads, int refine)
{
    if (n <= 0) return -1;
    int64_t E = offs[n];
    int64_t m2 = 0; /* thrust::reduce of the weights, louvain.cu:165-167 */
    for (int64_t e = 0; e < E; ++e) m2 += w ? w[e] : 1;
    if (m2 <= 0) return -1;

    int64_t *go = (int64_t *)malloc(((size_t)n + 1) * sizeof(int64_t));
    int32_t *gn = (int32_t *)malloc((size_t)(E > 0 ? E : 1) * sizeof(int32_t));
    int64_t *gw = (int64_t *)malloc((size_t)(E > 0 ? E : 1) * sizeof(int64_t));
    int64_t *no = (int64_t *)malloc(((size_t)n + 1) * sizeof(int64_t));
    int32_t *nn = (int32_t *)malloc((size_t)(E > 0 ? E : 1) * sizeof(int32_t));
    int64_t *nw = (int64_t *)malloc((size_t)(E > 0 ? E : 1) * sizeof(int64_t));
    int32_t *lab = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    int32_t *rl = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    int32_t *rlab = refine ? (int32_t *)malloc((size_t)n * sizeof(int32_t)) : NULL;
    int32_t *init = refine ? (int32_t *)malloc((size_t)n * sizeof(int32_t)) : NULL;
    int32_t *pmin = refine ? (int32_t *)malloc((size_t)n * sizeof(int32_t)) : NULL;
    int have_init = 0;
    memcpy(go, offs, ((size_t)n + 1) * sizeof(int64_t));
    memcpy(gn, nbr, (size_t)E * sizeof(int32_t));
    for (int64_t e = 0; e < E; ++e) gw[e] = w ? w[e] : 1;
    for (int32_t i = 0; i < n; ++i) comm_out[i] = i;

    int32_t cn = n, rounds = 0, nq_total = 0;
    double prev_mod = -1, cur_mod = -1;
    for (;;) {
        double q = 0;
        int32_t nq = 0;
        double *tr = iter_q ? iter_q + (nq_total < iter_cap ? nq_total : iter_cap) : NULL;
        int32_t cap = iter_q ? (iter_cap > nq_total ? iter_cap - nq_total : 0) : 0;
        int32_t it = phase1_w64(cn, go, gn, gw, m2, min_mod, lab, &q, tr, cap, &nq, nthreads,
                                have_init ? init : NULL);
        nq_total += nq;
        int64_t ne = 0;
        const int started_refined = have_init;
        const int gained = q - cur_mod >= min_mod;
        const int last = (!gained && !started_refined) || (max_levels > 0 && rounds + 1 >= max_levels);
        int32_t C;
        if (refine && !last && gained) {
            refine_w64(cn, go, gn, gw, m2, lab, rlab);
            C = contract_w64(cn, go, gn, gw, rlab, rl, no, nn, nw, &ne);
            for (int32_t v = 0; v < cn; ++v) pmin[v] = 0x7fffffff;
            for (int32_t v = 0; v < cn; ++v)
                if (rl[v] < pmin[lab[v]]) pmin[lab[v]] = rl[v];
            for (int32_t v = 0; v < cn; ++v) init[rl[v]] = pmin[lab[v]];
        } else {
            C = contract_w64(cn, go, gn, gw, lab, rl, no, nn, nw, &ne);
        }
        have_init = refine && !last && gained;
        /* labels of the input vertices follow the contraction (the gather of
         * louvain.cu:188-189, composed in the intended direction) */
        for (int32_t i = 0; i < n; ++i) comm_out[i] = rl[comm_out[i]];
        if (rounds < level_cap) {
            if (level_q) level_q[rounds] = q;
            if (level_c) level_c[rounds] = C;
            if (level_iters) level_iters[rounds] = it;
        }
        rounds++;
        prev_mod = cur_mod;
        cur_mod = q;
        int64_t *t64 = go; go = no; no = t64;
        int32_t *t32 = gn; gn = nn; nn = t32;
        t64 = gw; gw = nw; nw = t64;
        cn = C;
        /* round loop condition, louvain.cu:202 (a refined round that gained
         * less goes on with a plain contraction) */
        if (!(cur_mod - prev_mod >= min_mod) && !started_refined) break;
        if (max_levels > 0 && rounds >= max_levels) break;
    }
    if (n_iter_q) *n_iter_q = nq_total;
    free(go); free(gn); free(gw); free(no); free(nn); free(nw); free(lab); free(rl);
    free(rlab); free(init); free(pmin);
    return rounds;
}

int32_t orc_louvain(int32_t n, const int64_t *offs, const int32_t *nbr, const int32_t *w,
                    double min_mod, int32_t max_levels, int32_t *comm_out, double *level_q,
                    int32_t *level_c, int32_t *level_iters, int32_t level_cap, double *iter_q,
                    int32_t iter_cap, int32_t *n_iter_q, int32_t nthreads)
{
    if (n <= 0) return -1;
    int64_t *w64 = promote(w, offs[n]);
    int32_t r = louvain_w64(n, offs, nbr, w64, min_mod, max_levels, comm_out, level_q, level_c, level_iters,
                            level_cap, iter_q, iter_cap, n_iter_q, nthreads, 0);
    free(w64);
    return r;
}

int32_t orc_louvain_refine(int32_t n, const int64_t *offs, const int32_t *nbr, const int32_t *w,
                           double min_mod, int32_t max_levels, int32_t *comm_out, double *level_q,
                           int32_t *level_c, int32_t *level_iters, int32_t level_cap, double *iter_q,
                           int32_t iter_cap, int32_t *n_iter_q, int32_t nthreads)
{
    if (n <= 0) return -1;
    int64_t *w64 = promote(w, offs[n]);
    int32_t r = louvain_w64(n, offs, nbr, w64, min_mod, max_levels, comm_out, level_q, level_c, level_iters,
                            level_cap, iter_q, iter_cap, n_iter_q, nthreads, 1);
    free(w64);
    return r;
}

int32_t orc_louvain_fixed(int32_t n, const int64_t *offs, const int32_t *nbr, const int64_t *w,
                          double min_mod, int32_t max_levels, int32_t *comm_out, double *level_q,
                          int32_t *level_c, int32_t *level_iters, int32_t level_cap, double *iter_q,
                          int32_t iter_cap, int32_t *n_iter_q, int32_t nthreads)
{
    return louvain_w64(n, offs, nbr, w, min_mod, max_levels, comm_out, level_q, level_c, level_iters, level_cap,
                       iter_q, iter_cap, n_iter_q, nthreads, 0);
}

int32_t orc_louvain_fixed_refine(int32_t n, const int64_t *offs, const int32_t *nbr, const int64_t *w,
                                 double min_mod, int32_t max_levels, int32_t *comm_out, double *level_q,
                                 int32_t *level_c, int32_t *level_iters, int32_t level_cap, double *iter_q,
                                 int32_t iter_cap, int32_t *n_iter_q, int32_t nthreads)
{
    return louvain_w64(n, offs, nbr, w, min_mod, max_levels, comm_out, level_q, level_c, level_iters, level_cap,
                       iter_q, iter_cap, n_iter_q, nthreads, 1);
}

double orc_modularity_f32(int32_t n, const int64_t *offs, const int32_t *nbr, const float *w,
                          const int32_t *labels)
{
    /* the host check of kernel_functions.cu:1037-1079 with FP64 sums of the
     * float weights */
    double m2 = 0;
    for (int64_t e = 0; e < offs[n]; ++e) m2 += (double)w[e];
    double constant = 1.0 / m2;
    double *Tot = (double *)calloc((size_t)n, sizeof(double));
    double *In = (double *)calloc((size_t)n, sizeof(double));
    for (int32_t i = 0; i < n; ++i) {
        double degree = 0;
        for (int64_t j = offs[i]; j < offs[i + 1]; ++j) {
            degree += (double)w[j];
            if (labels[nbr[j]] == labels[i]) In[i] += (double)w[j];
        }
        Tot[labels[i]] += degree;
    }
    double q = 0;
    for (int32_t i = 0; i < n; ++i) q += In[i] * constant - Tot[i] * Tot[i] * constant * constant;
    free(Tot);
    free(In);
    return q;
}

double orc_modularity(int32_t n, const int64_t *offs, const int32_t *nbr, const int32_t *w,
                      const int32_t *labels)
{
    /* kernel_functions.cu:1037-1079: In per vertex, Tot per community, then
     * q += In[i]*c - Tot[i]^2*c^2 vertex by vertex. */
    int64_t m2 = 0;
    for (int64_t e = 0; e < offs[n]; ++e) m2 += w ? w[e] : 1;
    double constant = 1.0 / (double)m2;
    int64_t *Tot = (int64_t *)calloc((size_t)n, sizeof(int64_t));
    int64_t *In = (int64_t *)calloc((size_t)n, sizeof(int64_t));
    for (int32_t i = 0; i < n; ++i) {
        int64_t degree = 0;
        for (int64_t j = offs[i]; j < offs[i + 1]; ++j) {
            int32_t wt = w ? w[j] : 1;
            degree += wt;
            if (labels[nbr[j]] == labels[i]) In[i] += wt;
        }
        Tot[labels[i]] += degree;
    }
    double q = 0;
    for (int32_t i = 0; i < n; ++i)
        q += (double)In[i] * constant - (double)Tot[i] * (double)Tot[i] * constant * constant;
    free(Tot);
    free(In);
    return q;
}
