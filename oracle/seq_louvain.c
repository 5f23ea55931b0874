/*
 * seq_louvain.c - the classic sequential Louvain method on one CPU thread.
 *
 * TEST INFRASTRUCTURE ONLY: the timed sequential CPU baseline of bench.py
 * (a reported baseline, not the checker of the engine and not a restatement
 * of the reference, which has no host Louvain).  The engine never calls it.
 *
 * Algorithm: Blondel, Guillaume, Lambiotte & Lefebvre, "Fast unfolding of
 * communities in large networks" (J. Stat. Mech. 2008).  Local moving is
 * asynchronous: vertices are visited in id order, each leaves its community
 * and joins the neighbouring community of largest gain
 *     gain(c) = w(v, c) - Tot_c * K_v / m2
 * (strictly larger than its own community's to move; ties keep the first
 * community met in row order), and later vertices of the same pass see the
 * move at once.  Passes repeat while a pass raises Q by at least min_mod;
 * a level that raised Q by less than min_mod ends the run (the same 1e-6
 * rule the reference applies to iterations and rounds,
 * src/louvain_gpu/louvain_main_process.cu:1004-1007 and louvain.cu:202).
 * Otherwise the communities are contracted into a weighted graph (self-loop
 * entry = weight inside the community, both directions) and the next level
 * starts from singletons.
 *
 * Weights are int64 (int32 input weights, or all 1); Q is computed from exact
 * integer sums with one FP64 expression.
 */
#include "oracle.h"

#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 u128_t;

/* Q = sum_c In_c / m2 - sum_c Tot_c^2 / m2^2 with exact sums */
static double seq_q(int32_t n, const int64_t *offs, const int32_t *nbr, const int64_t *w, const int32_t *comm,
                    const int64_t *tot, int64_t m2)
{
    int64_t in = 0;
    for (int32_t v = 0; v < n; ++v)
        for (int64_t j = offs[v]; j < offs[v + 1]; ++j)
            if (comm[nbr[j]] == comm[v]) in += w[j];
    u128_t t2 = 0;
    for (int32_t c = 0; c < n; ++c) t2 += (u128_t)tot[c] * (u128_t)tot[c];
    return orc_q_from_sums128(in, (uint64_t)t2, (uint64_t)(t2 >> 64), m2);
}

int32_t orc_seq_louvain(int32_t n0, const int64_t *offs0, const int32_t *nbr0, const int32_t *w0, double min_mod,
                        int32_t max_levels, int32_t *comm_out, double *level_q, int32_t *level_c, int32_t level_cap,
                        int64_t *moves_out)
{
    if (n0 <= 0 || !offs0 || !comm_out) return -1;
    /* level graph (owned copies after level 0) */
    int32_t n = n0;
    int64_t E = offs0[n0];
    int64_t *offs = (int64_t *)malloc(((size_t)n + 1) * sizeof(int64_t));
    int32_t *nbr = (int32_t *)malloc((size_t)(E > 0 ? E : 1) * sizeof(int32_t));
    int64_t *w = (int64_t *)malloc((size_t)(E > 0 ? E : 1) * sizeof(int64_t));
    int64_t *K = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    int64_t *tot = (int64_t *)malloc((size_t)n * sizeof(int64_t));
    int32_t *comm = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    int64_t *acc = (int64_t *)calloc((size_t)n, sizeof(int64_t));
    int32_t *touched = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    int32_t *renum = (int32_t *)malloc((size_t)n * sizeof(int32_t));
    if (!offs || !nbr || !w || !K || !tot || !comm || !acc || !touched || !renum) return -1;
    memcpy(offs, offs0, ((size_t)n + 1) * sizeof(int64_t));
    memcpy(nbr, nbr0, (size_t)E * sizeof(int32_t));
    int64_t m2 = 0;
    for (int64_t j = 0; j < E; ++j) {
        w[j] = w0 ? (int64_t)w0[j] : 1;
        m2 += w[j];
    }
    for (int32_t v = 0; v < n0; ++v) comm_out[v] = v;
    if (m2 <= 0) {
        if (level_cap > 0) {
            level_q[0] = 0.0;
            level_c[0] = n0;
        }
        free(offs); free(nbr); free(w); free(K); free(tot); free(comm); free(acc); free(touched); free(renum);
        return 1;
    }
    const double inv_m2 = 1.0 / (double)m2;
    int64_t moves_total = 0;
    int32_t levels = 0;
    double q_prev_level = -1.0;
    for (;;) {
        for (int32_t v = 0; v < n; ++v) {
            int64_t k = 0;
            for (int64_t j = offs[v]; j < offs[v + 1]; ++j) k += w[j];
            K[v] = k;
            tot[v] = k;
            comm[v] = v;
        }
        double q = seq_q(n, offs, nbr, w, comm, tot, m2);
        const double q_start = q;
        /* local moving: passes until one gains less than min_mod */
        for (;;) {
            int64_t moves = 0;
            for (int32_t v = 0; v < n; ++v) {
                const int32_t cur = comm[v];
                int32_t nt = 0;
                for (int64_t j = offs[v]; j < offs[v + 1]; ++j) {
                    const int32_t u = nbr[j];
                    if (u == v) continue;
                    const int32_t c = comm[u];
                    if (acc[c] == 0) touched[nt++] = c;
                    acc[c] += w[j];
                }
                const double kv = (double)K[v];
                tot[cur] -= K[v];
                int32_t best = cur;
                double best_gain = (double)acc[cur] - (double)tot[cur] * kv * inv_m2;
                for (int32_t t = 0; t < nt; ++t) {
                    const int32_t c = touched[t];
                    const double g = (double)acc[c] - (double)tot[c] * kv * inv_m2;
                    if (g > best_gain) {
                        best_gain = g;
                        best = c;
                    }
                }
                tot[best] += K[v];
                if (best != cur) {
                    comm[v] = best;
                    ++moves;
                }
                for (int32_t t = 0; t < nt; ++t) acc[touched[t]] = 0;
            }
            moves_total += moves;
            const double q_new = seq_q(n, offs, nbr, w, comm, tot, m2);
            const double gain = q_new - q;
            q = q_new;
            if (moves == 0 || gain < min_mod) break;
        }
        /* community count and dense renumbering in ascending id */
        for (int32_t c = 0; c < n; ++c) renum[c] = -1;
        for (int32_t v = 0; v < n; ++v) renum[comm[v]] = 0;
        int32_t C = 0;
        for (int32_t c = 0; c < n; ++c)
            if (renum[c] == 0) renum[c] = C++;
        for (int32_t v = 0; v < n0; ++v) comm_out[v] = renum[comm[comm_out[v]]];
        if (levels < level_cap) {
            level_q[levels] = q;
            level_c[levels] = C;
        }
        ++levels;
        const double level_gain = q - (levels == 1 ? q_start : q_prev_level);
        q_prev_level = q;
        if (level_gain < min_mod || C == n || (max_levels > 0 && levels >= max_levels)) break;
        /* contraction: members grouped by community, rows aggregated with the
         * dense accumulator, entries in order of first appearance */
        int64_t *cstart = (int64_t *)calloc((size_t)C + 1, sizeof(int64_t));
        int32_t *members = (int32_t *)malloc((size_t)n * sizeof(int32_t));
        for (int32_t v = 0; v < n; ++v) cstart[renum[comm[v]] + 1]++;
        for (int32_t c = 0; c < C; ++c) cstart[c + 1] += cstart[c];
        int64_t *fill = (int64_t *)malloc((size_t)C * sizeof(int64_t));
        memcpy(fill, cstart, (size_t)C * sizeof(int64_t));
        for (int32_t v = 0; v < n; ++v) members[fill[renum[comm[v]]]++] = v;
        free(fill);
        int64_t *noffs = (int64_t *)malloc(((size_t)C + 1) * sizeof(int64_t));
        int32_t *nnbr = (int32_t *)malloc((size_t)(E > 0 ? E : 1) * sizeof(int32_t));
        int64_t *nw = (int64_t *)malloc((size_t)(E > 0 ? E : 1) * sizeof(int64_t));
        int64_t ne = 0;
        noffs[0] = 0;
        for (int32_t c = 0; c < C; ++c) {
            int32_t nt = 0;
            for (int64_t mi = cstart[c]; mi < cstart[c + 1]; ++mi) {
                const int32_t v = members[mi];
                for (int64_t j = offs[v]; j < offs[v + 1]; ++j) {
                    const int32_t d = renum[comm[nbr[j]]];
                    if (acc[d] == 0) touched[nt++] = d;
                    acc[d] += w[j];
                }
            }
            for (int32_t t = 0; t < nt; ++t) {
                nnbr[ne] = touched[t];
                nw[ne] = acc[touched[t]];
                acc[touched[t]] = 0;
                ++ne;
            }
            noffs[c + 1] = ne;
        }
        free(cstart);
        free(members);
        free(offs);
        free(nbr);
        free(w);
        offs = noffs;
        nbr = nnbr;
        w = nw;
        n = C;
        E = ne;
    }
    if (moves_out) *moves_out = moves_total;
    free(offs); free(nbr); free(w); free(K); free(tot); free(comm); free(acc); free(touched); free(renum);
    return levels;
}
