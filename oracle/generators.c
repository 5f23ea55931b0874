/*
 * generators.c - seeded synthetic graphs on the CPU side.
 *
 * TEST INFRASTRUCTURE ONLY: the CPU arm of bench.py (the timed reference arm
 * and the CPU baselines) builds its input here, so that it never loads the
 * engine library; tests/ check that the graphs are byte-identical to the
 * engine's own generator (gala_generate_rmat in
 * gala-mg_gb300/csrc/graph_host.cpp), which the GPU arm uses.
 *
 * R-MAT (Chakrabarti, Zhan & Faloutsos, 2004): every edge descends `scale`
 * levels of the adjacency matrix's quadrants with probabilities a, b, c and
 * d = 1 - a - b - c (optionally each perturbed by a factor in
 * [1 - noise, 1 + noise] and renormalised).  The draws come from splitmix64
 * (Steele, Lea & Flood, 2014), one stream per chunk of 2^20 edges seeded
 * from (seed, chunk index), so the graph does not depend on the thread
 * count.  Self-loops are dropped; the CSR is symmetrised, every row sorted
 * ascending and deduplicated (as the reference's preprocess does,
 * src/graph/graph.cpp:46-74), and ids without edges are dropped and the rest
 * renumbered in id order (graph.cpp:76-107) unless keep_isolated is set.
 */
#include "oracle.h"

#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline uint64_t sm64_next(uint64_t *x)
{
    uint64_t z = (*x += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

/* uniform in [0, 1) from the top 53 bits */
static inline double unit01(uint64_t *s) { return (double)(sm64_next(s) >> 11) * (1.0 / 9007199254740992.0); }

static int cmp_i32(const void *x, const void *y)
{
    const int32_t a = *(const int32_t *)x, b = *(const int32_t *)y;
    return (a > b) - (a < b);
}

void orc_free(void *p) { free(p); }

int32_t orc_generate_rmat(int32_t scale, int64_t nedges, double a, double b, double c, double noise,
                          int32_t keep_isolated, uint64_t seed, int32_t nthreads, int32_t *n_out,
                          int64_t **offs_out, int32_t **nbr_out)
{
    if (!n_out || !offs_out || !nbr_out || scale < 1 || scale > 30 || nedges <= 0 || a < 0 || b < 0 || c < 0 ||
        a + b + c > 1 || noise < 0 || noise >= 1)
        return -1;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
    const int64_t nid = (int64_t)1 << scale;
    const int64_t chunk = (int64_t)1 << 20;
    const int64_t nchunks = (nedges + chunk - 1) / chunk;
    int32_t *eu = (int32_t *)malloc((size_t)nedges * sizeof(int32_t));
    int32_t *ev = (int32_t *)malloc((size_t)nedges * sizeof(int32_t));
    int64_t *deg = (int64_t *)calloc((size_t)nid + 1, sizeof(int64_t));
    if (!eu || !ev || !deg) {
        free(eu);
        free(ev);
        free(deg);
        return -1;
    }
    const double ab = a + b, abc = a + b + c;
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t ch = 0; ch < nchunks; ++ch) {
        uint64_t s = seed ^ (0xD1B54A32D192ED03ULL * (uint64_t)(ch + 1));
        const int64_t lo = ch * chunk, hi = lo + chunk < nedges ? lo + chunk : nedges;
        for (int64_t i = lo; i < hi; ++i) {
            uint32_t u = 0, v = 0;
            for (int l = 0; l < scale; ++l) {
                double pa = a, pab = ab, pabc = abc;
                if (noise > 0) {
                    const double na = a * (1 - noise + 2 * noise * unit01(&s));
                    const double nb = b * (1 - noise + 2 * noise * unit01(&s));
                    const double nc = c * (1 - noise + 2 * noise * unit01(&s));
                    const double nd = (1 - abc) * (1 - noise + 2 * noise * unit01(&s));
                    const double inv = 1.0 / (na + nb + nc + nd);
                    pa = na * inv;
                    pab = (na + nb) * inv;
                    pabc = (na + nb + nc) * inv;
                }
                const double r = unit01(&s);
                u <<= 1;
                v <<= 1;
                if (r < pa) {
                } else if (r < pab) {
                    v |= 1;
                } else if (r < pabc) {
                    u |= 1;
                } else {
                    u |= 1;
                    v |= 1;
                }
            }
            eu[i] = (int32_t)u;
            ev[i] = (int32_t)v;
        }
    }
    /* symmetrised row lengths (self-loops dropped) */
    for (int64_t i = 0; i < nedges; ++i)
        if (eu[i] != ev[i]) {
            deg[eu[i] + 1]++;
            deg[ev[i] + 1]++;
        }
    for (int64_t i = 0; i < nid; ++i) deg[i + 1] += deg[i];
    int32_t *col = (int32_t *)malloc((size_t)(deg[nid] > 0 ? deg[nid] : 1) * sizeof(int32_t));
    int64_t *pos = (int64_t *)malloc((size_t)nid * sizeof(int64_t));
    int64_t *len = (int64_t *)calloc((size_t)nid, sizeof(int64_t));
    if (!col || !pos || !len) {
        free(eu);
        free(ev);
        free(deg);
        free(col);
        free(pos);
        free(len);
        return -1;
    }
    memcpy(pos, deg, (size_t)nid * sizeof(int64_t));
    for (int64_t i = 0; i < nedges; ++i)
        if (eu[i] != ev[i]) {
            col[pos[eu[i]]++] = ev[i];
            col[pos[ev[i]]++] = eu[i];
        }
    free(eu);
    free(ev);
    free(pos);
    /* sort and deduplicate every row in place */
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t r = 0; r < nid; ++r) {
        const int64_t s = deg[r], e = deg[r + 1];
        if (s == e) continue;
        qsort(col + s, (size_t)(e - s), sizeof(int32_t), cmp_i32);
        int64_t o = s + 1;
        for (int64_t j = s + 1; j < e; ++j)
            if (col[j] != col[o - 1]) col[o++] = col[j];
        len[r] = o - s;
    }
    /* renumber: every id when keep_isolated, else ids with edges in order */
    int32_t *renum = (int32_t *)malloc((size_t)nid * sizeof(int32_t));
    int32_t n = 0;
    for (int64_t i = 0; i < nid; ++i) renum[i] = (len[i] > 0 || keep_isolated) ? n++ : -1;
    int64_t *offs = (int64_t *)malloc(((size_t)n + 1) * sizeof(int64_t));
    offs[0] = 0;
    for (int64_t i = 0; i < nid; ++i)
        if (renum[i] >= 0) offs[renum[i] + 1] = offs[renum[i]] + len[i];
    int32_t *nbr = (int32_t *)malloc((size_t)(offs[n] > 0 ? offs[n] : 1) * sizeof(int32_t));
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t r = 0; r < nid; ++r) {
        if (len[r] == 0) continue;
        const int64_t o = offs[renum[r]];
        for (int64_t k = 0; k < len[r]; ++k) nbr[o + k] = renum[col[deg[r] + k]];
    }
    free(col);
    free(deg);
    free(len);
    free(renum);
    *n_out = n;
    *offs_out = offs;
    *nbr_out = nbr;
    return 0;
}
