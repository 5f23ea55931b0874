// graph_host.cpp - host side of libgala: errors, the .bin CSR format, text
// preprocessing, seeded graph generators and the host modularity check.
// Compiled with -ffp-contract=off (no fused multiply-add in FP64 sums).
#include <cuda_runtime.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <fstream>
#include <random>
#include <string>
#include <thread>
#include <vector>

#include "internal.h"

namespace gala {

static thread_local std::string g_err;
static std::atomic<long long> g_launches{0};

void set_error(const char *fmt, ...)
{
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
}

void clear_error() { g_err.clear(); }

gala_status cuda_fail(cudaError_t e, const char *what)
{
    set_error("%s: CUDA error %d (%s)", what, (int)e, cudaGetErrorString(e));
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? GALA_ERR_OOM : GALA_ERR_CUDA;
}

void note_launch(int k) { g_launches.fetch_add(k, std::memory_order_relaxed); }

static int hw_threads(int want)
{
    if (want > 0) return want;
    unsigned h = std::thread::hardware_concurrency();
    return h ? (int)h : 1;
}

template <typename F>
static void parallel_for(int nthreads, long long n, F f)
{
    if (nthreads <= 1 || n < 4096) {
        f(0, 0, n);
        return;
    }
    std::vector<std::thread> th;
    long long chunk = (n + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; ++t) {
        long long a = t * chunk, b = std::min(n, a + chunk);
        if (a >= b) break;
        th.emplace_back([=, &f] { f(t, a, b); });
    }
    for (auto &x : th) x.join();
}

// Validate a CSR in reference layout.
static gala_status validate(const gala_graph *g)
{
    if (g->n <= 0) {
        set_error("graph has no vertices");
        return GALA_ERR_INVALID;
    }
    int64_t prev = 0;
    for (int32_t v = 0; v < g->n; ++v) {
        if (g->offs[v] < prev) {
            set_error("offsets decrease at vertex %d", v);
            return GALA_ERR_FORMAT;
        }
        prev = g->offs[v];
    }
    const int64_t E = g->entries();
    for (int64_t e = 0; e < E; ++e)
        if (g->nbr[e] < 0 || g->nbr[e] >= g->n) {
            set_error("neighbour id %d at entry %lld out of range [0, %d)", g->nbr[e], (long long)e, g->n);
            return GALA_ERR_FORMAT;
        }
    if (g->weighted)
        for (int64_t e = 0; e < E; ++e)
            if (g->w[e] <= 0) {
                set_error("weight %d at entry %lld is not positive", g->w[e], (long long)e);
                return GALA_ERR_FORMAT;
            }
    return GALA_OK;
}

// Build a CSR (reference layout) from an undirected edge list: symmetrise,
// sort and deduplicate every row (weights of duplicates summed when
// weighted, the first kept otherwise - graph.cpp:55-74), drop ids without
// edges and renumber in id order (graph.cpp:76-107).  A self-loop line adds
// the loop twice to its row before deduplication, as graph.cpp:47-48 does.
static gala_graph *build_csr(std::vector<std::pair<int32_t, int32_t>> &edges, const std::vector<int32_t> *wts,
                             bool weighted, int nthreads, int64_t keep_ids = 0)
{
    int32_t maxid = -1;
    for (auto &e : edges) maxid = std::max(maxid, std::max(e.first, e.second));
    const int64_t nid = std::max((int64_t)maxid + 1, keep_ids);
    std::vector<int64_t> deg(nid + 1, 0);
    for (auto &e : edges) {
        deg[e.first + 1]++;
        deg[e.second + 1]++;
    }
    for (int64_t i = 0; i < nid; ++i) deg[i + 1] += deg[i];
    std::vector<int32_t> col(deg[nid]);
    std::vector<int32_t> cw(weighted ? deg[nid] : 0);
    std::vector<int64_t> pos(deg.begin(), deg.end() - 1);
    for (size_t i = 0; i < edges.size(); ++i) {
        int32_t a = edges[i].first, b = edges[i].second;
        int32_t wt = wts ? (*wts)[i] : 1;
        int64_t pa = pos[a]++;
        col[pa] = b;
        if (weighted) cw[pa] = wt;
        int64_t pb = pos[b]++;
        col[pb] = a;
        if (weighted) cw[pb] = wt;
    }
    // per-row sort + dedup, in parallel
    std::vector<int64_t> newlen(nid, 0);
    parallel_for(nthreads, nid, [&](int, long long a, long long b) {
        std::vector<std::pair<int32_t, int32_t>> tmp;
        for (long long r = a; r < b; ++r) {
            int64_t s = deg[r], e = deg[r + 1];
            if (s == e) continue;
            tmp.clear();
            for (int64_t j = s; j < e; ++j) tmp.emplace_back(col[j], weighted ? cw[j] : 1);
            std::stable_sort(tmp.begin(), tmp.end(),
                             [](const std::pair<int32_t, int32_t> &x, const std::pair<int32_t, int32_t> &y) {
                                 return x.first < y.first;
                             });
            int64_t o = s;
            for (size_t k = 0; k < tmp.size(); ++k) {
                if (k > 0 && tmp[k].first == tmp[k - 1].first) {
                    if (weighted) cw[o - 1] += tmp[k].second;
                    continue;
                }
                col[o] = tmp[k].first;
                if (weighted) cw[o] = tmp[k].second;
                ++o;
            }
            newlen[r] = o - s;
        }
    });
    // renumber ids with edges, in id order (all ids when keep_ids is set)
    std::vector<int32_t> renum(nid, -1);
    int32_t n = 0;
    for (int64_t i = 0; i < nid; ++i)
        if (newlen[i] > 0 || keep_ids > 0) renum[i] = n++;
    gala_graph *g = new gala_graph();
    g->n = n;
    g->weighted = weighted;
    g->offs.resize(n);
    int64_t acc = 0;
    for (int64_t i = 0; i < nid; ++i)
        if (renum[i] >= 0) {
            acc += newlen[i];
            g->offs[renum[i]] = acc;
        }
    g->nbr.resize(acc);
    if (weighted) g->w.resize(acc);
    parallel_for(nthreads, nid, [&](int, long long a, long long b) {
        for (long long r = a; r < b; ++r) {
            if (newlen[r] == 0) continue;
            int32_t v = renum[r];
            int64_t o = v == 0 ? 0 : g->offs[v - 1];
            for (int64_t k = 0; k < newlen[r]; ++k) {
                g->nbr[o + k] = renum[col[deg[r] + k]];
                if (weighted) g->w[o + k] = cw[deg[r] + k];
            }
        }
    });
    return g;
}

}  // namespace gala

using namespace gala;

gala_graph::~gala_graph()
{
    if (pinned) {
        if (!offs.empty()) cudaHostUnregister(offs.data());
        if (!nbr.empty()) cudaHostUnregister(nbr.data());
        if (!w.empty()) cudaHostUnregister(w.data());
        cudaGetLastError();
    }
}

extern "C" {

gala_status gala_graph_pin(gala_graph *g)
{
    clear_error();
    if (!g) {
        set_error("gala_graph_pin: null graph");
        return GALA_ERR_INVALID;
    }
    if (g->pinned) return GALA_OK;
    cudaError_t e = cudaSuccess;
    if (!g->offs.empty()) e = cudaHostRegister(g->offs.data(), g->offs.size() * sizeof(int64_t), 0);
    if (e == cudaSuccess && !g->nbr.empty()) e = cudaHostRegister(g->nbr.data(), g->nbr.size() * sizeof(int32_t), 0);
    if (e == cudaSuccess && !g->w.empty()) e = cudaHostRegister(g->w.data(), g->w.size() * sizeof(int32_t), 0);
    if (e != cudaSuccess) {
        cudaHostUnregister(g->offs.data());
        cudaHostUnregister(g->nbr.data());
        if (!g->w.empty()) cudaHostUnregister(g->w.data());
        return cuda_fail(e, "gala_graph_pin");
    }
    g->pinned = true;
    return GALA_OK;
}

const char *gala_last_error(void) { return g_err.c_str(); }

const char *gala_status_string(gala_status s)
{
    switch (s) {
    case GALA_OK: return "ok";
    case GALA_ERR_INVALID: return "invalid argument";
    case GALA_ERR_IO: return "i/o error";
    case GALA_ERR_FORMAT: return "malformed graph";
    case GALA_ERR_CUDA: return "CUDA error";
    case GALA_ERR_NO_DEVICE: return "no CUDA device";
    case GALA_ERR_OOM: return "out of memory";
    case GALA_ERR_OVERFLOW: return "device table overflow";
    case GALA_ERR_CAPACITY: return "graph exceeds context capacity";
    }
    return "unknown";
}

int64_t gala_kernel_launch_count(void) { return g_launches.load(); }

void gala_graph_destroy(gala_graph *g) { delete g; }

gala_status gala_graph_info(const gala_graph *g, int32_t *n, int64_t *num_entries, int32_t *weighted)
{
    if (!g) {
        set_error("gala_graph_info: null graph");
        return GALA_ERR_INVALID;
    }
    if (n) *n = g->n;
    if (num_entries) *num_entries = g->entries();
    if (weighted) *weighted = g->weighted ? 1 : 0;
    return GALA_OK;
}

gala_status gala_graph_arrays(const gala_graph *g, const int64_t **offsets_inclusive, const int32_t **neighbors,
                              const int32_t **weights)
{
    if (!g) {
        set_error("gala_graph_arrays: null graph");
        return GALA_ERR_INVALID;
    }
    if (offsets_inclusive) *offsets_inclusive = g->offs.data();
    if (neighbors) *neighbors = g->nbr.data();
    if (weights) *weights = g->weighted ? g->w.data() : nullptr;
    return GALA_OK;
}

gala_status gala_graph_load_bin(const char *path, int32_t weighted, gala_graph **out)
{
    clear_error();
    if (!path || !out) {
        set_error("gala_graph_load_bin: bad arguments");
        return GALA_ERR_INVALID;
    }
    *out = nullptr;
    FILE *f = fopen(path, "rb");
    if (!f) {
        set_error("cannot open %s", path);
        return GALA_ERR_IO;
    }
    fseek(f, 0, SEEK_END);
    long long fsize = ftell(f);
    fseek(f, 0, SEEK_SET);
    int32_t n = 0;
    if (fread(&n, sizeof(n), 1, f) != 1 || n <= 0) {
        fclose(f);
        set_error("%s: bad vertex count", path);
        return GALA_ERR_FORMAT;
    }
    if (4LL + 8LL * n > fsize) {
        fclose(f);
        set_error("%s: truncated offsets (%d vertices, %lld bytes)", path, n, fsize);
        return GALA_ERR_FORMAT;
    }
    gala_graph *g = new gala_graph();
    g->n = n;
    g->offs.resize(n);
    if (fread(g->offs.data(), sizeof(int64_t), n, f) != (size_t)n) {
        fclose(f);
        delete g;
        set_error("%s: short read of offsets", path);
        return GALA_ERR_FORMAT;
    }
    const int64_t E = g->offs[n - 1];
    const long long need = 4LL + 8LL * n + 4LL * E * (weighted ? 2 : 1);
    if (E < 0 || E % 2 != 0 || need > fsize) {
        fclose(f);
        delete g;
        set_error("%s: %lld CSR entries need %lld bytes, file has %lld%s", path, (long long)E, need, fsize,
                  (E % 2) ? " (odd entry count: the writer dropped the last entry)" : "");
        return GALA_ERR_FORMAT;
    }
    g->nbr.resize(E);
    size_t got = fread(g->nbr.data(), sizeof(int32_t), (size_t)E, f);
    g->weighted = weighted != 0;
    if (weighted) {
        g->w.resize(E);
        got += fread(g->w.data(), sizeof(int32_t), (size_t)E, f);
    }
    fclose(f);
    if (got != (size_t)E * (weighted ? 2 : 1)) {
        delete g;
        set_error("%s: short read of neighbours/weights", path);
        return GALA_ERR_FORMAT;
    }
    gala_status s = validate(g);
    if (s != GALA_OK) {
        delete g;
        return s;
    }
    *out = g;
    return GALA_OK;
}

gala_status gala_graph_store_bin(const gala_graph *g, const char *path)
{
    clear_error();
    if (!g || !path) {
        set_error("gala_graph_store_bin: bad arguments");
        return GALA_ERR_INVALID;
    }
    FILE *f = fopen(path, "wb");
    if (!f) {
        set_error("cannot create %s", path);
        return GALA_ERR_IO;
    }
    const int64_t E = g->entries();
    bool ok = fwrite(&g->n, sizeof(int32_t), 1, f) == 1 &&
              fwrite(g->offs.data(), sizeof(int64_t), (size_t)g->n, f) == (size_t)g->n &&
              fwrite(g->nbr.data(), sizeof(int32_t), (size_t)E, f) == (size_t)E;
    if (ok && g->weighted) ok = fwrite(g->w.data(), sizeof(int32_t), (size_t)E, f) == (size_t)E;
    ok = (fclose(f) == 0) && ok;
    if (!ok) {
        set_error("write error on %s", path);
        return GALA_ERR_IO;
    }
    return GALA_OK;
}

gala_status gala_graph_from_csr(int32_t n, const int64_t *offsets_inclusive, const int32_t *neighbors,
                                const int32_t *weights, gala_graph **out)
{
    clear_error();
    if (!out || n <= 0 || !offsets_inclusive || (!neighbors && offsets_inclusive[n - 1] > 0)) {
        set_error("gala_graph_from_csr: bad arguments");
        return GALA_ERR_INVALID;
    }
    gala_graph *g = new gala_graph();
    g->n = n;
    g->offs.assign(offsets_inclusive, offsets_inclusive + n);
    const int64_t E = g->offs[n - 1];
    if (E < 0) {
        delete g;
        set_error("negative entry count");
        return GALA_ERR_INVALID;
    }
    g->nbr.assign(neighbors, neighbors + E);
    if (weights) {
        g->weighted = true;
        g->w.assign(weights, weights + E);
    }
    gala_status s = validate(g);
    if (s != GALA_OK) {
        delete g;
        return s;
    }
    *out = g;
    return GALA_OK;
}

// Text edge list -> CSR (graph.cpp:18-151).  Lines are parsed in parallel
// chunks; lines that are empty, start with '#' or do not hold two integers
// are skipped.
gala_status gala_graph_from_text(const char *path, int32_t weighted, int32_t nthreads, gala_graph **out)
{
    clear_error();
    if (!path || !out) {
        set_error("gala_graph_from_text: bad arguments");
        return GALA_ERR_INVALID;
    }
    *out = nullptr;
    FILE *f = fopen(path, "rb");
    if (!f) {
        set_error("cannot open %s", path);
        return GALA_ERR_IO;
    }
    fseek(f, 0, SEEK_END);
    long long fsize = ftell(f);
    fseek(f, 0, SEEK_SET);
    std::string text((size_t)fsize, '\0');
    if (fsize > 0 && fread(&text[0], 1, (size_t)fsize, f) != (size_t)fsize) {
        fclose(f);
        set_error("short read of %s", path);
        return GALA_ERR_IO;
    }
    fclose(f);
    const int nt = hw_threads(nthreads);
    // chunk boundaries at line starts
    std::vector<size_t> cut(nt + 1, 0);
    cut[nt] = text.size();
    for (int t = 1; t < nt; ++t) {
        size_t p = text.size() * (size_t)t / (size_t)nt;
        while (p < text.size() && p > 0 && text[p - 1] != '\n') ++p;
        cut[t] = std::max(p, cut[t - 1]);
    }
    std::vector<std::vector<std::pair<int32_t, int32_t>>> parts(nt);
    std::vector<std::vector<int32_t>> wparts(nt);
    std::vector<int> bad(nt, 0);
    auto worker = [&](int t) {
        const char *p = text.data() + cut[t];
        const char *end = text.data() + cut[t + 1];
        while (p < end) {
            const char *eol = (const char *)memchr(p, '\n', (size_t)(end - p));
            if (!eol) eol = end;
            if (p < eol && *p != '#' && *p != '\r') {
                long long a, b, w = 1;
                const char *q = p;
                char *nx;
                a = strtoll(q, &nx, 10);
                bool ok = nx != q && nx <= eol;
                if (ok) {
                    q = nx;
                    b = strtoll(q, &nx, 10);
                    ok = nx != q && nx <= eol;
                    q = nx;
                }
                if (ok && weighted) {
                    w = strtoll(q, &nx, 10);
                    if (nx == q || nx > eol) w = 1;
                }
                if (ok && a >= 0 && b >= 0 && a < 0x7fffffffLL && b < 0x7fffffffLL) {
                    parts[t].emplace_back((int32_t)a, (int32_t)b);
                    if (weighted) wparts[t].push_back((int32_t)w);
                } else if (!ok) {
                    bad[t]++;
                }
            }
            p = eol + 1;
        }
    };
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t) th.emplace_back(worker, t);
    for (auto &x : th) x.join();
    std::vector<std::pair<int32_t, int32_t>> edges;
    std::vector<int32_t> wts;
    size_t total = 0;
    for (auto &p : parts) total += p.size();
    edges.reserve(total);
    if (weighted) wts.reserve(total);
    for (int t = 0; t < nt; ++t) {
        edges.insert(edges.end(), parts[t].begin(), parts[t].end());
        if (weighted) wts.insert(wts.end(), wparts[t].begin(), wparts[t].end());
        std::vector<std::pair<int32_t, int32_t>>().swap(parts[t]);
    }
    if (edges.empty()) {
        set_error("%s: no edges", path);
        return GALA_ERR_FORMAT;
    }
    *out = build_csr(edges, weighted ? &wts : nullptr, weighted != 0, nt);
    return GALA_OK;
}

// ---- generators ----------------------------------------------------------

static inline uint64_t splitmix64(uint64_t &x)
{
    uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
static inline double u01(uint64_t &s) { return (double)(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

gala_status gala_generate_sbm(int32_t n, int32_t k, double p_in, double p_out, uint64_t seed, gala_graph **out)
{
    clear_error();
    if (!out || n <= 1 || k <= 0 || k > n || p_in < 0 || p_in > 1 || p_out < 0 || p_out > 1) {
        set_error("gala_generate_sbm: bad arguments");
        return GALA_ERR_INVALID;
    }
    // vertex i is in block i * k / n; every pair (i<j) is sampled by
    // geometric skips over the row-major upper triangle of each block pair
    std::vector<std::pair<int32_t, int32_t>> edges;
    uint64_t s = seed * 0x2545F4914F6CDD1DULL + 1;
    std::vector<int32_t> bstart(k + 1);
    for (int b = 0; b <= k; ++b) bstart[b] = (int32_t)((int64_t)b * n / k);
    for (int a = 0; a < k; ++a)
        for (int b = a; b < k; ++b) {
            double p = a == b ? p_in : p_out;
            if (p <= 0) continue;
            int64_t na = bstart[a + 1] - bstart[a], nb = bstart[b + 1] - bstart[b];
            int64_t npairs = a == b ? na * (na - 1) / 2 : na * nb;
            double lq = std::log1p(-std::min(p, 1 - 1e-16));
            int64_t idx = -1;
            for (;;) {
                if (p >= 1) {
                    idx++;
                } else {
                    double r = u01(s);
                    idx += 1 + (int64_t)std::floor(std::log1p(-r) / lq);
                }
                if (idx >= npairs) break;
                int32_t u, v;
                if (a == b) {  // idx -> (i<j) within the block
                    int64_t i = (int64_t)((std::sqrt(8.0 * (double)idx + 1) - 1) / 2);
                    while (i * (i + 1) / 2 > idx) --i;
                    while ((i + 1) * (i + 2) / 2 <= idx) ++i;
                    int64_t j = idx - i * (i + 1) / 2;
                    u = bstart[a] + (int32_t)j;
                    v = bstart[a] + (int32_t)(i + 1);
                } else {
                    u = bstart[a] + (int32_t)(idx / nb);
                    v = bstart[b] + (int32_t)(idx % nb);
                }
                edges.emplace_back(u, v);
            }
        }
    if (edges.empty()) {
        set_error("gala_generate_sbm: no edges drawn");
        return GALA_ERR_INVALID;
    }
    *out = build_csr(edges, nullptr, false, 1);
    return GALA_OK;
}

gala_status gala_generate_sbm_batch(int32_t count, int32_t n_min, int32_t n_max, int32_t k_min, int32_t k_max,
                                    double deg_min, double deg_max, double mix_min, double mix_max, uint64_t seed,
                                    int32_t nthreads, gala_graph **out)
{
    clear_error();
    if (!out || count <= 0 || n_min < 4 || n_max < n_min || k_min < 1 || k_max < k_min || deg_min <= 0 ||
        deg_max < deg_min || mix_min < 0 || mix_max > 1 || mix_max < mix_min) {
        set_error("gala_generate_sbm_batch: bad arguments");
        return GALA_ERR_INVALID;
    }
    for (int i = 0; i < count; ++i) out[i] = nullptr;
    // parameters drawn serially (graph i depends only on seed and i)
    struct P {
        int32_t n, k;
        double pin, pout;
        uint64_t seed;
    };
    std::vector<P> ps((size_t)count);
    uint64_t s = seed * 0x9E3779B97F4A7C15ULL + 0x632BE59BD9B4E019ULL;
    const double l0 = std::log((double)n_min), l1 = std::log((double)n_max);
    for (int i = 0; i < count; ++i) {
        P &p = ps[i];
        p.n = (int32_t)std::llround(std::exp(l0 + (l1 - l0) * u01(s)));
        p.n = std::max(n_min, std::min(n_max, p.n));
        int32_t k = k_min + (int32_t)std::floor((k_max - k_min + 1) * u01(s));
        k = std::min(k, k_max);
        const double d = deg_min + (deg_max - deg_min) * u01(s);
        const double mu = mix_min + (mix_max - mix_min) * u01(s);
        // blocks large enough to hold the intra-block degree
        const int32_t kmax_fit = std::max(1, (int32_t)(p.n / (d * (1 - mu) + 2)));
        p.k = std::max(1, std::min(k, kmax_fit));
        const double bs = (double)p.n / p.k;
        p.pin = std::min(1.0, d * (1 - mu) / std::max(1.0, bs - 1));
        p.pout = p.k > 1 ? std::min(1.0, d * mu / std::max(1.0, p.n - bs)) : 0.0;
        p.seed = seed * 1000003ULL + (uint64_t)i;
    }
    std::atomic<int> failed{-1};
    const int nt = hw_threads(nthreads);
    std::vector<std::thread> th;
    std::atomic<int> next{0};
    for (int t = 0; t < std::min(nt, count); ++t)
        th.emplace_back([&] {
            for (int i = next++; i < count; i = next++) {
                gala_graph *g = nullptr;
                if (gala_generate_sbm(ps[i].n, ps[i].k, ps[i].pin, ps[i].pout, ps[i].seed, &g) != GALA_OK) {
                    failed = i;
                    continue;
                }
                out[i] = g;
            }
        });
    for (auto &x : th) x.join();
    if (failed >= 0) {
        const int i = failed;
        for (int j = 0; j < count; ++j) {
            gala_graph_destroy(out[j]);
            out[j] = nullptr;
        }
        set_error("gala_generate_sbm_batch: graph %d (n %d, k %d) drew no edges", i, ps[i].n, ps[i].k);
        return GALA_ERR_INVALID;
    }
    return GALA_OK;
}

gala_status gala_generate_rmat(int32_t scale, int64_t nedges, double a, double b, double c, double noise,
                               int32_t keep_isolated, uint64_t seed, int32_t nthreads, gala_graph **out)
{
    clear_error();
    if (!out || scale < 1 || scale > 30 || nedges <= 0 || a < 0 || b < 0 || c < 0 || a + b + c > 1 ||
        noise < 0 || noise >= 1) {
        set_error("gala_generate_rmat: bad arguments");
        return GALA_ERR_INVALID;
    }
    const int nt = hw_threads(nthreads);
    // fixed chunking so the graph does not depend on the thread count
    const int64_t chunk = 1 << 20;
    const int64_t nchunks = (nedges + chunk - 1) / chunk;
    std::vector<std::pair<int32_t, int32_t>> edges((size_t)nedges);
    std::vector<char> keep((size_t)nedges, 0);
    const double ab = a + b, abc = a + b + c;
    parallel_for(nt, nchunks, [&](int, long long c0, long long c1) {
        for (long long ch = c0; ch < c1; ++ch) {
            uint64_t s = seed ^ (0xD1B54A32D192ED03ULL * (uint64_t)(ch + 1));
            int64_t lo = ch * chunk, hi = std::min(nedges, lo + chunk);
            for (int64_t i = lo; i < hi; ++i) {
                uint32_t u = 0, v = 0;
                for (int l = 0; l < scale; ++l) {
                    double pa = a, pab = ab, pabc = abc;
                    if (noise > 0) {
                        double na = a * (1 - noise + 2 * noise * u01(s));
                        double nb = b * (1 - noise + 2 * noise * u01(s));
                        double nc = c * (1 - noise + 2 * noise * u01(s));
                        double nd = (1 - abc) * (1 - noise + 2 * noise * u01(s));
                        double inv = 1.0 / (na + nb + nc + nd);
                        pa = na * inv;
                        pab = (na + nb) * inv;
                        pabc = (na + nb + nc) * inv;
                    }
                    double r = u01(s);
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
                edges[i] = {(int32_t)u, (int32_t)v};
                keep[i] = u != v;  // self-loops removed
            }
        }
    });
    size_t o = 0;
    for (size_t i = 0; i < edges.size(); ++i)
        if (keep[i]) edges[o++] = edges[i];
    edges.resize(o);
    std::vector<char>().swap(keep);
    *out = build_csr(edges, nullptr, false, nt, keep_isolated ? (int64_t)1 << scale : 0);
    return GALA_OK;
}

gala_status gala_modularity_host(const gala_graph *g, const int32_t *community, double *q)
{
    clear_error();
    if (!g || !community || !q) {
        set_error("gala_modularity_host: bad arguments");
        return GALA_ERR_INVALID;
    }
    const int32_t n = g->n;
    for (int32_t v = 0; v < n; ++v)
        if (community[v] < 0 || community[v] >= n) {
            set_error("community id %d of vertex %d out of range", community[v], v);
            return GALA_ERR_INVALID;
        }
    // kernel_functions.cu:1037-1079: In per vertex, Tot per community
    int64_t m2 = 0;
    for (int64_t e = 0; e < g->entries(); ++e) m2 += g->weighted ? g->w[e] : 1;
    if (m2 <= 0) {
        set_error("graph has no edges");
        return GALA_ERR_INVALID;
    }
    const double constant = 1.0 / (double)m2;
    std::vector<int64_t> Tot(n, 0), In(n, 0);
    for (int32_t i = 0; i < n; ++i) {
        int64_t s = i == 0 ? 0 : g->offs[i - 1], e = g->offs[i], degree = 0;
        for (int64_t j = s; j < e; ++j) {
            int32_t wt = g->weighted ? g->w[j] : 1;
            degree += wt;
            if (community[g->nbr[j]] == community[i]) In[i] += wt;
        }
        Tot[community[i]] += degree;
    }
    double acc = 0;
    for (int32_t i = 0; i < n; ++i)
        acc += (double)In[i] * constant - (double)Tot[i] * (double)Tot[i] * constant * constant;
    *q = acc;
    return GALA_OK;
}

}  // extern "C"
