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
#include <functional>
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
    if (g->float_w) {
        const int32_t s = fixed_shift_of(g->wf.data(), E);
        if (s < 0) {
            set_error("float weights must be positive, finite and not below 2^-(fixed-point shift)");
            return GALA_ERR_FORMAT;
        }
        const_cast<gala_graph *>(g)->fixed_shift = s;
    }
    return GALA_OK;
}

// Float weights are held as round(w * 2^S) in int64: S = 61 - e with
// 2^e >= sum(w) (frexp of the sum in entry order), capped to [0, 40], so the
// total weight stays below 2^62.
int32_t fixed_shift_of(const float *w, int64_t E)
{
    double sum = 0, mn = INFINITY;
    for (int64_t e = 0; e < E; ++e) {
        const double x = (double)w[e];
        if (!(x > 0) || !std::isfinite(x)) return -1;
        sum += x;
        if (x < mn) mn = x;
    }
    int ex = 0;
    std::frexp(sum > 0 ? sum : 1.0, &ex);
    int s = 61 - ex;
    if (s > 40) s = 40;
    if (s < 0) s = 0;
    if (E > 0 && std::llrint(mn * std::ldexp(1.0, s)) <= 0) return -1;
    return s;
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
    g->rows_distinct = true;
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
        if (!wf.empty()) cudaHostUnregister(wf.data());
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
    if (e == cudaSuccess && !g->wf.empty()) e = cudaHostRegister(g->wf.data(), g->wf.size() * sizeof(float), 0);
    if (e != cudaSuccess) {
        cudaHostUnregister(g->offs.data());
        cudaHostUnregister(g->nbr.data());
        if (!g->w.empty()) cudaHostUnregister(g->w.data());
        if (!g->wf.empty()) cudaHostUnregister(g->wf.data());
        return cuda_fail(e, "gala_graph_pin");
    }
    g->pinned = true;
    // device-mapped addresses, for kernels that read the graph in place
    // (registered memory is mapped under unified addressing); a graph
    // without them is copied by the host instead
    void *p = nullptr;
    if (!g->offs.empty() && cudaHostGetDevicePointer(&p, g->offs.data(), 0) == cudaSuccess)
        g->dev_offs = (const int64_t *)p;
    if (!g->nbr.empty() && cudaHostGetDevicePointer(&p, g->nbr.data(), 0) == cudaSuccess)
        g->dev_nbr = (const int32_t *)p;
    if (!g->w.empty() && cudaHostGetDevicePointer(&p, g->w.data(), 0) == cudaSuccess) g->dev_w = (const int32_t *)p;
    cudaGetLastError();
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
    if (weighted) *weighted = g->float_w ? 2 : (g->weighted ? 1 : 0);
    return GALA_OK;
}

gala_status gala_graph_weights_f32(const gala_graph *g, const float **weights)
{
    if (!g || !weights) {
        set_error("gala_graph_weights_f32: bad arguments");
        return GALA_ERR_INVALID;
    }
    *weights = g->float_w ? g->wf.data() : nullptr;
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
    if (weighted < 0 || weighted > 2) {
        fclose(f);
        delete g;
        set_error("gala_graph_load_bin: weighted must be 0, 1 (int32) or 2 (float32)");
        return GALA_ERR_INVALID;
    }
    const long long need = 4LL + 8LL * n + 4LL * E * (weighted ? 2 : 1);
    // (an odd entry count is legal - a contracted graph has one self-loop
    // entry per community - but the reference's writer drops the last entry
    // of such a graph, graph.cpp:75,166, which the size check catches)
    if (E < 0 || need > fsize) {
        fclose(f);
        delete g;
        set_error("%s: %lld CSR entries need %lld bytes, file has %lld%s", path, (long long)E, need, fsize,
                  (E % 2) ? " (odd entry count: a writer that drops the last entry made this file)" : "");
        return GALA_ERR_FORMAT;
    }
    g->nbr.resize(E);
    size_t got = fread(g->nbr.data(), sizeof(int32_t), (size_t)E, f);
    g->weighted = weighted == 1;
    g->float_w = weighted == 2;
    if (weighted == 1) {
        g->w.resize(E);
        got += fread(g->w.data(), sizeof(int32_t), (size_t)E, f);
    } else if (weighted == 2) {
        g->wf.resize(E);
        got += fread(g->wf.data(), sizeof(float), (size_t)E, f);
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
    if (ok && g->float_w) ok = fwrite(g->wf.data(), sizeof(float), (size_t)E, f) == (size_t)E;
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

gala_status gala_graph_from_csr_f32(int32_t n, const int64_t *offsets_inclusive, const int32_t *neighbors,
                                    const float *weights, gala_graph **out)
{
    clear_error();
    if (!out || n <= 0 || !offsets_inclusive || !weights || (!neighbors && offsets_inclusive[n - 1] > 0)) {
        set_error("gala_graph_from_csr_f32: bad arguments");
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
    g->float_w = true;
    g->wf.assign(weights, weights + E);
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

// ---- LFR-style planted graph ---------------------------------------------
// Power-law degree d ~ x^-tau1 on [dmin, dmax] and community size ~ x^-tau2
// on [cmin, cmax] (continuous inverse-CDF draws, rounded down); a fraction
// 1 - mu of every vertex's stubs stays inside its community.  Vertices are
// placed, largest internal degree first, into random communities large
// enough to hold that degree; stubs are paired by the configuration model
// inside every community and, for the mixing stubs, across random buckets.
// Self-loops are dropped and parallel edges merged (weights summed).
// Weights are lognormal(0, 1) float32 (Box-Muller on splitmix64).  The graph
// depends only on the arguments, not on nthreads.
static inline double powerlaw_draw(uint64_t &s, double lo, double hi, double tau)
{
    const double a = std::pow(lo, 1 - tau), b = std::pow(hi, 1 - tau);
    return std::pow(a + (b - a) * u01(s), 1 / (1 - tau));
}

static inline float lognormal_draw(uint64_t &s)
{
    double u1 = u01(s);
    const double u2 = u01(s);
    if (u1 < 1e-300) u1 = 1e-300;
    const double z = std::sqrt(-2 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    return (float)std::exp(z);
}

gala_status gala_generate_lfr(int32_t n, double tau1, int32_t dmin, int32_t dmax, double tau2, int32_t cmin,
                              int32_t cmax, double mu, int32_t float_weights, uint64_t seed, int32_t nthreads,
                              gala_graph **out)
{
    clear_error();
    if (!out || n < 2 || dmin < 1 || dmax < dmin || cmin < 2 || cmax < cmin || tau1 <= 1 || tau2 <= 1 || mu < 0 ||
        mu > 1 || cmin > n) {
        set_error("gala_generate_lfr: bad arguments");
        return GALA_ERR_INVALID;
    }
    *out = nullptr;
    const int nt = hw_threads(nthreads);
    const int64_t chunk = 1 << 16;
    const int64_t nchunks = (n + chunk - 1) / chunk;
    auto par = [&](int64_t items, const std::function<void(int64_t)> &f) {
        std::atomic<int64_t> next{0};
        std::vector<std::thread> th;
        auto run = [&] {
            for (int64_t i = next++; i < items; i = next++) f(i);
        };
        for (int t = 1; t < std::min<int64_t>(nt, items); ++t) th.emplace_back(run);
        run();
        for (auto &x : th) x.join();
    };
    // degrees and internal degrees
    std::vector<int32_t> deg(n), kin(n);
    par(nchunks, [&](int64_t c) {
        uint64_t s = seed * 0xD1B54A32D192ED03ULL + (uint64_t)c * 0x9E3779B97F4A7C15ULL + 1;
        for (int64_t v = c * chunk; v < std::min<int64_t>(n, (c + 1) * chunk); ++v) {
            int32_t d = (int32_t)powerlaw_draw(s, dmin, dmax + 1.0, tau1);
            d = std::max(dmin, std::min(dmax, d));
            deg[v] = d;
            kin[v] = (int32_t)std::llround((1 - mu) * d);
        }
    });
    // community sizes summing to n
    std::vector<int32_t> csize;
    {
        uint64_t s = seed * 0x9E3779B97F4A7C15ULL + 7;
        int64_t tot = 0;
        while (tot < n) {
            int32_t c = (int32_t)powerlaw_draw(s, cmin, cmax + 1.0, tau2);
            c = std::max(cmin, std::min(cmax, c));
            if (tot + c > n) c = (int32_t)(n - tot);
            csize.push_back(c);
            tot += c;
        }
        if (csize.size() > 1 && csize.back() < cmin) {  // fold a short last community into the previous one
            csize[csize.size() - 2] += csize.back();
            csize.pop_back();
        }
        std::sort(csize.begin(), csize.end(), std::greater<int32_t>());
    }
    const int32_t K = (int32_t)csize.size();
    // placement: vertices by internal degree (descending), each into a random
    // community with room whose size exceeds the internal degree
    std::vector<int32_t> order(n);
    {
        std::vector<int64_t> cnt((size_t)dmax + 2, 0);
        for (int32_t v = 0; v < n; ++v) cnt[kin[v]]++;
        int64_t acc = 0;
        for (int32_t k = dmax + 1; k >= 0; --k) {  // descending k
            const int64_t c = cnt[k];
            cnt[k] = acc;
            acc += c;
        }
        for (int32_t v = 0; v < n; ++v) order[cnt[kin[v]]++] = v;
    }
    std::vector<int32_t> comm(n), room(csize.begin(), csize.end());
    {
        uint64_t s = seed * 0xA24BAED4963EE407ULL + 11;
        std::vector<int32_t> eligible;  // communities with room, size > current k
        int32_t next_c = 0;
        for (int32_t idx = 0; idx < n; ++idx) {
            const int32_t v = order[idx];
            while (next_c < K && csize[next_c] > kin[v]) eligible.push_back(next_c++);
            int32_t c = -1;
            while (!eligible.empty()) {
                const size_t r = (size_t)(splitmix64(s) % eligible.size());
                if (room[eligible[r]] > 0) {
                    c = eligible[r];
                    break;
                }
                eligible[r] = eligible.back();
                eligible.pop_back();
            }
            if (c < 0) {  // no community large enough left: the largest one with room
                for (int32_t q = 0; q < K && c < 0; ++q)
                    if (room[q] > 0) c = q;
                kin[v] = std::min(kin[v], csize[c] - 1);
                while (next_c < K && csize[next_c] > kin[v]) eligible.push_back(next_c++);
            }
            comm[v] = c;
            room[c]--;
        }
    }
    // members per community
    std::vector<int64_t> coff((size_t)K + 1, 0);
    for (int32_t v = 0; v < n; ++v) coff[comm[v] + 1]++;
    for (int32_t c = 0; c < K; ++c) coff[c + 1] += coff[c];
    std::vector<int32_t> members(n);
    {
        std::vector<int64_t> pos(coff.begin(), coff.end() - 1);
        for (int32_t v = 0; v < n; ++v) members[pos[comm[v]]++] = v;
    }
    // edges: intra-community pairing per community, mixing pairing per bucket
    constexpr int kBuckets = 256;
    std::vector<std::vector<int32_t>> eu((size_t)K + kBuckets), ev((size_t)K + kBuckets);
    std::vector<std::vector<float>> ew((size_t)K + kBuckets);
    auto pair_up = [&](std::vector<int32_t> &stubs, uint64_t s, size_t slot) {
        for (size_t i = stubs.size(); i > 1; --i) std::swap(stubs[i - 1], stubs[splitmix64(s) % i]);
        for (size_t i = 0; i + 1 < stubs.size(); i += 2) {
            const int32_t a = stubs[i], b = stubs[i + 1];
            if (a == b) continue;
            eu[slot].push_back(std::min(a, b));
            ev[slot].push_back(std::max(a, b));
            ew[slot].push_back(float_weights ? lognormal_draw(s) : 1.0f);
        }
    };
    par(K, [&](int64_t c) {
        std::vector<int32_t> stubs;
        for (int64_t i = coff[c]; i < coff[c + 1]; ++i)
            for (int32_t k = 0; k < kin[members[i]]; ++k) stubs.push_back(members[i]);
        pair_up(stubs, seed * 0x94D049BB133111EBULL + (uint64_t)c * 0x9E3779B97F4A7C15ULL + 3, (size_t)c);
    });
    {
        // mixing stubs: bucket of every stub drawn per vertex chunk
        std::vector<int64_t> bcnt((size_t)nchunks * kBuckets, 0);
        auto stub_bucket_rng = [&](int64_t c) {
            return seed * 0xBF58476D1CE4E5B9ULL + (uint64_t)c * 0x9E3779B97F4A7C15ULL + 5;
        };
        par(nchunks, [&](int64_t c) {
            uint64_t s = stub_bucket_rng(c);
            for (int64_t v = c * chunk; v < std::min<int64_t>(n, (c + 1) * chunk); ++v)
                for (int32_t k = kin[v]; k < deg[v]; ++k) bcnt[(size_t)c * kBuckets + splitmix64(s) % kBuckets]++;
        });
        std::vector<int64_t> boff((size_t)nchunks * kBuckets + 1, 0);  // bucket-major
        std::vector<int64_t> bstart(kBuckets + 1, 0);
        int64_t acc = 0;
        for (int b = 0; b < kBuckets; ++b) {
            bstart[b] = acc;
            for (int64_t c = 0; c < nchunks; ++c) {
                boff[(size_t)b * nchunks + c] = acc;
                acc += bcnt[(size_t)c * kBuckets + b];
            }
        }
        bstart[kBuckets] = acc;
        std::vector<int32_t> mix((size_t)acc);
        par(nchunks, [&](int64_t c) {
            uint64_t s = stub_bucket_rng(c);
            std::vector<int64_t> pos(kBuckets);
            for (int b = 0; b < kBuckets; ++b) pos[b] = boff[(size_t)b * nchunks + c];
            for (int64_t v = c * chunk; v < std::min<int64_t>(n, (c + 1) * chunk); ++v)
                for (int32_t k = kin[v]; k < deg[v]; ++k) mix[pos[splitmix64(s) % kBuckets]++] = (int32_t)v;
        });
        par(kBuckets, [&](int64_t b) {
            std::vector<int32_t> stubs(mix.begin() + bstart[b], mix.begin() + bstart[b + 1]);
            pair_up(stubs, seed * 0x2545F4914F6CDD1DULL + (uint64_t)b * 0x9E3779B97F4A7C15ULL + 9, (size_t)K + b);
        });
    }
    // CSR: both directions, rows sorted by (neighbour, weight), parallel
    // edges merged with summed weights
    std::vector<int64_t> slot_off(eu.size() + 1, 0);
    for (size_t i = 0; i < eu.size(); ++i) slot_off[i + 1] = slot_off[i] + (int64_t)eu[i].size();
    std::vector<int64_t> rdeg((size_t)n + 1, 0);
    for (size_t i = 0; i < eu.size(); ++i)
        for (size_t j = 0; j < eu[i].size(); ++j) {
            rdeg[eu[i][j] + 1]++;
            rdeg[ev[i][j] + 1]++;
        }
    for (int32_t v = 0; v < n; ++v) rdeg[v + 1] += rdeg[v];
    std::vector<int32_t> col((size_t)rdeg[n]);
    std::vector<float> cw((size_t)rdeg[n]);
    {
        std::vector<int64_t> pos(rdeg.begin(), rdeg.end() - 1);
        for (size_t i = 0; i < eu.size(); ++i) {
            for (size_t j = 0; j < eu[i].size(); ++j) {
                const int32_t a = eu[i][j], b = ev[i][j];
                const float w = ew[i][j];
                col[pos[a]] = b;
                cw[pos[a]++] = w;
                col[pos[b]] = a;
                cw[pos[b]++] = w;
            }
            std::vector<int32_t>().swap(eu[i]);
            std::vector<int32_t>().swap(ev[i]);
            std::vector<float>().swap(ew[i]);
        }
    }
    std::vector<int64_t> newlen(n, 0);
    par(nchunks, [&](int64_t c) {
        std::vector<std::pair<int32_t, float>> tmp;
        for (int64_t r = c * chunk; r < std::min<int64_t>(n, (c + 1) * chunk); ++r) {
            const int64_t s0 = rdeg[r], e0 = rdeg[r + 1];
            tmp.clear();
            for (int64_t j = s0; j < e0; ++j) tmp.emplace_back(col[j], cw[j]);
            std::sort(tmp.begin(), tmp.end());
            int64_t o = s0;
            for (size_t k = 0; k < tmp.size(); ++k) {
                if (k > 0 && tmp[k].first == tmp[k - 1].first) {
                    cw[o - 1] += tmp[k].second;
                    continue;
                }
                col[o] = tmp[k].first;
                cw[o] = tmp[k].second;
                ++o;
            }
            newlen[r] = o - s0;
        }
    });
    gala_graph *g = new gala_graph();
    g->n = n;
    g->rows_distinct = true;
    g->offs.resize(n);
    int64_t acc = 0;
    for (int32_t v = 0; v < n; ++v) {
        acc += newlen[v];
        g->offs[v] = acc;
    }
    g->nbr.resize((size_t)acc);
    if (float_weights) {
        g->float_w = true;
        g->wf.resize((size_t)acc);
    }
    par(nchunks, [&](int64_t c) {
        for (int64_t r = c * chunk; r < std::min<int64_t>(n, (c + 1) * chunk); ++r) {
            const int64_t o = r == 0 ? 0 : g->offs[r - 1];
            for (int64_t k = 0; k < newlen[r]; ++k) {
                g->nbr[o + k] = col[rdeg[r] + k];
                if (float_weights) g->wf[o + k] = cw[rdeg[r] + k];
            }
        }
    });
    gala_status st = validate(g);
    if (st != GALA_OK) {
        delete g;
        return st;
    }
    *out = g;
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
    if (g->float_w) {  // FP64 sums of the float weights
        double m2f = 0;
        for (int64_t e = 0; e < g->entries(); ++e) m2f += (double)g->wf[e];
        const double cf = 1.0 / m2f;
        std::vector<double> Tf(n, 0.0), If(n, 0.0);
        for (int32_t i = 0; i < n; ++i) {
            int64_t s = i == 0 ? 0 : g->offs[i - 1], e = g->offs[i];
            double degree = 0;
            for (int64_t j = s; j < e; ++j) {
                degree += (double)g->wf[j];
                if (community[g->nbr[j]] == community[i]) If[i] += (double)g->wf[j];
            }
            Tf[community[i]] += degree;
        }
        double acc = 0;
        for (int32_t i = 0; i < n; ++i) acc += If[i] * cf - Tf[i] * Tf[i] * cf * cf;
        *q = acc;
        return GALA_OK;
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
