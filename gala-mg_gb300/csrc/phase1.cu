// phase1.cu - phase-1 kernels of the GB300 Louvain engine (sm_103a).
//
// One phase-1 iteration (louvain_main_process.cu:571-1034 in the reference):
//   decide  : every active vertex aggregates the weights to its neighbour
//             communities, picks the best gain (ties -> lowest id) and, when it
//             moves, appends (v, old, new) to a mover list
//   apply   : movers update comm, Tot and size with integer atomics
//   reduce  : min over non-empty Tot and sum of Tot^2
//   update  : In[v] (weight to the own community) for every vertex, the
//             pruning bound, the next active lists and sum of In
// All reads of a sweep see the previous iteration's labels (synchronous
// semantics, as in the reference), so results do not depend on the order in
// which vertices are processed.
#include "common.cuh"
#include "internal.h"
#include "scan.cuh"

namespace gala {

static int g_num_sms = 0;
static int num_sms()
{
    if (g_num_sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (g_num_sms <= 0) g_num_sms = 148;
    }
    return g_num_sms;
}
int hub_grid_size() { return num_sms(); }

constexpr int kCountBlock = 1024;


// Exact 128-bit block sum added to the (lo, hi) counter pair (carry from the
// low word's atomic result, so the total does not depend on the order).
__device__ __forceinline__ void block_add_u128(unsigned __int128 v, unsigned long long *lo, unsigned long long *hi)
{
    __shared__ unsigned long long rlo[32], rhi[32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        const unsigned long long l = __shfl_xor_sync(GALA_FULL_MASK, (unsigned long long)v, o);
        const unsigned long long h = __shfl_xor_sync(GALA_FULL_MASK, (unsigned long long)(v >> 64), o);
        v += ((unsigned __int128)h << 64) | l;
    }
    if (lane == 0) {
        rlo[wid] = (unsigned long long)v;
        rhi[wid] = (unsigned long long)(v >> 64);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned __int128 t = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += ((unsigned __int128)rhi[w] << 64) | rlo[w];
        const unsigned long long l = (unsigned long long)t;
        unsigned long long h = (unsigned long long)(t >> 64);
        if (l) {
            const unsigned long long old = atomicAdd(lo, l);
            if (old + l < old) h += 1;
        }
        if (h) atomicAdd(hi, h);
    }
    __syncthreads();
}

// Square sums of community weights: u64 for int32 weights, exact u128 for
// 64-bit fixed-point weights (Tot^2 up to 2^124).
template <typename WT>
struct SqSum {
    using T = unsigned long long;
    static __device__ __forceinline__ T sq(WT t) { return (T)((long long)t * t); }
    static __device__ __forceinline__ void add(T v, DevStats *st) { block_add_u64(v, &st->sum_tot2); }
};
template <>
struct SqSum<long long> {
    using T = unsigned __int128;
    static __device__ __forceinline__ T sq(long long t)
    {
        return (T)(unsigned long long)t * (unsigned long long)t;
    }
    static __device__ __forceinline__ void add(T v, DevStats *st) { block_add_u128(v, &st->sum_tot2, &st->sum_tot2_hi); }
};

// ------------------------------------------------------------------------
// Level init: labels = own id, size 1 (louvain_main_process.cu:323-353),
// then a stable counting sort of the vertices into degree bins (the reference
// uses 8 count_if + a radix sort_by_key, :298-375).
// ------------------------------------------------------------------------
template <typename WT>
__global__ void k_init_vertices(int n, int32_t *comm, WT *K, WT *Self, WT *Tot, int32_t *size, WT *In)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        comm[v] = v;
        size[v] = 1;
        K[v] = 0;
        Self[v] = 0;
        Tot[v] = 0;
        In[v] = 0;
    }
}

// Level init of a contracted level whose K and Self the contraction wrote:
// labels and sizes as above, Tot = K, In = Self, and the sums sum(K),
// sum(K^2), sum(Self) of the singleton partition without a row scan.
template <typename WT>
__global__ void __launch_bounds__(256) k_init_vertices_ks(int n, int32_t *comm, const WT *__restrict__ K,
                                                          const WT *__restrict__ Self, WT *Tot, int32_t *size,
                                                          WT *In, DevStats *st)
{
    unsigned long long sk = 0, ss = 0;
    typename SqSum<WT>::T sk2 = 0;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const WT k = K[v], sf = Self[v];
        comm[v] = v;
        size[v] = 1;
        Tot[v] = k;
        In[v] = sf;
        sk += (unsigned long long)k;
        sk2 += SqSum<WT>::sq(k);
        ss += (unsigned long long)sf;
    }
    block_add_u64(sk, &st->sum_k);
    SqSum<WT>::add(sk2, st);
    block_add_u64(ss, &st->sum_in);
}

__global__ void __launch_bounds__(kCountBlock) k_bin_count(int n, const int64_t *__restrict__ offs,
                                                           int32_t *blockcnt, int nblk, DevStats *st, BinLimits lim)
{
    __shared__ int cnt[kNumBinSlots];
    if (threadIdx.x < kNumBinSlots) cnt[threadIdx.x] = 0;
    __syncthreads();
    int v = blockIdx.x * kCountBlock + threadIdx.x;
    int deg = 0;
    if (v < n) {
        deg = (int)(offs[v + 1] - offs[v]);
        atomicAdd(&cnt[bin_of_degree(deg, lim)], 1);
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) deg = max(deg, __shfl_xor_sync(GALA_FULL_MASK, deg, o));
    if ((threadIdx.x & 31) == 0 && deg > 0) atomicMax(&st->max_deg, deg);
    __syncthreads();
    if (threadIdx.x < kNumBinSlots) blockcnt[threadIdx.x * nblk + blockIdx.x] = cnt[threadIdx.x];
}

__global__ void __launch_bounds__(kCountBlock) k_bin_scatter(int n, const int64_t *__restrict__ offs,
                                                             const int32_t *__restrict__ blockoff, int nblk,
                                                             int32_t *order, DevStats *st, BinLimits lim)
{
    __shared__ int wcnt[kCountBlock / 32][kNumBinSlots];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int v = blockIdx.x * kCountBlock + threadIdx.x;
    int b = -1;
    if (v < n) b = bin_of_degree(offs[v + 1] - offs[v], lim);
    unsigned mine = 0;
#pragma unroll
    for (int bb = 0; bb < kNumBinSlots; ++bb) {
        unsigned bal = __ballot_sync(GALA_FULL_MASK, b == bb);
        if (b == bb) mine = bal;
        if (lane == 0) wcnt[wid][bb] = __popc(bal);
    }
    __syncthreads();
    if (threadIdx.x < kNumBinSlots) {
        int acc = 0;
        for (int w = 0; w < kCountBlock / 32; ++w) {
            int t = wcnt[w][threadIdx.x];
            wcnt[w][threadIdx.x] = acc;
            acc += t;
        }
    }
    __syncthreads();
    if (b >= 0) order[blockoff[b * nblk + blockIdx.x] + wcnt[wid][b] + __popc(mine & lanemask_lt())] = v;
    if (blockIdx.x == 0 && threadIdx.x <= kNumBinSlots)
        st->bin_start[threadIdx.x] = threadIdx.x < kNumBinSlots ? blockoff[threadIdx.x * nblk] : n;
}

// Symmetry hash of one entry: h(v, u, w) - h(u, v, w), summed over all
// entries modulo 2^64 (stats->sym_hash), is 0 when every entry has a mirror.
// Two rounds of the murmur3 finaliser per 32-bit half.
__device__ __forceinline__ unsigned fmix32(unsigned h)
{
    h ^= h >> 16;
    h *= 0x85EBCA6Bu;
    h ^= h >> 13;
    h *= 0xC2B2AE35u;
    return h ^ (h >> 16);
}
__device__ __forceinline__ unsigned long long dir_hash(int a, int b, unsigned long long w)
{
    const unsigned wl = (unsigned)w, wh = (unsigned)(w >> 32);
    const unsigned x = fmix32((unsigned)a ^ fmix32((unsigned)b ^ 0x9E3779B9u) ^ wl);
    const unsigned y = fmix32((unsigned)b + fmix32((unsigned)a + 0x7F4A7C15u) + wh * 0x85EBCA77u + wl);
    return ((unsigned long long)x << 32) | y;
}
__device__ __forceinline__ unsigned long long sym_term(int v, int u, unsigned long long w)
{
    return dir_hash(v, u, w) - dir_hash(u, v, w);
}

// K = row weight sum, Self = self-loop weight (init_communities,
// kernel_functions.cu:34-73); Tot = K, In = Self.  Accumulates sum(K),
// sum(K^2) and sum(Self) for the modularity of the singleton partition, and
// the symmetry hash.
template <typename WT, int G, bool W>
__global__ void __launch_bounds__(256) k_init_rows_group(const int32_t *__restrict__ list, int count,
                                                         const int64_t *__restrict__ offs,
                                                         const int32_t *__restrict__ nbr,
                                                         const WT *__restrict__ w, WT *K, WT *Self, WT *Tot,
                                                         WT *In, DevStats *st)
{
    const int lane = threadIdx.x & 31, sub = lane & (G - 1), gw = lane / G;
    constexpr int GPW = 32 / G;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    unsigned long long sk = 0, ss = 0, hs = 0;
    typename SqSum<WT>::T sk2 = 0;
    for (int base = wg * GPW; base < count; base += nw * GPW) {
        const int idx = base + gw;
        const bool has = idx < count;
        int v = 0;
        long long s = 0, e = 0;
        if (has) {
            v = list[idx];
            s = offs[v];
            e = offs[v + 1];
        }
        WT k = 0, sf = 0;
        for (long long j = s + sub; j < e; j += G) {
            WT wt = W ? w[j] : 1;
            const int u = nbr[j];
            k += wt;
            if (u == v) sf = wt;
            hs += sym_term(v, u, (unsigned long long)wt);
        }
#pragma unroll
        for (int o = G / 2; o >= 1; o >>= 1) {
            k += __shfl_xor_sync(GALA_FULL_MASK, k, o);
            sf += __shfl_xor_sync(GALA_FULL_MASK, sf, o);
        }
        if (has && sub == 0) {
            K[v] = k;
            Tot[v] = k;
            Self[v] = sf;
            In[v] = sf;
            sk += (unsigned long long)k;
            sk2 += SqSum<WT>::sq(k);
            ss += (unsigned long long)sf;
        }
    }
    block_add_u64(sk, &st->sum_k);
    SqSum<WT>::add(sk2, st);
    block_add_u64(ss, &st->sum_in);
    block_add_u64(hs, &st->sym_hash);
}

template <typename WT, bool W>
__global__ void __launch_bounds__(256) k_init_rows_cta(const int32_t *__restrict__ list, int count,
                                                       const int64_t *__restrict__ offs,
                                                       const int32_t *__restrict__ nbr,
                                                       const WT *__restrict__ w, WT *K, WT *Self, WT *Tot, WT *In,
                                                       DevStats *st)
{
    __shared__ WT rk[8], rs[8];
    unsigned long long sk = 0, ss = 0, hs = 0;
    typename SqSum<WT>::T sk2 = 0;
    for (int i = blockIdx.x; i < count; i += gridDim.x) {
        int v = list[i];
        long long s = offs[v], e = offs[v + 1];
        WT k = 0, sf = 0;
        for (long long j = s + threadIdx.x; j < e; j += blockDim.x) {
            WT wt = W ? w[j] : 1;
            const int u = nbr[j];
            k += wt;
            if (u == v) sf = wt;
            hs += sym_term(v, u, (unsigned long long)wt);
        }
        k = warp_sum(k);
        sf = warp_sum(sf);
        if ((threadIdx.x & 31) == 0) {
            rk[threadIdx.x >> 5] = k;
            rs[threadIdx.x >> 5] = sf;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            k = 0;
            sf = 0;
            for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
                k += rk[q];
                sf += rs[q];
            }
            K[v] = k;
            Tot[v] = k;
            Self[v] = sf;
            In[v] = sf;
            sk += (unsigned long long)k;
            sk2 += SqSum<WT>::sq(k);
            ss += (unsigned long long)sf;
        }
        __syncthreads();
    }
    block_add_u64(sk, &st->sum_k);
    SqSum<WT>::add(sk2, st);
    block_add_u64(ss, &st->sum_in);
    block_add_u64(hs, &st->sym_hash);
}

__global__ void k_reset_level_stats(DevStats *st)
{
    st->sum_in = 0;
    st->sum_tot2 = 0;
    st->sum_tot2_hi = 0;
    st->sum_self = 0;
    st->sum_k = 0;
    st->max_deg = 0;
    st->err = 0;
    st->n_movers = 0;
    st->sym_hash = 0;
}

void p1_reset_level_stats(Phase1Buffers &b, cudaStream_t st)
{
    k_reset_level_stats<<<1, 1, 0, st>>>(b.stats);
    note_launch(1);
}

template <typename WT>
static void launch_init_rows(const LevelGraph &g, Phase1Buffers &b, int bin, const int32_t *list, int cnt,
                             cudaStream_t st, DevStats *stats = nullptr)
{
    if (cnt <= 0) return;
    if (!stats) stats = b.stats;
    const bool W = g.w != nullptr;
    const WT *w = (const WT *)g.w;
    WT *K = (WT *)b.K, *Self = (WT *)b.Self, *Tot = (WT *)b.Tot, *In = (WT *)b.In;
    const int cap = num_sms() * 8;
    auto grid_for = [&](int G) {
        long long blocks = ((long long)cnt * G + 255) / 256;
        return (int)(blocks < cap ? blocks : cap);
    };
#define GALA_INIT_GROUP(GV)                                                                              \
    do {                                                                                                 \
        if (W)                                                                                           \
            k_init_rows_group<WT, GV, true><<<grid_for(GV), 256, 0, st>>>(list, cnt, g.offs, g.nbr, w, K,  \
                                                                          Self, Tot, In, stats);         \
        else                                                                                             \
            k_init_rows_group<WT, GV, false><<<grid_for(GV), 256, 0, st>>>(list, cnt, g.offs, g.nbr, w, K, \
                                                                           Self, Tot, In, stats);        \
    } while (0)
    switch (bin) {
    case 0: GALA_INIT_GROUP(4); break;
    case 1: GALA_INIT_GROUP(8); break;
    case 2: GALA_INIT_GROUP(16); break;
    case 3:
    case 4:
    case 5: GALA_INIT_GROUP(32); break;
    default: {
        int grid = cnt < cap ? cnt : cap;
        if (W)
            k_init_rows_cta<WT, true><<<grid, 256, 0, st>>>(list, cnt, g.offs, g.nbr, w, K, Self, Tot, In, stats);
        else
            k_init_rows_cta<WT, false><<<grid, 256, 0, st>>>(list, cnt, g.offs, g.nbr, w, K, Self, Tot, In, stats);
    }
    }
#undef GALA_INIT_GROUP
    note_launch(1);
}

// Level init part 1: labels/sizes, degree-bin counting sort.  The caller reads
// bin_start back before calling p1_level_init_rows.
void p1_level_init(const LevelGraph &g, Phase1Buffers &b, cudaStream_t st)
{
    const int n = g.n;
    const int nblk = (n + kCountBlock - 1) / kCountBlock;
    const int grid = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
    if (g.ks_ready && g.wide)
        k_init_vertices_ks<long long><<<grid, 256, 0, st>>>(n, b.comm, (const long long *)b.K,
                                                            (const long long *)b.Self, (long long *)b.Tot, b.size,
                                                            (long long *)b.In, b.stats);
    else if (g.ks_ready)
        k_init_vertices_ks<int><<<grid, 256, 0, st>>>(n, b.comm, b.K, b.Self, b.Tot, b.size, b.In, b.stats);
    else if (g.wide)
        k_init_vertices<long long><<<grid, 256, 0, st>>>(n, b.comm, (long long *)b.K, (long long *)b.Self,
                                                         (long long *)b.Tot, b.size, (long long *)b.In);
    else
        k_init_vertices<int><<<grid, 256, 0, st>>>(n, b.comm, b.K, b.Self, b.Tot, b.size, b.In);
    k_bin_count<<<nblk, kCountBlock, 0, st>>>(n, g.offs, b.blockcnt, nblk, b.stats, b.lim);
    exclusive_scan(b.blockcnt, b.blockoff, (long long)kNumBinSlots * nblk, OpIdentity(), b.scan_partial,
                   &b.stats->total, st, &b.stats->err);
    k_bin_scatter<<<nblk, kCountBlock, 0, st>>>(n, g.offs, b.blockoff, nblk, b.order, b.stats, b.lim);
    note_launch(3);
}

// Unweighted level whose rows are still being copied: K = Tot = degree of
// every vertex from the offsets alone, so a vertex's first sweep needs only
// its own row.
__global__ void k_init_degree(int n, const int64_t *__restrict__ offs, int32_t *K, int32_t *Tot)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const int d = (int)(offs[v + 1] - offs[v]);
        K[v] = d;
        Tot[v] = d;
    }
}

// Sub-ranges of the degree bins per row chunk: lo[k][bin] = first position in
// the bin's segment of the order list (ascending ids within a bin) of a vertex
// id >= vstart[k]; cnt[k][bin] = lo[k + 1][bin] - lo[k][bin].
__global__ void k_chunk_bounds(const int32_t *__restrict__ order, const DevStats *__restrict__ st, ChunkStarts vs,
                               int P, int32_t *lo, int32_t *cnt)
{
    const int32_t *vstart = vs.v;
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (P + 1) * kNumBins) return;
    const int k = t / kNumBins, bin = t % kNumBins;
    const int bs = st->bin_start[bin], be = st->bin_start[bin + 1];
    auto first_ge = [&](int id) {
        int l = bs, h = be;  // first position in [bs, be) with order >= id
        while (l < h) {
            const int m = (l + h) >> 1;
            if (order[m] < id) l = m + 1;
            else h = m;
        }
        return l - bs;
    };
    const int a = k < P ? first_ge(vstart[k]) : be - bs;
    lo[k * kNumBins + bin] = a;
    if (k < P) cnt[k * kNumBins + bin] = (k + 1 < P ? first_ge(vstart[k + 1]) : be - bs) - a;
}

void p1_init_degree(const LevelGraph &g, Phase1Buffers &b, cudaStream_t st)
{
    const int grid = std::min((g.n + 255) / 256, num_sms() * 8);
    k_init_degree<<<grid > 0 ? grid : 1, 256, 0, st>>>(g.n, g.offs, b.K, b.Tot);
    note_launch(1);
}

void p1_chunk_bounds(Phase1Buffers &b, const ChunkStarts &vs, int P, int32_t *d_lo, int32_t *d_cnt, cudaStream_t st)
{
    const int t = (P + 1) * kNumBins;
    k_chunk_bounds<<<(t + 127) / 128, 128, 0, st>>>(b.order, b.stats, vs, P, d_lo, d_cnt);
    note_launch(1);
}

void p1_init_rows_range(const LevelGraph &g, Phase1Buffers &b, int bin, const int32_t *list, int cnt, DevStats *stats,
                        cudaStream_t st)
{
    if (g.wide)
        launch_init_rows<long long>(g, b, bin, list, cnt, st, stats);
    else
        launch_init_rows<int>(g, b, bin, list, cnt, st, stats);
}

void p1_level_init_rows(const LevelGraph &g, Phase1Buffers &b, const int *bin_start, cudaStream_t st)
{
    if (g.ks_ready) return;  // K, Self, Tot, In and the sums came with the level init
    for (int bin = 0; bin < kNumBins; ++bin) {
        if (g.wide)
            launch_init_rows<long long>(g, b, bin, b.order + bin_start[bin], bin_start[bin + 1] - bin_start[bin], st);
        else
            launch_init_rows<int>(g, b, bin, b.order + bin_start[bin], bin_start[bin + 1] - bin_start[bin], st);
    }
}

// ------------------------------------------------------------------------
// Decide-and-move
// ------------------------------------------------------------------------
template <typename WT>
struct DecideArgs {
    const int64_t *__restrict__ offs;
    const int32_t *__restrict__ nbr;
    const WT *__restrict__ w;
    const int32_t *__restrict__ comm;
    const WT *__restrict__ K;
    const WT *__restrict__ Self;
    const WT *__restrict__ Tot;
    const int32_t *__restrict__ size;
    int32_t *mv_v, *mv_old, *mv_new;
    DevStats *st;
    double constant;  // 1 / m2
    long long m2;
    int fp64_only;    // 1 = evaluate every vertex with the FP64 expressions
    float *feat_gain;   // proposal features (null when no proposal mode is on)
    int32_t *feat_ndist;
    // batched graphs (null for one graph): graph of each vertex, its total
    // weight m2 and 1/m2, and the graphs whose phase 1 has stopped
    const int32_t *__restrict__ gid;
    const long long *__restrict__ m2g;
    const double *__restrict__ cg;
    const uint8_t *__restrict__ stop;
};

// Gain scale of a vertex: m2 and 1/m2 of its graph.
struct Scale {
    long long m2;
    double c;
};
template <typename WT>
__device__ __forceinline__ Scale scale_of(const DecideArgs<WT> &a, int v)
{
    if (a.gid) {
        const int g = a.gid[v];
        return Scale{a.m2g[g], a.cg[g]};
    }
    return Scale{a.m2, a.constant};
}
// Vertex of a batched graph whose phase 1 has stopped: not decided.
template <typename WT>
__device__ __forceinline__ bool stopped(const DecideArgs<WT> &a, int v)
{
    return a.stop && a.stop[a.gid[v]];
}

// Proposal features of a decided vertex: its best corrected gain
// (max(X, 0) - (w_cur - Self) m2, normalised by K m2) and the number of
// distinct neighbour communities (-1 when the schedule does not count them).
template <typename WT>
__device__ __forceinline__ void write_features(const DecideArgs<WT> &a, const Scale &sc, int v, long long x, WT w_cur,
                                               WT self_w, WT ki, int ndist)
{
    if constexpr (!WideOf<WT>::exact) return;  // no proposal modes on fixed-point weights
    if (!a.feat_gain) return;
    const long long y = (x > 0 ? x : 0) - (long long)(w_cur - self_w) * sc.m2;
    a.feat_gain[v] = ki > 0 ? (float)y / ((float)sc.m2 * (float)ki) : 0.f;
    a.feat_ndist[v] = ndist;
}

// Singleton swap guard (kernel_functions.cu:386): two singletons never move
// towards the larger id.
template <typename WT>
__device__ __forceinline__ bool guard_ok(const DecideArgs<WT> &a, int cur, int best)
{
    return !(a.size[best] == 1 && a.size[cur] == 1 && best > cur);
}

// ---- exact integer gains ---------------------------------------------------
// The reference's gain dq = 2w - 2K((Tot_c - Tot_cur) + K)/m2 equals
// (2/m2) * X with the integer X = w*m2 - K*((Tot_c - Tot_cur) + K), which fits
// int64 for m2 < 2^31.  Distinct X differ by at least 2/m2 in dq, while the
// FP64 evaluation errs by at most K * 2^-50; so for K*m2 < 2^49 the FP64 order
// of distinct X is the exact order and the sign of a non-zero X (or of the
// corrected gain) is exact.  Three cases can still round either way and are
// re-evaluated with the FP64 expressions of the reference: equal best X from
// different weights (FP64 may order them by value, not by id), X = 0 when
// the vertex has no other weight in its community, and a corrected gain of
// exactly 0.  Everything else is decided in integer arithmetic (GB300 runs
// FP64 at a small fraction of its integer rate).
// (Fixed-point weights have no exact-integer path: X is 0 for every
// candidate and int_decision sends the vertex to the FP64 evaluation.)
template <typename WT>
__device__ __forceinline__ long long gain_x(WT w, WT ki, WT tc, WT tcur, long long m2)
{
    if constexpr (!WideOf<WT>::exact) return 0;
    return (long long)w * m2 - (long long)ki * ((long long)tc - (long long)tcur + (long long)ki);
}

// Merge candidate (ox, oc, ow, ot) into (x, c, w, t): larger X first, then the
// lower id; t records a tie on the best X between different weights.
// Commutative, so butterfly reductions agree on every lane.
template <typename WT>
__device__ __forceinline__ void cand_merge(long long &x, int &c, WT &w, int &t, long long ox, int oc, WT ow, int ot)
{
    if (ox == x) {
        int tie = t | ot | (ow != w);
        if (oc < c) {
            c = oc;
            w = ow;
        }
        t = tie;
    } else if (ox > x) {
        x = ox;
        c = oc;
        w = ow;
        t = ot;
    }
}

// 0 = stay, 1 = move (before the singleton guard), 2 = evaluate in FP64.
template <typename WT>
__device__ __forceinline__ int int_decision(const DecideArgs<WT> &a, const Scale &sc, long long x, int t, int cur,
                                            int best, WT w_cur, WT self_w, WT ki)
{
    if constexpr (!WideOf<WT>::exact) return 2;
    if (a.fp64_only || (long long)ki * sc.m2 >= (1LL << 49)) return 2;
    if (best == cur) return 0;  // every candidate has X < 0: every FP64 gain is < 0
    if (x == 0) return w_cur == self_w ? 2 : 0;
    if (t) return 2;
    const long long y = x - (long long)(w_cur - self_w) * sc.m2;
    if (y == 0) return 2;
    return y > 0 ? 1 : 0;
}

template <typename WT>
__device__ __forceinline__ void warp_merge_int(long long &x, int &c, WT &w, int &t, WT &wc, int width)
{
    for (int o = width / 2; o >= 1; o >>= 1) {
        long long ox = __shfl_xor_sync(GALA_FULL_MASK, x, o);
        int oc = __shfl_xor_sync(GALA_FULL_MASK, c, o);
        WT ow = __shfl_xor_sync(GALA_FULL_MASK, w, o);
        int ot = __shfl_xor_sync(GALA_FULL_MASK, t, o);
        wc += __shfl_xor_sync(GALA_FULL_MASK, wc, o);
        cand_merge(x, c, w, t, ox, oc, ow, ot);
    }
}

template <typename WT>
__device__ __forceinline__ void append_mover(const DecideArgs<WT> &a, bool move, int v, int cur, int best)
{
    unsigned b = __ballot_sync(GALA_FULL_MASK, move);
    if (b == 0) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(b) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&a.st->n_movers, __popc(b));
    base = __shfl_sync(GALA_FULL_MASK, base, leader);
    if (move) {
        int p = base + __popc(b & lanemask_lt());
        a.mv_v[p] = v;
        a.mv_old[p] = cur;
        a.mv_new[p] = best;
    }
}

// Degree <= G: one lane per neighbour.  Lanes holding the same neighbour
// community are found with __match_any_sync (the key carries the group index
// so groups of one warp stay apart) and their weights summed with
// __reduce_add_sync; the lowest lane of each set evaluates the gain.
constexpr int kStageN = 256;  // staged active-list appends per warp
constexpr int kStageM = 128;  // staged movers per warp
template <typename WT, int G, bool W>
__global__ void __launch_bounds__(256) k_decide_group(DecideArgs<WT> a, const int32_t *__restrict__ list,
                                                      const int *__restrict__ count_ptr)
{
    const int lane = threadIdx.x & 31, sub = lane & (G - 1), gw = lane / G;
    constexpr int GPW = 32 / G;
    const int count = *count_ptr;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    __shared__ int stage_buf[8][3 * kStageM];
    WarpStage<kStageM, 3> stage{stage_buf[threadIdx.x >> 5], 0};
    int *const mlists[3] = {a.mv_v, a.mv_old, a.mv_new};
    for (int base = wg * GPW; base < count; base += nw * GPW) {
        const int idx = base + gw;
        bool has = idx < count;
        int v = 0, cur = -1, deg = 0;
        WT ki = 0, sf = 0, tcur = 0;
        long long s = 0;
        Scale sc{a.m2, a.constant};
        if (has) {
            v = list[idx];
            has = !stopped(a, v);
        }
        if (has) {
            sc = scale_of(a, v);
            s = a.offs[v];
            deg = (int)(a.offs[v + 1] - s);
            cur = a.comm[v];
            ki = a.K[v];
            sf = a.Self[v];
            tcur = a.Tot[cur];
        }
        const bool valid = has && sub < deg;
        int c = -1;
        WT wt = 0;
        if (valid) {
            c = a.comm[a.nbr[s + sub]];
            wt = W ? a.w[s + sub] : 1;
        }
        // lanes of the group holding the same community: the lowest leads and
        // sums the weights (G - 1 shuffles for small groups, a key match for
        // whole warps)
        WT wsum;
        bool leader;
        if constexpr (G == 32) {
            const unsigned m = __match_any_sync(GALA_FULL_MASK, c);
            wsum = W ? group_sum(m, wt) : (WT)__popc(m);
            leader = valid && (__ffs(m) - 1 == lane);
        } else {
            wsum = wt;
            leader = valid;
#pragma unroll
            for (int o = 1; o < G; ++o) {
                const int osub = (sub + o) & (G - 1);
                const int src = (lane & ~(G - 1)) | osub;
                const int oc = __shfl_sync(GALA_FULL_MASK, c, src);
                const WT ow = __shfl_sync(GALA_FULL_MASK, wt, src);
                if (oc == c) {
                    wsum += ow;
                    if (osub < sub) leader = false;
                }
            }
        }
        const WT wc_own = (leader && c == cur) ? wsum : 0;
        WT wc = wc_own;
        WT tc = 0;
        long long x = -1;
        int bc = cur, bt = 0;
        WT bw = 0;
        if (leader && c != cur) {
            tc = a.Tot[c];
            const long long xx = gain_x(wsum, ki, tc, tcur, sc.m2);
            if (xx >= 0) {
                x = xx;
                bc = c;
                bw = wsum;
            }
        }
        warp_merge_int(x, bc, bw, bt, wc, G);
        int dec = 0;
        if (has && sub == 0) dec = int_decision(a, sc, x, bt, cur, bc, wc, sf, ki);
        const bool fp = dec == 2;
        if (__any_sync(GALA_FULL_MASK, fp)) {
            // the reference's FP64 evaluation of the same candidates
            double dq = 0.0;
            int fc = cur;
            if (leader && c != cur) {
                const double d = gain_dq(wsum, ki, tc, tcur, sc.c);
                if (d > 0.0) {
                    dq = d;
                    fc = c;
                }
            }
#pragma unroll
            for (int o = G / 2; o >= 1; o >>= 1) {
                const double od = __shfl_xor_sync(GALA_FULL_MASK, dq, o);
                const int oc = __shfl_xor_sync(GALA_FULL_MASK, fc, o);
                if (cand_better(od, oc, dq, fc)) {
                    dq = od;
                    fc = oc;
                }
            }
            if (fp) {
                bc = fc;
                dec = (fc != cur && gain_correct(dq, wc, sf) > 0.0) ? 1 : 0;
                atomicAdd(&a.st->fp64_decisions, 1ull);
            }
        }
        const bool move = has && sub == 0 && dec == 1 && guard_ok(a, cur, bc);
        if (a.feat_gain) {
            const unsigned lb = __ballot_sync(GALA_FULL_MASK, leader);
            const unsigned gmask = G == 32 ? GALA_FULL_MASK : (((1u << G) - 1u) << (gw * G));
            if (has && sub == 0) write_features(a, sc, v, x, wc, sf, ki, __popc(lb & gmask));
        }
        const int item[3] = {v, cur, bc};
        stage.push(move, item, mlists, &a.st->n_movers);
    }
    stage.flush(mlists, &a.st->n_movers);
}

// Scan a hash table: this thread's best candidate by exact X and its share of
// the weight to the own community.
template <typename WT>
__device__ __forceinline__ void scan_table_int(const DecideArgs<WT> &a, const Scale &sc, const int *keys,
                                               const WT *vals, int T, int first, int stride, int cur, WT ki,
                                               WT tcur, long long &x, int &bc, WT &bw, int &bt, WT &wc)
{
    for (int j = first; j < T; j += stride) {
        const int c = keys[j];
        if (c < 0) continue;
        const WT wv = vals[j];
        if (c == cur) {
            wc += wv;
        } else {
            const long long xx = gain_x(wv, ki, a.Tot[c], tcur, sc.m2);
            if (xx >= 0) cand_merge(x, bc, bw, bt, xx, c, wv, 0);
        }
    }
}

// The same scan with the reference's FP64 gains (vertices int_decision
// cannot settle).
template <typename WT>
__device__ __forceinline__ void scan_table(const DecideArgs<WT> &a, const Scale &sc, const int *keys, const WT *vals,
                                           int T, int first, int stride, int cur, WT ki, WT tcur, double &dq,
                                           int &bc)
{
    for (int j = first; j < T; j += stride) {
        int c = keys[j];
        if (c < 0 || c == cur) continue;
        double d = gain_dq(vals[j], ki, a.Tot[c], tcur, sc.c);
        if (d > 0.0 && cand_better(d, c, dq, bc)) {
            dq = d;
            bc = c;
        }
    }
}

__device__ __forceinline__ void warp_argmax(double &dq, int &bc)
{
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        double od = __shfl_xor_sync(GALA_FULL_MASK, dq, o);
        int oc = __shfl_xor_sync(GALA_FULL_MASK, bc, o);
        if (cand_better(od, oc, dq, bc)) {
            dq = od;
            bc = oc;
        }
    }
}

// Insert (key, w) into a table of T slots (power of two); returns the slot
// and sets `created` when this call claimed it, -1 when the probe ran out.
template <typename VT>
__device__ __forceinline__ int hash_add_slot(int *keys, VT *vals, int T, int log2t, int key, VT w, bool &created)
{
    // one compare-and-swap per probe: it claims an empty slot or returns the
    // key that holds it
    unsigned h = hash_slot(key, log2t);
    created = false;
    for (int p = 0; p < T; ++p) {
        const int k = atomicCAS(&keys[h], -1, key);
        if (k == -1 || k == key) {
            created = k == -1;
            atomic_add_w(&vals[h], w);
            return (int)h;
        }
        h = (h + 1) & (unsigned)(T - 1);
    }
    return -1;
}

// Scans over the list of occupied slots (slot indices in occ[0, nocc)).
template <typename WT>
__device__ __forceinline__ void scan_list_int(const DecideArgs<WT> &a, const Scale &sc, const int *keys,
                                              const WT *vals, const unsigned short *occ, int nocc, int first,
                                              int stride, int cur, WT ki, WT tcur, long long &x, int &bc, WT &bw,
                                              int &bt, WT &wc)
{
    // X = w m2 - K Tot_c - K (K - Tot_cur): the last term is per vertex
    const long long xbase = WideOf<WT>::exact ? (long long)ki * ((long long)ki - (long long)tcur) : 0;
    for (int q = first; q < nocc; q += stride) {
        const int j = occ[q];
        const int c = keys[j];
        const WT wv = vals[j];
        if (c == cur) {
            wc += wv;
        } else {
            const long long xx = WideOf<WT>::exact
                                     ? (long long)wv * sc.m2 - (long long)ki * (long long)a.Tot[c] - xbase
                                     : 0;
            if (xx >= 0) cand_merge(x, bc, bw, bt, xx, c, wv, 0);
        }
    }
}

template <typename WT>
__device__ __forceinline__ void scan_list(const DecideArgs<WT> &a, const Scale &sc, const int *keys, const WT *vals,
                                          const unsigned short *occ, int nocc, int first, int stride, int cur, WT ki,
                                          WT tcur, double &dq, int &bc)
{
    for (int q = first; q < nocc; q += stride) {
        const int j = occ[q];
        const int c = keys[j];
        if (c == cur) continue;
        const double d = gain_dq(vals[j], ki, a.Tot[c], tcur, sc.c);
        if (d > 0.0 && cand_better(d, c, dq, bc)) {
            dq = d;
            bc = c;
        }
    }
}

// Degree 33-256: one warp per vertex with a private shared-memory hash table
// of TW slots (two launches: 256 slots for rows up to 128 entries, with eight
// resident blocks per SM at 32 registers a thread, and 512 slots for longer
// rows).  The table is cleared once per warp; per vertex the slots it claims
// are listed, and only those are scanned and cleared again.
constexpr int kWarpTable = 512;  // the full table; rows up to kWarpTable / 4 use half of it
constexpr int kWarpWarps = 8;  // warps per block
// TW slots per warp for rows up to TW / 2 entries (a vertex claims at most
// as many slots as it has entries)
template <typename WT, int TW>
constexpr size_t warp_smem()
{
    return (size_t)kWarpWarps * (TW * (sizeof(int) + sizeof(WT)) + (TW / 2) * sizeof(unsigned short));
}
template <typename WT, bool W, int TW, int MINB>
__global__ void __launch_bounds__(256, MINB) k_decide_warp(DecideArgs<WT> a, const int32_t *__restrict__ list,
                                                     const int *__restrict__ count_ptr, int dlo, int dhi)
{
    extern __shared__ long long wsm_ll[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    constexpr int TL = TW == 256 ? 8 : 9;
    static_assert((1 << TL) == TW, "table size");
    WT *vals = (WT *)wsm_ll + wib * TW;
    int *keys = (int *)((WT *)wsm_ll + kWarpWarps * TW) + wib * TW;
    unsigned short *occ =
        (unsigned short *)((int *)((WT *)wsm_ll + kWarpWarps * TW) + kWarpWarps * TW) + wib * (TW / 2);
    for (int j = lane; j < TW; j += 32) {
        keys[j] = -1;
        vals[j] = 0;
    }
    __syncwarp();
    const int count = *count_ptr;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = wg; i < count; i += nw) {
        const int v = list[i];
        if (stopped(a, v)) continue;
        const Scale sc = scale_of(a, v);
        const long long s = a.offs[v];
        const int deg = (int)(a.offs[v + 1] - s);
        if (deg <= dlo || deg > dhi) continue;  // the other launch of this bin decides it
        const int cur = a.comm[v];
        int nocc = 0;
        const int32_t *rn = a.nbr + s;
        const WT *rw = W ? a.w + s : nullptr;
        for (int e0 = 0; e0 < deg; e0 += 32) {
            const int e = e0 + lane;
            const bool valid = e < deg;
            int c = -1;
            WT wt = 0;
            if (valid) {
                c = a.comm[rn[e]];
                wt = W ? rw[e] : 1;
            }
            // every entry goes to the table on its own: repeated communities
            // meet at their slot (a warp-level match of equal keys costs more
            // than the repeated adds it saves)
            bool created = false;
            int slot = -1;
            if (valid) {
                slot = hash_add_slot(keys, vals, TW, TL, c, wt, created);
                if (slot < 0) atomicOr(&a.st->err, kErrHashOverflow);
            }
            const unsigned cb = __ballot_sync(GALA_FULL_MASK, created);
            if (created) occ[nocc + __popc(cb & lanemask_lt())] = (unsigned short)slot;
            nocc += __popc(cb);
        }
        __syncwarp();
        const WT ki = a.K[v], tcur = a.Tot[cur], sf = a.Self[v];
        long long x = -1;
        int bc = cur, bt = 0;
        WT bw = 0, wc = 0;
        scan_list_int(a, sc, keys, vals, occ, nocc, lane, 32, cur, ki, tcur, x, bc, bw, bt, wc);
        warp_merge_int(x, bc, bw, bt, wc, 32);
        int dec = int_decision(a, sc, x, bt, cur, bc, wc, sf, ki);  // warp-uniform
        if (dec == 2) {
            double dq = 0.0;
            int fc = cur;
            scan_list(a, sc, keys, vals, occ, nocc, lane, 32, cur, ki, tcur, dq, fc);
            warp_argmax(dq, fc);
            bc = fc;
            dec = (fc != cur && gain_correct(dq, wc, sf) > 0.0) ? 1 : 0;
            if (lane == 0) atomicAdd(&a.st->fp64_decisions, 1ull);
        }
        const bool move = lane == 0 && dec == 1 && guard_ok(a, cur, bc);
        if (lane == 0) write_features(a, sc, v, x, wc, sf, ki, nocc);
        append_mover(a, move, v, cur, bc);
        __syncwarp();
        for (int q = lane; q < nocc; q += 32) {
            const int j = occ[q];
            keys[j] = -1;
            vals[j] = 0;
        }
        __syncwarp();
    }
}

// Resident 256-thread blocks per SM of the 33-256 kernel (occupancy query,
// cached per instantiation).
template <typename WT, int TW, int MINB>
int warp_resident(bool W)
{
    static int cached[2] = {0, 0};
    int &r = cached[W ? 1 : 0];
    if (r == 0) {
        int k = 0;
        if (W)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, k_decide_warp<WT, true, TW, MINB>, 256,
                                                          warp_smem<WT, TW>());
        else
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, k_decide_warp<WT, false, TW, MINB>, 256,
                                                          warp_smem<WT, TW>());
        r = k > 0 ? k : 1;
    }
    return r;
}

// Degree 257-8192: one CTA per vertex with a shared-memory hash table of tmax
// slots (int keys, WT values) and the list of claimed slots, cleared once per
// CTA and then slot by slot after every vertex.
template <typename WT>
constexpr size_t cta_smem(int tmax)
{
    // a vertex claims at most deg <= tmax / 2 slots
    return (size_t)tmax * (sizeof(int) + sizeof(WT)) + (size_t)(tmax / 2) * sizeof(unsigned short);
}
template <typename WT, int BLOCK, bool W>
__global__ void __launch_bounds__(BLOCK) k_decide_cta(DecideArgs<WT> a, const int32_t *__restrict__ list,
                                                      const int *__restrict__ count_ptr, int tmax, int dlo,
                                                      int dhi)
{
    extern __shared__ long long dyn_smem_ll[];
    __shared__ double r_dq[BLOCK / 32];
    __shared__ long long r_x[BLOCK / 32];
    __shared__ int r_c[BLOCK / 32];
    __shared__ WT r_w[BLOCK / 32];
    __shared__ int r_t[BLOCK / 32];
    __shared__ WT r_wc[BLOCK / 32];
    __shared__ int s_dec, s_bc, s_nocc;
    __shared__ WT s_wc;
    WT *vals = (WT *)dyn_smem_ll;
    int *keys = (int *)(vals + tmax);
    unsigned short *occ = (unsigned short *)(keys + tmax);
    const int lg = __ffs(tmax) - 1;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int j = threadIdx.x; j < tmax; j += BLOCK) {
        keys[j] = -1;
        vals[j] = 0;
    }
    if (threadIdx.x == 0) s_nocc = 0;
    __syncthreads();
    const int count = *count_ptr;
    for (int i = blockIdx.x; i < count; i += gridDim.x) {
        const int v = list[i];
        if (stopped(a, v)) continue;
        const Scale sc = scale_of(a, v);
        const long long s = a.offs[v];
        const long long e = a.offs[v + 1];
        const int deg = (int)(e - s);
        const int cur = a.comm[v];
        if (deg <= dlo || deg > dhi) continue;  // the other launch of this bin decides it
        if (2LL * deg > tmax) {  // cannot happen for the bin limits; recorded, vertex stays
            if (threadIdx.x == 0) atomicOr(&a.st->err, kErrHashOverflow);
            continue;
        }
        for (long long b0 = s; b0 < e; b0 += BLOCK) {
            const long long j = b0 + threadIdx.x;
            const bool valid = j < e;
            int c = -1;
            WT wt = 0;
            if (valid) {
                c = a.comm[a.nbr[j]];
                wt = W ? a.w[j] : 1;
            }
            bool created = false;
            int slot = -1;
            if (valid) {
                slot = hash_add_slot(keys, vals, tmax, lg, c, wt, created);
                if (slot < 0) atomicOr(&a.st->err, kErrHashOverflow);
            }
            const unsigned cb = __ballot_sync(GALA_FULL_MASK, created);
            if (cb) {
                const int leader = __ffs(cb) - 1;
                int base = 0;
                if (lane == leader) base = atomicAdd(&s_nocc, __popc(cb));
                base = __shfl_sync(GALA_FULL_MASK, base, leader);
                if (created) occ[base + __popc(cb & lanemask_lt())] = (unsigned short)slot;
            }
        }
        __syncthreads();
        const int nocc = s_nocc;
        const WT ki = a.K[v], tcur = a.Tot[cur], sf = a.Self[v];
        constexpr int NW = BLOCK / 32;
        long long x = -1;
        int bc = cur, bt = 0;
        WT bw = 0, wc = 0;
        scan_list_int(a, sc, keys, vals, occ, nocc, threadIdx.x, BLOCK, cur, ki, tcur, x, bc, bw, bt, wc);
        warp_merge_int(x, bc, bw, bt, wc, 32);
        if (lane == 0) {
            r_x[wid] = x;
            r_c[wid] = bc;
            r_w[wid] = bw;
            r_t[wid] = bt;
            r_wc[wid] = wc;
        }
        __syncthreads();
        if (wid == 0) {
            x = lane < NW ? r_x[lane] : -1;
            bc = lane < NW ? r_c[lane] : cur;
            bw = lane < NW ? r_w[lane] : 0;
            bt = lane < NW ? r_t[lane] : 0;
            wc = lane < NW ? r_wc[lane] : 0;
            warp_merge_int(x, bc, bw, bt, wc, 32);
            if (lane == 0) {
                s_dec = int_decision(a, sc, x, bt, cur, bc, wc, sf, ki);
                s_bc = bc;
                s_wc = wc;
            }
        }
        __syncthreads();
        if (s_dec == 2) {  // block-uniform: the reference's FP64 evaluation
            double dq = 0.0;
            int fc = cur;
            scan_list(a, sc, keys, vals, occ, nocc, threadIdx.x, BLOCK, cur, ki, tcur, dq, fc);
            warp_argmax(dq, fc);
            if (lane == 0) {
                r_dq[wid] = dq;
                r_c[wid] = fc;
            }
            __syncthreads();
            if (wid == 0) {
                dq = lane < NW ? r_dq[lane] : 0.0;
                fc = lane < NW ? r_c[lane] : cur;
                warp_argmax(dq, fc);
                if (lane == 0) {
                    s_bc = fc;
                    s_dec = (fc != cur && gain_correct(dq, s_wc, sf) > 0.0) ? 1 : 0;
                    atomicAdd(&a.st->fp64_decisions, 1ull);
                }
            }
            __syncthreads();
        }
        if (wid == 0) {
            const bool move = lane == 0 && s_dec == 1 && guard_ok(a, cur, s_bc);
            if (lane == 0) write_features(a, sc, v, x, s_wc, sf, ki, nocc);
            append_mover(a, move, v, cur, s_bc);
        }
        for (int q = threadIdx.x; q < nocc; q += BLOCK) {
            const int j = occ[q];
            keys[j] = -1;
            vals[j] = 0;
        }
        __syncthreads();
        if (threadIdx.x == 0) s_nocc = 0;
        __syncthreads();
    }
}

// First sweep of a level: every vertex is its own community (comm[u] = u
// after the level init), and rows hold distinct neighbours, so every entry
// is its own candidate community: no aggregation table.  One group of
// GROUP threads (a warp, or the whole CTA) per vertex.
template <typename WT, bool W>
__device__ __forceinline__ void first_scan_int(const DecideArgs<WT> &a, const Scale &sc, long long s, int deg, int v,
                                               int first, int stride, WT ki, WT tcur, long long &x, int &bc, WT &bw,
                                               int &bt, WT &wc)
{
    for (int j = first; j < deg; j += stride) {
        const int u = a.nbr[s + j];
        const WT w = W ? a.w[s + j] : (WT)1;
        if (u == v) {
            wc += w;
        } else {
            const long long xx = gain_x(w, ki, a.Tot[u], tcur, sc.m2);
            if (xx >= 0) cand_merge(x, bc, bw, bt, xx, u, w, 0);
        }
    }
}

template <typename WT, bool W>
__device__ __forceinline__ void first_scan(const DecideArgs<WT> &a, const Scale &sc, long long s, int deg, int v,
                                           int first, int stride, WT ki, WT tcur, double &dq, int &bc)
{
    for (int j = first; j < deg; j += stride) {
        const int u = a.nbr[s + j];
        if (u == v) continue;
        const double d = gain_dq(W ? a.w[s + j] : (WT)1, ki, a.Tot[u], tcur, sc.c);
        if (d > 0.0 && cand_better(d, u, dq, bc)) {
            dq = d;
            bc = u;
        }
    }
}

template <typename WT, bool W>
__global__ void __launch_bounds__(256) k_first_warp(DecideArgs<WT> a, const int32_t *__restrict__ list,
                                                    const int *__restrict__ count_ptr)
{
    const int lane = threadIdx.x & 31;
    const int count = *count_ptr;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = wg; i < count; i += nw) {
        const int v = list[i];
        if (stopped(a, v)) continue;
        const Scale sc = scale_of(a, v);
        const long long s = a.offs[v];
        const int deg = (int)(a.offs[v + 1] - s);
        const int cur = a.comm[v];  // = v
        const WT ki = a.K[v], tcur = a.Tot[cur], sf = a.Self[v];
        long long x = -1;
        int bc = cur, bt = 0;
        WT bw = 0, wc = 0;
        first_scan_int<WT, W>(a, sc, s, deg, v, lane, 32, ki, tcur, x, bc, bw, bt, wc);
        warp_merge_int(x, bc, bw, bt, wc, 32);
        int dec = int_decision(a, sc, x, bt, cur, bc, wc, sf, ki);  // warp-uniform
        if (dec == 2) {
            double dq = 0.0;
            int fc = cur;
            first_scan<WT, W>(a, sc, s, deg, v, lane, 32, ki, tcur, dq, fc);
            warp_argmax(dq, fc);
            bc = fc;
            dec = (fc != cur && gain_correct(dq, wc, sf) > 0.0) ? 1 : 0;
            if (lane == 0) atomicAdd(&a.st->fp64_decisions, 1ull);
        }
        const bool move = lane == 0 && dec == 1 && guard_ok(a, cur, bc);
        if (lane == 0) write_features(a, sc, v, x, wc, sf, ki, deg);
        append_mover(a, move, v, cur, bc);
    }
}

template <typename WT, int BLOCK, bool W>
__global__ void __launch_bounds__(BLOCK) k_first_cta(DecideArgs<WT> a, const int32_t *__restrict__ list,
                                                     const int *__restrict__ count_ptr)
{
    __shared__ double r_dq[BLOCK / 32];
    __shared__ long long r_x[BLOCK / 32];
    __shared__ int r_c[BLOCK / 32];
    __shared__ WT r_w[BLOCK / 32];
    __shared__ int r_t[BLOCK / 32];
    __shared__ WT r_wc[BLOCK / 32];
    __shared__ int s_dec, s_bc;
    __shared__ WT s_wc;
    constexpr int NW = BLOCK / 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int count = *count_ptr;
    for (int i = blockIdx.x; i < count; i += gridDim.x) {
        const int v = list[i];
        if (stopped(a, v)) continue;
        const Scale sc = scale_of(a, v);
        const long long s = a.offs[v];
        const int deg = (int)(a.offs[v + 1] - s);
        const int cur = a.comm[v];  // = v
        const WT ki = a.K[v], tcur = a.Tot[cur], sf = a.Self[v];
        long long x = -1;
        int bc = cur, bt = 0;
        WT bw = 0, wc = 0;
        first_scan_int<WT, W>(a, sc, s, deg, v, threadIdx.x, BLOCK, ki, tcur, x, bc, bw, bt, wc);
        warp_merge_int(x, bc, bw, bt, wc, 32);
        if (lane == 0) {
            r_x[wid] = x;
            r_c[wid] = bc;
            r_w[wid] = bw;
            r_t[wid] = bt;
            r_wc[wid] = wc;
        }
        __syncthreads();
        if (wid == 0) {
            x = lane < NW ? r_x[lane] : -1;
            bc = lane < NW ? r_c[lane] : cur;
            bw = lane < NW ? r_w[lane] : 0;
            bt = lane < NW ? r_t[lane] : 0;
            wc = lane < NW ? r_wc[lane] : 0;
            warp_merge_int(x, bc, bw, bt, wc, 32);
            if (lane == 0) {
                s_dec = int_decision(a, sc, x, bt, cur, bc, wc, sf, ki);
                s_bc = bc;
                s_wc = wc;
            }
        }
        __syncthreads();
        if (s_dec == 2) {  // block-uniform
            double dq = 0.0;
            int fc = cur;
            first_scan<WT, W>(a, sc, s, deg, v, threadIdx.x, BLOCK, ki, tcur, dq, fc);
            warp_argmax(dq, fc);
            if (lane == 0) {
                r_dq[wid] = dq;
                r_c[wid] = fc;
            }
            __syncthreads();
            if (wid == 0) {
                dq = lane < NW ? r_dq[lane] : 0.0;
                fc = lane < NW ? r_c[lane] : cur;
                warp_argmax(dq, fc);
                if (lane == 0) {
                    s_bc = fc;
                    s_dec = (fc != cur && gain_correct(dq, s_wc, sf) > 0.0) ? 1 : 0;
                    atomicAdd(&a.st->fp64_decisions, 1ull);
                }
            }
            __syncthreads();
        }
        if (wid == 0) {
            const bool move = lane == 0 && s_dec == 1 && guard_ok(a, cur, s_bc);
            if (lane == 0) write_features(a, sc, v, x, s_wc, sf, ki, deg);
            append_mover(a, move, v, cur, s_bc);
        }
        __syncthreads();
    }
}

constexpr int kCtaTable5 = 4096;
constexpr int kCtaTable6 = 16384;
// Resident blocks per SM of a CTA decide kernel with a tmax-slot table (cached).
template <typename WT, int BLOCK>
int cta_resident(bool W, int tmax)
{
    static int cached[2][32] = {};
    int &r = cached[W ? 1 : 0][__builtin_ctz((unsigned)tmax)];
    if (r == 0) {
        int k = 0;
        if (W)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, k_decide_cta<WT, BLOCK, true>, BLOCK, cta_smem<WT>(tmax));
        else
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&k, k_decide_cta<WT, BLOCK, false>, BLOCK,
                                                          cta_smem<WT>(tmax));
        r = k > 0 ? k : 1;
    }
    return r;
}

// Arguments of the decide kernels for the weight type WT.
template <typename WT>
static DecideArgs<WT> decide_args(const LevelGraph &g, Phase1Buffers &b, double constant, long long m2,
                                  int fp64_only)
{
    DecideArgs<WT> a;
    a.offs = g.offs;
    a.nbr = g.nbr;
    a.w = (const WT *)g.w;
    a.comm = b.comm;
    a.K = (const WT *)b.K;
    a.Self = (const WT *)b.Self;
    a.Tot = (const WT *)b.Tot;
    a.size = b.size;
    a.mv_v = b.mv_v;
    a.mv_old = b.mv_old;
    a.mv_new = b.mv_new;
    a.st = b.stats;
    a.constant = constant;
    a.m2 = m2;
    a.fp64_only = fp64_only;
    a.feat_gain = b.features_on ? b.feat_gain : nullptr;
    a.feat_ndist = b.feat_ndist;
    a.gid = b.gid;
    a.m2g = b.m2g;
    a.cg = b.cg;
    a.stop = b.gstop;
    return a;
}

template <typename WT>
static void decide_t(const LevelGraph &g, Phase1Buffers &b, int bin, const int32_t *list, const int *count_ptr,
                     int level_count, double constant, long long m2, int fp64_only, bool first, cudaStream_t st)
{
    const DecideArgs<WT> a = decide_args<WT>(g, b, constant, m2, fp64_only);
    const bool W = g.w != nullptr;
    const int cap = num_sms() * 8;
    auto grid_lanes = [&](int lanes_per_item) {
        long long blocks = ((long long)level_count * lanes_per_item + 255) / 256;
        return (int)(blocks < cap ? blocks : cap);
    };
    if (first && bin >= 4 && bin <= 6) {  // singleton partition: no aggregation tables
        if (bin == 4) {
            if (W)
                k_first_warp<WT, true><<<grid_lanes(32), 256, 0, st>>>(a, list, count_ptr);
            else
                k_first_warp<WT, false><<<grid_lanes(32), 256, 0, st>>>(a, list, count_ptr);
        } else {
            const int grid = level_count < num_sms() * 8 ? level_count : num_sms() * 8;
            if (W)
                k_first_cta<WT, 256, true><<<grid, 256, 0, st>>>(a, list, count_ptr);
            else
                k_first_cta<WT, 256, false><<<grid, 256, 0, st>>>(a, list, count_ptr);
        }
        note_launch(1);
        return;
    }
#define GALA_DG(GV)                                                                                    \
    do {                                                                                               \
        if (W)                                                                                         \
            k_decide_group<WT, GV, true><<<grid_lanes(GV), 256, 0, st>>>(a, list, count_ptr);          \
        else                                                                                           \
            k_decide_group<WT, GV, false><<<grid_lanes(GV), 256, 0, st>>>(a, list, count_ptr);         \
    } while (0)
    switch (bin) {
    case 0: GALA_DG(4); break;
    case 1: GALA_DG(8); break;
    case 2: GALA_DG(16); break;
    case 3: GALA_DG(32); break;
    case 4: {
        // as many CTAs as can reside (tables and registers): no second wave
        // two launches: rows up to 128 entries with 256-slot tables (more
        // resident warps), longer rows with 512-slot tables
        {
            const int cap4 = num_sms() * warp_resident<WT, kWarpTable / 2, 8>(W);
            const int g4 = grid_lanes(32) < cap4 ? grid_lanes(32) : cap4;
            const size_t sm = warp_smem<WT, kWarpTable / 2>();
            if (W)
                k_decide_warp<WT, true, kWarpTable / 2, 8><<<g4, 256, sm, st>>>(a, list, count_ptr, 0, kWarpTable / 4);
            else
                k_decide_warp<WT, false, kWarpTable / 2, 8><<<g4, 256, sm, st>>>(a, list, count_ptr, 0, kWarpTable / 4);
        }
        {
            const int cap4 = num_sms() * warp_resident<WT, kWarpTable, 1>(W);
            const int g4 = grid_lanes(32) < cap4 ? grid_lanes(32) : cap4;
            const size_t sm = warp_smem<WT, kWarpTable>();
            if (W)
                k_decide_warp<WT, true, kWarpTable, 1><<<g4, 256, sm, st>>>(a, list, count_ptr, kWarpTable / 4, INT_MAX);
            else
                k_decide_warp<WT, false, kWarpTable, 1><<<g4, 256, sm, st>>>(a, list, count_ptr, kWarpTable / 4, INT_MAX);
        }
        note_launch(1);
        break;
    }
    case 5: {  // 256 (default) or 512 threads per vertex
        if (b.b5_block == 256) {
            // two launches: rows up to 1024 entries with a 2048-slot table
            // (more resident CTAs), longer rows with the 4096-slot table
            const int splits[2][3] = {{kCtaTable5 / 2, 0, kCtaTable5 / 4}, {kCtaTable5, kCtaTable5 / 4, INT_MAX}};
            for (const auto &sp : splits) {
                const int cap5 = num_sms() * cta_resident<WT, 256>(W, sp[0]);
                const int grid = level_count < cap5 ? level_count : cap5;
                const size_t sm = cta_smem<WT>(sp[0]);
                if (W)
                    k_decide_cta<WT, 256, true><<<grid, 256, sm, st>>>(a, list, count_ptr, sp[0], sp[1], sp[2]);
                else
                    k_decide_cta<WT, 256, false><<<grid, 256, sm, st>>>(a, list, count_ptr, sp[0], sp[1], sp[2]);
            }
            note_launch(1);
        } else {
            const size_t sm = cta_smem<WT>(kCtaTable5);
            int grid = level_count < num_sms() * 4 ? level_count : num_sms() * 4;
            if (W)
                k_decide_cta<WT, 512, true><<<grid, 512, sm, st>>>(a, list, count_ptr, kCtaTable5, 0, INT_MAX);
            else
                k_decide_cta<WT, 512, false><<<grid, 512, sm, st>>>(a, list, count_ptr, kCtaTable5, 0, INT_MAX);
        }
        break;
    }
    case 6: {
        const int splits[2][3] = {{kCtaTable6 / 2, 0, kCtaTable6 / 4}, {kCtaTable6, kCtaTable6 / 4, INT_MAX}};
        for (const auto &sp : splits) {
            const int cap6 = num_sms() * cta_resident<WT, 1024>(W, sp[0]);
            const int grid = level_count < cap6 ? level_count : cap6;
            const size_t sm = cta_smem<WT>(sp[0]);
            if (W)
                k_decide_cta<WT, 1024, true><<<grid, 1024, sm, st>>>(a, list, count_ptr, sp[0], sp[1], sp[2]);
            else
                k_decide_cta<WT, 1024, false><<<grid, 1024, sm, st>>>(a, list, count_ptr, sp[0], sp[1], sp[2]);
        }
        note_launch(1);
        break;
    }
    default: return;  // hub vertices: p1_hub_decide
    }
#undef GALA_DG
    note_launch(1);
}

void p1_decide(const LevelGraph &g, Phase1Buffers &b, int bin, const int32_t *list, const int *count_ptr,
               int level_count, double constant, long long m2, int fp64_only, bool first, cudaStream_t st)
{
    if (level_count <= 0) return;
    if (g.wide)
        decide_t<long long>(g, b, bin, list, count_ptr, level_count, constant, m2, fp64_only, first, st);
    else
        decide_t<int>(g, b, bin, list, count_ptr, level_count, constant, m2, fp64_only, first, st);
}

template <typename WT>
static void configure_t()
{
    cudaFuncSetAttribute(k_decide_cta<WT, 1024, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)cta_smem<WT>(kCtaTable6));
    cudaFuncSetAttribute(k_decide_cta<WT, 1024, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)cta_smem<WT>(kCtaTable6));
    cudaFuncSetAttribute(k_decide_cta<WT, 512, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)cta_smem<WT>(kCtaTable5));
    cudaFuncSetAttribute(k_decide_cta<WT, 256, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)cta_smem<WT>(kCtaTable5));
    cudaFuncSetAttribute(k_decide_cta<WT, 256, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)cta_smem<WT>(kCtaTable5));
    cudaFuncSetAttribute(k_decide_cta<WT, 512, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)cta_smem<WT>(kCtaTable5));
    cudaFuncSetAttribute(k_decide_warp<WT, true, kWarpTable, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)warp_smem<WT, kWarpTable>());
    cudaFuncSetAttribute(k_decide_warp<WT, false, kWarpTable, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)warp_smem<WT, kWarpTable>());
    cudaFuncSetAttribute(k_decide_warp<WT, true, kWarpTable / 2, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)warp_smem<WT, kWarpTable / 2>());
    cudaFuncSetAttribute(k_decide_warp<WT, false, kWarpTable / 2, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)warp_smem<WT, kWarpTable / 2>());
}

void p1_configure_kernels()
{
    configure_t<int>();
    configure_t<long long>();
}

// ------------------------------------------------------------------------
// Apply (sign = +1) or revert (sign = -1) the movers of an iteration
// (Tot += Tot_update, size += size_update, louvain_main_process.cu:949-953).
// ------------------------------------------------------------------------
template <typename WT>
__global__ void k_apply_movers(const int32_t *__restrict__ mv_v, const int32_t *__restrict__ mv_old,
                               const int32_t *__restrict__ mv_new, DevStats *stp, int sign, int32_t *comm, WT *Tot,
                               int32_t *size, const WT *__restrict__ K, int32_t *last_move, int iteration,
                               const int64_t *__restrict__ offs, uint8_t *moved)
{
    // whole warps step together: movers of one warp that share a source or a
    // target community add to its Tot and size once (many movers of a sweep
    // head for the same large community)
    const int nm = stp->n_movers;
    const int lane = threadIdx.x & 31;
    unsigned long long deg = 0;
    for (int i0 = blockIdx.x * blockDim.x + threadIdx.x - lane; i0 < nm; i0 += gridDim.x * blockDim.x) {
        const int i = i0 + lane;
        const bool valid = i < nm;
        int from = -1, to = -1;
        WT k = 0;
        if (valid) {
            const int v = mv_v[i];
            from = sign > 0 ? mv_old[i] : mv_new[i];
            to = sign > 0 ? mv_new[i] : mv_old[i];
            k = K[v];
            comm[v] = to;
            if (last_move && sign > 0) last_move[v] = iteration;
            if (offs) deg += (unsigned long long)(offs[v + 1] - offs[v]);
            if (moved) moved[v] = 1;
        }
        const unsigned mt = __match_any_sync(GALA_FULL_MASK, to);
        const WT kt = group_sum(mt, k);
        if (valid && lane == __ffs(mt) - 1) {
            atomic_add_w(&Tot[to], kt);
            atomicAdd(&size[to], __popc(mt));
        }
        const unsigned mf = __match_any_sync(GALA_FULL_MASK, from);
        const WT kf = group_sum(mf, k);
        if (valid && lane == __ffs(mf) - 1) {
            atomic_add_w(&Tot[from], (WT)-kf);
            atomicSub(&size[from], __popc(mf));
        }
    }
    if (offs) block_add_u64(deg, &stp->mv_edges);
}

void p1_apply_movers(Phase1Buffers &b, int sign, int n, cudaStream_t st, int iteration, const int64_t *offs,
                     uint8_t *moved)
{
    if (sign < 0) offs = nullptr, moved = nullptr;
    int grid = (n + 255) / 256;
    int cap = num_sms() * 4;
    if (grid > cap) grid = cap;
    if (grid < 1) grid = 1;
    if (b.wide)
        k_apply_movers<long long><<<grid, 256, 0, st>>>(b.mv_v, b.mv_old, b.mv_new, b.stats, sign, b.comm,
                                                        (long long *)b.Tot, b.size, (const long long *)b.K, nullptr,
                                                        iteration, offs, moved);
    else
        k_apply_movers<int><<<grid, 256, 0, st>>>(b.mv_v, b.mv_old, b.mv_new, b.stats, sign, b.comm, b.Tot, b.size,
                                                  b.K, b.features_on ? b.last_move : nullptr, iteration, offs, moved);
    note_launch(1);
}

// min over non-empty Tot (Tot_op, kernel_functions.cuh:112-121) and sum Tot^2.
template <typename WT>
__global__ void k_tot_reduce(const WT *__restrict__ Tot, int n, DevStats *st)
{
    long long mn = 0x7fffffffffffffffLL;
    typename SqSum<WT>::T s2 = 0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
        const WT t = Tot[c];
        if (t != 0) {
            mn = min(mn, (long long)t);
            s2 += SqSum<WT>::sq(t);
        }
    }
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) mn = min(mn, __shfl_xor_sync(GALA_FULL_MASK, mn, o));
    if ((threadIdx.x & 31) == 0 && mn != 0x7fffffffffffffffLL) atomicMin(&st->min_tot, mn);
    SqSum<WT>::add(s2, st);
}

void p1_tot_reduce(Phase1Buffers &b, int n, cudaStream_t st)
{
    int grid = (n + 1023) / 1024;
    int cap = num_sms() * 4;
    if (grid > cap) grid = cap;
    if (grid < 1) grid = 1;
    if (b.wide)
        k_tot_reduce<long long><<<grid, 1024, 0, st>>>((const long long *)b.Tot, n, b.stats);
    else
        k_tot_reduce<int><<<grid, 1024, 0, st>>>(b.Tot, n, b.stats);
    note_launch(1);
}

__global__ void k_iter_reset(DevStats *st, int next, long long min_tot_init)
{
    st->n_movers = 0;
    st->mv_edges = 0;
    st->push_mode = 0;
    st->push_len = 0;
    st->sum_in = 0;
    st->sum_tot2 = 0;
    st->sum_tot2_hi = 0;
    st->min_tot = min_tot_init;
    st->act_edges[next] = 0;
    st->act_vertices[next] = 0;
    for (int i = 0; i < kNumBins; ++i) st->act_count[next][i] = 0;
}

void p1_iter_reset(Phase1Buffers &b, int next, long long min_tot_init, cudaStream_t st)
{
    k_iter_reset<<<1, 1, 0, st>>>(b.stats, next, min_tot_init);
    note_launch(1);
}

// ------------------------------------------------------------------------
// Weight update + pruning (compute_In / compute_In_blk,
// kernel_functions.cu:890-1034): In[v] over the new labels, the pruning
// bound, next active lists, sum of In.
// ------------------------------------------------------------------------
template <typename WT>
struct UpdateArgs {
    const int64_t *__restrict__ offs;
    const int32_t *__restrict__ nbr;
    const WT *__restrict__ w;
    const int32_t *__restrict__ comm;
    const WT *__restrict__ K;
    const WT *__restrict__ Self;
    const WT *__restrict__ Tot;
    WT *In;
    uint8_t *act_flag;  // per-vertex copy of the next active set
    int32_t *act_list;  // next active list, segment of this bin
    int *act_counter;
    DevStats *st;
    double constant;
    long long m2;
    int next;
    // batched graphs (null for one graph)
    const int32_t *__restrict__ gid;
    const long long *__restrict__ m2g;
    const double *__restrict__ cg;
    const uint8_t *__restrict__ stop;
    const int32_t *__restrict__ min_tot_g;
};

// Per-vertex prune parameters: the graph's m2, 1/m2 and min Tot; `stop` when
// the vertex's graph has stopped (no update, never active).
struct PruneScale {
    long long m2;
    double c;
    long long min_tot;
    bool stop;
};
template <typename WT>
__device__ __forceinline__ PruneScale prune_scale(const UpdateArgs<WT> &a, int v, long long min_tot)
{
    if (a.gid) {
        const int g = a.gid[v];
        return PruneScale{a.m2g[g], a.cg[g], a.min_tot_g[g], a.stop[g] != 0};
    }
    return PruneScale{a.m2, a.constant, min_tot, false};
}

template <typename WT, int G, bool W>
__global__ void __launch_bounds__(256) k_update_group(UpdateArgs<WT> a, const int32_t *__restrict__ list, int count)
{
    if (a.st->push_mode) return;  // the incremental update runs instead
    const int lane = threadIdx.x & 31, sub = lane & (G - 1), gw = lane / G;
    constexpr int GPW = 32 / G;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const long long min_tot = a.st->min_tot;
    unsigned long long s_in = 0, s_edges = 0;
    int s_act = 0;
    __shared__ int stage_buf[8][kStageN];
    WarpStage<kStageN, 1> stage{stage_buf[threadIdx.x >> 5], 0};
    int *const lists[1] = {a.act_list};
    for (int base = wg * GPW; base < count; base += nw * GPW) {
        const int idx = base + gw;
        bool has = idx < count;
        int v = 0, cur = -1;
        long long s = 0, e = 0;
        PruneScale ps{a.m2, a.constant, min_tot, false};
        if (has) {
            v = list[idx];
            ps = prune_scale(a, v, min_tot);
            if (ps.stop) has = false;
        }
        if (has) {
            s = a.offs[v];
            e = a.offs[v + 1];
            cur = a.comm[v];
        }
        WT sum = 0;
#pragma unroll 4
        for (long long j = s + sub; j < e; j += G)
            if (a.comm[a.nbr[j]] == cur) sum += W ? a.w[j] : 1;
#pragma unroll
        for (int o = G / 2; o >= 1; o >>= 1) sum += __shfl_xor_sync(GALA_FULL_MASK, sum, o);
        bool active = false;
        if (ps.stop && sub == 0) a.act_flag[v] = 0;
        if (has && sub == 0) {
            a.In[v] = sum;
            const WT ki = a.K[v];
            active = !prune_bound_fast<WT>(sum, a.Self[v], ki, (WT)ps.min_tot, a.Tot[cur], ps.c, ps.m2);
            a.act_flag[v] = active;
            s_in += (unsigned long long)sum;
            if (active) {
                s_edges += (unsigned long long)(e - s);
                s_act += 1;
            }
        }
        const int item[1] = {v};
        stage.push(active, item, lists, a.act_counter);
    }
    stage.flush(lists, a.act_counter);
    block_add_u64(s_in, &a.st->sum_in);
    block_add_u64(s_edges, &a.st->act_edges[a.next]);
    block_add_i32(s_act, &a.st->act_vertices[a.next]);
}

template <typename WT, bool W>
__global__ void __launch_bounds__(256) k_update_cta(UpdateArgs<WT> a, const int32_t *__restrict__ list, int count)
{
    if (a.st->push_mode) return;  // the incremental update runs instead
    __shared__ WT red[8];
    const long long min_tot = a.st->min_tot;
    unsigned long long s_in = 0, s_edges = 0;
    int s_act = 0;
    for (int i = blockIdx.x; i < count; i += gridDim.x) {
        const int v = list[i];
        const PruneScale ps = prune_scale(a, v, min_tot);
        if (ps.stop) {  // block-uniform
            if (threadIdx.x == 0) a.act_flag[v] = 0;
            continue;
        }
        const long long s = a.offs[v], e = a.offs[v + 1];
        const int cur = a.comm[v];
        WT sum = 0;
#pragma unroll 4
        for (long long j = s + threadIdx.x; j < e; j += blockDim.x)
            if (a.comm[a.nbr[j]] == cur) sum += W ? a.w[j] : 1;
        sum = warp_sum(sum);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
        __syncthreads();
        if (threadIdx.x == 0) {
            sum = 0;
            for (int q = 0; q < (int)(blockDim.x >> 5); ++q) sum += red[q];
            a.In[v] = sum;
            const WT ki = a.K[v];
            bool active = !prune_bound_fast<WT>(sum, a.Self[v], ki, (WT)ps.min_tot, a.Tot[cur], ps.c, ps.m2);
            a.act_flag[v] = active;
            s_in += (unsigned long long)sum;
            if (active) {
                a.act_list[atomicAdd(a.act_counter, 1)] = v;
                s_edges += (unsigned long long)(e - s);
                s_act += 1;
            }
        }
        __syncthreads();
    }
    block_add_u64(s_in, &a.st->sum_in);
    block_add_u64(s_edges, &a.st->act_edges[a.next]);
    block_add_i32(s_act, &a.st->act_vertices[a.next]);
}

template <typename WT>
static UpdateArgs<WT> update_args(const LevelGraph &g, Phase1Buffers &b, int bin, int next, int bin_start,
                                  double constant, long long m2)
{
    UpdateArgs<WT> a;
    a.offs = g.offs;
    a.nbr = g.nbr;
    a.w = (const WT *)g.w;
    a.comm = b.comm;
    a.K = (const WT *)b.K;
    a.Self = (const WT *)b.Self;
    a.Tot = (const WT *)b.Tot;
    a.In = (WT *)b.In;
    a.act_flag = b.act_flag;
    a.act_list = b.act[next] + bin_start;
    a.act_counter = &b.stats->act_count[next][bin];
    a.st = b.stats;
    a.constant = constant;
    a.m2 = m2;
    a.next = next;
    a.gid = b.gid;
    a.m2g = b.m2g;
    a.cg = b.cg;
    a.stop = b.gstop;
    a.min_tot_g = b.min_tot_g;
    return a;
}

template <typename WT>
static void update_t(const LevelGraph &g, Phase1Buffers &b, int bin, const int32_t *list, int count, int next,
                     int bin_start, double constant, long long m2, cudaStream_t st)
{
    const UpdateArgs<WT> a = update_args<WT>(g, b, bin, next, bin_start, constant, m2);
    const bool W = g.w != nullptr;
    const int cap = num_sms() * 8;
    auto grid_lanes = [&](int G) {
        long long blocks = ((long long)count * G + 255) / 256;
        return (int)(blocks < cap ? blocks : cap);
    };
#define GALA_UG(GV)                                                                                    \
    do {                                                                                               \
        if (W)                                                                                         \
            k_update_group<WT, GV, true><<<grid_lanes(GV), 256, 0, st>>>(a, list, count);              \
        else                                                                                           \
            k_update_group<WT, GV, false><<<grid_lanes(GV), 256, 0, st>>>(a, list, count);             \
    } while (0)
    // bins 2-4 use groups narrower than their rows: a lane sums several
    // entries (independent loads) and a warp serves several vertices, more
    // rows in flight than one lane per entry (measured on R-MAT levels)
    switch (bin) {
    case 0: GALA_UG(4); break;
    case 1: GALA_UG(8); break;
    case 2: GALA_UG(8); break;
    case 3: GALA_UG(16); break;
    case 4: GALA_UG(8); break;
    case 5: GALA_UG(32); break;
    default: {
        int grid = count < cap ? count : cap;
        if (W)
            k_update_cta<WT, true><<<grid, 256, 0, st>>>(a, list, count);
        else
            k_update_cta<WT, false><<<grid, 256, 0, st>>>(a, list, count);
    }
    }
#undef GALA_UG
    note_launch(1);
}

void p1_update(const LevelGraph &g, Phase1Buffers &b, int bin, const int32_t *list, int count, int next,
               int bin_start, double constant, long long m2, cudaStream_t st)
{
    if (count <= 0) return;
    if (g.wide)
        update_t<long long>(g, b, bin, list, count, next, bin_start, constant, m2, st);
    else
        update_t<int>(g, b, bin, list, count, next, bin_start, constant, m2, st);
}

// ------------------------------------------------------------------------
// Hub vertices (degree > 8192): one global hash table per hub, filled by
// many CTAs in 4096-entry chunks of the hub's row, scanned by many CTAs in
// 4096-slot chunks (each writes the best candidate of its chunk), and merged
// by one warp per hub.  A hub's work is spread over all SMs instead of one.
// ------------------------------------------------------------------------
constexpr int kHubChunk = 4096;

__global__ void k_hub_plan(HubPlan p, const int64_t *__restrict__ offs)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.H; i += gridDim.x * blockDim.x) {
        const int v = p.hubs[i];
        const long long deg = offs[v + 1] - offs[v];
        long long T = next_pow2_ll(deg + deg / 2);  // load at most 2/3
        if (p.t_cap > 0 && T > p.t_cap) T = p.t_cap;  // capped: inserts may run out of slots
        p.T[i] = T;
        p.chunks[i] = (deg + kHubChunk - 1) / kHubChunk;
        p.tchunks[i] = (T + kHubChunk - 1) / kHubChunk;
    }
}

__global__ void k_hub_tail(HubPlan p, const DevStats *st)
{
    p.toff[p.H] = st->total;
    p.coff[p.H] = st->total2;
    p.tcoff[p.H] = st->total3;
}

__global__ void k_hub_work(HubPlan p)
{
    const int lane = threadIdx.x & 31;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = wg; i < p.H; i += nw) {
        long long o = p.coff[i], k = p.coff[i + 1] - o;
        for (long long j = lane; j < k; j += 32) p.work[o + j] = i;
        o = p.tcoff[i];
        k = p.tcoff[i + 1] - o;
        for (long long j = lane; j < k; j += 32) p.twork[o + j] = i;
    }
}

// Values of a hub table (WT per slot, after the keys of all tables).
template <typename WT>
__device__ __forceinline__ WT *hub_vals(const HubPlan &p, long long i)
{
    return (WT *)(p.pool + p.half) + p.toff[i];
}

template <typename WT, bool W>
__global__ void __launch_bounds__(256) k_hub_insert(DecideArgs<WT> a, HubPlan p, const uint8_t *__restrict__ flag)
{
    // a small shared-memory table in front of the hub's global table: an
    // entry whose community finds a slot within kHubCacheProbe probes is
    // summed there, the rest go to the global table directly; the cached sums
    // are added to the global table at the end of the chunk (integer adds:
    // the totals do not depend on the split)
    constexpr int kHubCache = 512, kHubCacheLog = 9, kHubCacheProbe = 2;
    __shared__ int ckeys[kHubCache];
    __shared__ WT cvals[kHubCache];
    for (int q = threadIdx.x; q < kHubCache; q += blockDim.x) {
        ckeys[q] = -1;
        cvals[q] = 0;
    }
    __syncthreads();
    for (long long wi = blockIdx.x; wi < p.nwork; wi += gridDim.x) {
        const int i = p.work[wi];
        const int v = p.hubs[i];
        if (!flag[v] || stopped(a, v)) continue;  // block-uniform
        const long long e = a.offs[v + 1];
        const long long s = a.offs[v] + (wi - p.coff[i]) * kHubChunk;
        const long long e2 = s + kHubChunk < e ? s + kHubChunk : e;
        const int T = (int)p.T[i];
        const int lg = __ffs(T) - 1;
        int *keys = p.pool + p.toff[i];
        WT *vals = hub_vals<WT>(p, i);
        for (long long b0 = s; b0 < e2; b0 += blockDim.x) {
            const long long j = b0 + threadIdx.x;
            if (j < e2) {
                const int c = a.comm[a.nbr[j]];
                const WT wt = W ? a.w[j] : 1;
                unsigned h = hash_slot(c, kHubCacheLog);
                bool cached = false;
#pragma unroll
                for (int q = 0; q < kHubCacheProbe; ++q) {
                    const int k = atomicCAS(&ckeys[h], -1, c);
                    if (k == -1 || k == c) {
                        atomic_add_w(&cvals[h], wt);
                        cached = true;
                        break;
                    }
                    h = (h + 1) & (unsigned)(kHubCache - 1);
                }
                if (!cached && !hash_add(keys, vals, T, lg, c, wt)) atomicOr(&a.st->err, kErrHashOverflow);
            }
        }
        __syncthreads();
        for (int q = threadIdx.x; q < kHubCache; q += blockDim.x) {
            const int k = ckeys[q];
            if (k != -1) {
                if (!hash_add(keys, vals, T, lg, k, cvals[q])) atomicOr(&a.st->err, kErrHashOverflow);
                ckeys[q] = -1;
                cvals[q] = 0;
            }
        }
        __syncthreads();
    }
}

// FP64 evaluation needed whatever the candidates: K*m2 out of the range where
// the integer order equals the FP64 order (or FP64 forced).
template <typename WT>
__device__ __forceinline__ bool needs_fp64(const DecideArgs<WT> &a, const Scale &sc, WT ki)
{
    if constexpr (!WideOf<WT>::exact) return true;
    return a.fp64_only || (long long)ki * sc.m2 >= (1LL << 49);
}

template <typename WT>
__global__ void __launch_bounds__(256) k_hub_scan(DecideArgs<WT> a, HubPlan p, const uint8_t *__restrict__ flag)
{
    __shared__ long long r_x[8];
    __shared__ double r_dq[8];
    __shared__ int r_c[8], r_t[8];
    __shared__ WT r_w[8], r_wc[8];
    WT *pw = (WT *)p.pw, *pwc = (WT *)p.pwc;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (long long wi = blockIdx.x; wi < p.ntwork; wi += gridDim.x) {
        const int i = p.twork[wi];
        const int v = p.hubs[i];
        if (!flag[v] || stopped(a, v)) continue;
        const Scale sc = scale_of(a, v);
        const int cur = a.comm[v];
        const WT ki = a.K[v], tcur = a.Tot[cur];
        const long long j0 = (wi - p.tcoff[i]) * kHubChunk;
        const long long T = p.T[i];
        const long long j1 = j0 + kHubChunk < T ? j0 + kHubChunk : T;
        const int *keys = p.pool + p.toff[i];
        const WT *vals = hub_vals<WT>(p, i);
        long long x = -1;
        int bc = cur, bt = 0;
        WT bw = 0, wc = 0;
        scan_table_int(a, sc, keys + j0, vals + j0, (int)(j1 - j0), threadIdx.x, blockDim.x, cur, ki, tcur, x, bc,
                       bw, bt, wc);
        warp_merge_int(x, bc, bw, bt, wc, 32);
        if (lane == 0) {
            r_x[wid] = x;
            r_c[wid] = bc;
            r_w[wid] = bw;
            r_t[wid] = bt;
            r_wc[wid] = wc;
        }
        __syncthreads();
        if (wid == 0) {
            const int nwp = blockDim.x >> 5;
            x = lane < nwp ? r_x[lane] : -1;
            bc = lane < nwp ? r_c[lane] : cur;
            bw = lane < nwp ? r_w[lane] : 0;
            bt = lane < nwp ? r_t[lane] : 0;
            wc = lane < nwp ? r_wc[lane] : 0;
            warp_merge_int(x, bc, bw, bt, wc, 32);
            if (lane == 0) {
                p.px[wi] = x;
                p.pc[wi] = bc;
                pw[wi] = bw;
                p.pt[wi] = bt;
                pwc[wi] = wc;
            }
        }
        __syncthreads();
        if (needs_fp64(a, sc, ki)) {  // uniform per chunk: the reference's FP64 gains, chunk-wise
            double dq = 0.0;
            int fc = cur;
            scan_table(a, sc, keys + j0, vals + j0, (int)(j1 - j0), threadIdx.x, blockDim.x, cur, ki, tcur, dq, fc);
            warp_argmax(dq, fc);
            if (lane == 0) {
                r_dq[wid] = dq;
                r_c[wid] = fc;
            }
            __syncthreads();
            if (wid == 0) {
                const int nwp = blockDim.x >> 5;
                dq = lane < nwp ? r_dq[lane] : 0.0;
                fc = lane < nwp ? r_c[lane] : cur;
                warp_argmax(dq, fc);
                if (lane == 0) {
                    p.pdq[wi] = dq;
                    p.pfc[wi] = fc;
                }
            }
            __syncthreads();
        }
    }
}

template <typename WT>
__global__ void __launch_bounds__(256) k_hub_final(DecideArgs<WT> a, HubPlan p, const uint8_t *__restrict__ flag)
{
    const WT *pw = (const WT *)p.pw, *pwc = (const WT *)p.pwc;
    const int lane = threadIdx.x & 31;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = wg; i < p.H; i += nw) {
        const int v = p.hubs[i];
        if (!flag[v] || stopped(a, v)) continue;
        const Scale sc = scale_of(a, v);
        const int cur = a.comm[v];
        const WT ki = a.K[v], sf = a.Self[v], tcur = a.Tot[cur];
        long long x = -1;
        int bc = cur, bt = 0;
        WT bw = 0, wc = 0;
        for (long long q = p.tcoff[i] + lane; q < p.tcoff[i + 1]; q += 32) {
            wc += pwc[q];
            if (p.px[q] >= 0) cand_merge(x, bc, bw, bt, p.px[q], p.pc[q], pw[q], p.pt[q]);
        }
        warp_merge_int(x, bc, bw, bt, wc, 32);
        int dec = int_decision(a, sc, x, bt, cur, bc, wc, sf, ki);  // warp-uniform
        if (dec == 2) {
            double dq = 0.0;
            int fc = cur;
            if (needs_fp64(a, sc, ki)) {  // chunk-wise FP64 partials from k_hub_scan
                for (long long q = p.tcoff[i] + lane; q < p.tcoff[i + 1]; q += 32)
                    if (cand_better(p.pdq[q], p.pfc[q], dq, fc)) {
                        dq = p.pdq[q];
                        fc = p.pfc[q];
                    }
            } else {  // rare rounding cases: rescan the table in FP64
                scan_table(a, sc, p.pool + p.toff[i], hub_vals<WT>(p, i), (int)p.T[i], lane, 32, cur, ki, tcur, dq,
                           fc);
            }
            warp_argmax(dq, fc);
            bc = fc;
            dec = (fc != cur && gain_correct(dq, wc, sf) > 0.0) ? 1 : 0;
            if (lane == 0) atomicAdd(&a.st->fp64_decisions, 1ull);
        }
        const bool move = lane == 0 && dec == 1 && guard_ok(a, cur, bc);
        append_mover(a, move, v, cur, bc);
    }
}

// Per level: table sizes, chunk counts and their offsets (the caller reads
// the three totals from the stats block before p1_hub_work_launch).
void p1_hub_plan_launch(const LevelGraph &g, Phase1Buffers &b, HubPlan &p, cudaStream_t st)
{
    const int grid = (p.H + 255) / 256;
    k_hub_plan<<<grid, 256, 0, st>>>(p, g.offs);
    exclusive_scan(p.T, p.toff, p.H, OpIdentity(), b.scan_partial, &b.stats->total, st, &b.stats->err);
    exclusive_scan(p.chunks, p.coff, p.H, OpIdentity(), b.scan_partial, &b.stats->total2, st, &b.stats->err);
    exclusive_scan(p.tchunks, p.tcoff, p.H, OpIdentity(), b.scan_partial, &b.stats->total3, st, &b.stats->err);
    k_hub_tail<<<1, 1, 0, st>>>(p, b.stats);
    note_launch(2);
}

void p1_hub_work_launch(HubPlan &p, cudaStream_t st)
{
    k_hub_work<<<(p.H * 32 + 255) / 256, 256, 0, st>>>(p);
    note_launch(1);
}

template <typename WT>
static void hub_decide_t(const LevelGraph &g, Phase1Buffers &b, const HubPlan &p, double constant, long long m2,
                         int fp64_only, cudaStream_t st)
{
    const DecideArgs<WT> a = decide_args<WT>(g, b, constant, m2, fp64_only);
    const int cap = num_sms() * 8;
    cudaMemsetAsync(p.pool, 0xff, (size_t)p.half * sizeof(int32_t), st);
    cudaMemsetAsync(p.pool + p.half, 0, (size_t)p.half * sizeof(WT), st);
    const int g1 = (int)(p.nwork < cap ? p.nwork : cap);
    if (g.w)
        k_hub_insert<WT, true><<<g1, 256, 0, st>>>(a, p, b.act_flag);
    else
        k_hub_insert<WT, false><<<g1, 256, 0, st>>>(a, p, b.act_flag);
    k_hub_scan<WT><<<(int)(p.ntwork < cap ? p.ntwork : cap), 256, 0, st>>>(a, p, b.act_flag);
    k_hub_final<WT><<<(p.H * 32 + 255) / 256, 256, 0, st>>>(a, p, b.act_flag);
    note_launch(3);
}

// One iteration's decide-and-move of the hub bin.  The values of the hub
// tables follow all keys: p.half int32 keys, then p.half values of the
// weight type (the caller sized the pool for it).
void p1_hub_decide(const LevelGraph &g, Phase1Buffers &b, const HubPlan &p, double constant, long long m2,
                   int fp64_only, cudaStream_t st)
{
    if (p.H <= 0) return;
    if (g.wide)
        hub_decide_t<long long>(g, b, p, constant, m2, fp64_only, st);
    else
        hub_decide_t<int>(g, b, p, constant, m2, fp64_only, st);
}

// ------------------------------------------------------------------------
// Weight update of the hub bin: In[v] of a hub row summed by many CTAs (one
// per 4096-entry chunk, the chunks of the hub plan) with integer atomics,
// then one thread per hub evaluates the pruning bound.
// ------------------------------------------------------------------------
template <typename WT>
__global__ void k_hub_in_zero(HubPlan p, WT *In, const DevStats *st)
{
    if (st->push_mode) return;  // the incremental update runs instead
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < p.H; i += gridDim.x * blockDim.x) In[p.hubs[i]] = 0;
}

template <typename WT, bool W>
__global__ void __launch_bounds__(256) k_hub_in_partial(UpdateArgs<WT> a, HubPlan p)
{
    if (a.st->push_mode) return;  // the incremental update runs instead
    __shared__ WT red[8];
    for (long long wi = blockIdx.x; wi < p.nwork; wi += gridDim.x) {
        const int i = p.work[wi];
        const int v = p.hubs[i];
        if (a.gid && a.stop[a.gid[v]]) continue;  // block-uniform
        const long long e = a.offs[v + 1];
        const long long s = a.offs[v] + (wi - p.coff[i]) * kHubChunk;
        const long long e2 = s + kHubChunk < e ? s + kHubChunk : e;
        const int cur = a.comm[v];
        WT sum = 0;
#pragma unroll 4
        for (long long j = s + threadIdx.x; j < e2; j += blockDim.x)
            if (a.comm[a.nbr[j]] == cur) sum += W ? a.w[j] : 1;
        sum = warp_sum(sum);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sum;
        __syncthreads();
        if (threadIdx.x == 0) {
            WT t = 0;
            for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += red[q];
            if (t) atomic_add_w(&a.In[v], t);
        }
        __syncthreads();
    }
}

template <typename WT>
__global__ void __launch_bounds__(256) k_hub_in_final(UpdateArgs<WT> a, HubPlan p)
{
    if (a.st->push_mode) return;  // the incremental update runs instead
    const long long min_tot = a.st->min_tot;
    unsigned long long s_in = 0, s_edges = 0;
    int s_act = 0;
    const int stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x; base < p.H; base += stride) {  // warp-uniform trip count
        const int i = base + threadIdx.x;
        bool active = false;
        int v = 0;
        if (i < p.H) {
            v = p.hubs[i];
            const PruneScale ps = prune_scale(a, v, min_tot);
            if (ps.stop) {
                a.act_flag[v] = 0;
            } else {
                const WT sum = a.In[v];
                const WT ki = a.K[v];
                active = !prune_bound_fast<WT>(sum, a.Self[v], ki, (WT)ps.min_tot, a.Tot[a.comm[v]], ps.c, ps.m2);
                a.act_flag[v] = active;
                s_in += (unsigned long long)sum;
                if (active) {
                    s_edges += (unsigned long long)(a.offs[v + 1] - a.offs[v]);
                    s_act += 1;
                }
            }
        }
        warp_append(active, v, a.act_list, a.act_counter);
    }
    block_add_u64(s_in, &a.st->sum_in);
    block_add_u64(s_edges, &a.st->act_edges[a.next]);
    block_add_i32(s_act, &a.st->act_vertices[a.next]);
}

template <typename WT>
static void hub_update_t(const LevelGraph &g, Phase1Buffers &b, const HubPlan &p, int next, int bin_start,
                         double constant, long long m2, cudaStream_t st)
{
    UpdateArgs<WT> a = update_args<WT>(g, b, 7, next, bin_start, constant, m2);
    const int cap = num_sms() * 8;
    const int hg = (p.H + 255) / 256;
    k_hub_in_zero<WT><<<hg, 256, 0, st>>>(p, a.In, b.stats);
    const int g1 = (int)(p.nwork < cap ? p.nwork : cap);
    if (g.w)
        k_hub_in_partial<WT, true><<<g1, 256, 0, st>>>(a, p);
    else
        k_hub_in_partial<WT, false><<<g1, 256, 0, st>>>(a, p);
    k_hub_in_final<WT><<<hg, 256, 0, st>>>(a, p);
    note_launch(3);
}

void p1_hub_update(const LevelGraph &g, Phase1Buffers &b, const HubPlan &p, int next, int bin_start, double constant,
                   long long m2, cudaStream_t st)
{
    if (p.H <= 0) return;
    if (g.wide)
        hub_update_t<long long>(g, b, p, next, bin_start, constant, m2, st);
    else
        hub_update_t<int>(g, b, p, next, bin_start, constant, m2, st);
}

}  // namespace gala
