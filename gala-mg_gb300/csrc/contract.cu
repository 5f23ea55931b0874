// contract.cu - phase 2 (contraction) of the GB300 Louvain engine.
//
// Replaces build_compressed_graph (build_compressed_graph.cu:5-173 and the
// kernels at kernel_functions.cu:1083-1694 of the reference).  Steps:
//   1. community sizes (histogram) and dense renumbering in ascending label
//      order: exclusive scan of (size > 0), no sort
//   2. members of each community (counting-sort buckets)
//   3. the community-ordered edge stream: for every member edge the new id of
//      the neighbour's community and the weight, contiguous per community
//   4. per community, sum the weights per neighbour community, by row length:
//        <= 32 entries      one warp, __match_any_sync + __reduce_add_sync
//        <= 512 entries     one 128-thread CTA, shared-memory hash table
//        <= 4096 entries    one CTA (1024 threads; 256 when rows are sorted),
//                           shared-memory hash table
//        <= 8192 entries    one 1024-thread CTA (rows in table order only)
//        larger             a global table per community filled by many CTAs
//                           (4096-entry chunks of the stream); a dense table
//                           indexed by community id when a hash table would not
//                           be smaller
//      and emit the distinct neighbours in ascending id order (rank by
//      shuffle compare, bitonic sort in shared memory, or - rows with more
//      than 16384 distinct neighbours - a bitmap over all communities ranked
//      by a prefix sum of popcounts, all spread over many CTAs)
//   5. CSR offsets by scan and a compaction copy.
// Rows come out sorted by neighbour id, so the contracted graph of a given
// partition is unique and can be compared bit for bit.
//
// The stream fill and the compaction walk contiguous entry ranges: every
// warp takes 1024 consecutive CSR entries and finds the row of each entry
// with a 5-step shuffle search over a window of 32 row ends, so the work is
// balanced whatever the row lengths (hub rows, empty rows of isolated
// vertices).
#include <limits.h>

#include <algorithm>

#include "common.cuh"
#include "internal.h"
#include "scan.cuh"
#include "walk.cuh"

namespace gala {

static int sm_count()
{
    static int s = 0;
    if (s == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev);
        if (s <= 0) s = 148;
    }
    return s;
}

constexpr int kSmallMax = 32;
constexpr int kMid1Max = 512;
constexpr int kMid2Max = 4096;
constexpr int kMid3Max = 8192;  // rows in hash-table order only (a 16384-slot table)
constexpr int kLongCls = 4;     // class of the rows aggregated in global tables
constexpr int kWarpCls = 5;     // rows of 33..kWarpAggMax entries in table order: one warp each
constexpr int kWarpAggMax = 128;
constexpr int kNumCls = 6;
constexpr int kChunk = 4096;
constexpr int kSortMax = 16384;
constexpr int kRangeEntries = 1024;  // CSR entries per warp task

struct OpDegOf {
    const int64_t *offs;
    __device__ __forceinline__ long long operator()(int32_t v, long long) const
    {
        return (long long)(offs[v + 1] - offs[v]);
    }
};
struct OpPopc {
    __device__ __forceinline__ long long operator()(unsigned x, long long) const { return __popc(x); }
};
struct OpRowNonEmpty {  // in = offs: row idx has entries
    const int64_t *offs;
    __device__ __forceinline__ long long operator()(int64_t x, long long idx) const
    {
        return offs[idx + 1] > x ? 1 : 0;
    }
};

// Walk list of the rows that have entries: nz_rows[i] (row id) and
// nz_offs[i] (its first entry), nz_offs[count] = E, count in st->nz_rows.
// Row walks over it never step through runs of empty rows.
// (E, or *dE on the device when dE is set)
__global__ void k_nz_tail(DevStats *st, long long *nz_offs, long long E, const long long *dE)
{
    const int cnt = (int)st->total;
    st->nz_rows = cnt;
    nz_offs[cnt] = dE ? *dE : E;
}

// Rows [0, n), or [0, min(n, *dn)) when dn is set.  Besides the row and its
// first entry, every listed row gets the value its walk kernel adds to an
// entry index (nz_shift, from shift(row, first entry)), and every 1024-entry
// task its first row (task_row): a walk then loads one coalesced value per
// row and starts its tasks without a search.
template <typename Shift>
__global__ void k_nz_scatter(const int64_t *__restrict__ offs, int n, const int32_t *__restrict__ pos,
                             int32_t *nz_rows, long long *nz_offs, long long *nz_shift, int32_t *task_row,
                             const long long *dn, Shift shift)
{
    if (dn && *dn < n) n = (int)*dn;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const long long s = offs[i], e = offs[i + 1];
        if (e > s) {
            const int p = pos[i];
            nz_rows[p] = i;
            nz_offs[p] = s;
            nz_shift[p] = shift(i, s);
            for (long long t = (s + kRangeEntries - 1) / kRangeEntries; t * kRangeEntries < e; ++t)
                task_row[t] = p;
        }
    }
}

// Shifts of the two walks: the stream fill writes entry j of vertex v's row
// to medge[mpos[v]] + (j - offs[v]); the compaction reads entry j of
// community c's new row from tmp_off[c] + (j - new_offs[c]).
struct ShiftStream {
    const int32_t *__restrict__ mpos;
    const long long *__restrict__ medge;
    __device__ __forceinline__ long long operator()(int v, long long s) const { return medge[mpos[v]] - s; }
};
struct ShiftCompact {
    const long long *__restrict__ tmp_off;
    __device__ __forceinline__ long long operator()(int c, long long s) const { return tmp_off[c] - s; }
};

// Caller-supplied labels must lie in [0, n) before they index any array.
__global__ void k_check_labels(const int32_t *__restrict__ comm, int n, DevStats *st)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        int c = comm[v];
        if (c < 0 || c >= n) atomicOr(&st->err, kErrBadLabel);
    }
}

__global__ void k_hist(const int32_t *__restrict__ comm, int n, int32_t *cnt)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        atomicAdd(&cnt[comm[v]], 1);
}

// New label of every vertex and member count of every new community (its
// entry count ec and, with self_out, its Self start at 0); with tot/k_out,
// K_new of community c is its total Tot[c] (the weight of the new row equals
// the weighted degrees of its members, exactly).
template <typename WT>
__global__ void k_relabel(const int32_t *__restrict__ comm, const int32_t *__restrict__ newid,
                          const int32_t *__restrict__ cnt, int n, int32_t *lab, int32_t *csz, long long *ec,
                          const WT *__restrict__ tot, WT *k_out, WT *self_out)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        lab[v] = newid[comm[v]];
        int k = cnt[v];
        if (k > 0) {
            const int c = newid[v];
            csz[c] = k;
            ec[c] = 0;
            if (k_out) k_out[c] = tot[v];
            if (self_out) self_out[c] = 0;
        }
    }
}

__global__ void k_compose(int32_t *orig, int n_orig, const int32_t *__restrict__ lab)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_orig; i += gridDim.x * blockDim.x)
        orig[i] = lab[orig[i]];
}

// Member buckets: csz[c] counts down to 0, so the members of c fill
// [moff[c], moff[c] + size) from the end (no cursor copy of moff).
__global__ void k_member_scatter(const int32_t *__restrict__ lab, const int64_t *__restrict__ offs, int n,
                                 const int32_t *__restrict__ moff, int32_t *csz, int32_t *members, int32_t *mpos,
                                 long long *ec)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        int c = lab[v];
        int p = moff[c] + atomicSub(&csz[c], 1) - 1;
        members[p] = v;
        mpos[v] = p;
        long long d = offs[v + 1] - offs[v];
        if (d) atomicAdd((unsigned long long *)&ec[c], (unsigned long long)d);
    }
}

// Community-ordered edge stream over contiguous entry ranges: entry j of row
// v goes to medge[mpos[v]] + (j - offs[v]).  Unweighted levels (W false)
// write no weights: the aggregation counts every entry as 1.  Rows are walked through the
// list of rows with entries (nz_rows / nz_offs); each row's destination
// (medge[mpos[v]] - offs[v]) is loaded once per row window.
template <typename WT, bool W>
__global__ void __launch_bounds__(256) k_stream_fill(long long E, const int32_t *__restrict__ nbr,
                                                     const WT *__restrict__ w, const int32_t *__restrict__ lab,
                                                     int32_t *skey, WT *sw,
                                                     const long long *__restrict__ nz_offs,
                                                     const long long *__restrict__ nz_shift,
                                                     const int32_t *__restrict__ task_row, DevStats *st)
{
    const long long wg = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const int nnz = st->nz_rows;
    // per row: pa = destination of the row's entry j minus j, pb = 1 (rows
    // past the list keep pb = 0)
    auto rowval = [=](int r, long long &pa, long long &pb) {
        pa = nz_shift[r];
        pb = 1;
    };
    constexpr int U = kWalkUnroll;
    const int lane = threadIdx.x & 31;
    auto cur = row_cursor(nz_offs, nnz, rowval);
    for (long long t = wg; t * kRangeEntries < E; t += nw) {
        const long long j0 = t * kRangeEntries;
        const long long j1 = j0 + kRangeEntries < E ? j0 + kRangeEntries : E;
        cur.start_row(task_row[t]);
        for (long long jb = j0; jb < j1; jb += 32 * U) {
            long long src[U], dst[U];
            bool ok[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const long long b0 = jb + 32 * u;
                ok[u] = false;
                src[u] = dst[u] = 0;
                if (b0 < j1) {  // warp-uniform
                    const long long j = b0 + lane;
                    long long d, valid;
                    const bool in = cur.resolve(b0, b0 + 31 < j1 ? b0 + 31 : j1 - 1, j, d, valid);
                    if (j < j1) {
                        const long long to = j + d;
                        if (!in || !valid || to < 0 || to >= E)  // recorded, never written
                            atomicOr(&st->err, kErrBadIndex);
                        else {
                            ok[u] = true;
                            src[u] = j;
                            dst[u] = to;
                        }
                    }
                }
            }
            int key[U];
            WT wv[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                key[u] = ok[u] ? nbr[src[u]] : 0;
                wv[u] = (W && ok[u]) ? w[src[u]] : (WT)0;
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (ok[u]) key[u] = lab[key[u]];
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (ok[u]) {
                    skey[dst[u]] = key[u];
                    if (W) sw[dst[u]] = wv[u];
                }
        }
    }
}

__device__ __forceinline__ int row_class(long long E, int sort_rows)
{
    if (E == 0) return -1;
    if (E <= kSmallMax) return 0;
    if (E <= kWarpAggMax && !sort_rows) return kWarpCls;
    if (E <= kMid1Max) return 1;
    if (E <= kMid2Max) return 2;
    if (E <= kMid3Max && !sort_rows) return 3;
    return kLongCls;
}

// Size classes: every block lists the communities of a contiguous range with
// one counter add per class (a first pass counts the range); class k lists
// its communities from lists + k * lstride.  Communities without entries get
// an empty row right away.
__global__ void __launch_bounds__(256) k_classify(const long long *__restrict__ ec, int32_t *lists, long long lstride,
                                                  int32_t *kc, DevStats *st, int sort_rows)
{
    __shared__ int wc[8][kNumCls];  // per-warp counts of a tile
    __shared__ int next[kNumCls];   // the block's next list position per class
    const int C = (int)st->ccount;
    const long long per = ((long long)C + gridDim.x - 1) / gridDim.x;
    const int c0 = (int)((long long)blockIdx.x * per < C ? (long long)blockIdx.x * per : C);
    const int c1 = (int)(c0 + per < C ? c0 + per : C);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int cnt[kNumCls];
#pragma unroll
    for (int k = 0; k < kNumCls; ++k) cnt[k] = 0;
    for (int c = c0 + threadIdx.x; c < c1; c += blockDim.x) {
        const int cls = row_class(ec[c], sort_rows);
#pragma unroll
        for (int k = 0; k < kNumCls; ++k) cnt[k] += cls == k;
    }
    if (threadIdx.x < kNumCls) next[threadIdx.x] = 0;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kNumCls; ++k) {
        const int t = __reduce_add_sync(GALA_FULL_MASK, (unsigned)cnt[k]);
        if (lane == 0 && t) atomicAdd(&next[k], t);
    }
    __syncthreads();
    if (threadIdx.x < kNumCls && next[threadIdx.x])
        next[threadIdx.x] = atomicAdd(&st->small_cnt[threadIdx.x], next[threadIdx.x]);
    __syncthreads();
    for (int t0 = c0; t0 < c1; t0 += blockDim.x) {  // block-uniform
        const int c = t0 + threadIdx.x;
        const int cls = c < c1 ? row_class(ec[c], sort_rows) : -2;
        if (cls == -1) kc[c] = 0;
        int rank = 0;
#pragma unroll
        for (int k = 0; k < kNumCls; ++k) {
            const unsigned b = __ballot_sync(GALA_FULL_MASK, cls == k);
            if (cls == k) rank = __popc(b & lanemask_lt());
            if (lane == 0) wc[wid][k] = __popc(b);
        }
        __syncthreads();
        if (cls >= 0) {
            int off = next[cls] + rank;
            for (int w = 0; w < wid; ++w) off += wc[w][cls];
            lists[cls * lstride + off] = c;
        }
        __syncthreads();
        if (threadIdx.x < kNumCls) {
            int s = 0;
            for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += wc[w][threadIdx.x];
            next[threadIdx.x] += s;
        }
        __syncthreads();
    }
}

template <typename WT>
struct AggArgs {
    const int32_t *__restrict__ moff;
    const long long *__restrict__ medge;
    const long long *__restrict__ ec;
    const int32_t *__restrict__ skey;
    const WT *__restrict__ sw;  // null: unweighted level, every entry weighs 1
    const long long *__restrict__ tmp_off;
    int32_t *tmp_nbr;
    WT *tmp_w;
    int32_t *kc;
    DevStats *st;  // st->ccount = C
    __device__ __forceinline__ WT w_at(long long i) const { return sw ? sw[i] : (WT)1; }
};

// Rows of at most 32 entries: one warp, rank of each distinct key by a
// shuffle compare against all others.
template <typename WT>
__global__ void __launch_bounds__(256) k_agg_small(AggArgs<WT> a, const int32_t *__restrict__ list)
{
    const int lane = threadIdx.x & 31;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int cnt = a.st->small_cnt[0];
    for (int i = wg; i < cnt; i += nw) {
        const int c = list[i];
        const long long st = a.medge[a.moff[c]];
        const int E = (int)a.ec[c];
        const bool valid = lane < E;
        int key = -1;
        WT wt = 0;
        if (valid) {
            key = a.skey[st + lane];
            wt = a.w_at(st + lane);
        }
        const unsigned m = __match_any_sync(GALA_FULL_MASK, key);
        const WT sum = group_sum(m, wt);
        const bool head = valid && (__ffs(m) - 1 == lane);
        const unsigned hm = __ballot_sync(GALA_FULL_MASK, head);
        int rank = 0;
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            int kj = __shfl_sync(GALA_FULL_MASK, key, j);
            rank += ((hm >> j) & 1u) && kj < key;
        }
        if (head) {
            a.tmp_nbr[a.tmp_off[c] + rank] = key;
            a.tmp_w[a.tmp_off[c] + rank] = sum;
        }
        if (lane == 0) a.kc[c] = __popc(hm);
    }
}

// Sort (key, val) pairs in shared memory by key, P a power of two.
template <typename VT>
__device__ __forceinline__ void bitonic_sort_smem(int *k, VT *v, int P)
{
    for (int size = 2; size <= P; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = threadIdx.x; t < (P >> 1); t += blockDim.x) {
                int i = 2 * t - (t & (stride - 1));
                int j = i + stride;
                bool asc = (i & size) == 0;
                int ki = k[i], kj = k[j];
                if ((ki > kj) == asc) {
                    k[i] = kj;
                    k[j] = ki;
                    VT tv = v[i];
                    v[i] = v[j];
                    v[j] = tv;
                }
            }
            __syncthreads();
        }
    }
}

// Insert stream entries [st, st + len) into a table (dense when keys is
// null).  Returns this thread's count of newly created keys.  All threads of
// the block call it.
__device__ __forceinline__ bool add_was_zero(int *p, int v) { return atomicAdd(p, v) == 0; }
__device__ __forceinline__ bool add_was_zero(long long *p, long long v)
{
    return atomicAdd((unsigned long long *)p, (unsigned long long)v) == 0ull;
}

template <typename WT>
__device__ __forceinline__ int agg_insert(const AggArgs<WT> &a, long long st, int len, int *keys, WT *vals, int T,
                                          int lg)
{
    const int lane = threadIdx.x & 31;
    int created = 0;
    for (int b0 = 0; b0 < len; b0 += blockDim.x) {
        const int j = b0 + threadIdx.x;
        const bool valid = j < len;
        int key = -1;
        WT wt = 0;
        if (valid) {
            key = a.skey[st + j];
            wt = a.w_at(st + j);
        }
        const unsigned m = __match_any_sync(GALA_FULL_MASK, key);
        const WT sum = group_sum(m, wt);
        if (valid && __ffs(m) - 1 == lane) {
            if (!keys) {
                created += add_was_zero(&vals[key], sum);
            } else {
                unsigned h = hash_slot(key, lg);
                bool ok = false;
                for (int p = 0; p < T; ++p) {
                    int k = *(volatile int *)&keys[h];
                    if (k == -1) {
                        k = atomicCAS(&keys[h], -1, key);
                        if (k == -1) {
                            k = key;
                            created++;
                        }
                    }
                    if (k == key) {
                        atomic_add_w(&vals[h], sum);
                        ok = true;
                        break;
                    }
                    h = (h + 1) & (unsigned)(T - 1);
                }
                if (!ok) atomicOr(&a.st->err, kErrHashOverflow);
            }
        }
    }
    return created;
}

// Add (key, w) to a table (dense when keys is null); returns 1 when this call
// created the key, 0 when it existed, -1 when the probe ran out.  `slot`
// receives the slot (hash tables).
template <typename WT>
__device__ __forceinline__ int table_add(int *keys, WT *vals, int T, int lg, int key, WT w, int &slot)
{
    if (!keys) {
        slot = key;
        return add_was_zero(&vals[key], w) ? 1 : 0;
    }
    unsigned h = hash_slot(key, lg);
    for (int p = 0; p < T; ++p) {
        int k = *(volatile int *)&keys[h];
        int created = 0;
        if (k == -1) {
            k = atomicCAS(&keys[h], -1, key);
            if (k == -1) {
                k = key;
                created = 1;
            }
        }
        if (k == key) {
            atomic_add_w(&vals[h], w);
            slot = (int)h;
            return created;
        }
        h = (h + 1) & (unsigned)(T - 1);
    }
    slot = -1;
    return -1;
}

// Insert stream entries [st, st + len) into a shared-memory hash table (T
// slots) and list every slot a key claims in occ (counter *nocc, shared).
// All threads of the block call it.
template <typename WT>
__device__ __forceinline__ void agg_insert_list(const AggArgs<WT> &a, long long st, int len, int *keys, WT *vals,
                                                int T, int lg, unsigned short *occ, int *nocc)
{
    const int lane = threadIdx.x & 31;
    for (int b0 = 0; b0 < len; b0 += blockDim.x) {
        const int j = b0 + threadIdx.x;
        const bool valid = j < len;
        int key = -1;
        WT wt = 0;
        if (valid) {
            key = a.skey[st + j];
            wt = a.w_at(st + j);
        }
        // shared-memory tables take every entry on its own (cheaper than a
        // warp-level match of equal keys); the global tables of long rows do
        // match first, where repeated keys would queue on one address
        int created = 0, slot = -1;
        if (valid) {
            created = table_add(keys, vals, T, lg, key, wt, slot);
            if (created < 0) {
                atomicOr(&a.st->err, kErrHashOverflow);
                created = 0;
            }
        }
        const unsigned cb = __ballot_sync(GALA_FULL_MASK, created == 1);
        if (cb) {
            const int leader = __ffs(cb) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(nocc, __popc(cb));
            base = __shfl_sync(GALA_FULL_MASK, base, leader);
            if (created == 1) occ[base + __popc(cb & lanemask_lt())] = (unsigned short)slot;
        }
    }
}

// Rows of 33..kWarpAggMax entries in hash-table order: one warp per
// community with its own shared-memory table (2 kWarpAggMax slots) and list
// of claimed slots; warps work independently (no block barriers), so eight
// communities per block are in flight.
template <typename WT>
__global__ void __launch_bounds__(256) k_agg_warp_list(AggArgs<WT> a, const int32_t *__restrict__ list)
{
    constexpr int T = 2 * kWarpAggMax, LG = 8;
    static_assert((1 << LG) == T, "table size");
    __shared__ int skeys[8][T];
    __shared__ WT svals[8][T];
    __shared__ unsigned char socc[8][kWarpAggMax];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int *keys = skeys[wid];
    WT *vals = svals[wid];
    unsigned char *occ = socc[wid];
    for (int j = lane; j < T; j += 32) {
        keys[j] = -1;
        vals[j] = 0;
    }
    __syncwarp();
    const int cnt = a.st->small_cnt[kWarpCls];
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = wg; i < cnt; i += nw) {
        const int c = list[i];
        const long long st = a.medge[a.moff[c]];
        const int E = (int)a.ec[c];  // 33..kWarpAggMax
        int nocc = 0;
        for (int b0 = 0; b0 < E; b0 += 32) {
            const int j = b0 + lane;
            int created = 0, slot = -1;
            if (j < E) {
                created = table_add(keys, vals, T, LG, a.skey[st + j], a.w_at(st + j), slot);
                if (created < 0) {
                    atomicOr(&a.st->err, kErrHashOverflow);
                    created = 0;
                }
            }
            const unsigned cb = __ballot_sync(GALA_FULL_MASK, created == 1);
            if (created == 1) occ[nocc + __popc(cb & lanemask_lt())] = (unsigned char)slot;
            nocc += __popc(cb);
        }
        __syncwarp();
        const long long o = a.tmp_off[c];
        for (int q = lane; q < nocc; q += 32) {
            const int j = occ[q];
            a.tmp_nbr[o + q] = keys[j];
            a.tmp_w[o + q] = vals[j];
            keys[j] = -1;
            vals[j] = 0;
        }
        if (lane == 0) a.kc[c] = nocc;
        __syncwarp();
    }
}

// Rows of 33..kMid2Max entries in hash-table order (level-to-level
// contraction): one CTA per community; the shared-memory table of TMAX slots
// is cleared once per CTA, per community only the claimed slots (listed) are
// emitted and cleared.
template <typename WT, int BLOCK, int TMAX>
__global__ void __launch_bounds__(BLOCK) k_agg_mid_list(AggArgs<WT> a, const int32_t *__restrict__ list, int cls)
{
    extern __shared__ long long sml_ll[];
    WT *vals = (WT *)sml_ll;
    int *keys = (int *)(vals + TMAX);
    unsigned short *occ = (unsigned short *)(keys + TMAX);
    __shared__ int s_k;
    constexpr int lg = (TMAX == 1024) ? 10 : (TMAX == 2048 ? 11 : (TMAX == 4096 ? 12 : (TMAX == 8192 ? 13 : 14)));
    static_assert((1 << lg) == TMAX, "table size");
    for (int j = threadIdx.x; j < TMAX; j += BLOCK) {
        keys[j] = -1;
        vals[j] = 0;
    }
    if (threadIdx.x == 0) s_k = 0;
    __syncthreads();
    const int cnt = a.st->small_cnt[cls];
    for (int i = blockIdx.x; i < cnt; i += gridDim.x) {
        const int c = list[i];
        const long long st = a.medge[a.moff[c]];
        const int E = (int)a.ec[c];
        agg_insert_list(a, st, E, keys, vals, TMAX, lg, occ, &s_k);
        __syncthreads();
        const int k = s_k;
        const long long o = a.tmp_off[c];
        for (int q = threadIdx.x; q < k; q += BLOCK) {
            const int j = occ[q];
            a.tmp_nbr[o + q] = keys[j];
            a.tmp_w[o + q] = vals[j];
            keys[j] = -1;
            vals[j] = 0;
        }
        if (threadIdx.x == 0) a.kc[c] = k;
        __syncthreads();
        if (threadIdx.x == 0) s_k = 0;
        __syncthreads();
    }
}

// Rows of 33..kMid2Max entries: one CTA per community, shared-memory hash
// table of TMAX slots, distinct keys sorted by a bitonic sort of LMAX slots.
template <typename WT, int BLOCK, int TMAX, int LMAX>
__global__ void __launch_bounds__(BLOCK) k_agg_mid(AggArgs<WT> a, const int32_t *__restrict__ list, int cls)
{
    extern __shared__ long long sm_ll[];
    int *keys = (int *)sm_ll;
    WT *vals = (WT *)(keys + TMAX);
    int *lk = (int *)(vals + TMAX);
    WT *lv = (WT *)(lk + LMAX);
    __shared__ int s_k;
    const int cnt = a.st->small_cnt[cls];
    for (int i = blockIdx.x; i < cnt; i += gridDim.x) {
        const int c = list[i];
        const long long st = a.medge[a.moff[c]];
        const int E = (int)a.ec[c];
        const int C = (int)a.st->ccount;
        const int cap = E < C ? E : C;
        int T = next_pow2_int(2LL * cap);
        if (T < 64) T = 64;
        if (T > TMAX) T = TMAX;
        const int lg = __ffs(T) - 1;
        for (int j = threadIdx.x; j < T; j += BLOCK) {
            keys[j] = -1;
            vals[j] = 0;
        }
        if (threadIdx.x == 0) s_k = 0;
        __syncthreads();
        agg_insert(a, st, E, keys, vals, T, lg);
        __syncthreads();
        for (int j = threadIdx.x; j < T; j += BLOCK) {
            int kk = keys[j];
            if (kk >= 0) {
                int p = atomicAdd(&s_k, 1);
                lk[p] = kk;
                lv[p] = vals[j];
            }
        }
        __syncthreads();
        const int k = s_k;
        const int P = next_pow2_int(k);
        for (int j = k + threadIdx.x; j < P; j += BLOCK) {
            lk[j] = 0x7fffffff;
            lv[j] = 0;
        }
        __syncthreads();
        bitonic_sort_smem(lk, lv, P);
        const long long o = a.tmp_off[c];
        for (int j = threadIdx.x; j < k; j += BLOCK) {
            a.tmp_nbr[o + j] = lk[j];
            a.tmp_w[o + j] = lv[j];
        }
        if (threadIdx.x == 0) a.kc[c] = k;
        __syncthreads();
    }
}

// ---- rows of more than kMid2Max entries --------------------------------

struct BigArgs {
    const int32_t *__restrict__ list;  // class-3 communities
    long long *T;
    long long *chunks;
    long long *tchunks;
    const long long *__restrict__ toff;
    const long long *__restrict__ coff;
    const long long *__restrict__ tcoff;
    int32_t *mode;
    int32_t *work;
    int32_t *twork;
    int32_t *kdist;
    int32_t *cursor;
    long long *gwords;
    const long long *__restrict__ gofs;
    int32_t *pool;
    long long pool_half;  // keys at pool[0, half), values (WT, 8-byte aligned) from pool[half]
    long long work_cap;   // capacity of work
    long long twork_cap;  // capacity of twork
    unsigned *bits;       // bitmaps of the rows ranked by bitmap
    unsigned *pref;       // exclusive prefix of their popcounts
};

// Long-row kernels run only while the tables fit their scratch.
__device__ __forceinline__ bool big_off(const DevStats *st) { return (st->err & kErrCapacity) != 0; }

// Table size and chunk counts of every class-3 community.  A dense table
// (slot = community id) is used when a hash table would not be smaller.
template <typename WT>
__global__ void k_big_plan(AggArgs<WT> a, BigArgs b)
{
    const int cnt = a.st->small_cnt[kLongCls];
    const long long C = a.st->ccount;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        const long long E = a.ec[b.list[i]];
        const long long cap = E < C ? E : C;
        long long T = next_pow2_ll(cap + cap / 2);  // load at most 2/3
        int dense = T >= C;
        if (dense) T = C;
        b.T[i] = T;
        b.mode[i] = dense;
        b.chunks[i] = (E + kChunk - 1) / kChunk;
        b.tchunks[i] = (T + kChunk - 1) / kChunk;
        b.kdist[i] = 0;
        b.cursor[i] = 0;
    }
}

// toff[cnt] / coff[cnt] / tcoff[cnt] close the last segments; tables or
// chunk lists beyond their scratch set kErrCapacity, which stops the other
// long-row kernels (the host reports it after the contraction).
__global__ void k_big_tail(BigArgs b, DevStats *st)
{
    const int cnt = st->small_cnt[kLongCls];
    ((long long *)b.toff)[cnt] = st->big_slots;
    ((long long *)b.coff)[cnt] = st->big_nwork;
    ((long long *)b.tcoff)[cnt] = st->big_ntwork;
    if (st->big_slots > b.pool_half || st->big_nwork > b.work_cap || st->big_ntwork > b.twork_cap)
        st->err |= kErrCapacity;
}

// Empty tables: keys -1, values 0, over the slots the plan counted.
template <typename WT>
__global__ void k_big_clear(BigArgs b, const DevStats *st)
{
    if (big_off(st)) return;
    const long long slots = st->big_slots;
    WT *vals = (WT *)(b.pool + b.pool_half);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < slots;
         i += (long long)gridDim.x * blockDim.x) {
        b.pool[i] = -1;
        vals[i] = 0;
    }
}

// stream chunk -> community and table chunk -> community, one warp per
// community (list index)
template <typename WT>
__global__ void k_big_work(AggArgs<WT> a, BigArgs b)
{
    const int lane = threadIdx.x & 31;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int cnt = big_off(a.st) ? 0 : a.st->small_cnt[kLongCls];
    for (int i = wg; i < cnt; i += nw) {
        long long o = b.coff[i], k = b.coff[i + 1] - o;
        for (long long j = lane; j < k; j += 32) b.work[o + j] = i;
        o = b.tcoff[i];
        k = b.tcoff[i + 1] - o;
        for (long long j = lane; j < k; j += 32) b.twork[o + j] = i;
    }
}

// Values of a community's global table (after the keys of all tables).
template <typename WT>
__device__ __forceinline__ WT *big_vals(const BigArgs &b, long long i)
{
    return (WT *)(b.pool + b.pool_half) + b.toff[i];
}

// Every CTA aggregates one chunk of kChunk stream entries of a long row in a
// shared-memory table first, then adds the chunk's distinct keys to the row's
// global table (many CTAs share one row); new keys are counted.
constexpr int kSmT = 8192;  // shared-memory slots for a kChunk-entry chunk
template <typename WT>
constexpr size_t big_sm_smem()
{
    return (size_t)kSmT * (sizeof(WT) + sizeof(int) + sizeof(unsigned short));
}
template <typename WT>
__global__ void __launch_bounds__(512) k_big_insert_sm(AggArgs<WT> a, BigArgs b, int lists)
{
    const long long nwork = big_off(a.st) ? 0 : a.st->big_nwork;
    if (nwork <= blockIdx.x) return;
    extern __shared__ long long bsm_ll[];
    WT *svals = (WT *)bsm_ll;
    int *skeys = (int *)(svals + kSmT);
    unsigned short *socc = (unsigned short *)(skeys + kSmT);
    __shared__ int s_n, s_base;
    __shared__ int red[16];
    for (int q = threadIdx.x; q < kSmT; q += blockDim.x) {
        skeys[q] = -1;
        svals[q] = 0;
    }
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    constexpr int slg = 13;
    static_assert((1 << slg) == kSmT, "table size");
    for (long long wi = blockIdx.x; wi < nwork; wi += gridDim.x) {
        const int i = b.work[wi];
        const long long j = wi - b.coff[i];
        const int c = b.list[i];
        const long long E = a.ec[c];
        const long long st = a.medge[a.moff[c]] + j * kChunk;
        const int len = (int)((E - j * kChunk) < kChunk ? (E - j * kChunk) : kChunk);
        const long long T = b.T[i];
        WT *vals = big_vals<WT>(b, i);
        int *keys = b.mode[i] ? nullptr : b.pool + b.toff[i];
        const int lg = keys ? __ffs((int)T) - 1 : 0;
        for (int q = threadIdx.x; q < len; q += blockDim.x) {
            const int key = a.skey[st + q];
            const WT wt = a.w_at(st + q);
            unsigned h = hash_slot(key, slg);
            for (int p = 0; p < kSmT; ++p) {
                int k = *(volatile int *)&skeys[h];  // a repeated key skips the claim
                if (k == -1) k = atomicCAS(&skeys[h], -1, key);
                if (k == -1 || k == key) {
                    atomic_add_w(&svals[h], wt);
                    if (k == -1) socc[atomicAdd(&s_n, 1)] = (unsigned short)h;
                    break;
                }
                h = (h + 1) & (unsigned)(kSmT - 1);
            }
        }
        __syncthreads();
        const int n = s_n;
        // the chunk's distinct keys go to the global table; with lists, the
        // slots this chunk created are appended to the row's slot list (in the
        // row's own tmp range), one counter add per chunk
        constexpr int kIt = kChunk / 512;
        int made[kIt];
        unsigned mask = 0;
#pragma unroll
        for (int it = 0; it < kIt; ++it) {
            const int q = threadIdx.x + it * 512;
            made[it] = 0;
            if (q < n) {
                const int h = socc[q];
                int slot;
                const int r = table_add(keys, vals, (int)T, lg, skeys[h], svals[h], slot);
                if (r < 0) atomicOr(&a.st->err, kErrHashOverflow);
                if (r == 1) {
                    mask |= 1u << it;
                    made[it] = slot;
                }
                skeys[h] = -1;
                svals[h] = 0;
            }
        }
        const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
        const int mine = __popc(mask);
        int incl = mine;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(GALA_FULL_MASK, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) red[wid] = incl;
        __syncthreads();
        if (threadIdx.x == 0) {
            int tot = 0;
            for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
                const int t = red[q];
                red[q] = tot;
                tot += t;
            }
            if (tot) atomicAdd(&b.kdist[i], tot);
            s_base = (lists && tot) ? atomicAdd(&b.cursor[i], tot) : 0;
            s_n = 0;
        }
        __syncthreads();
        if (lists && mask) {
            int p = s_base + red[wid] + incl - mine;
            const long long o = a.tmp_off[c];
#pragma unroll
            for (int it = 0; it < kIt; ++it)
                if (mask & (1u << it)) a.tmp_nbr[o + p++] = made[it];
        }
        __syncthreads();
    }
}

// Rows with more distinct neighbours than a shared-memory sort holds are
// ranked by a bitmap over all communities: words per row (0 for the others);
// every class-3 row gets its final length here.
template <typename WT>
__global__ void k_big_mark(AggArgs<WT> a, BigArgs b, int sort_rows)
{
    const int cnt = a.st->small_cnt[kLongCls];
    const long long words = (a.st->ccount + 31) >> 5;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        const int k = b.kdist[i];
        b.gwords[i] = (sort_rows && k > kSortMax) ? words : 0;
        a.kc[b.list[i]] = k;
    }
}

// Rows in table order: every kChunk entries of a row's slot list (written by
// the inserts into the row's own tmp range) are replaced in place by the
// (key, value) of their slot.  Work items: lcoff is the exclusive scan of
// the list chunks per row, *total their number.
template <typename WT>
__global__ void __launch_bounds__(256) k_big_collect_list(AggArgs<WT> a, BigArgs b, const long long *lcoff,
                                                          const long long *total)
{
    const int cnt = a.st->small_cnt[kLongCls];
    const long long nw = *total;
    for (long long w = blockIdx.x; w < nw; w += gridDim.x) {
        int lo = 0, hi = cnt - 1;  // last row with lcoff <= w
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (lcoff[mid] <= w) lo = mid;
            else hi = mid - 1;
        }
        const int i = lo;
        const int c = b.list[i];
        const long long q0 = (w - lcoff[i]) * kChunk;
        const long long k = b.cursor[i];
        const long long q1 = q0 + kChunk < k ? q0 + kChunk : k;
        const long long o = a.tmp_off[c];
        const bool dense = b.mode[i];
        const WT *vals = big_vals<WT>(b, i);
        const int *keys = b.pool + b.toff[i];
        for (long long q = q0 + threadIdx.x; q < q1; q += blockDim.x) {
            const int slot = a.tmp_nbr[o + q];
            a.tmp_nbr[o + q] = dense ? slot : keys[slot];
            a.tmp_w[o + q] = vals[slot];
        }
    }
}

// Row length of every long row in table order: its slot-list length.
template <typename WT>
__global__ void k_big_len(AggArgs<WT> a, BigArgs b)
{
    const int cnt = a.st->small_cnt[kLongCls];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
        a.kc[b.list[i]] = b.cursor[i];
}

__global__ void k_big_lchunks(const int *cursor, const DevStats *st, long long *lch)
{
    const int cnt = st->small_cnt[kLongCls];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x)
        lch[i] = (cursor[i] + kChunk - 1) / kChunk;
}

// ---- long rows by key range (rows in table order) ----------------------
//
// Every kChunk-entry chunk of a long row is summed per key in shared memory
// first; its distinct (key, sum) pairs go back to the chunk's own stream
// range, ordered by bucket (key >> kRadLg: 8192 communities each), together
// with the chunk's bucket offsets and the pair counts per (row, bucket).
// Work items then cover one bucket, or a run of small buckets, of one row: a
// CTA sums the item's pairs from every chunk of the row in one shared-memory
// table (dense over the bucket's 8192 keys, or hashed) and appends the
// distinct keys to the row.  A bucket of more than kRadPiece pairs is split
// by chunk range over several CTAs that add their sums into a global dense
// table of the bucket; the last of them emits it.  Against the global hash
// tables of the other path this takes no table clear, no global probing and
// no slot-list collection.
constexpr int kRadLg = 13;
constexpr int kRadW = 1 << kRadLg;  // communities per bucket
constexpr int kRadNbMax = 2048;     // buckets per row (C <= 2^24)
constexpr int kRadH = 2048;         // buckets of at most kRadH pairs are grouped (< 2 kRadH pairs per item)
constexpr int kRadPiece = 32768;    // pairs per CTA of a split bucket
static_assert(kSmT == kRadW, "the chunk table and a bucket have the same size");

struct RadItem {
    long long sbase;  // first stream entry of the row
    long long dst;    // first tmp entry of the row
    long long w0;     // first chunk of the row (index over all long rows)
    long long erow;   // entries of the row
    int i;            // row (list index)
    int b0, b1;       // buckets [b0, b1)
    int k0, k1;       // chunks [k0, k1) of the row
    int acc;          // global table of a split bucket (-1: none)
    int pieces;       // CTAs of the bucket
    int total;        // pairs of the buckets over all chunks of the row
};
constexpr int kRadItemInts = (int)(sizeof(RadItem) / sizeof(int));

// Global table of a split bucket: kRadW values, a bitmap of the slots that
// received a non-positive sum, a counter of finished pieces.
__host__ __device__ constexpr long long rad_acc_ints(long long vints) { return kRadW * vints + kRadW / 32 + 8; }

struct RadLayout {
    long long offm, items, acc, max_items, max_acc, end;
};
__host__ __device__ inline long long rad_up8(long long x) { return (x + 7) & ~7LL; }
// Pool layout (ints): pair counts per (row, bucket) at 0, then the chunks'
// bucket offsets (uint16, nb + 1 per chunk), the items and the global tables.
// Items per row are at most pairs (4 / kRadH + 1 / kRadPiece) + 2: big
// buckets, the runs after them and one run per kRadH-pair window, plus the
// extra pieces of split buckets.
__host__ __device__ inline RadLayout rad_layout(long long cnt, long long nwork, long long nb, long long vints)
{
    RadLayout L;
    L.offm = rad_up8(cnt * nb);
    L.items = rad_up8(L.offm + (nwork * (nb + 1) + 1) / 2);
    L.max_items = 5 * nwork * kChunk / kRadH + 2 * cnt + 16;
    L.acc = rad_up8(L.items + L.max_items * kRadItemInts);
    L.max_acc = nwork * kChunk / kRadPiece + 1;
    L.end = L.acc + L.max_acc * rad_acc_ints(vints);
    return L;
}

// Exclusive prefix of x over the block (all threads call; ws: 33 ints);
// total receives the block sum.  Ends with a barrier.
__device__ __forceinline__ int block_excl_scan(int x, int *ws, int &total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int incl = x;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(GALA_FULL_MASK, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) ws[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const int w = lane < nw ? ws[lane] : 0;
        int wi = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(GALA_FULL_MASK, wi, o);
            if (lane >= o) wi += t;
        }
        if (lane < nw) ws[lane] = wi - w;
        if (lane == 31) ws[32] = wi;
    }
    __syncthreads();
    total = ws[32];
    const int r = ws[wid] + incl - x;
    __syncthreads();
    return r;
}

// Chunk counts per row, cursors, zeroed pair counts, buckets per row.
template <typename WT>
__global__ void k_rad_plan(AggArgs<WT> a, BigArgs b, int32_t *tot, long long pool_ints)
{
    const int cnt = a.st->small_cnt[kLongCls];
    const long long C = a.st->ccount;
    const int nb = (int)((C + kRadW - 1) >> kRadLg);
    const long long tid = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const long long nt = (long long)gridDim.x * blockDim.x;
    for (long long i = tid; i < cnt; i += nt) {
        const long long E = a.ec[b.list[i]];
        b.chunks[i] = (E + kChunk - 1) / kChunk;
        b.cursor[i] = 0;
    }
    const long long ntot = (long long)cnt * nb;
    if (nb <= kRadNbMax && ntot <= pool_ints)
        for (long long q = tid; q < ntot; q += nt) tot[q] = 0;
    if (tid == 0) a.st->rad_nb = nb;
}

// coff[cnt] closes the chunk list; the layout is fixed and checked against
// the pool (kErrCapacity stops the other kernels).
__global__ void k_rad_tail(BigArgs b, DevStats *st, long long vints, long long pool_ints)
{
    const int cnt = st->small_cnt[kLongCls];
    const long long nwork = st->big_nwork;
    ((long long *)b.coff)[cnt] = nwork;
    const int nb = st->rad_nb;
    const RadLayout L = rad_layout(cnt, nwork, nb, vints);
    st->rad_offm = L.offm;
    st->rad_items = L.items;
    st->rad_acc = L.acc;
    st->rad_max_items = L.max_items;
    st->rad_max_acc = L.max_acc;
    if (nb > kRadNbMax || L.end > pool_ints) st->err |= kErrCapacity;
}

template <typename WT>
constexpr size_t rad_combine_smem()
{
    return (size_t)kSmT * (sizeof(WT) + sizeof(int) + sizeof(unsigned short)) + (kRadNbMax + 1) * sizeof(int);
}

// One chunk per CTA iteration: sum the chunk's entries per key (shared-memory
// hash table), then write the distinct pairs back over the chunk in bucket
// order.  pk / pw are the stream's keys and weight slots (the weight slots
// are written even on an unweighted level, where the stream has no weights).
constexpr int kRadCombineThreads = 1024;  // two CTAs per SM: 32 registers a thread
template <typename WT>
__global__ void __launch_bounds__(kRadCombineThreads, 2) k_rad_combine(AggArgs<WT> a, BigArgs b, int32_t *pool, int32_t *pk, WT *pw)
{
    DevStats *st = a.st;
    const long long nwork = big_off(st) ? 0 : st->big_nwork;
    if (nwork <= blockIdx.x) return;
    const int cnt = st->small_cnt[kLongCls];
    const int nb = st->rad_nb;
    int32_t *tot = pool;
    unsigned short *offm = (unsigned short *)(pool + st->rad_offm);
    extern __shared__ long long rsm_ll[];
    WT *svals = (WT *)rsm_ll;
    int *skeys = (int *)(svals + kSmT);
    int *hist = skeys + kSmT;
    unsigned short *socc = (unsigned short *)(hist + kRadNbMax + 1);
    __shared__ int s_n;
    __shared__ int ws[33];
    for (int q = threadIdx.x; q < kSmT; q += blockDim.x) {
        skeys[q] = -1;
        svals[q] = 0;
    }
    for (int q = threadIdx.x; q <= kRadNbMax; q += blockDim.x) hist[q] = 0;
    if (threadIdx.x == 0) s_n = 0;
    __syncthreads();
    for (long long wi = blockIdx.x; wi < nwork; wi += gridDim.x) {
        int lo = 0, hi = cnt - 1;  // row of the chunk: last i with coff[i] <= wi
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (b.coff[mid] <= wi) lo = mid;
            else hi = mid - 1;
        }
        const int i = lo;
        const int c = b.list[i];
        const long long j = wi - b.coff[i];
        const long long E = a.ec[c];
        const long long s0 = a.medge[a.moff[c]] + j * kChunk;
        const int len = (int)((E - j * kChunk) < kChunk ? (E - j * kChunk) : kChunk);
        constexpr int kPer = kChunk / kRadCombineThreads;  // entries per thread, loaded before the inserts
        int kk[kPer];
        WT ww[kPer];
#pragma unroll
        for (int u = 0; u < kPer; ++u) {
            const int q = threadIdx.x + u * kRadCombineThreads;
            kk[u] = 0;
            ww[u] = 0;
            if (q < len) {
                kk[u] = pk[s0 + q];
                ww[u] = a.sw ? pw[s0 + q] : (WT)1;
            }
        }
#pragma unroll
        for (int u = 0; u < kPer; ++u) {
            if (threadIdx.x + u * kRadCombineThreads >= len) break;
            const int key = kk[u];
            const WT wt = ww[u];
            unsigned h = hash_slot(key, kRadLg);
            for (int p = 0; p < kSmT; ++p) {
                int k = *(volatile int *)&skeys[h];  // a repeated key skips the claim
                if (k == -1) k = atomicCAS(&skeys[h], -1, key);
                if (k == -1 || k == key) {
                    atomic_add_w(&svals[h], wt);
                    if (k == -1) {
                        socc[atomicAdd(&s_n, 1)] = (unsigned short)h;
                        const int bk = key >> kRadLg;
                        if (bk < nb) atomicAdd(&hist[bk], 1);
                        else atomicOr(&st->err, kErrBadIndex);
                    }
                    break;
                }
                h = (h + 1) & (unsigned)(kSmT - 1);
            }
        }
        __syncthreads();
        const int n = s_n;
        // bucket offsets of the chunk: exclusive scan of hist, kHistPer buckets per thread
        constexpr int kHistPer = kRadNbMax / kRadCombineThreads;
        int v[kHistPer], sum = 0;
        const int t4 = threadIdx.x * kHistPer;
#pragma unroll
        for (int u = 0; u < kHistPer; ++u) {
            v[u] = (t4 + u < nb) ? hist[t4 + u] : 0;
            sum += v[u];
        }
        int total;
        int run = block_excl_scan(sum, ws, total);
        unsigned short *orow = offm + wi * (nb + 1);
#pragma unroll
        for (int u = 0; u < kHistPer; ++u) {
            const int bk = t4 + u;
            if (bk < nb) {
                if (v[u]) atomicAdd(&tot[(long long)i * nb + bk], v[u]);
                orow[bk] = (unsigned short)run;
                hist[bk] = run;  // the scatter's cursor of the bucket
                run += v[u];
            }
        }
        if (threadIdx.x == 0) orow[nb] = (unsigned short)n;
        __syncthreads();
        for (int q = threadIdx.x; q < n; q += blockDim.x) {
            const int h = socc[q];
            const int key = skeys[h];
            const int bk = key >> kRadLg;
            if (bk < nb) {
                const int p = atomicAdd(&hist[bk], 1);
                pk[s0 + p] = key;
                pw[s0 + p] = svals[h];
            }
            skeys[h] = -1;
            svals[h] = 0;
        }
        __syncthreads();
        for (int q = threadIdx.x; q < nb; q += blockDim.x) hist[q] = 0;
        if (threadIdx.x == 0) s_n = 0;
        __syncthreads();
    }
}

// Work items of every long row, one warp per row: a bucket of more than
// kRadH pairs is an item of its own (split into pieces of about kRadPiece
// pairs by chunk range), runs of smaller buckets are grouped while their
// pair prefix stays in one kRadH window.  Split buckets get a zeroed global
// table.
template <typename WT>
__global__ void k_rad_items(AggArgs<WT> a, BigArgs b, int32_t *pool, long long vints)
{
    DevStats *st = a.st;
    const int cnt = big_off(st) ? 0 : st->small_cnt[kLongCls];
    const int nb = st->rad_nb;
    const int lane = threadIdx.x & 31;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    RadItem *items = (RadItem *)(pool + st->rad_items);
    int32_t *accs = pool + st->rad_acc;
    const long long max_items = st->rad_max_items, max_acc = st->rad_max_acc;
    const long long acc_ints = rad_acc_ints(vints);
    for (int i = wg; i < cnt; i += nw) {
        const int nch = (int)b.chunks[i];
        const int c = b.list[i];
        const long long r_sbase = a.medge[a.moff[c]], r_dst = a.tmp_off[c], r_w0 = b.coff[i], r_e = a.ec[c];
        const int32_t *trow = pool + (long long)i * nb;
        long long carry = 0;  // pairs of the buckets before the tile
        int prev_big = 0;
        long long prev_win = -1;
        int open_b = -1;  // first bucket of the item still open, and its prefix
        long long open_s = 0;
        for (int t0 = 0; t0 <= nb; t0 += 32) {  // bucket nb closes the last item
            const int bk = t0 + lane;
            const int m = bk < nb ? trow[bk] : 0;
            int incl = m;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(GALA_FULL_MASK, incl, o);
                if (lane >= o) incl += t;
            }
            const long long S = carry + incl - m;
            const int big = m > kRadH;
            const long long win = S / kRadH;
            int pb = __shfl_up_sync(GALA_FULL_MASK, big, 1);
            long long pwin = __shfl_up_sync(GALA_FULL_MASK, win, 1);
            if (lane == 0) {
                pb = prev_big;
                pwin = prev_win;
            }
            const bool start = bk <= nb && (bk == 0 || bk == nb || big || pb || win != pwin);
            const unsigned sm = __ballot_sync(GALA_FULL_MASK, start);
            // every start closes the item that began at the previous start
            const unsigned below = sm & lanemask_lt();
            const int pl = below ? 31 - __clz(below) : 0;
            const int sb = __shfl_sync(GALA_FULL_MASK, bk, pl);
            const long long sS = __shfl_sync(GALA_FULL_MASK, S, pl);
            const int ps = below ? sb : open_b;
            const long long pS = below ? sS : open_s;
            int np = 0;
            RadItem it{};
            if (start && ps >= 0) {
                const long long t = S - pS;
                if (t > 0) {
                    np = 1;
                    if (bk - ps == 1 && t > kRadH) {
                        const long long P = (t + kRadPiece - 1) / kRadPiece;
                        np = (int)(P < nch ? P : nch);
                    }
                    it.sbase = r_sbase;
                    it.dst = r_dst;
                    it.w0 = r_w0;
                    it.erow = r_e;
                    it.i = i;
                    it.b0 = ps;
                    it.b1 = bk;
                    it.acc = -1;
                    it.pieces = np;
                    it.total = (int)t;
                }
            }
            int ex = np;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(GALA_FULL_MASK, ex, o);
                if (lane >= o) ex += t;
            }
            const int wsum = __shfl_sync(GALA_FULL_MASK, ex, 31);
            ex -= np;
            long long base = 0;
            if (lane == 0 && wsum) base = atomicAdd(&st->rad_nitems, wsum);
            base = __shfl_sync(GALA_FULL_MASK, base, 0);
            int acc = -1;
            if (np) {
                if (base + ex + np > max_items) {
                    atomicOr(&st->err, kErrCapacity);
                } else {
                    if (np > 1) {
                        acc = atomicAdd(&st->rad_nacc, 1);
                        if (acc >= max_acc) {
                            atomicOr(&st->err, kErrCapacity);
                            acc = -1;
                        }
                    }
                    if (np == 1 || acc >= 0) {
                        it.acc = acc;
                        for (int p = 0; p < np; ++p) {
                            it.k0 = (int)((long long)p * nch / np);
                            it.k1 = (int)((long long)(p + 1) * nch / np);
                            items[base + ex + p] = it;
                        }
                    }
                }
            }
            unsigned am = __ballot_sync(GALA_FULL_MASK, acc >= 0);
            while (am) {  // zero the global tables this warp took
                const int l = __ffs(am) - 1;
                am &= am - 1;
                const long long ac = __shfl_sync(GALA_FULL_MASK, acc, l);
                int4 *z = (int4 *)(accs + ac * acc_ints);
                for (long long q = lane; q < acc_ints / 4; q += 32) z[q] = make_int4(0, 0, 0, 0);
            }
            carry += __shfl_sync(GALA_FULL_MASK, incl, 31);
            prev_big = __shfl_sync(GALA_FULL_MASK, big, 31);
            prev_win = __shfl_sync(GALA_FULL_MASK, win, 31);
            if (sm) {
                const int hl = 31 - __clz(sm);
                open_b = __shfl_sync(GALA_FULL_MASK, bk, hl);
                open_s = __shfl_sync(GALA_FULL_MASK, S, hl);
            }
        }
    }
}

// Hashed items hold under 2 kRadH pairs, so their slot lists need 2 kRadH
// entries; chunk ranges are scanned kRadBatch at a time.  With int weights
// three CTAs fit an SM.
constexpr int kRadOcc = 2 * kRadH;
constexpr int kRadBatch = 256;
template <typename WT>
constexpr size_t rad_agg_smem()
{
    return (size_t)kRadW * (sizeof(WT) + sizeof(int)) + kRadOcc * sizeof(unsigned short);
}

// One warp appends the present slots [wid * 512, wid * 512 + 512) of a
// dense bucket table (values v, bitmap nbits of non-positive sums) to row i
// with one cursor add: keys kbase + slot.  GLOBAL: the table is a split
// bucket's global one (read past L1); otherwise the values are zeroed.
template <typename WT, bool GLOBAL>
__device__ __forceinline__ void rad_emit_warp(const AggArgs<WT> &a, int32_t *cursor, int i, long long dst,
                                              int kbase, WT *v, const unsigned *nbits)
{
    const int lane = threadIdx.x & 31;
    const int s0 = (threadIdx.x >> 5) * 512;
    auto present = [&](int s) -> unsigned {
        const WT x = GLOBAL ? __ldcg(&v[s]) : v[s];
        const unsigned wb = GLOBAL ? __ldcg(&nbits[s >> 5]) : nbits[s >> 5];
        return __ballot_sync(GALA_FULL_MASK, x != 0 || ((wb >> lane) & 1u));
    };
    int cnt = 0;
#pragma unroll 4
    for (int r = 0; r < 16; ++r) cnt += __popc(present(s0 + r * 32 + lane));
    long long base = 0;
    if (lane == 0 && cnt) base = atomicAdd(&cursor[i], cnt);
    long long d = dst + __shfl_sync(GALA_FULL_MASK, base, 0);
    const unsigned lt = lanemask_lt();
#pragma unroll 4
    for (int r = 0; r < 16; ++r) {
        const int s = s0 + r * 32 + lane;
        const unsigned m = present(s);
        if ((m >> lane) & 1u) {
            const long long p = d + __popc(m & lt);
            a.tmp_nbr[p] = kbase + s;
            a.tmp_w[p] = GLOBAL ? __ldcg(&v[s]) : v[s];
        }
        d += __popc(m);
        if (!GLOBAL) v[s] = 0;
    }
}

// The items, taken from a queue by persistent CTAs of 512 threads (the next
// index is fetched while an item runs).  An item's pairs are spread over all
// threads: the chunks' pair ranges (kRadBatch chunks at a time) are scanned
// into a prefix in shared memory, and every thread walks it forward to find
// the chunk of its next pair.  Every warp emits its share of the distinct
// keys with its own cursor add.
template <typename WT>
__global__ void __launch_bounds__(512) k_rad_agg(AggArgs<WT> a, BigArgs b, int32_t *pool, const int32_t *pk,
                                                 const WT *pw, long long vints)
{
    DevStats *st = a.st;
    if (big_off(st)) return;
    long long nitems = st->rad_nitems;
    if (nitems > st->rad_max_items) nitems = st->rad_max_items;
    const int nb1 = st->rad_nb + 1;
    const RadItem *items = (const RadItem *)(pool + st->rad_items);
    const unsigned short *offm = (const unsigned short *)(pool + st->rad_offm);
    int32_t *accs = pool + st->rad_acc;
    const long long acc_ints = rad_acc_ints(vints);
    extern __shared__ long long asm_ll[];
    WT *vals = (WT *)asm_ll;
    int *keys = (int *)(vals + kRadW);
    unsigned *bits = (unsigned *)keys;  // dense items: the first kRadW / 32 key slots
    unsigned short *occ = (unsigned short *)(keys + kRadW);
    __shared__ int s_it, s_n, s_last;
    __shared__ int ws[33];
    __shared__ int cps[kRadBatch + 1];  // prefix of the pair ranges of a batch of chunks
    __shared__ int clo[kRadBatch];      // first pair of each chunk of the batch
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int q = threadIdx.x; q < kRadW; q += blockDim.x) {
        keys[q] = -1;
        vals[q] = 0;
    }
    int nxt = 0;
    if (threadIdx.x == 0) s_it = atomicAdd(&st->rad_next, 1);
    for (;;) {
        __syncthreads();
        const int itn = s_it;
        if (itn >= nitems) break;
        if (threadIdx.x == 0) {
            nxt = atomicAdd(&st->rad_next, 1);
            s_n = 0;
        }
        const RadItem it = items[itn];
        const bool dense = it.b1 - it.b0 == 1 && it.total > kRadH;
        const int kbase = it.b0 << kRadLg;
        int T = kRadW, lg = kRadLg;
        if (dense) {
            for (int q = threadIdx.x; q < kRadW / 32; q += blockDim.x) bits[q] = 0;
        } else {
            T = next_pow2_int(2LL * it.total);
            if (T < 64) T = 64;
            if (T > kRadW) T = kRadW;
            lg = __ffs(T) - 1;
        }
        // (the barriers of the scan below order the resets before the inserts)
        for (int kb = it.k0; kb < it.k1; kb += kRadBatch) {
            const int kn = it.k1 - kb < kRadBatch ? it.k1 - kb : kRadBatch;
            int lo = 0, len = 0;
            if (threadIdx.x < kn) {
                const long long k = kb + threadIdx.x;
                const unsigned short *orow = offm + (it.w0 + k) * nb1;
                const long long rem = it.erow - k * kChunk;  // entries of the chunk
                lo = orow[it.b0];
                long long hi = orow[it.b1];
                if (hi > rem) hi = rem;
                len = hi > lo ? (int)hi - lo : 0;
            }
            int tot;
            const int ex = block_excl_scan(len, ws, tot);
            if (threadIdx.x < kn) {
                cps[threadIdx.x] = ex;
                clo[threadIdx.x] = lo;
            }
            if (threadIdx.x == 0) cps[kn] = tot;
            __syncthreads();
            constexpr int U = 4;
            int ch = 0;
            for (int q0 = 0; q0 < tot; q0 += 512 * U) {
                int key[U];
                WT v[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int q = q0 + u * 512 + threadIdx.x;
                    key[u] = 0;
                    v[u] = 0;
                    if (q < tot) {
                        while (cps[ch + 1] <= q) ++ch;
                        const long long pos = it.sbase + (long long)(kb + ch) * kChunk + clo[ch] + (q - cps[ch]);
                        key[u] = pk[pos];
                        v[u] = pw[pos];
                    }
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    if (q0 + u * 512 + threadIdx.x >= tot) break;
                    if (dense) {
                        const unsigned s = (unsigned)(key[u] - kbase);
                        if (s < (unsigned)kRadW) {
                            atomic_add_w(&vals[s], v[u]);
                            if (v[u] <= 0) atomicOr(&bits[s >> 5], 1u << (s & 31));
                        } else {
                            atomicOr(&st->err, kErrBadIndex);
                        }
                    } else {
                        int slot;
                        const int r = table_add(keys, vals, T, lg, key[u], v[u], slot);
                        if (r < 0) atomicOr(&st->err, kErrHashOverflow);
                        else if (r == 1) {
                            const int o = atomicAdd(&s_n, 1);
                            if (o < kRadOcc) occ[o] = (unsigned short)slot;
                            else atomicOr(&st->err, kErrHashOverflow);
                        }
                    }
                }
            }
            __syncthreads();  // the inserts are done; cps / clo are free
        }
        if (!dense) {
            const int n = s_n < kRadOcc ? s_n : kRadOcc;
            const int per = ((n + 15) / 16 + 31) & ~31;  // list entries per warp
            const int wlo = wid * per;
            const int whi = wlo + per < n ? wlo + per : n;
            if (wlo < whi) {
                long long base = 0;
                if (lane == 0) base = atomicAdd(&b.cursor[it.i], whi - wlo);
                const long long d = it.dst + __shfl_sync(GALA_FULL_MASK, base, 0) - wlo;
                for (int q = wlo + lane; q < whi; q += 32) {
                    const int h = occ[q];
                    a.tmp_nbr[d + q] = keys[h];
                    a.tmp_w[d + q] = vals[h];
                    keys[h] = -1;
                    vals[h] = 0;
                }
            }
        } else if (it.pieces == 1) {
            rad_emit_warp<WT, false>(a, b.cursor, it.i, it.dst, kbase, vals, bits);
        } else {
            // add this piece to the bucket's global table; the last piece emits it
            WT *gv = (WT *)(accs + it.acc * acc_ints);
            unsigned *gb = (unsigned *)(gv + kRadW);
            int *gcnt = (int *)(gb + kRadW / 32);
            for (int s = threadIdx.x; s < kRadW; s += blockDim.x) {
                const WT x = vals[s];
                if (x != 0) atomic_add_w(&gv[s], x);
                vals[s] = 0;
            }
            for (int q = threadIdx.x; q < kRadW / 32; q += blockDim.x)
                if (bits[q]) atomicOr(&gb[q], bits[q]);
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0) s_last = atomicAdd(gcnt, 1) == it.pieces - 1;
            __syncthreads();
            if (s_last) {
                __threadfence();
                rad_emit_warp<WT, true>(a, b.cursor, it.i, it.dst, kbase, gv, gb);
            }
        }
        if (dense && lane < 16) keys[wid * 16 + lane] = -1;  // the bitmap words of this warp's slots
        if (threadIdx.x == 0) s_it = nxt;
    }
}

// Table chunks: distinct entries of sorted rows go to the row unsorted
// (atomic cursor); rows ranked by bitmap set their bits.
template <typename WT>
__global__ void __launch_bounds__(256) k_big_collect(AggArgs<WT> a, BigArgs b, long long ntwork)
{
    for (long long wi = blockIdx.x; wi < ntwork; wi += gridDim.x) {
        const int i = b.twork[wi];
        const long long j0 = (wi - b.tcoff[i]) * kChunk;
        const long long T = b.T[i];
        const int c = b.list[i];
        const WT *vals = big_vals<WT>(b, i);
        const int *keys = b.pool + b.toff[i];
        const bool dense = b.mode[i];
        const bool bitmap = b.gwords[i] > 0;
        const long long o = a.tmp_off[c];
        unsigned *bits = bitmap ? b.bits + b.gofs[i] : nullptr;
        for (long long s0 = j0; s0 < j0 + kChunk && s0 < T; s0 += blockDim.x) {
            const long long s = s0 + threadIdx.x;
            int key = -1;
            WT val = 0;
            if (s < T && s < j0 + kChunk) {
                val = vals[s];
                key = dense ? (val > 0 ? (int)s : -1) : keys[s];
            }
            const bool occ = key >= 0;
            if (bitmap) {
                if (occ) atomicOr(&bits[key >> 5], 1u << (key & 31));
            } else {
                const unsigned bal = __ballot_sync(GALA_FULL_MASK, occ);
                if (bal) {
                    const int lane = threadIdx.x & 31, leader = __ffs(bal) - 1;
                    int base = 0;
                    if (lane == leader) base = atomicAdd(&b.cursor[i], __popc(bal));
                    base = __shfl_sync(GALA_FULL_MASK, base, leader);
                    if (occ) {
                        const long long p = o + base + __popc(bal & lanemask_lt());
                        a.tmp_nbr[p] = key;
                        a.tmp_w[p] = val;
                    }
                }
            }
        }
    }
}

// Table chunks of bitmap-ranked rows: rank = popcounts of the row's bitmap
// before the key.
template <typename WT>
__global__ void __launch_bounds__(256) k_big_rank(AggArgs<WT> a, BigArgs b, long long ntwork)
{
    for (long long wi = blockIdx.x; wi < ntwork; wi += gridDim.x) {
        const int i = b.twork[wi];
        if (b.gwords[i] == 0) continue;
        const long long j0 = (wi - b.tcoff[i]) * kChunk;
        const long long T = b.T[i];
        const int c = b.list[i];
        const WT *vals = big_vals<WT>(b, i);
        const int *keys = b.pool + b.toff[i];
        const bool dense = b.mode[i];
        const long long o = a.tmp_off[c];
        const unsigned *bits = b.bits + b.gofs[i];
        const unsigned *pref = b.pref + b.gofs[i];
        const unsigned base = pref[0];
        for (long long s = j0 + threadIdx.x; s < j0 + kChunk && s < T; s += blockDim.x) {
            const WT val = vals[s];
            const int key = dense ? (val > 0 ? (int)s : -1) : keys[s];
            if (key < 0) continue;
            const unsigned r = pref[key >> 5] - base + __popc(bits[key >> 5] & ((1u << (key & 31)) - 1u));
            a.tmp_nbr[o + r] = key;
            a.tmp_w[o + r] = val;
        }
    }
}

// Rows with at most kSortMax distinct neighbours: one CTA sorts the row in
// shared memory.
template <typename WT>
__global__ void __launch_bounds__(1024) k_big_sort(AggArgs<WT> a, BigArgs b)
{
    extern __shared__ long long sm_ll[];
    int *lk = (int *)sm_ll;
    WT *lv = (WT *)(lk + kSortMax);
    const int cnt = a.st->small_cnt[kLongCls];
    for (int i = blockIdx.x; i < cnt; i += gridDim.x) {
        if (b.gwords[i] != 0) continue;
        const int c = b.list[i];
        const int k = b.kdist[i];
        const long long o = a.tmp_off[c];
        const int P = next_pow2_int(k);
        for (int j = threadIdx.x; j < P; j += blockDim.x) {
            lk[j] = j < k ? a.tmp_nbr[o + j] : 0x7fffffff;
            lv[j] = j < k ? a.tmp_w[o + j] : 0;
        }
        __syncthreads();
        bitonic_sort_smem(lk, lv, P);
        for (int j = threadIdx.x; j < k; j += blockDim.x) {
            a.tmp_nbr[o + j] = lk[j];
            a.tmp_w[o + j] = lv[j];
        }
        __syncthreads();
    }
}

// Compaction over contiguous output ranges: output entry j of community c
// comes from tmp_off[c] + (j - new_offs[c]); c and that shift are loaded once
// per row window.  C and the entry count are read on the device.
template <typename WT>
__global__ void __launch_bounds__(256) k_compact(const int64_t *__restrict__ new_offs,
                                                 const long long *__restrict__ tmp_off,
                                                 const int32_t *__restrict__ tmp_nbr, const WT *__restrict__ tmp_w,
                                                 int32_t *out_nbr, WT *out_w, long long tmp_cap,
                                                 const int32_t *__restrict__ nz_rows,
                                                 const long long *__restrict__ nz_offs,
                                                 const long long *__restrict__ nz_shift,
                                                 const int32_t *__restrict__ task_row, DevStats *st,
                                                 WT *self_out)
{
    const long long wg = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const int nnz = st->nz_rows;
    const int C = (int)st->ccount;
    const long long Enew = st->new_entries;
    // per row: pa = the community (-1 when out of range), pb = source shift
    auto rowval = [=](int r, long long &pa, long long &pb) {
        const int c = nz_rows[r];
        if (c < 0 || c >= C) return;
        pa = c;
        pb = nz_shift[r];
    };
    constexpr int U = kWalkUnroll;
    const int lane = threadIdx.x & 31;
    auto cur = row_cursor(nz_offs, nnz, rowval);
    for (long long t = wg; t * kRangeEntries < Enew; t += nw) {
        const long long j0 = t * kRangeEntries;
        const long long j1 = j0 + kRangeEntries < Enew ? j0 + kRangeEntries : Enew;
        cur.start_row(task_row[t]);
        for (long long jb = j0; jb < j1; jb += 32 * U) {
            long long src[U], com[U];
            bool ok[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const long long b0 = jb + 32 * u;
                ok[u] = false;
                src[u] = 0;
                com[u] = -1;
                if (b0 < j1) {  // warp-uniform
                    const long long j = b0 + lane;
                    long long c, d;
                    const bool in = cur.resolve(b0, b0 + 31 < j1 ? b0 + 31 : j1 - 1, j, c, d);
                    if (j < j1) {
                        const long long from = j + d;
                        if (!in || c < 0 || from < 0 || from >= tmp_cap)  // recorded, never read or written
                            atomicOr(&st->err, kErrBadIndex);
                        else {
                            ok[u] = true;
                            src[u] = from;
                            com[u] = c;
                        }
                    }
                }
            }
            int32_t nb[U];
            WT wt[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                nb[u] = ok[u] ? tmp_nbr[src[u]] : 0;
                wt[u] = ok[u] ? tmp_w[src[u]] : (WT)0;
            }
#pragma unroll
            for (int u = 0; u < U; ++u)
                if (ok[u]) {
                    const long long j = jb + 32 * u + lane;
                    out_nbr[j] = nb[u];
                    out_w[j] = wt[u];
                    if (self_out && nb[u] == com[u]) self_out[com[u]] = wt[u];
                }
        }
    }
}

__global__ void k_contract_set_tail(int32_t *moff, const DevStats *st, int n, long long *medge, long long E)
{
    moff[st->ccount] = n;
    medge[n] = E;
}

__global__ void k_set_last_offset(int64_t *offs, const DevStats *st) { offs[st->ccount] = st->new_entries; }

__global__ void k_contract_reset(DevStats *st)
{
    for (int k = 0; k < kNumCls; ++k) st->small_cnt[k] = 0;
    st->err = 0;
    st->ccount = 0;
    st->new_entries = 0;
    st->big_slots = st->big_nwork = st->big_ntwork = st->big_lwork = 0;
    st->rad_nb = st->rad_nitems = st->rad_nacc = st->rad_next = 0;
}

// Shared memory of the table kernels: int keys plus WT values per slot.
template <typename WT>
constexpr size_t mid1_smem()
{
    return (1024 + kMid1Max) * (sizeof(int) + sizeof(WT));
}
template <typename WT>
constexpr size_t mid2_smem()
{
    return (8192 + kMid2Max) * (sizeof(int) + sizeof(WT));
}
template <typename WT>
constexpr size_t sort_smem()
{
    return kSortMax * (sizeof(int) + sizeof(WT));
}

template <typename WT>
static void configure_mid()
{
    cudaFuncSetAttribute(k_agg_mid<WT, 128, 1024, kMid1Max>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)mid1_smem<WT>());
    cudaFuncSetAttribute(k_agg_mid<WT, 256, 8192, kMid2Max>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)mid2_smem<WT>());
}

template <typename WT>
constexpr size_t list_smem(int tmax)
{
    return (size_t)tmax * (sizeof(WT) + sizeof(int) + sizeof(unsigned short));
}

template <typename WT>
static void configure_t()
{
    configure_mid<WT>();

    cudaFuncSetAttribute(k_big_sort<WT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sort_smem<WT>());
    cudaFuncSetAttribute(k_big_insert_sm<WT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)big_sm_smem<WT>());
    cudaFuncSetAttribute(k_rad_combine<WT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rad_combine_smem<WT>());
    cudaFuncSetAttribute(k_rad_agg<WT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)rad_agg_smem<WT>());
    cudaFuncSetAttribute(k_agg_mid_list<WT, 1024, 8192>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)list_smem<WT>(8192));
    cudaFuncSetAttribute(k_agg_mid_list<WT, 1024, 16384>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)list_smem<WT>(16384));
}

void contract_configure_kernels()
{
    configure_t<int>();
    configure_t<long long>();
}

static int grid_cap(long long items, int per_block, int cap)
{
    long long g = (items + per_block - 1) / per_block;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

// Blocks of a grid-stride kernel that are resident at once (threads per
// block, dynamic shared memory): a larger grid runs a second, partial wave.
template <typename K>
static int resident_grid(K kernel, int threads, size_t smem = 0)
{
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem) != cudaSuccess || per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
    }
    return per_sm * sm_count();
}

// Walk list of the rows of (offs, n) that have entries (E entries in total).
// With dn / dE (device) the rows are [0, min(n, *dn)) and the entries *dE:
// nothing waits for the host.
template <typename Shift>
static void build_walk_list(const int64_t *offs, int n, long long E, ContractBuffers &b, cudaStream_t st, Shift shift,
                            const long long *dn = nullptr, const long long *dE = nullptr)
{
    const int cap = sm_count() * 8;
    if (dn)
        exclusive_scan_dev(offs, b.nz_pos, n, dn, OpRowNonEmpty{offs}, b.scan_partial, &b.stats->total, st,
                           &b.stats->err);
    else
        exclusive_scan(offs, b.nz_pos, n, OpRowNonEmpty{offs}, b.scan_partial, &b.stats->total, st, &b.stats->err);
    k_nz_tail<<<1, 1, 0, st>>>(b.stats, b.nz_offs, E, dE);
    k_nz_scatter<Shift><<<grid_cap(n, 256, cap), 256, 0, st>>>(offs, n, b.nz_pos, b.nz_rows, b.nz_offs, b.nz_shift,
                                                               b.task_row, dn, shift);
    note_launch(2);
}

static bool read_stats(DevStats *h, DevStats *d, cudaStream_t st, gala_status *status, const char *what)
{
    cudaError_t ce;
    if ((ce = cudaGetLastError()) != cudaSuccess ||  // a failed launch
        (ce = cudaMemcpyAsync(h, d, sizeof(DevStats), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (ce = cudaStreamSynchronize(st)) != cudaSuccess) {
        *status = cuda_fail(ce, what);
        return false;
    }
    return true;
}

// Keys of the long-row tables take pool[0, half), their values (WT) the rest.
template <typename WT>
static long long big_pool_half(const ContractBuffers &b)
{
    constexpr long long vints = sizeof(WT) / sizeof(int32_t);
    return (b.big_pool_ints / (1 + vints)) & ~1LL;  // even: the values start 8-byte aligned
}

// Rows longer than kMid3Max entries (kMid2Max when sorted; class kLongCls),
// at most cnt_max of them.  Counts, table sizes and the scratch check stay on
// the device; only sorted rows read their bitmap sizes on the host.  Returns
// false on failure.
// Whether the key-range path fits the pool for any level of n rows and E
// entries (C <= n, every long row longer than kMid3Max entries).
template <typename WT>
static bool rad_fits(long long n, long long E, const ContractBuffers &b)
{
    constexpr long long vints = sizeof(WT) / sizeof(int32_t);
    if (E >= (1LL << 31)) return false;  // pair counts are 32-bit
    const long long nb = (n + kRadW - 1) / kRadW;
    if (nb > kRadNbMax) return false;
    const long long cnt = std::min(n, E / (kMid3Max + 1));
    return rad_layout(cnt, E / kChunk + cnt, nb, vints).end <= b.big_pool_ints;
}

template <typename WT>
static bool contract_long_rows(const AggArgs<WT> &a, ContractBuffers &b, const int32_t *list, int cnt_max,
                               cudaStream_t st, gala_status *status, bool sort_rows, long long n, long long E)
{
    const int nsm = sm_count();
    const int cap = nsm * 8;
    DevStats *ds = b.stats;
    const int *dcnt = &ds->small_cnt[kLongCls];
    BigArgs ba{};
    ba.list = list;
    ba.T = b.big_T;
    ba.chunks = b.big_chunks;
    ba.tchunks = b.big_tchunks;
    ba.toff = b.big_toff;
    ba.coff = b.big_coff;
    ba.tcoff = b.big_tcoff;
    ba.mode = b.big_mode;
    ba.work = b.big_work;
    ba.twork = b.big_twork;
    ba.kdist = b.big_kdist;
    ba.cursor = b.big_cursor;
    ba.gwords = b.big_gwords;
    ba.gofs = b.big_gofs;
    ba.pool = b.big_pool;
    ba.pool_half = big_pool_half<WT>(b);
    ba.work_cap = b.big_work_cap;
    ba.twork_cap = b.big_twork_cap;
    if (!sort_rows && b.long_rows_mode == 0 && rad_fits<WT>(n, E, b)) {
        constexpr long long vints = sizeof(WT) / sizeof(int32_t);
        k_rad_plan<WT><<<grid_cap(cnt_max, 256, cap), 256, 0, st>>>(a, ba, b.big_pool, b.big_pool_ints);
        exclusive_scan_dev(b.big_chunks, b.big_coff, cnt_max, dcnt, OpIdentity(), b.scan_partial, &ds->big_nwork, st,
                           &ds->err);
        k_rad_tail<<<1, 1, 0, st>>>(ba, ds, vints, b.big_pool_ints);
        k_rad_combine<WT><<<resident_grid(k_rad_combine<WT>, kRadCombineThreads, rad_combine_smem<WT>()),
                            kRadCombineThreads,
                            rad_combine_smem<WT>(), st>>>(a, ba, b.big_pool, b.stream_key, (WT *)b.stream_w);
        k_rad_items<WT><<<grid_cap((long long)cnt_max * 32, 256, cap), 256, 0, st>>>(a, ba, b.big_pool, vints);
        k_rad_agg<WT><<<resident_grid(k_rad_agg<WT>, 512, rad_agg_smem<WT>()), 512, rad_agg_smem<WT>(), st>>>(
            a, ba, b.big_pool, b.stream_key, (const WT *)b.stream_w, vints);
        k_big_len<WT><<<grid_cap(cnt_max, 256, cap), 256, 0, st>>>(a, ba);
        note_launch(6);
        return true;
    }
    k_big_plan<WT><<<grid_cap(cnt_max, 256, cap), 256, 0, st>>>(a, ba);
    exclusive_scan_dev(b.big_T, b.big_toff, cnt_max, dcnt, OpIdentity(), b.scan_partial, &ds->big_slots, st,
                       &ds->err);
    exclusive_scan_dev(b.big_chunks, b.big_coff, cnt_max, dcnt, OpIdentity(), b.scan_partial, &ds->big_nwork, st,
                       &ds->err);
    exclusive_scan_dev(b.big_tchunks, b.big_tcoff, cnt_max, dcnt, OpIdentity(), b.scan_partial, &ds->big_ntwork,
                       st, &ds->err);
    k_big_tail<<<1, 1, 0, st>>>(ba, ds);
    k_big_clear<WT><<<cap, 256, 0, st>>>(ba, ds);
    k_big_work<WT><<<grid_cap((long long)cnt_max * 32, 256, cap), 256, 0, st>>>(a, ba);
    k_big_insert_sm<WT><<<nsm * 2, 512, big_sm_smem<WT>(), st>>>(a, ba, sort_rows ? 0 : 1);
    note_launch(5);
    if (!sort_rows) {
        // rows in table order: collect from the slot lists, no table scans
        long long *lch = b.big_tchunks, *lcoff = b.big_tcoff;
        k_big_lchunks<<<grid_cap(cnt_max, 256, cap), 256, 0, st>>>(ba.cursor, ds, lch);
        exclusive_scan_dev(lch, lcoff, cnt_max, dcnt, OpIdentity(), b.scan_partial, &ds->big_lwork, st, &ds->err);
        k_big_collect_list<WT><<<nsm * 8, 256, 0, st>>>(a, ba, lcoff, &ds->big_lwork);
        k_big_len<WT><<<grid_cap(cnt_max, 256, cap), 256, 0, st>>>(a, ba);
        note_launch(3);
        return true;
    }
    // sorted rows: the bitmap sizes come back to the host
    DevStats hs;
    if (!read_stats(&hs, ds, st, status, "contraction: long rows")) return false;
    const int cnt3 = hs.small_cnt[kLongCls];
    if (cnt3 == 0 || (hs.err & kErrCapacity)) return true;  // a capacity error is reported at the end
    const long long ntwork = hs.big_ntwork;
    k_big_mark<WT><<<grid_cap(cnt3, 256, cap), 256, 0, st>>>(a, ba, 1);
    exclusive_scan(b.big_gwords, b.big_gofs, cnt3, OpIdentity(), b.scan_partial, &ds->total, st, &ds->err);
    note_launch(1);
    if (!read_stats(&hs, ds, st, status, "contraction: long-row bitmaps")) return false;
    const long long words = hs.total;
    if (2 * words > b.big_bitmap_words) {
        set_error("contraction: %lld bitmap words needed, scratch holds %lld", 2 * words, b.big_bitmap_words);
        *status = GALA_ERR_CAPACITY;
        return false;
    }
    ba.bits = (unsigned *)b.big_bitmap;
    ba.pref = (unsigned *)b.big_bitmap + words;
    if (words > 0) cudaMemsetAsync(ba.bits, 0, (size_t)words * sizeof(unsigned), st);
    const int tgrid = (int)(ntwork < nsm * 8 ? ntwork : nsm * 8);
    if (tgrid > 0) {
        k_big_collect<WT><<<tgrid, 256, 0, st>>>(a, ba, ntwork);
        note_launch(1);
    }
    if (words > 0 && tgrid > 0) {
        exclusive_scan(ba.bits, ba.pref, words, OpPopc(), b.scan_partial, &ds->total, st, &ds->err);
        k_big_rank<WT><<<tgrid, 256, 0, st>>>(a, ba, ntwork);
        note_launch(1);
    }
    k_big_sort<WT><<<cnt3 < nsm * 2 ? cnt3 : nsm * 2, 1024, sort_smem<WT>(), st>>>(a, ba);
    note_launch(1);
    return true;
}

// Returns the community count C (>= 1) or -1 on failure (*status set).
// new_offs receives C+1 offsets (leading 0).  orig_map (length n_orig) is
// composed with the new labels.  C, the size classes and the new entry count
// stay on the device: the host reads them once, after the compaction (and,
// for sorted long rows, once more for their bitmap sizes).
template <typename WT>
static int contract_t(const LevelGraph &g, const int32_t *comm, ContractBuffers &b, int64_t *new_offs,
                      int32_t *new_nbr, WT *new_w, int32_t *orig_map, int32_t n_orig, int64_t *new_E,
                      cudaStream_t st, gala_status *status, bool validate_labels, bool sort_rows,
                      const NextLevelInit &nli, bool labels_only)
{
    const int n = g.n;
    const long long E = g.E;
    const int nsm = sm_count();
    const int cap = nsm * 8;
    *status = GALA_OK;
    DevStats hs;
    DevStats *ds = b.stats;
    const long long *dC = &ds->ccount;

    k_contract_reset<<<1, 1, 0, st>>>(ds);
    note_launch(1);
    if (validate_labels) {
        k_check_labels<<<grid_cap(n, 256, cap), 256, 0, st>>>(comm, n, ds);
        note_launch(1);
        if (!read_stats(&hs, ds, st, status, "contraction: label check")) return -1;
        if (hs.err) {
            set_error("contraction: a community label lies outside [0, %d)", n);
            *status = GALA_ERR_INVALID;
            return -1;
        }
    }
    cudaMemsetAsync(b.cnt, 0, ((size_t)n + 1) * sizeof(int32_t), st);
    k_hist<<<grid_cap(n, 256, cap), 256, 0, st>>>(comm, n, b.cnt);
    exclusive_scan(b.cnt, b.newid, n, OpPositive(), b.scan_partial, &ds->ccount, st, &ds->err);
    k_relabel<WT><<<grid_cap(n, 256, cap), 256, 0, st>>>(comm, b.newid, b.cnt, n, b.lab, b.csz, b.ec,
                                                         (const WT *)nli.tot, (WT *)nli.k, (WT *)nli.self);
    note_launch(2);
    if (orig_map) {
        k_compose<<<grid_cap(n_orig, 256, cap), 256, 0, st>>>(orig_map, n_orig, b.lab);
        note_launch(1);
    }
    if (labels_only) {
        if (!read_stats(&hs, ds, st, status, "contraction: community count")) return -1;
        *new_E = 0;
        return (int)hs.ccount;
    }
    exclusive_scan_dev(b.csz, b.moff, n, dC, OpIdentity(), b.scan_partial, &ds->total, st, &ds->err);
    k_member_scatter<<<grid_cap(n, 256, cap), 256, 0, st>>>(b.lab, g.offs, n, b.moff, b.csz, b.members, b.mpos,
                                                            b.ec);
    exclusive_scan(b.members, b.medge, n, OpDegOf{g.offs}, b.scan_partial, &ds->total, st, &ds->err);
    // moff[C] = n and medge[n] = E close the last segments
    k_contract_set_tail<<<1, 1, 0, st>>>(b.moff, ds, n, b.medge, E);
    note_launch(2);
    const bool weighted = g.w != nullptr;
    if (E > 0) {
        build_walk_list(g.offs, n, E, b, st, ShiftStream{b.mpos, b.medge});
        const int tasks = grid_cap((E + kRangeEntries - 1) / kRangeEntries * 32, 256, cap);
        if (weighted) {
            const int grid = std::min(tasks, resident_grid(k_stream_fill<WT, true>, 256));
            k_stream_fill<WT, true><<<grid, 256, 0, st>>>(E, g.nbr, (const WT *)g.w, b.lab, b.stream_key,
                                                          (WT *)b.stream_w, b.nz_offs, b.nz_shift, b.task_row, ds);
        } else {
            const int grid = std::min(tasks, resident_grid(k_stream_fill<WT, false>, 256));
            k_stream_fill<WT, false><<<grid, 256, 0, st>>>(E, g.nbr, nullptr, b.lab, b.stream_key, nullptr, b.nz_offs,
                                                           b.nz_shift, b.task_row, ds);
        }
        note_launch(1);
    }
    k_classify<<<grid_cap(n, 256, cap), 256, 0, st>>>(b.ec, b.cls_list, n, b.kc, ds, sort_rows ? 1 : 0);
    exclusive_scan_dev(b.ec, b.tmp_off, n, dC, OpCapDev{dC}, b.scan_partial, &ds->total, st, &ds->err);
    note_launch(1);

    AggArgs<WT> a;
    a.moff = b.moff;
    a.medge = b.medge;
    a.ec = b.ec;
    a.skey = b.stream_key;
    a.sw = weighted ? (const WT *)b.stream_w : nullptr;
    a.tmp_off = b.tmp_off;
    a.tmp_nbr = b.tmp_nbr;
    a.tmp_w = (WT *)b.tmp_w;
    a.kc = b.kc;
    a.st = ds;
    // Every class kernel reads its count on the device; its grid is bounded
    // by the most communities the class can hold (E / its shortest row).
    auto most = [&](long long min_entries) -> int {
        const long long c = E / min_entries;
        return (int)(c < n ? c : n);
    };
    const int n_small = most(1), n_warp = sort_rows ? 0 : most(kSmallMax + 1);
    const int n_mid1 = most(sort_rows ? kSmallMax + 1 : kWarpAggMax + 1), n_mid2 = most(kMid1Max + 1);
    const int n_mid3 = sort_rows ? 0 : most(kMid2Max + 1), n_long = most((sort_rows ? kMid2Max : kMid3Max) + 1);
    // The classes are independent (disjoint tmp ranges and kc entries): with
    // auxiliary streams they aggregate concurrently, the long rows (the
    // longest chain of launches) first.
    cudaStream_t cs[ContractBuffers::kAux];
    const bool par = b.aux[0] != nullptr && b.fork_ev != nullptr;
    if (par) cudaEventRecord(b.fork_ev, st);
    for (int i = 0; i < ContractBuffers::kAux; ++i) {
        cs[i] = par ? b.aux[i] : st;
        if (par) cudaStreamWaitEvent(cs[i], b.fork_ev, 0);
    }
    bool ok = n_long == 0 ||
              contract_long_rows(a, b, b.cls_list + (long long)kLongCls * n, n_long, cs[3], status, sort_rows, n, E);
    if (ok && n_mid2 > 0) {
        const int grid = n_mid2 < nsm * 2 ? n_mid2 : nsm * 2;
        if (sort_rows)
            k_agg_mid<WT, 256, 8192, kMid2Max><<<grid, 256, mid2_smem<WT>(), cs[2]>>>(a, b.cls_list + 2LL * n, 2);
        else
            k_agg_mid_list<WT, 1024, 8192><<<grid, 1024, list_smem<WT>(8192), cs[2]>>>(a, b.cls_list + 2LL * n, 2);
        note_launch(1);
    }
    if (ok && n_mid3 > 0) {  // 4097-8192 entries, rows in table order
        const int grid = n_mid3 < nsm ? n_mid3 : nsm;
        k_agg_mid_list<WT, 1024, 16384><<<grid, 1024, list_smem<WT>(16384), cs[2]>>>(a, b.cls_list + 3LL * n, 3);
        note_launch(1);
    }
    if (ok && n_mid1 > 0) {
        const int grid = n_mid1 < nsm * 16 ? n_mid1 : nsm * 16;
        if (sort_rows)
            k_agg_mid<WT, 128, 1024, kMid1Max><<<grid, 128, mid1_smem<WT>(), cs[1]>>>(a, b.cls_list + (long long)n, 1);
        else
            k_agg_mid_list<WT, 128, 1024><<<grid, 128, list_smem<WT>(1024), cs[1]>>>(a, b.cls_list + (long long)n,
                                                                                      1);
        note_launch(1);
    }
    if (ok && n_small > 0) {
        k_agg_small<WT><<<grid_cap((long long)n_small * 32, 256, cap), 256, 0, cs[0]>>>(a, b.cls_list);
        note_launch(1);
    }
    if (ok && n_warp > 0) {
        k_agg_warp_list<WT><<<grid_cap((long long)n_warp * 32, 256, cap), 256, 0, cs[0]>>>(
            a, b.cls_list + (long long)kWarpCls * n);
        note_launch(1);
    }
    if (par)
        for (int i = 0; i < ContractBuffers::kAux; ++i) {
            cudaEventRecord(b.join_ev[i], cs[i]);
            cudaStreamWaitEvent(st, b.join_ev[i], 0);
        }
    if (!ok) return -1;
    exclusive_scan_dev(b.kc, new_offs, n, dC, OpIdentity(), b.scan_partial, &ds->new_entries, st, &ds->err);
    k_set_last_offset<<<1, 1, 0, st>>>(new_offs, ds);
    note_launch(1);
    if (E > 0) {  // the new level has at most E entries
        build_walk_list(new_offs, n, 0, b, st, ShiftCompact{b.tmp_off}, dC, &ds->new_entries);
        // a second wave of blocks measured faster here than a resident grid
        k_compact<WT><<<grid_cap((E + kRangeEntries - 1) / kRangeEntries * 32, 256, cap), 256, 0, st>>>(
            new_offs, b.tmp_off, b.tmp_nbr, (const WT *)b.tmp_w, new_nbr, new_w, E, b.nz_rows, b.nz_offs, b.nz_shift,
            b.task_row, ds, (WT *)nli.self);
        note_launch(1);
    }
    if (!read_stats(&hs, ds, st, status, "contraction")) return -1;
    if (hs.err & kErrCapacity) {
        set_error("contraction: long rows need %lld table slots / %lld + %lld chunks, scratch holds %lld / %lld / "
                  "%lld",
                  hs.big_slots, hs.big_nwork, hs.big_ntwork, big_pool_half<WT>(b), b.big_work_cap, b.big_twork_cap);
        *status = GALA_ERR_CAPACITY;
        return -1;
    }
    if (hs.err) {
        set_error("contraction: hash table overflow (error bits %d)", hs.err);
        *status = GALA_ERR_OVERFLOW;
        return -1;
    }
    *new_E = hs.new_entries;
    return (int)hs.ccount;
}

int contract_run(const LevelGraph &g, const int32_t *comm, ContractBuffers &b, int64_t *new_offs,
                 int32_t *new_nbr, void *new_w, int32_t *orig_map, int32_t n_orig, int64_t *new_E,
                 cudaStream_t st, gala_status *status, bool validate_labels, bool sort_rows,
                 const NextLevelInit &nli, bool labels_only)
{
    if ((nli.k != nullptr) != (nli.tot != nullptr)) {
        set_error("contraction: K_new needs the community totals");
        *status = GALA_ERR_INVALID;
        return -1;
    }
    if (g.wide)
        return contract_t<long long>(g, comm, b, new_offs, new_nbr, (long long *)new_w, orig_map, n_orig, new_E, st,
                                     status, validate_labels, sort_rows, nli, labels_only);
    return contract_t<int>(g, comm, b, new_offs, new_nbr, (int *)new_w, orig_map, n_orig, new_E, st, status,
                           validate_labels, sort_rows, nli, labels_only);
}

}  // namespace gala
