// contract.cu - phase 2 (contraction) of the GB300 Louvain engine.
//
// Replaces build_compressed_graph (build_compressed_graph.cu:5-173 and the
// kernels at kernel_functions.cu:1083-1694 of the reference).  Steps:
//   1. community sizes (histogram) and dense renumbering in ascending label
//      order: exclusive scan of (size > 0), no sort
//   2. members of each community (counting-sort buckets)
//   3. the community-ordered edge stream: for every member edge the new id of
//      the neighbour's community and the weight, contiguous per community
//   4. per community, sum the weights per neighbour community:
//        <= 32 entries    one warp, __match_any_sync + __reduce_add_sync
//        <= 4096 entries  one CTA, shared-memory hash table
//        larger           one CTA, global-memory hash table (per-CTA slice)
//      and emit the distinct neighbours in ascending id order (rank by
//      shuffle compare, bitonic sort in shared memory, or a bitmap over all
//      communities for very long rows)
//   5. CSR offsets by scan and a compaction copy.
// Rows come out sorted by neighbour id, so the contracted graph of a given
// partition is unique and can be compared bit for bit.
#include "common.cuh"
#include "internal.h"
#include "scan.cuh"

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
constexpr int kMidMax = 4096;
constexpr int kMidTable = 8192;
constexpr int kBigList = 16384;

struct OpDegOf {
    const int64_t *offs;
    __device__ __forceinline__ long long operator()(int32_t v, long long) const
    {
        return (long long)(offs[v + 1] - offs[v]);
    }
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

__global__ void k_relabel(const int32_t *__restrict__ comm, const int32_t *__restrict__ newid,
                          const int32_t *__restrict__ cnt, int n, int32_t *lab, int32_t *csz)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        lab[v] = newid[comm[v]];
        int k = cnt[v];
        if (k > 0) csz[newid[v]] = k;
    }
}

__global__ void k_compose(int32_t *orig, int n_orig, const int32_t *__restrict__ lab)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_orig; i += gridDim.x * blockDim.x)
        orig[i] = lab[orig[i]];
}

__global__ void k_member_scatter(const int32_t *__restrict__ lab, const int64_t *__restrict__ offs, int n,
                                 int32_t *cursor, int32_t *members, int32_t *mpos, long long *ec)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        int c = lab[v];
        int p = atomicAdd(&cursor[c], 1);
        members[p] = v;
        mpos[v] = p;
        long long d = offs[v + 1] - offs[v];
        if (d) atomicAdd((unsigned long long *)&ec[c], (unsigned long long)d);
    }
}

// Community-ordered edge stream: one warp per vertex (rows read in vertex
// order, written to the vertex's slot in its community's segment).
template <bool W>
__global__ void __launch_bounds__(256) k_stream_fill(int n, const int64_t *__restrict__ offs,
                                                     const int32_t *__restrict__ nbr,
                                                     const int32_t *__restrict__ w,
                                                     const int32_t *__restrict__ lab,
                                                     const int32_t *__restrict__ mpos,
                                                     const long long *__restrict__ medge, int32_t *skey,
                                                     int32_t *sw)
{
    const int lane = threadIdx.x & 31;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int v = wg; v < n; v += nw) {
        const long long s = offs[v], e = offs[v + 1];
        const long long base = medge[mpos[v]] - s;
        for (long long j = s + lane; j < e; j += 32) {
            skey[base + j] = lab[nbr[j]];
            sw[base + j] = W ? w[j] : 1;
        }
    }
}

__global__ void k_classify(int C, const long long *__restrict__ ec, int32_t *lists, DevStats *st)
{
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < C; c += gridDim.x * blockDim.x) {
        long long E = ec[c];
        int cls = E <= kSmallMax ? 0 : (E <= kMidMax ? 1 : 2);
        int p = atomicAdd(&st->small_cnt[cls], 1);
        lists[(long long)cls * C + p] = c;
        if (cls == 2) {
            long long cap = E < C ? E : C;
            atomicMax((unsigned long long *)&st->large_max_cap, (unsigned long long)cap);
        }
    }
}

struct AggArgs {
    const int32_t *__restrict__ moff;
    const long long *__restrict__ medge;
    const long long *__restrict__ ec;
    const int32_t *__restrict__ skey;
    const int32_t *__restrict__ sw;
    const long long *__restrict__ tmp_off;
    int32_t *tmp_nbr;
    int32_t *tmp_w;
    int32_t *kc;
    DevStats *st;
    int C;
};

// Rows of at most 32 entries: one warp, rank of each distinct key by a
// shuffle compare against all others.
__global__ void __launch_bounds__(256) k_agg_small(AggArgs a, const int32_t *__restrict__ list)
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
        int key = -1, wt = 0;
        if (valid) {
            key = a.skey[st + lane];
            wt = a.sw[st + lane];
        }
        const unsigned m = __match_any_sync(GALA_FULL_MASK, key);
        const int sum = (int)__reduce_add_sync(m, (unsigned)wt);
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
__device__ __forceinline__ void bitonic_sort_smem(int *k, int *v, int P)
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
                    int tv = v[i];
                    v[i] = v[j];
                    v[j] = tv;
                }
            }
            __syncthreads();
        }
    }
}

// Insert a block-wide chunk of the stream into a hash table (all threads).
__device__ __forceinline__ void agg_insert(const AggArgs &a, long long st, int E, int *keys, int *vals, int T,
                                           int lg)
{
    const int lane = threadIdx.x & 31;
    for (int b0 = 0; b0 < E; b0 += blockDim.x) {
        const int j = b0 + threadIdx.x;
        const bool valid = j < E;
        int key = -1, wt = 0;
        if (valid) {
            key = a.skey[st + j];
            wt = a.sw[st + j];
        }
        const unsigned m = __match_any_sync(GALA_FULL_MASK, key);
        const int sum = (int)__reduce_add_sync(m, (unsigned)wt);
        if (valid && __ffs(m) - 1 == lane)
            if (!hash_add(keys, vals, T, lg, key, sum)) atomicOr(&a.st->err, kErrHashOverflow);
    }
}

// Rows of 33..4096 entries: one CTA, shared-memory table and bitonic sort.
__global__ void __launch_bounds__(256) k_agg_mid(AggArgs a, const int32_t *__restrict__ list)
{
    extern __shared__ int sm[];
    int *keys = sm;
    int *vals = sm + kMidTable;
    int *lk = sm + 2 * kMidTable;
    int *lv = lk + kMidMax;
    __shared__ int s_k;
    const int cnt = a.st->small_cnt[1];
    for (int i = blockIdx.x; i < cnt; i += gridDim.x) {
        const int c = list[i];
        const long long st = a.medge[a.moff[c]];
        const int E = (int)a.ec[c];
        const int cap = E < a.C ? E : a.C;
        int T = next_pow2_int(2LL * cap);
        if (T < 64) T = 64;
        const int lg = __ffs(T) - 1;
        for (int j = threadIdx.x; j < T; j += blockDim.x) {
            keys[j] = -1;
            vals[j] = 0;
        }
        if (threadIdx.x == 0) s_k = 0;
        __syncthreads();
        agg_insert(a, st, E, keys, vals, T, lg);
        __syncthreads();
        for (int j = threadIdx.x; j < T; j += blockDim.x) {
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
        for (int j = k + threadIdx.x; j < P; j += blockDim.x) {
            lk[j] = 0x7fffffff;
            lv[j] = 0;
        }
        __syncthreads();
        bitonic_sort_smem(lk, lv, P);
        const long long o = a.tmp_off[c];
        for (int j = threadIdx.x; j < k; j += blockDim.x) {
            a.tmp_nbr[o + j] = lk[j];
            a.tmp_w[o + j] = lv[j];
        }
        if (threadIdx.x == 0) a.kc[c] = k;
        __syncthreads();
    }
}

// Rows of more than 4096 entries: one CTA with a global-memory table slice;
// distinct keys sorted in shared memory when they fit, otherwise ranked with
// a bitmap over all C communities and a prefix of its popcounts.
__global__ void __launch_bounds__(1024) k_agg_big(AggArgs a, const int32_t *__restrict__ list, int tmax,
                                                  int32_t *gtab, int32_t *gbits, long long bit_words)
{
    extern __shared__ int sm[];
    int *lk = sm;
    int *lv = sm + kBigList;
    __shared__ int s_k;
    __shared__ long long wt_s[32];
    __shared__ long long tot_s;
    int *keys = gtab + (long long)blockIdx.x * 2 * tmax;
    int *vals = keys + tmax;
    unsigned *bits = (unsigned *)gbits + (long long)blockIdx.x * 2 * bit_words;
    unsigned *pref = bits + bit_words;
    const int cnt = a.st->small_cnt[2];
    const int nwords = (a.C + 31) >> 5;
    for (int i = blockIdx.x; i < cnt; i += gridDim.x) {
        const int c = list[i];
        const long long st = a.medge[a.moff[c]];
        const int E = (int)a.ec[c];
        const int cap = E < a.C ? E : a.C;
        int T = next_pow2_int(2LL * cap);
        if (T < 64) T = 64;
        if (T > tmax) {
            if (threadIdx.x == 0) atomicOr(&a.st->err, kErrHashOverflow);
            continue;
        }
        const int lg = __ffs(T) - 1;
        for (int j = threadIdx.x; j < T; j += blockDim.x) {
            keys[j] = -1;
            vals[j] = 0;
        }
        if (threadIdx.x == 0) s_k = 0;
        __syncthreads();
        agg_insert(a, st, E, keys, vals, T, lg);
        __syncthreads();
        for (int j = threadIdx.x; j < T; j += blockDim.x)
            if (keys[j] >= 0) atomicAdd(&s_k, 1);
        __syncthreads();
        const int k = s_k;
        const long long o = a.tmp_off[c];
        if (k <= kBigList) {
            __syncthreads();
            if (threadIdx.x == 0) s_k = 0;
            __syncthreads();
            for (int j = threadIdx.x; j < T; j += blockDim.x) {
                int kk = keys[j];
                if (kk >= 0) {
                    int p = atomicAdd(&s_k, 1);
                    lk[p] = kk;
                    lv[p] = vals[j];
                }
            }
            __syncthreads();
            const int P = next_pow2_int(k);
            for (int j = k + threadIdx.x; j < P; j += blockDim.x) {
                lk[j] = 0x7fffffff;
                lv[j] = 0;
            }
            __syncthreads();
            bitonic_sort_smem(lk, lv, P);
            for (int j = threadIdx.x; j < k; j += blockDim.x) {
                a.tmp_nbr[o + j] = lk[j];
                a.tmp_w[o + j] = lv[j];
            }
        } else {
            for (int j = threadIdx.x; j < nwords; j += blockDim.x) bits[j] = 0u;
            __syncthreads();
            for (int j = threadIdx.x; j < T; j += blockDim.x) {
                int kk = keys[j];
                if (kk >= 0) atomicOr(&bits[kk >> 5], 1u << (kk & 31));
            }
            __syncthreads();
            long long carry = 0;
            for (int b0 = 0; b0 < nwords; b0 += blockDim.x) {
                int j = b0 + threadIdx.x;
                long long pc = j < nwords ? __popc(bits[j]) : 0;
                long long ex = block_exclusive_scan<long long>(pc, wt_s, &tot_s);
                if (j < nwords) pref[j] = (unsigned)(ex + carry);
                carry += tot_s;
                __syncthreads();
            }
            for (int j = threadIdx.x; j < T; j += blockDim.x) {
                int kk = keys[j];
                if (kk >= 0) {
                    unsigned r = pref[kk >> 5] + __popc(bits[kk >> 5] & ((1u << (kk & 31)) - 1u));
                    a.tmp_nbr[o + r] = kk;
                    a.tmp_w[o + r] = vals[j];
                }
            }
        }
        if (threadIdx.x == 0) a.kc[c] = k;
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) k_compact(int C, const int32_t *__restrict__ kc,
                                                 const int64_t *__restrict__ new_offs,
                                                 const long long *__restrict__ tmp_off,
                                                 const int32_t *__restrict__ tmp_nbr,
                                                 const int32_t *__restrict__ tmp_w, int32_t *out_nbr,
                                                 int32_t *out_w)
{
    const int lane = threadIdx.x & 31;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int c = wg; c < C; c += nw) {
        const int k = kc[c];
        const long long src = tmp_off[c], dst = new_offs[c];
        for (int j = lane; j < k; j += 32) {
            out_nbr[dst + j] = tmp_nbr[src + j];
            out_w[dst + j] = tmp_w[src + j];
        }
    }
}

__global__ void k_contract_set_tail(int32_t *moff, int C, int n, long long *medge, long long E)
{
    moff[C] = n;
    medge[n] = E;
}

__global__ void k_set_last_offset(int64_t *offs, int C, const long long *total) { offs[C] = *total; }

__global__ void k_contract_reset(DevStats *st)
{
    st->small_cnt[0] = st->small_cnt[1] = st->small_cnt[2] = 0;
    st->large_max_cap = 0;
    st->err = 0;
}

void contract_configure_kernels()
{
    cudaFuncSetAttribute(k_agg_mid, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (2 * kMidTable + 2 * kMidMax) * (int)sizeof(int));
    cudaFuncSetAttribute(k_agg_big, cudaFuncAttributeMaxDynamicSharedMemorySize, 2 * kBigList * (int)sizeof(int));
}

static int grid_cap(long long items, int per_block, int cap)
{
    long long g = (items + per_block - 1) / per_block;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

// Returns the community count C (>= 1) or -1 on failure (*status set).
// new_offs receives C+1 offsets (leading 0).  orig_map (length n_orig) is
// composed with the new labels.
int contract_run(const LevelGraph &g, const int32_t *comm, ContractBuffers &b, int64_t *new_offs,
                 int32_t *new_nbr, int32_t *new_w, int32_t *orig_map, int32_t n_orig, int64_t *new_E,
                 cudaStream_t st, gala_status *status, bool validate_labels)
{
    const int n = g.n;
    const int cap = sm_count() * 8;
    cudaError_t ce;
    *status = GALA_OK;
    DevStats hs;

    k_contract_reset<<<1, 1, 0, st>>>(b.stats);
    note_launch(1);
    if (validate_labels) {
        k_check_labels<<<grid_cap(n, 256, cap), 256, 0, st>>>(comm, n, b.stats);
        note_launch(1);
        if ((ce = cudaMemcpyAsync(&hs.err, &b.stats->err, sizeof(int), cudaMemcpyDeviceToHost, st)) !=
                cudaSuccess ||
            (ce = cudaStreamSynchronize(st)) != cudaSuccess) {
            *status = cuda_fail(ce, "contraction: label check");
            return -1;
        }
        if (hs.err) {
            set_error("contraction: a community label lies outside [0, %d)", n);
            *status = GALA_ERR_INVALID;
            return -1;
        }
    }
    cudaMemsetAsync(b.cnt, 0, ((size_t)n + 1) * sizeof(int32_t), st);
    k_hist<<<grid_cap(n, 256, cap), 256, 0, st>>>(comm, n, b.cnt);
    exclusive_scan(b.cnt, b.newid, n, OpPositive(), b.scan_partial, &b.stats->total, st);
    note_launch(2);
    if ((ce = cudaMemcpyAsync(&hs.total, &b.stats->total, sizeof(long long), cudaMemcpyDeviceToHost, st)) !=
            cudaSuccess ||
        (ce = cudaStreamSynchronize(st)) != cudaSuccess) {
        *status = cuda_fail(ce, "contraction: community count");
        return -1;
    }
    const int C = (int)hs.total;

    k_relabel<<<grid_cap(n, 256, cap), 256, 0, st>>>(comm, b.newid, b.cnt, n, b.lab, b.csz);
    if (orig_map) k_compose<<<grid_cap(n_orig, 256, cap), 256, 0, st>>>(orig_map, n_orig, b.lab);
    exclusive_scan(b.csz, b.moff, C, OpIdentity(), b.scan_partial, &b.stats->total, st);
    cudaMemcpyAsync(b.cursor, b.moff, (size_t)C * sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
    cudaMemsetAsync(b.ec, 0, ((size_t)C + 1) * sizeof(long long), st);
    k_member_scatter<<<grid_cap(n, 256, cap), 256, 0, st>>>(b.lab, g.offs, n, b.cursor, b.members, b.mpos, b.ec);
    exclusive_scan(b.members, b.medge, n, OpDegOf{g.offs}, b.scan_partial, &b.stats->total, st);
    // moff[C] = n and medge[n] = E close the last segments
    k_contract_set_tail<<<1, 1, 0, st>>>(b.moff, C, n, b.medge, g.E);
    if (g.w)
        k_stream_fill<true><<<grid_cap((long long)n * 32, 256, cap), 256, 0, st>>>(
            n, g.offs, g.nbr, g.w, b.lab, b.mpos, b.medge, b.stream_key, b.stream_w);
    else
        k_stream_fill<false><<<grid_cap((long long)n * 32, 256, cap), 256, 0, st>>>(
            n, g.offs, g.nbr, g.w, b.lab, b.mpos, b.medge, b.stream_key, b.stream_w);
    k_classify<<<grid_cap(C, 256, cap), 256, 0, st>>>(C, b.ec, b.cls_list, b.stats);
    exclusive_scan(b.ec, b.tmp_off, C, OpCap{C}, b.scan_partial, &b.stats->total, st);
    note_launch(6 + (orig_map ? 1 : 0));
    if ((ce = cudaMemcpyAsync(&hs, b.stats, sizeof(DevStats), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (ce = cudaStreamSynchronize(st)) != cudaSuccess) {
        *status = cuda_fail(ce, "contraction: classification");
        return -1;
    }

    AggArgs a;
    a.moff = b.moff;
    a.medge = b.medge;
    a.ec = b.ec;
    a.skey = b.stream_key;
    a.sw = b.stream_w;
    a.tmp_off = b.tmp_off;
    a.tmp_nbr = b.tmp_nbr;
    a.tmp_w = b.tmp_w;
    a.kc = b.kc;
    a.st = b.stats;
    a.C = C;
    if (hs.small_cnt[0] > 0) {
        k_agg_small<<<grid_cap((long long)hs.small_cnt[0] * 32, 256, cap), 256, 0, st>>>(a, b.cls_list);
        note_launch(1);
    }
    if (hs.small_cnt[1] > 0) {
        int grid = hs.small_cnt[1] < sm_count() * 2 ? hs.small_cnt[1] : sm_count() * 2;
        k_agg_mid<<<grid, 256, (2 * kMidTable + 2 * kMidMax) * sizeof(int), st>>>(a, b.cls_list + (long long)C);
        note_launch(1);
    }
    if (hs.small_cnt[2] > 0) {
        int tmax = next_pow2_int(2LL * hs.large_max_cap);
        if (tmax < 64) tmax = 64;
        long long words = ((long long)C + 31) / 32;
        long long per_cta_table = 2LL * tmax;
        long long per_cta_bits = 2LL * words;
        long long g1 = b.big_table_slots / per_cta_table;
        long long g2 = b.big_bitmap_words / per_cta_bits;
        long long grid = hs.small_cnt[2];
        if (grid > sm_count()) grid = sm_count();
        if (grid > g1) grid = g1;
        if (grid > g2) grid = g2;
        if (grid < 1) {
            set_error("contraction: community row of %lld entries exceeds the scratch table", hs.large_max_cap);
            *status = GALA_ERR_CAPACITY;
            return -1;
        }
        k_agg_big<<<(int)grid, 1024, 2 * kBigList * sizeof(int), st>>>(a, b.cls_list + 2LL * C, tmax, b.big_table,
                                                                      b.big_bitmap, words);
        note_launch(1);
    }
    exclusive_scan(b.kc, new_offs, C, OpIdentity(), b.scan_partial, &b.stats->total, st);
    k_set_last_offset<<<1, 1, 0, st>>>(new_offs, C, &b.stats->total);
    k_compact<<<grid_cap((long long)C * 32, 256, cap), 256, 0, st>>>(C, b.kc, new_offs, b.tmp_off, b.tmp_nbr,
                                                                     b.tmp_w, new_nbr, new_w);
    note_launch(2);
    if ((ce = cudaMemcpyAsync(&hs, b.stats, sizeof(DevStats), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (ce = cudaStreamSynchronize(st)) != cudaSuccess) {
        *status = cuda_fail(ce, "contraction: compaction");
        return -1;
    }
    if (hs.err) {
        set_error("contraction: hash table overflow (error bits %d)", hs.err);
        *status = GALA_ERR_OVERFLOW;
        return -1;
    }
    *new_E = hs.total;
    return C;
}

}  // namespace gala
