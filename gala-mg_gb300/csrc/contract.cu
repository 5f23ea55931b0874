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
//        <= 4096 entries    one 256-thread CTA, shared-memory hash table
//        larger             a global table per community filled by many CTAs
//                           (4096-entry chunks of the stream); a dense table
//                           indexed by community id when the row can hold a
//                           large share of all communities
//      and emit the distinct neighbours in ascending id order (rank by
//      shuffle compare, bitonic sort in shared memory, a scan of the dense
//      table, or a bitmap over all communities for very long rows)
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
constexpr int kMid1Max = 512;
constexpr int kMid2Max = 4096;
constexpr int kChunk = 4096;
constexpr int kEmitList = 16384;

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
        if (s == e) continue;
        const long long base = medge[mpos[v]] - s;
        for (long long j = s + lane; j < e; j += 32) {
            skey[base + j] = lab[nbr[j]];
            sw[base + j] = W ? w[j] : 1;
        }
    }
}

__device__ __forceinline__ int row_class(long long E)
{
    return E <= kSmallMax ? 0 : (E <= kMid1Max ? 1 : (E <= kMid2Max ? 2 : 3));
}

// Size classes with warp-aggregated appends (one atomic per warp and class).
__global__ void __launch_bounds__(256) k_classify(int C, const long long *__restrict__ ec, int32_t *lists,
                                                  DevStats *st)
{
    const int stride = gridDim.x * blockDim.x;
    for (int base = blockIdx.x * blockDim.x; base < C; base += stride) {
        const int c = base + threadIdx.x;
        const int cls = c < C ? row_class(ec[c]) : -1;
#pragma unroll
        for (int k = 0; k < 4; ++k) warp_append(cls == k, c, lists + (long long)k * C, &st->small_cnt[k]);
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

// Insert stream entries [st + lo, st + hi) into a hash table (or a dense
// table when keys == nullptr).  Called by all threads of the block.
__device__ __forceinline__ void agg_insert(const AggArgs &a, long long st, int lo, int hi, int *keys, int *vals,
                                           int T, int lg)
{
    const int lane = threadIdx.x & 31;
    for (int b0 = lo; b0 < hi; b0 += blockDim.x) {
        const int j = b0 + threadIdx.x;
        const bool valid = j < hi;
        int key = -1, wt = 0;
        if (valid) {
            key = a.skey[st + j];
            wt = a.sw[st + j];
        }
        const unsigned m = __match_any_sync(GALA_FULL_MASK, key);
        const int sum = (int)__reduce_add_sync(m, (unsigned)wt);
        if (valid && __ffs(m) - 1 == lane) {
            if (!keys)
                atomicAdd(&vals[key], sum);
            else if (!hash_add(keys, vals, T, lg, key, sum))
                atomicOr(&a.st->err, kErrHashOverflow);
        }
    }
}

// Rows of 33..kMid2Max entries: one CTA per community, shared-memory hash
// table of TMAX slots, distinct keys sorted by a bitonic sort of LMAX slots.
template <int BLOCK, int TMAX, int LMAX>
__global__ void __launch_bounds__(BLOCK) k_agg_mid(AggArgs a, const int32_t *__restrict__ list, int cls)
{
    extern __shared__ int sm[];
    int *keys = sm;
    int *vals = sm + TMAX;
    int *lk = sm + 2 * TMAX;
    int *lv = lk + LMAX;
    __shared__ int s_k;
    const int cnt = a.st->small_cnt[cls];
    for (int i = blockIdx.x; i < cnt; i += gridDim.x) {
        const int c = list[i];
        const long long st = a.medge[a.moff[c]];
        const int E = (int)a.ec[c];
        const int cap = E < a.C ? E : a.C;
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
        agg_insert(a, st, 0, E, keys, vals, T, lg);
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
    const long long *__restrict__ toff;
    const long long *__restrict__ coff;
    int32_t *mode;
    int32_t *work;
    int32_t *pool;
    long long pool_half;  // keys at pool[0, half), values at pool[half, 2 half)
};

// Table size and chunk count of every class-3 community.  A dense table
// (slot = community id) is used when a hash table would not be smaller.
__global__ void k_big_plan(AggArgs a, BigArgs b)
{
    const int cnt = a.st->small_cnt[3];
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < cnt; i += gridDim.x * blockDim.x) {
        const long long E = a.ec[b.list[i]];
        const long long cap = E < a.C ? E : a.C;
        long long T = next_pow2_ll(2LL * cap);
        int dense = T >= a.C;
        if (dense) T = a.C;
        b.T[i] = T;
        b.mode[i] = dense;
        b.chunks[i] = (E + kChunk - 1) / kChunk;
    }
}

__global__ void k_big_tail(BigArgs b, const DevStats *st)
{
    // toff[cnt] / coff[cnt] close the last segments (totals of the scans)
    const int cnt = st->small_cnt[3];
    ((long long *)b.toff)[cnt] = st->total;
    ((long long *)b.coff)[cnt] = st->total2;
}

// chunk -> community (list index), one warp per community
__global__ void k_big_work(AggArgs a, BigArgs b)
{
    const int lane = threadIdx.x & 31;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int cnt = a.st->small_cnt[3];
    for (int i = wg; i < cnt; i += nw) {
        const long long o = b.coff[i], k = b.coff[i + 1] - o;
        for (long long j = lane; j < k; j += 32) b.work[o + j] = i;
    }
}

// Every CTA inserts one chunk of kChunk stream entries into its community's
// global table (hash or dense); many CTAs share one community.
__global__ void __launch_bounds__(256) k_big_insert(AggArgs a, BigArgs b, long long nwork)
{
    for (long long wi = blockIdx.x; wi < nwork; wi += gridDim.x) {
        const int i = b.work[wi];
        const long long j = wi - b.coff[i];
        const int c = b.list[i];
        const long long E = a.ec[c];
        const long long st = a.medge[a.moff[c]] + j * kChunk;
        const int len = (int)((E - j * kChunk) < kChunk ? (E - j * kChunk) : kChunk);
        const long long T = b.T[i];
        int *vals = b.pool + b.pool_half + b.toff[i];
        int *keys = b.mode[i] ? nullptr : b.pool + b.toff[i];
        agg_insert(a, st, 0, len, keys, vals, (int)T, __ffs((int)T) - 1);
    }
}

// One CTA per class-3 community: rank the distinct keys and write the row.
__global__ void __launch_bounds__(1024) k_big_emit(AggArgs a, BigArgs b, unsigned *gbits, long long bit_words)
{
    extern __shared__ int sm[];
    int *lk = sm;
    int *lv = sm + kEmitList;
    __shared__ int s_k;
    __shared__ long long wt_s[32];
    __shared__ long long tot_s;
    unsigned *bits = gbits + (long long)blockIdx.x * 2 * bit_words;
    unsigned *pref = bits + bit_words;
    const int cnt = a.st->small_cnt[3];
    const int nwords = (a.C + 31) >> 5;
    for (int i = blockIdx.x; i < cnt; i += gridDim.x) {
        const int c = b.list[i];
        const long long T = b.T[i];
        const int *vals = b.pool + b.pool_half + b.toff[i];
        const int *keys = b.pool + b.toff[i];
        const long long o = a.tmp_off[c];
        int k = 0;
        if (b.mode[i]) {
            // dense: slot = neighbour community, ascending by construction
            long long carry = 0;
            for (long long b0 = 0; b0 < T; b0 += blockDim.x) {
                const long long x = b0 + threadIdx.x;
                const int wv = x < T ? vals[x] : 0;
                const long long f = wv > 0 ? 1 : 0;
                const long long ex = block_exclusive_scan<long long>(f, wt_s, &tot_s);
                if (f) {
                    a.tmp_nbr[o + carry + ex] = (int)x;
                    a.tmp_w[o + carry + ex] = wv;
                }
                carry += tot_s;
                __syncthreads();
            }
            k = (int)carry;
        } else {
            if (threadIdx.x == 0) s_k = 0;
            __syncthreads();
            int mine = 0;
            for (long long j = threadIdx.x; j < T; j += blockDim.x) mine += keys[j] >= 0;
            mine = warp_sum(mine);
            if ((threadIdx.x & 31) == 0 && mine) atomicAdd(&s_k, mine);
            __syncthreads();
            k = s_k;
            __syncthreads();
            if (k <= kEmitList) {
                if (threadIdx.x == 0) s_k = 0;
                __syncthreads();
                for (long long j = threadIdx.x; j < T; j += blockDim.x) {
                    const int kk = keys[j];
                    if (kk >= 0) {
                        const int p = atomicAdd(&s_k, 1);
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
                for (long long j = threadIdx.x; j < T; j += blockDim.x) {
                    const int kk = keys[j];
                    if (kk >= 0) atomicOr(&bits[kk >> 5], 1u << (kk & 31));
                }
                __syncthreads();
                long long carry = 0;
                for (int b0 = 0; b0 < nwords; b0 += blockDim.x) {
                    const int j = b0 + threadIdx.x;
                    const long long pc = j < nwords ? __popc(bits[j]) : 0;
                    const long long ex = block_exclusive_scan<long long>(pc, wt_s, &tot_s);
                    if (j < nwords) pref[j] = (unsigned)(ex + carry);
                    carry += tot_s;
                    __syncthreads();
                }
                for (long long j = threadIdx.x; j < T; j += blockDim.x) {
                    const int kk = keys[j];
                    if (kk >= 0) {
                        const unsigned r = pref[kk >> 5] + __popc(bits[kk >> 5] & ((1u << (kk & 31)) - 1u));
                        a.tmp_nbr[o + r] = kk;
                        a.tmp_w[o + r] = vals[j];
                    }
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
    st->small_cnt[0] = st->small_cnt[1] = st->small_cnt[2] = st->small_cnt[3] = 0;
    st->err = 0;
}

constexpr size_t kMid1Smem = (2 * 1024 + 2 * kMid1Max) * sizeof(int);
constexpr size_t kMid2Smem = (2 * 8192 + 2 * kMid2Max) * sizeof(int);
constexpr size_t kEmitSmem = 2 * kEmitList * sizeof(int);

void contract_configure_kernels()
{
    cudaFuncSetAttribute(k_agg_mid<256, 8192, kMid2Max>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kMid2Smem);
    cudaFuncSetAttribute(k_big_emit, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kEmitSmem);
}

static int grid_cap(long long items, int per_block, int cap)
{
    long long g = (items + per_block - 1) / per_block;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

static bool read_stats(DevStats *h, DevStats *d, cudaStream_t st, gala_status *status, const char *what)
{
    cudaError_t ce;
    if ((ce = cudaMemcpyAsync(h, d, sizeof(DevStats), cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
        (ce = cudaStreamSynchronize(st)) != cudaSuccess) {
        *status = cuda_fail(ce, what);
        return false;
    }
    return true;
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
    *status = GALA_OK;
    DevStats hs;

    k_contract_reset<<<1, 1, 0, st>>>(b.stats);
    note_launch(1);
    if (validate_labels) {
        k_check_labels<<<grid_cap(n, 256, cap), 256, 0, st>>>(comm, n, b.stats);
        note_launch(1);
        if (!read_stats(&hs, b.stats, st, status, "contraction: label check")) return -1;
        if (hs.err) {
            set_error("contraction: a community label lies outside [0, %d)", n);
            *status = GALA_ERR_INVALID;
            return -1;
        }
    }
    cudaMemsetAsync(b.cnt, 0, ((size_t)n + 1) * sizeof(int32_t), st);
    k_hist<<<grid_cap(n, 256, cap), 256, 0, st>>>(comm, n, b.cnt);
    exclusive_scan(b.cnt, b.newid, n, OpPositive(), b.scan_partial, &b.stats->total, st);
    note_launch(1);
    if (!read_stats(&hs, b.stats, st, status, "contraction: community count")) return -1;
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
    if (!read_stats(&hs, b.stats, st, status, "contraction: classification")) return -1;

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
    const int nsm = sm_count();
    if (hs.small_cnt[0] > 0) {
        k_agg_small<<<grid_cap((long long)hs.small_cnt[0] * 32, 256, cap), 256, 0, st>>>(a, b.cls_list);
        note_launch(1);
    }
    if (hs.small_cnt[1] > 0) {
        int grid = hs.small_cnt[1] < nsm * 12 ? hs.small_cnt[1] : nsm * 12;
        k_agg_mid<128, 1024, kMid1Max><<<grid, 128, kMid1Smem, st>>>(a, b.cls_list + (long long)C, 1);
        note_launch(1);
    }
    if (hs.small_cnt[2] > 0) {
        int grid = hs.small_cnt[2] < nsm * 2 ? hs.small_cnt[2] : nsm * 2;
        k_agg_mid<256, 8192, kMid2Max><<<grid, 256, kMid2Smem, st>>>(a, b.cls_list + 2LL * C, 2);
        note_launch(1);
    }
    if (hs.small_cnt[3] > 0) {
        const int cnt3 = hs.small_cnt[3];
        BigArgs ba;
        ba.list = b.cls_list + 3LL * C;
        ba.T = b.big_T;
        ba.chunks = b.big_chunks;
        ba.toff = b.big_toff;
        ba.coff = b.big_coff;
        ba.mode = b.big_mode;
        ba.work = b.big_work;
        ba.pool = b.big_pool;
        ba.pool_half = 0;
        k_big_plan<<<grid_cap(cnt3, 256, cap), 256, 0, st>>>(a, ba);
        exclusive_scan(b.big_T, b.big_toff, cnt3, OpIdentity(), b.scan_partial, &b.stats->total, st);
        exclusive_scan(b.big_chunks, b.big_coff, cnt3, OpIdentity(), b.scan_partial, &b.stats->total2, st);
        k_big_tail<<<1, 1, 0, st>>>(ba, b.stats);
        note_launch(2);
        if (!read_stats(&hs, b.stats, st, status, "contraction: large rows")) return -1;
        const long long slots = hs.total, nwork = hs.total2;
        if (2 * slots > b.big_pool_ints || nwork > b.big_work_cap) {
            set_error("contraction: large rows need %lld table slots / %lld chunks, pool holds %lld / %lld", slots,
                      nwork, b.big_pool_ints / 2, b.big_work_cap);
            *status = GALA_ERR_CAPACITY;
            return -1;
        }
        ba.pool_half = slots;
        cudaMemsetAsync(b.big_pool, 0xff, (size_t)slots * sizeof(int32_t), st);
        cudaMemsetAsync(b.big_pool + slots, 0, (size_t)slots * sizeof(int32_t), st);
        k_big_work<<<grid_cap((long long)cnt3 * 32, 256, cap), 256, 0, st>>>(a, ba);
        k_big_insert<<<(int)(nwork < nsm * 8 ? nwork : nsm * 8), 256, 0, st>>>(a, ba, nwork);
        const long long words = ((long long)C + 31) / 32;
        long long grid = cnt3 < nsm * 2 ? cnt3 : nsm * 2;
        const long long fit = b.big_bitmap_words / (2 * words);
        if (grid > fit) grid = fit;
        if (grid < 1) {
            set_error("contraction: %d communities need a %lld-word bitmap, scratch holds %lld", C, 2 * words,
                      b.big_bitmap_words);
            *status = GALA_ERR_CAPACITY;
            return -1;
        }
        k_big_emit<<<(int)grid, 1024, kEmitSmem, st>>>(a, ba, (unsigned *)b.big_bitmap, words);
        note_launch(3);
    }
    exclusive_scan(b.kc, new_offs, C, OpIdentity(), b.scan_partial, &b.stats->total, st);
    k_set_last_offset<<<1, 1, 0, st>>>(new_offs, C, &b.stats->total);
    k_compact<<<grid_cap((long long)C * 32, 256, cap), 256, 0, st>>>(C, b.kc, new_offs, b.tmp_off, b.tmp_nbr,
                                                                     b.tmp_w, new_nbr, new_w);
    note_launch(2);
    if (!read_stats(&hs, b.stats, st, status, "contraction: compaction")) return -1;
    if (hs.err) {
        set_error("contraction: hash table overflow (error bits %d)", hs.err);
        *status = GALA_ERR_OVERFLOW;
        return -1;
    }
    *new_E = hs.total;
    return C;
}

}  // namespace gala
