// update_push.cu - incremental weight update of a phase-1 sweep.
//
// The full update (compute_In / compute_In_blk, kernel_functions.cu:890-1034
// of the reference; the per-bin update kernels of phase1.cu) sums In[v], the
// weight from v to its own community, over every row after every sweep.
// Only movers and their neighbours can change it.  On a symmetric graph every
// entry (u, v, w) of a mover u's row mirrors the entry (v, u, w) of v's row,
// so a neighbour v that did not move loses w when its community is u's old
// one and gains w when it is u's new one; a mover's own In is summed again
// over its row.  Weights are integers (or 64-bit fixed point), the sums are
// exact, and In, the pruning bound, the next active lists and the sums equal
// those of the full update bit for bit.  A sweep takes this path when its
// movers' rows hold a small share of the level's entries, on a graph whose
// entries all have mirrors (the level-init row kernels of phase1.cu sum a
// hash of every entry minus its mirror).
#include "common.cuh"
#include "internal.h"
#include "scan.cuh"
#include "walk.cuh"

namespace gala {

namespace {

int sm_count_push()
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

constexpr int kPushRange = 1024;  // entries of the movers' rows per warp task

struct OpRowLen {  // row length of the vertex `in`
    const int64_t *offs;
    __device__ __forceinline__ long long operator()(int32_t v, long long) const
    {
        return (long long)(offs[v + 1] - offs[v]);
    }
};

// Incremental or full update of this sweep: incremental when allowed (a
// level's In is exact from the previous sweep on, the graph is symmetric)
// and, unless forced, when the movers' rows hold under a third of the
// level's entries.
__global__ void k_update_mode(DevStats *st, int allow, int force, long long E)
{
    const int push = allow && (force || st->mv_edges * 3ull < (unsigned long long)E);
    st->push_mode = push;
    st->push_len = push ? st->n_movers : 0;
}

// Incremental: pre[n_movers] = their entry total and In of every mover
// restarts at 0.  Full: the mover flags are cleared here (the prune pass
// clears them otherwise).
template <typename WT>
__global__ void k_push_prep(const int32_t *__restrict__ mv_v, long long *pre, WT *In, uint8_t *moved,
                            const DevStats *st)
{
    const int nm = st->n_movers;
    const bool push = st->push_mode != 0;
    if (push && blockIdx.x == 0 && threadIdx.x == 0) pre[nm] = st->push_total;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nm; i += gridDim.x * blockDim.x) {
        if (push)
            In[mv_v[i]] = 0;
        else
            moved[mv_v[i]] = 0;
    }
}

// The movers' rows as one walk list (row r = mover r, entries
// [pre[r], pre[r + 1])), 1024 entries per warp task.  Entry (u, v, w):
//   w counts towards In[u] when v lies in u's new community (summed over the
//   lanes of one row first, one atomic per row and batch);
//   v != u that did not move loses w when it lies in u's old community and
//   gains w when it lies in u's new one.
template <typename WT, bool W>
__global__ void __launch_bounds__(256) k_push_in(const int64_t *__restrict__ offs, const int32_t *__restrict__ nbr,
                                                 const WT *__restrict__ w, const int32_t *__restrict__ comm, WT *In,
                                                 const uint8_t *__restrict__ moved, const int32_t *__restrict__ mv_v,
                                                 const int32_t *__restrict__ mv_old,
                                                 const int32_t *__restrict__ mv_new, const long long *__restrict__ pre,
                                                 const DevStats *__restrict__ st)
{
    if (!st->push_mode) return;
    constexpr int U = kWalkUnroll;
    const int lane = threadIdx.x & 31;
    const long long wg = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const int nm = st->n_movers;
    const long long total = st->push_total;
    // per row: pa = physical index of the row's entry j minus j, pb = the row
    auto rowval = [=](int r, long long &pa, long long &pb) {
        pa = offs[mv_v[r]] - pre[r];
        pb = r;
    };
    auto cur = row_cursor(pre, nm, rowval);
    const unsigned le = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);  // lanes 0..lane
    for (long long t = wg; t * kPushRange < total; t += nw) {
        const long long j0 = t * kPushRange;
        const long long j1 = j0 + kPushRange < total ? j0 + kPushRange : total;
        cur.start(j0);
        for (long long jb = j0; jb < j1; jb += 32 * U) {
            long long src[U];
            int row[U];
            bool ok[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const long long b0 = jb + 32 * u;
                ok[u] = false;
                src[u] = 0;
                row[u] = -1;
                if (b0 < j1) {  // warp-uniform
                    const long long j = b0 + lane;
                    long long d, r;
                    const bool in = cur.resolve(b0, b0 + 31 < j1 ? b0 + 31 : j1 - 1, j, d, r);
                    if (j < j1 && in && r >= 0) {
                        ok[u] = true;
                        src[u] = j + d;
                        row[u] = (int)r;
                    }
                }
            }
            int v[U];
            WT wv[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                v[u] = ok[u] ? nbr[src[u]] : 0;
                wv[u] = ok[u] ? (W ? w[src[u]] : (WT)1) : (WT)0;
            }
            int cv[U], mu[U], old[U], nu[U];
            bool mf[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                cv[u] = mu[u] = old[u] = nu[u] = -1;
                mf[u] = true;
                if (ok[u]) {
                    cv[u] = comm[v[u]];
                    mu[u] = mv_v[row[u]];
                    old[u] = mv_old[row[u]];
                    nu[u] = mv_new[row[u]];
                    mf[u] = moved[v[u]] != 0;
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                if (jb + 32 * u < j1) {  // warp-uniform: every lane takes part in the row sums
                    const WT own = (ok[u] && cv[u] == nu[u]) ? wv[u] : (WT)0;
                    // lanes of one row are contiguous: segment [start, end]
                    const int rp = __shfl_up_sync(GALA_FULL_MASK, row[u], 1);
                    const bool head = lane == 0 || !ok[u] || row[u] != rp;
                    const unsigned heads = __ballot_sync(GALA_FULL_MASK, head);
                    const int start = 31 - __clz((int)(heads & le));
                    const unsigned above = heads & ~le;
                    const int end = above ? __ffs((int)above) - 2 : 31;
                    const unsigned seg = (end == 31 ? 0xffffffffu : ((2u << end) - 1u)) & ~((1u << start) - 1u);
                    const WT sum = group_sum(seg, own);
                    if (ok[u] && lane == start && sum != 0) atomic_add_w(&In[mu[u]], sum);
                }
                if (ok[u] && v[u] != mu[u] && !mf[u]) {
                    if (cv[u] == old[u])
                        atomic_add_w(&In[v[u]], (WT)-wv[u]);
                    else if (cv[u] == nu[u])
                        atomic_add_w(&In[v[u]], wv[u]);
                }
            }
        }
    }
}

struct BinStarts {
    int s[kNumBinSlots + 1];
};

// Every vertex of bins 0-7: the pruning bound on its In (the rule of the
// full update kernels), its flag, the next active list of its bin, and the
// sums; clears the mover flags.
template <typename WT>
__global__ void __launch_bounds__(256) k_prune_all(const int32_t *__restrict__ order, BinStarts bs, int next,
                                                   const int64_t *__restrict__ offs, const int32_t *__restrict__ comm,
                                                   const WT *__restrict__ K, const WT *__restrict__ Self,
                                                   const WT *__restrict__ Tot, const WT *__restrict__ In,
                                                   uint8_t *act_flag, uint8_t *moved, int32_t *act_list,
                                                   DevStats *st, double constant, long long m2)
{
    if (!st->push_mode) return;
    const long long min_tot = st->min_tot;
    const int end = bs.s[kNumBins];
    const int lane = threadIdx.x & 31;
    unsigned long long s_in = 0, s_edges = 0;
    int s_act = 0;
    for (int base = blockIdx.x * blockDim.x; base < end; base += gridDim.x * blockDim.x) {  // block-uniform
        const int i = base + threadIdx.x;
        bool active = false;
        int v = 0, bin = 0;
        if (i < end) {
            v = order[i];
            while (bin < kNumBins - 1 && i >= bs.s[bin + 1]) ++bin;
            const WT sum = In[v];
            active = !prune_bound_fast<WT>(sum, Self[v], K[v], (WT)min_tot, Tot[comm[v]], constant, m2);
            act_flag[v] = active;
            moved[v] = 0;
            s_in += (unsigned long long)sum;
            if (active) {
                s_edges += (unsigned long long)(offs[v + 1] - offs[v]);
                s_act += 1;
            }
        }
        // appends to the bin segments (a warp spans one bin or a few)
        unsigned todo = __ballot_sync(GALA_FULL_MASK, active);
        while (todo) {
            const int lb = __shfl_sync(GALA_FULL_MASK, bin, __ffs((int)todo) - 1);
            const bool mine = active && bin == lb;
            const unsigned m = __ballot_sync(GALA_FULL_MASK, mine);
            const int leader = __ffs((int)m) - 1;
            int pos = 0;
            if (lane == leader) pos = atomicAdd(&st->act_count[next][lb], __popc(m));
            pos = __shfl_sync(GALA_FULL_MASK, pos, leader);
            if (mine) act_list[bs.s[lb] + pos + __popc(m & lanemask_lt())] = v;
            todo &= ~m;
        }
    }
    block_add_u64(s_in, &st->sum_in);
    block_add_u64(s_edges, &st->act_edges[next]);
    block_add_i32(s_act, &st->act_vertices[next]);
}

template <typename WT>
void push_update_t(const LevelGraph &g, Phase1Buffers &b, const int *bin_start, int next, double constant,
                   long long m2, int allow, int force, cudaStream_t st)
{
    const int n = g.n;
    const int cap = sm_count_push() * 8;
    WT *In = (WT *)b.In;
    k_update_mode<<<1, 1, 0, st>>>(b.stats, allow, force, g.E);
    exclusive_scan_dev(b.mv_v, b.mv_pre, n, &b.stats->push_len, OpRowLen{g.offs}, b.scan_partial,
                       &b.stats->push_total, st, &b.stats->err);
    const int gv = (int)std::min<long long>(cap, ((long long)n + 255) / 256);
    k_push_prep<WT><<<gv, 256, 0, st>>>(b.mv_v, b.mv_pre, In, b.moved, b.stats);
    const int gw = (int)std::min<long long>(cap, (g.E / kPushRange + 1) * 32 / 256 + 1);
    if (g.w)
        k_push_in<WT, true><<<gw, 256, 0, st>>>(g.offs, g.nbr, (const WT *)g.w, b.comm, In, b.moved, b.mv_v,
                                                b.mv_old, b.mv_new, b.mv_pre, b.stats);
    else
        k_push_in<WT, false><<<gw, 256, 0, st>>>(g.offs, g.nbr, nullptr, b.comm, In, b.moved, b.mv_v, b.mv_old,
                                                 b.mv_new, b.mv_pre, b.stats);
    BinStarts bs;
    for (int i = 0; i <= kNumBinSlots; ++i) bs.s[i] = bin_start[i];
    const int gp = (int)std::min<long long>(cap, ((long long)bs.s[kNumBins] + 255) / 256);
    k_prune_all<WT><<<gp > 0 ? gp : 1, 256, 0, st>>>(b.order, bs, next, g.offs, b.comm, (const WT *)b.K,
                                                     (const WT *)b.Self, (const WT *)b.Tot, In, b.act_flag, b.moved,
                                                     b.act[next], b.stats, constant, m2);
    note_launch(4);
}

}  // namespace

void p1_push_update(const LevelGraph &g, Phase1Buffers &b, const int *bin_start, int next, double constant,
                    long long m2, int allow, int force, cudaStream_t st)
{
    if (g.wide)
        push_update_t<long long>(g, b, bin_start, next, constant, m2, allow, force, st);
    else
        push_update_t<int>(g, b, bin_start, next, constant, m2, allow, force, st);
}

}  // namespace gala
