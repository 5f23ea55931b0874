// batch_cta.cu - a batch of small graphs in one persistent launch: every CTA
// takes graphs from a queue (largest first) and runs the whole multi-round
// Louvain of a graph on its own - phase 1 sweeps, the convergence rule, the
// contraction and the round rule - with block barriers between the steps and
// no host round trip.  Batching has no counterpart in the reference; every
// graph follows the single-graph rules of the reference
// (louvain_main_process.cu:571-1034 for phase 1, build_compressed_graph.cu
// for the contraction, louvain.cu:193-226 for the rounds), so its partition,
// modularity and community count equal its single-graph run.
//
// Decisions follow the single-graph engine: candidates are ordered by the
// exact integer gain numerator X = w m2 - K ((Tot_c - Tot_cur) + K), and the
// cases where the reference's FP64 rounding could decide (equal best X from
// different weights, X = 0, a corrected gain of 0, K m2 >= 2^49) are
// re-evaluated with its FP64 expressions.  Neighbour-community weights are
// summed per warp: rows of at most kWRow entries in a shared-memory
// open-addressing table whose claimed slots are listed (only those are read
// and cleared); longer rows in a dense per-warp table in global memory
// indexed by community id (a level has at most kCtaMaxN vertices), read and
// cleared with one atomic exchange per entry.
#include "common.cuh"
#include "internal.h"
#include "scan.cuh"

namespace gala {

namespace {

constexpr int kCtaThreads = 512;
constexpr int kCtaWarps = kCtaThreads / 32;
constexpr int kWT = 512;  // slots of a warp's shared-memory table
constexpr int kWTLog = 9;
constexpr int kWRow = kWT / 2;  // longest row (entries) the table takes

// Level graph as seen by one graph's CTA: level 0 reads the union CSR
// (64-bit global offsets, union ids), later levels the graph's own
// contracted CSR (32-bit local offsets, local ids).
struct LevelView {
    const int64_t *o64;
    const int32_t *o32;
    long long obase;
    const int32_t *nbr;
    int shift;
    const int32_t *w;
    __device__ __forceinline__ int beg(int v) const { return o64 ? (int)(o64[v] - obase) : o32[v]; }
    __device__ __forceinline__ int end(int v) const { return o64 ? (int)(o64[v + 1] - obase) : o32[v + 1]; }
    __device__ __forceinline__ int nb(int j) const { return nbr[j] - shift; }
    __device__ __forceinline__ int wt(int j) const { return w ? w[j] : 1; }
};

struct WarpTable {
    int keys[kWT];
    int vals[kWT];
    unsigned short occ[kWRow];  // slots claimed by the current row
};

struct CtaShared {
    WarpTable *tab;  // kCtaWarps tables in dynamic shared memory
    long long red_ll[kCtaWarps];
    unsigned long long red_u[kCtaWarps];
    int red_i[kCtaWarps];
    long long scan_wt[32];
    long long scan_tot;
    int graph;
};

__device__ __forceinline__ long long cta_sum_ll(long long v, long long *red)
{
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    long long t = 0;
    for (int q = 0; q < kCtaWarps; ++q) t += red[q];
    return t;
}

__device__ __forceinline__ unsigned long long cta_sum_u64(unsigned long long v, unsigned long long *red)
{
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    unsigned long long t = 0;
    for (int q = 0; q < kCtaWarps; ++q) t += red[q];
    return t;
}

__device__ __forceinline__ int cta_min_int(int v, int *red)
{
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v = min(v, __shfl_xor_sync(GALA_FULL_MASK, v, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    int t = 0x7fffffff;
    for (int q = 0; q < kCtaWarps; ++q) t = min(t, red[q]);
    return t;
}

// out[i] = sum_{j<i} f(j) for i < n (block-wide; returns the total).
template <typename F>
__device__ __forceinline__ int cta_exclusive_scan(int n, F f, int *out, long long *wt, long long *tot)
{
    long long carry = 0;
    for (int base = 0; base < n; base += kCtaThreads) {
        const int i = base + threadIdx.x;
        const long long v = i < n ? f(i) : 0;
        const long long ex = block_exclusive_scan<long long>(v, wt, tot);
        if (i < n) out[i] = (int)(carry + ex);
        carry += *tot;
        __syncthreads();
    }
    return (int)carry;
}

// Best candidate across the warp: larger gain, then the lower id.
__device__ __forceinline__ void warp_best(double &dq, int &c)
{
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        const double od = __shfl_xor_sync(GALA_FULL_MASK, dq, o);
        const int oc = __shfl_xor_sync(GALA_FULL_MASK, c, o);
        if (cand_better(od, oc, dq, c)) {
            dq = od;
            c = oc;
        }
    }
}

// Q from exact sums with the engine's FP64 expression (sum_in/m2 - t2/m2^2).
__device__ __forceinline__ double q_of_sums(unsigned long long sum_in, unsigned long long sum_tot2, long long m2)
{
    const double c = 1.0 / (double)m2;
    return __dsub_rn(__dmul_rn((double)(long long)sum_in, c), __dmul_rn(__dmul_rn((double)sum_tot2, c), c));
}

// Add w to key's slot (claiming an empty one); at most kWRow distinct keys
// go to a table of kWT slots, so the probe always ends.
__device__ __forceinline__ int wt_add(WarpTable &t, int key, int w, bool &created)
{
    unsigned h = ((unsigned)key * 0x9E3779B1u) >> (32 - kWTLog);
    for (int p = 0; p < kWT; ++p) {
        const int k = atomicCAS(&t.keys[h], -1, key);
        if (k == -1 || k == key) {
            created = k == -1;
            atomicAdd(&t.vals[h], w);
            return (int)h;
        }
        h = (h + 1) & (kWT - 1);
    }
    created = false;
    return -1;
}

// Sum the weights per key over the entries of rows [r0, r1) (row r holds
// entries [rb(r), re(r)); entry j has key kf(j) and weight wf(j)); then
// emit(key, sum, pos) once per distinct key, pos = 0, 1, ... over the keys.
// total (warp-uniform) is the number of entries.  All 32 lanes call.
template <typename RB, typename RE, typename KF, typename WF, typename EM>
__device__ __forceinline__ void warp_aggregate(WarpTable &t, int *gacc, int r0, int r1, long long total, RB rb,
                                               RE re, KF kf, WF wf, EM emit)
{
    const int lane = threadIdx.x & 31;
    if (total <= kWRow) {
        int nocc = 0;
        for (int r = r0; r < r1; ++r) {
            const int b = rb(r), e = re(r);
            for (int j0 = b; j0 < e; j0 += 32) {
                const int j = j0 + lane;
                bool cr = false;
                int slot = -1;
                if (j < e) slot = wt_add(t, kf(j), wf(j), cr);
                const unsigned cb = __ballot_sync(GALA_FULL_MASK, cr);
                if (cr) t.occ[nocc + __popc(cb & lanemask_lt())] = (unsigned short)slot;
                nocc += __popc(cb);
            }
        }
        __syncwarp();
        for (int q = lane; q < nocc; q += 32) {
            const int sl = t.occ[q];
            const int key = t.keys[sl], sum = t.vals[sl];
            t.keys[sl] = -1;
            t.vals[sl] = 0;
            emit(key, sum, q);
        }
        __syncwarp();
    } else {
        for (int r = r0; r < r1; ++r)
            for (int j = rb(r) + lane; j < re(r); j += 32) atomicAdd(&gacc[kf(j)], wf(j));
        __syncwarp();
        int base = 0;
        for (int r = r0; r < r1; ++r) {
            const int b = rb(r), e = re(r);
            for (int j0 = b; j0 < e; j0 += 32) {
                const int j = j0 + lane;
                int key = -1, sum = 0;
                if (j < e) {
                    key = kf(j);
                    sum = atomicExch(&gacc[key], 0);
                }
                const unsigned got = __ballot_sync(GALA_FULL_MASK, sum != 0);
                if (sum != 0) emit(key, sum, base + __popc(got & lanemask_lt()));
                base += __popc(got);
            }
        }
        __syncwarp();
    }
}

// Candidate merge by exact gain numerator: larger X, then the lower id; t
// records a tie on the best X between different weights.
__device__ __forceinline__ void merge_x(long long &x, int &c, int &w, int &t, long long ox, int oc, int ow, int ot)
{
    if (ox == x) {
        const int tie = t | ot | (ow != w);
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

// Phase 1 of one level (the oracle's phase1 rule): labels in prev on return.
__device__ void cta_phase1(const BatchCtaArgs &a, const LevelView &g, int n, long long m2, int vb, int *gacc,
                           CtaShared &sh, double *q_out, int *iters_out)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    WarpTable &tab = sh.tab[wid];
    int *K = a.K + vb, *Self = a.Self + vb, *Tot = a.Tot + vb, *In = a.In + vb, *prev = a.prev + vb,
        *cur = a.cur + vb, *size = a.size + vb;
    uint8_t *active = a.active + vb;
    const double constant = 1.0 / (double)m2;
    // init_communities: K = Tot = row weight, Self = self-loop weight,
    // label = own id, size 1, In = Self, every vertex active
    unsigned long long s_in = 0, s_t2 = 0;
    for (int v = threadIdx.x; v < n; v += kCtaThreads) {
        int k = 0, sf = 0;
        for (int j = g.beg(v); j < g.end(v); ++j) {
            const int wt = g.wt(j);
            k += wt;
            if (g.nb(j) == v) sf = wt;
        }
        K[v] = k;
        Tot[v] = k;
        Self[v] = sf;
        In[v] = sf;
        size[v] = 1;
        prev[v] = v;
        cur[v] = v;
        active[v] = 1;
        s_in += (unsigned long long)sf;
        s_t2 += (unsigned long long)((long long)k * k);
    }
    s_in = cta_sum_u64(s_in, sh.red_u);
    s_t2 = cta_sum_u64(s_t2, sh.red_u);
    double prev_q = q_of_sums(s_in, s_t2, m2);
    int iters = 0;
    auto rb = [&](int v) { return g.beg(v); };
    auto re = [&](int v) { return g.end(v); };
    auto kf = [&](int j) { return prev[g.nb(j)]; };
    auto wf = [&](int j) { return g.wt(j); };
    for (;;) {
        // decide-and-move: one warp per active vertex, every decision reads
        // the labels and totals of the previous iteration
        for (int v = wid; v < n; v += kCtaWarps) {
            const int b = g.beg(v), e = g.end(v);
            int nv = prev[v];
            if (active[v] && e > b) {
                const int cv = nv;
                const int ki = K[v], sf = Self[v], tcur = Tot[cv];
                long long x = -1;
                int bc = cv, bw = 0, bt = 0, wc = 0;
                warp_aggregate(tab, gacc, v, v + 1, e - b, rb, re, kf, wf, [&](int c, int s, int) {
                    if (c == cv) {
                        wc += s;
                    } else {
                        const long long xx = (long long)s * m2 - (long long)ki * ((long long)Tot[c] - tcur + ki);
                        if (xx >= 0) merge_x(x, bc, bw, bt, xx, c, s, 0);
                    }
                });
#pragma unroll
                for (int o = 16; o >= 1; o >>= 1) {
                    const long long ox = __shfl_xor_sync(GALA_FULL_MASK, x, o);
                    const int oc = __shfl_xor_sync(GALA_FULL_MASK, bc, o);
                    const int ow = __shfl_xor_sync(GALA_FULL_MASK, bw, o);
                    const int ot = __shfl_xor_sync(GALA_FULL_MASK, bt, o);
                    wc += __shfl_xor_sync(GALA_FULL_MASK, wc, o);
                    merge_x(x, bc, bw, bt, ox, oc, ow, ot);
                }
                // 0 stay, 1 move, 2 the FP64 expressions decide (warp-uniform)
                int dec;
                if ((long long)ki * m2 >= (1LL << 49))
                    dec = 2;
                else if (bc == cv)
                    dec = 0;
                else if (x == 0)
                    dec = wc == sf ? 2 : 0;
                else if (bt)
                    dec = 2;
                else {
                    const long long y = x - (long long)(wc - sf) * m2;
                    dec = y == 0 ? 2 : (y > 0 ? 1 : 0);
                }
                if (dec == 2) {
                    double bdq = 0.0;
                    int fc = cv;
                    warp_aggregate(tab, gacc, v, v + 1, e - b, rb, re, kf, wf, [&](int c, int s, int) {
                        if (c == cv) return;
                        const double d = gain_dq<int>(s, ki, Tot[c], tcur, constant);
                        if (d > 0.0 && cand_better(d, c, bdq, fc)) {
                            bdq = d;
                            fc = c;
                        }
                    });
                    warp_best(bdq, fc);
                    bc = fc;
                    dec = (fc != cv && gain_correct<int>(bdq, wc, sf) > 0.0) ? 1 : 0;
                }
                if (dec == 1 && !(size[bc] == 1 && size[cv] == 1 && bc > cv)) nv = bc;
            }
            if (lane == 0) cur[v] = nv;
        }
        __syncthreads();
        // Tot += Tot_update, size += size_update
        for (int v = threadIdx.x; v < n; v += kCtaThreads) {
            const int to = cur[v], from = prev[v];
            if (to != from) {
                atomicAdd(&Tot[to], K[v]);
                atomicSub(&Tot[from], K[v]);
                atomicAdd(&size[to], 1);
                atomicSub(&size[from], 1);
            }
        }
        __syncthreads();
        // min Tot over non-empty communities (m2 when none) and sum Tot^2
        int mn = 0x7fffffff;
        s_t2 = 0;
        for (int c = threadIdx.x; c < n; c += kCtaThreads) {
            const int t = Tot[c];
            if (t != 0) {
                mn = min(mn, t);
                s_t2 += (unsigned long long)((long long)t * t);
            }
        }
        mn = cta_min_int(mn, sh.red_i);
        s_t2 = cta_sum_u64(s_t2, sh.red_u);
        const int min_tot = mn == 0x7fffffff ? (int)m2 : mn;
        // weight update and pruning (compute_In): one warp per vertex
        unsigned long long my_in = 0;
        for (int v = wid; v < n; v += kCtaWarps) {
            const int b = g.beg(v), e = g.end(v);
            if (e == b) {
                if (lane == 0) active[v] = 1;
                continue;
            }
            const int c = cur[v];
            int s = 0;
            for (int j = b + lane; j < e; j += 32)
                if (cur[g.nb(j)] == c) s += g.wt(j);
            s = warp_sum(s);
            if (lane == 0) {
                In[v] = s;
                my_in += (unsigned long long)s;
                active[v] = !prune_bound_fast<int>(s, Self[v], K[v], min_tot, Tot[c], constant, m2);
            }
        }
        s_in = cta_sum_u64(my_in, sh.red_u);
        const double q = q_of_sums(s_in, s_t2, m2);
        ++iters;
        if (q - prev_q < a.min_mod) break;  // the iteration's partition is dropped
        prev_q = q;
        for (int v = threadIdx.x; v < n; v += kCtaThreads) prev[v] = cur[v];
        __syncthreads();
    }
    __syncthreads();
    *q_out = prev_q;
    *iters_out = iters;
}

// Contraction of a level by its labels (prev): dense renumbering in
// ascending label order, member lists, new rows in buffer `nb` (entries in
// table order).  Returns C; rl receives every vertex's new id.
__device__ int cta_contract(const BatchCtaArgs &a, const LevelView &g, int n, int vb, long long eb, int g_idx,
                            int nb, int *gacc, CtaShared &sh)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    WarpTable &tab = sh.tab[wid];
    const int *lab = a.prev + vb;
    int *cnt = a.cnt + vb, *newid = a.newid + vb, *rl = a.rl + vb, *cursor = a.cursor + vb,
        *members = a.members + vb, *kc = a.kc + vb, *moff = a.moff + vb + g_idx, *ec = a.In + vb;
    int32_t *noffs = a.loffs[nb] + vb + g_idx;
    int32_t *nnbr = a.lnbr[nb] + eb, *nw = a.lw[nb] + eb;
    for (int c = threadIdx.x; c < n; c += kCtaThreads) cnt[c] = 0;
    __syncthreads();
    for (int v = threadIdx.x; v < n; v += kCtaThreads) atomicAdd(&cnt[lab[v]], 1);
    __syncthreads();
    const int C = cta_exclusive_scan(n, [&](int c) { return cnt[c] > 0 ? 1 : 0; }, newid, sh.scan_wt, &sh.scan_tot);
    // member starts: old communities in id order are new communities in id order
    cta_exclusive_scan(n, [&](int c) { return cnt[c]; }, cursor, sh.scan_wt, &sh.scan_tot);
    for (int c = threadIdx.x; c < n; c += kCtaThreads)
        if (cnt[c] > 0) moff[newid[c]] = cursor[c];
    if (threadIdx.x == 0) moff[C] = n;
    for (int v = threadIdx.x; v < n; v += kCtaThreads) rl[v] = newid[lab[v]];
    __syncthreads();
    for (int c = threadIdx.x; c < C; c += kCtaThreads) {
        cursor[c] = moff[c];
        ec[c] = 0;
    }
    __syncthreads();
    for (int v = threadIdx.x; v < n; v += kCtaThreads) {
        const int c = rl[v];
        members[atomicAdd(&cursor[c], 1)] = v;
        atomicAdd(&ec[c], g.end(v) - g.beg(v));
    }
    __syncthreads();
    // two passes over every community's member rows (one warp per
    // community): count the distinct neighbour communities, then, at the
    // scanned offsets, write (community, summed weight)
    auto rb = [&](int mi) { return g.beg(members[mi]); };
    auto re = [&](int mi) { return g.end(members[mi]); };
    auto kf = [&](int j) { return rl[g.nb(j)]; };
    auto wf = [&](int j) { return g.wt(j); };
    for (int pass = 0; pass < 2; ++pass) {
        for (int c = wid; c < C; c += kCtaWarps) {
            const int o = pass ? noffs[c] : 0;
            int k = 0;
            warp_aggregate(tab, gacc, moff[c], moff[c + 1], ec[c], rb, re, kf, wf, [&](int d, int s, int pos) {
                if (pass) {
                    nnbr[o + pos] = d;
                    nw[o + pos] = s;
                }
                ++k;
            });
            k = warp_sum(k);
            if (!pass && lane == 0) kc[c] = k;
        }
        __syncthreads();
        if (!pass) {
            const int Enew = cta_exclusive_scan(C, [&](int c) { return kc[c]; }, noffs, sh.scan_wt, &sh.scan_tot);
            if (threadIdx.x == 0) noffs[C] = Enew;
            __syncthreads();
        }
    }
    return C;
}

__global__ void __launch_bounds__(kCtaThreads) k_batch_cta(BatchCtaArgs a)
{
    extern __shared__ WarpTable cta_tabs[];
    __shared__ CtaShared sh;
    sh.tab = cta_tabs;  // every thread stores the same address before using it
    const int wid = threadIdx.x >> 5;
    // this warp's dense table for long rows (zero, and left zero by every use)
    int *gacc = a.gacc + ((size_t)blockIdx.x * kCtaWarps + wid) * (size_t)a.nmax;
    for (int i = threadIdx.x; i < kCtaWarps * kWT; i += kCtaThreads) {
        sh.tab[i / kWT].keys[i % kWT] = -1;
        sh.tab[i / kWT].vals[i % kWT] = 0;
    }
    __syncthreads();
    for (;;) {
        if (threadIdx.x == 0) {
            const int t = atomicAdd(a.queue, 1);
            sh.graph = t < a.G ? a.order[t] : -1;
        }
        __syncthreads();
        const int gi = sh.graph;
        __syncthreads();
        if (gi < 0) break;
        const int vb = (int)a.vstart[gi], n0 = (int)(a.vstart[gi + 1] - vb);
        const long long eb = a.estart[gi];
        const int E0 = (int)(a.estart[gi + 1] - eb);
        LevelView g{a.u_offs + vb, nullptr, eb, a.u_nbr + eb, vb, a.u_w ? a.u_w + eb : nullptr};
        long long m2 = 0;
        for (int j = threadIdx.x; j < E0; j += kCtaThreads) m2 += g.wt(j);
        m2 = cta_sum_ll(m2, sh.red_ll);
        int32_t *orig = a.labels + vb;
        for (int i = threadIdx.x; i < n0; i += kCtaThreads) orig[i] = i;
        __syncthreads();
        if (m2 <= 0 || m2 > 0x7fffffffLL) {  // no edges: singletons; too heavy for int32 sums: flagged
            if (threadIdx.x == 0) {
                if (m2 > 0) atomicOr(a.err, 1);
                a.q_out[gi] = 0.0;
                a.c_out[gi] = n0;
                a.rounds_out[gi] = 0;
                a.iters_out[gi] = 0;
            }
            __syncthreads();
            continue;
        }
        int n = n0, rounds = 0, iters_all = 0, C = n0, buf = 0;
        double prev_mod = -1.0, cur_mod = -1.0;
        for (;;) {
            double q = 0.0;
            int it = 0;
            cta_phase1(a, g, n, m2, vb, gacc, sh, &q, &it);
            iters_all += it;
            C = cta_contract(a, g, n, vb, eb, gi, buf, gacc, sh);
            const int *rl = a.rl + vb;
            for (int i = threadIdx.x; i < n0; i += kCtaThreads) orig[i] = rl[orig[i]];
            __syncthreads();
            ++rounds;
            prev_mod = cur_mod;
            cur_mod = q;
            if (!(cur_mod - prev_mod >= a.min_mod)) break;  // louvain.cu:202
            if (a.max_levels > 0 && rounds >= a.max_levels) break;
            g = LevelView{nullptr, a.loffs[buf] + vb + gi, 0, a.lnbr[buf] + eb, 0, a.lw[buf] + eb};
            n = C;
            buf ^= 1;
        }
        if (threadIdx.x == 0) {
            a.q_out[gi] = cur_mod;
            a.c_out[gi] = C;
            a.rounds_out[gi] = rounds;
            a.iters_out[gi] = iters_all;
        }
        __syncthreads();
    }
}

}  // namespace

constexpr size_t kCtaSmem = sizeof(WarpTable) * kCtaWarps;

void batch_cta_configure()
{
    cudaFuncSetAttribute(k_batch_cta, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kCtaSmem);
}

int batch_cta_grid(int G)
{
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_cta, kCtaThreads, kCtaSmem);
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long cap = (long long)(per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
    return (int)(G < cap ? G : cap);
}

size_t batch_cta_gacc_ints(int grid, int nmax) { return (size_t)grid * kCtaWarps * (size_t)nmax; }

void batch_cta_launch(const BatchCtaArgs &a, int grid, cudaStream_t st)
{
    k_batch_cta<<<grid, kCtaThreads, kCtaSmem, st>>>(a);
    note_launch(1);
}

}  // namespace gala
