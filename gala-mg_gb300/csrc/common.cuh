// common.cuh - device helpers shared by the phase-1, contraction and scan
// kernels of the GB300 Louvain engine (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "binlimits.h"

#define GALA_FULL_MASK 0xffffffffu

namespace gala {

// ---------------------------------------------------------------------------
// Degree bins of the decide-and-move and weight-update sweeps.
//   bin 0..3: deg 1-4 / 5-8 / 9-16 / 17-32 -> a group of 4/8/16/32 lanes per
//             vertex, one neighbour per lane, aggregation by shuffles (groups
//             of 4-16 lanes) or __match_any_sync (whole warps)
//   bin 4   : deg 33-256     -> one warp per vertex, 256-slot smem hash up to
//                               128 entries, else 512
//   bin 5   : deg 257-2048   -> one 256-thread CTA per vertex (512 by option),
//                               2048-slot smem hash up to 1024 entries, else 4096
//   bin 6   : deg 2049-8192  -> one 1024-thread CTA per vertex, 8192-slot smem
//                               hash up to 4096 entries, else 16384
//   bin 7   : deg > 8192     -> hub rows: global hash tables filled and scanned
//                               by many CTAs (4096-entry / 4096-slot chunks)
//   bin 8   : deg 0          -> never processed (the reference bins start at 1,
//                               louvain_main_process.cu:278)
// ---------------------------------------------------------------------------
constexpr int kNumBins = 8;
constexpr int kNumBinSlots = 9;

__host__ __device__ inline int bin_of_degree(int64_t d, const BinLimits &l)
{
    if (d <= 0) return 8;
    if (d <= 4) return 0;
    if (d <= 8) return 1;
    if (d <= 16) return 2;
    if (d <= 32) return 3;
    if (d <= l.m4) return 4;
    if (d <= l.m5) return 5;
    if (d <= l.m6) return 6;
    return 7;
}

__host__ __device__ inline int bin_of_degree(int64_t d)
{
    if (d <= 0) return 8;
    if (d <= 4) return 0;
    if (d <= 8) return 1;
    if (d <= 16) return 2;
    if (d <= 32) return 3;
    if (d <= 256) return 4;
    if (d <= 2048) return 5;
    if (d <= 8192) return 6;
    return 7;
}

// Device-side counters of one context (one instance in device memory, mirrored
// to pinned host memory once per iteration).
struct DevStats {
    unsigned long long sum_in;      // sum over vertices of In[v]
    unsigned long long sum_tot2;    // sum over communities of Tot[c]^2 (low word)
    unsigned long long sum_tot2_hi; // high word (64-bit fixed-point weights)
    unsigned long long sum_self;    // sum of self-loop weights (level init)
    unsigned long long sum_k;       // sum of K = total weight m2 (level init)
    unsigned long long act_edges[2];   // sum of degrees in the active lists
    int act_vertices[2];
    long long min_tot;              // min over non-empty communities of Tot
    int n_movers;                   // movers of the current iteration
    int err;                        // error bits (kErr*)
    int max_deg;
    int num_communities;            // contraction: C
    int nz_rows;                    // contraction: rows with entries (walk list)
    int bin_start[kNumBinSlots + 1];  // order list: start of each bin
    int act_count[2][kNumBins];       // active list counts (ping-pong)
    int small_cnt[6];                 // contraction: communities per size class
    long long total2;                 // scratch total of a second scan
    long long total3;                 // scratch total of a third scan
    long long total;                  // scratch total of the last scan
    unsigned long long fp64_decisions; // vertices decided with the FP64 expressions
    // move-proposal modes
    int prop_count[kNumBins];          // vertices the network proposes, per bin
    long long trace_mark;              // sample count before the current sweep
    unsigned long long skipped;        // active vertices not decided (proposal said stay)
    unsigned long long skipped_edges;  // row entries of the skipped vertices
    // contraction counts that stay on the device between its kernels
    long long ccount;       // communities C
    long long new_entries;  // entries of the contracted level
    long long big_slots;    // long rows: table slots
    long long big_nwork;    // long rows: stream chunks
    long long big_ntwork;   // long rows: table chunks
    long long big_lwork;    // long rows: slot-list chunks
    // long rows by key range: pool offsets (ints) and counts
    long long rad_offm;     // per-chunk bucket offsets (uint16)
    long long rad_items;    // work items
    long long rad_acc;      // accumulators of buckets split over several CTAs
    long long rad_max_items;
    long long rad_max_acc;
    int rad_nb;             // buckets per row: ceil(C / 8192)
    int rad_nitems;         // items planned
    int rad_nacc;           // accumulators taken
    int rad_next;           // item queue head
    // incremental weight update
    unsigned long long mv_edges;  // row entries of this sweep's movers
    long long push_total;         // the same, summed by the movers' prefix
    unsigned long long sym_hash;  // 0 when the graph is symmetric (hash of every entry minus its mirror)
    int push_mode;                // 1: this sweep updates In incrementally (the per-bin updates return at once)
    int push_len;                 // movers in the prefix scan (0 unless push_mode)
};

constexpr int kErrHashOverflow = 1;
constexpr int kErrProbeLimit = 2;
constexpr int kErrBadLabel = 4;
constexpr int kErrBadIndex = 8;
constexpr int kErrCapacity = 16;  // contraction: long-row tables exceed their scratch

// ---------------------------------------------------------------------------
// Weight types.  Integer graphs (the reference's int32 weights) run with
// WT = int32_t: weights, K, Self, Tot and In are int32 and most decisions are
// taken in exact integer arithmetic.  Float-weight graphs run with
// WT = int64_t: every float weight is held as an exact 64-bit fixed-point
// integer (weight * 2^S), so all sums (K, Tot, In, contracted weights) are
// exact and independent of the order of the atomics, and every gain is
// evaluated with the FP64 expressions.
// ---------------------------------------------------------------------------
template <typename WT>
struct WideOf {
    static constexpr bool exact = sizeof(WT) == 4;  // exact-integer decisions available
};

// Sum of w over the lanes of mask m (all lanes of m call with their w).
__device__ __forceinline__ int group_sum(unsigned m, int w) { return (int)__reduce_add_sync(m, (unsigned)w); }
// 64-bit values (0 <= w < 2^63) in three 21-bit limbs: a limb sum over 32
// lanes stays below 2^26.
__device__ __forceinline__ long long group_sum(unsigned m, long long w)
{
    const unsigned long long u = (unsigned long long)w;
    const unsigned l0 = __reduce_add_sync(m, (unsigned)(u & 0x1fffff));
    const unsigned l1 = __reduce_add_sync(m, (unsigned)((u >> 21) & 0x1fffff));
    const unsigned l2 = __reduce_add_sync(m, (unsigned)(u >> 42));
    return (long long)((unsigned long long)l0 + ((unsigned long long)l1 << 21) + ((unsigned long long)l2 << 42));
}

__device__ __forceinline__ void atomic_add_w(int *p, int v) { atomicAdd(p, v); }
__device__ __forceinline__ void atomic_add_w(long long *p, long long v)
{
    atomicAdd((unsigned long long *)p, (unsigned long long)v);  // two's complement: also subtracts
}

// ---------------------------------------------------------------------------
// FP64 gain of a candidate community, same operation order as the reference
// (kernel_functions.cu:136, :171, :202, :362):
//   2*w - 2*K*((Tot_c - Tot_cur) + K) * (1/m2)
// Written with explicit round-to-nearest intrinsics so that no FMA contraction
// changes the rounding; the CPU oracle is compiled with -ffp-contract=off.
// ---------------------------------------------------------------------------
template <typename WT>
__device__ __forceinline__ double gain_dq(WT w_to_c, WT ki, WT tot_c, WT tot_cur, double constant)
{
    double a = __dmul_rn(2.0, (double)w_to_c);
    double b = __dmul_rn(2.0, (double)ki);
    double t = __dadd_rn(__dsub_rn((double)tot_c, (double)tot_cur), (double)ki);
    return __dsub_rn(a, __dmul_rn(__dmul_rn(b, t), constant));
}

// (maxdq - 2*w_cur) + 2*Self  (kernel_functions.cu:381 / :532 / :748)
template <typename WT>
__device__ __forceinline__ double gain_correct(double maxdq, WT w_cur, WT self_w)
{
    return __dadd_rn(__dsub_rn(maxdq, (double)(2 * w_cur)), (double)(2 * self_w));
}

// Pruning bound of compute_In (kernel_functions.cu:944, :1028):
//   2*(In-Self) - (K-Self) + (double)(minTot - (Tot_c - K)) * (1/m2) * K > 0
template <typename WT>
__device__ __forceinline__ bool prune_bound(WT in_w, WT self_w, WT ki, WT min_tot, WT tot_c, double constant)
{
    WT ip = 2 * (in_w - self_w) - (ki - self_w);
    double d = __dmul_rn(__dmul_rn((double)(min_tot - (tot_c - ki)), constant), (double)ki);
    return __dadd_rn((double)ip, d) > 0.0;
}

// The same bound decided in exact integers: P = ip*m2 + (minTot - (Tot_c - K))*K
// has the sign of the FP64 expression whenever P != 0 and K*m2 < 2^49 (the
// FP64 error is below K*2^-50, non-zero P/m2 is at least 1/m2 away from 0);
// otherwise the FP64 expression decides, as in the reference.
template <typename WT>
__device__ __forceinline__ bool prune_bound_fast(WT in_w, WT self_w, WT ki, WT min_tot, WT tot_c, double constant,
                                                 long long m2)
{
    if constexpr (WideOf<WT>::exact) {
        if ((long long)ki * m2 < (1LL << 49)) {
            const int ip = 2 * (in_w - self_w) - (ki - self_w);
            const long long p = (long long)ip * m2 + (long long)(min_tot - (tot_c - ki)) * (long long)ki;
            if (p != 0) return p > 0;
        }
    }
    return prune_bound(in_w, self_w, ki, min_tot, tot_c, constant);
}

// Candidate order: larger gain first, then the lower community id.
__device__ __forceinline__ bool cand_better(double dq_a, int c_a, double dq_b, int c_b)
{
    return dq_a > dq_b || (dq_a == dq_b && c_a < c_b);
}

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Smallest power of two >= x (x <= 2^40).
__host__ __device__ inline long long next_pow2_ll(long long x)
{
    long long p = 1;
    while (p < x && p < (1LL << 40)) p <<= 1;
    return p;
}
__host__ __device__ inline int next_pow2_int(long long x)
{
    long long p = next_pow2_ll(x);
    return p > (1LL << 30) ? (1 << 30) : (int)p;
}

// Open-addressing hash table with linear probing; keys int32 (-1 = empty),
// int32 weight sums.  T is a power of two; at most T probes.
__device__ __forceinline__ unsigned hash_slot(int key, int log2t)
{
    return ((unsigned)key * 0x9E3779B1u) >> (32 - log2t);
}

template <typename VT>
__device__ __forceinline__ bool hash_add(int *keys, VT *vals, int T, int log2t, int key, VT w)
{
    unsigned h = hash_slot(key, log2t);
    for (int p = 0; p < T; ++p) {
        int k = *(volatile int *)&keys[h];
        if (k == -1) {
            k = atomicCAS(&keys[h], -1, key);
            if (k == -1) k = key;
        }
        if (k == key) {
            atomic_add_w(&vals[h], w);
            return true;
        }
        h = (h + 1) & (unsigned)(T - 1);
    }
    return false;
}

// Warp-aggregated append of one item per flagged lane to list[*counter ...].
// Must be called by all 32 lanes.
__device__ __forceinline__ void warp_append(bool flag, int value, int *list, int *counter)
{
    unsigned b = __ballot_sync(GALA_FULL_MASK, flag);
    if (b == 0) return;
    int lane = threadIdx.x & 31;
    int leader = __ffs(b) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(counter, __popc(b));
    base = __shfl_sync(GALA_FULL_MASK, base, leader);
    if (flag) list[base + __popc(b & lanemask_lt())] = value;
}

// Per-warp staging of list appends: a warp gathers its items in a
// shared-memory buffer of N slots and hands them out with one counter atomic
// per full buffer (appends of a whole grid to one counter otherwise queue on
// that counter).  All 32 lanes call push and flush; flush is needed at the end.
template <int N, int K>
struct WarpStage {
    int *buf;  // K * N ints of shared memory, this warp's
    int n;     // items held (warp-uniform)
    __device__ __forceinline__ void flush(int *const *lists, int *counter)
    {
        __syncwarp();
        if (n == 0) return;
        const int lane = threadIdx.x & 31;
        int base = 0;
        if (lane == 0) base = atomicAdd(counter, n);
        base = __shfl_sync(GALA_FULL_MASK, base, 0);
#pragma unroll
        for (int k = 0; k < K; ++k)
            for (int i = lane; i < n; i += 32) lists[k][base + i] = buf[k * N + i];
        __syncwarp();
        n = 0;
    }
    __device__ __forceinline__ void push(bool flag, const int (&vals)[K], int *const *lists, int *counter)
    {
        const unsigned b = __ballot_sync(GALA_FULL_MASK, flag);
        if (b == 0) return;
        if (n + 32 > N) flush(lists, counter);
        if (flag) {
            const int p = n + __popc(b & lanemask_lt());
#pragma unroll
            for (int k = 0; k < K; ++k) buf[k * N + p] = vals[k];
        }
        n += __popc(b);
    }
};

template <typename T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v += __shfl_xor_sync(GALA_FULL_MASK, v, o);
    return v;
}

// ---------------------------------------------------------------------------
// Block reductions into the device counters (all threads must call).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void block_add_u64(unsigned long long v, unsigned long long *dst)
{
    __shared__ unsigned long long red[32];
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        unsigned long long t = lane < (int)(blockDim.x >> 5) ? red[lane] : 0ull;
        t = warp_sum(t);
        if (lane == 0 && t) atomicAdd(dst, t);
    }
    __syncthreads();
}

__device__ __forceinline__ void block_add_i32(int v, int *dst)
{
    __shared__ int red[32];
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) red[wid] = v;
    __syncthreads();
    if (wid == 0) {
        int t = lane < (int)(blockDim.x >> 5) ? red[lane] : 0;
        t = warp_sum(t);
        if (lane == 0 && t) atomicAdd(dst, t);
    }
    __syncthreads();
}

}  // namespace gala
