// scan.cuh - exclusive prefix sum over device arrays in one pass (tiles chained
// by decoupled look-back).
// Used for the degree-bin counting sort, the community renumbering and the
// CSR offsets of the contraction.  Input values pass through a functor, so a
// flag (x > 0) or a cap (min(x, C)) needs no separate pass.
#pragma once
#include "common.cuh"

namespace gala {

constexpr int kScanThreads = 512;
constexpr int kScanItems = 8;  // per thread
constexpr int kScanTile = kScanThreads * kScanItems;

struct OpIdentity {
    template <typename T>
    __device__ __forceinline__ long long operator()(T x, long long) const { return (long long)x; }
};
struct OpPositive {
    template <typename T>
    __device__ __forceinline__ long long operator()(T x, long long) const { return x > 0 ? 1 : 0; }
};
struct OpCap {
    long long cap;
    template <typename T>
    __device__ __forceinline__ long long operator()(T x, long long) const
    {
        return (long long)x < cap ? (long long)x : cap;
    }
};
struct OpCapDev {  // cap read on the device
    const long long *cap;
    template <typename T>
    __device__ __forceinline__ long long operator()(T x, long long) const
    {
        const long long c = *cap;
        return (long long)x < c ? (long long)x : c;
    }
};

template <typename T>
__device__ __forceinline__ T block_exclusive_scan(T v, T *warp_tot, T *block_total)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    T incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(GALA_FULL_MASK, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) warp_tot[wid] = incl;
    __syncthreads();
    if (wid == 0) {
        const int nw = blockDim.x >> 5;
        T t = lane < nw ? warp_tot[lane] : (T)0;
        T ti = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(GALA_FULL_MASK, ti, o);
            if (lane >= o) ti += y;
        }
        if (lane < nw) warp_tot[lane] = ti - t;
        if (lane == nw - 1) *block_total = ti;
    }
    __syncthreads();
    T r = warp_tot[wid] + incl - v;
    __syncthreads();
    return r;
}

// Single-pass exclusive scan with decoupled look-back (Merrill & Garland,
// "Single-pass Parallel Prefix Scan with Decoupled Look-back", 2016).  Each
// tile of kScanTile items takes its id from a counter in launch order, so it
// only ever waits for tiles that already run; it publishes its aggregate,
// then (after looking back) its inclusive prefix, as one 64-bit word:
// flag in the top two bits, value below (values are non-negative and below
// 2^62).  The look-back reads 32 predecessors per step, one per lane of
// warp 0.  Every wait is bounded: a tile that waited kScanSpinLimit rounds
// records kScanErrBit in *err and counts that predecessor as 0.
constexpr unsigned long long kScanFlagAgg = 1ull << 62;
constexpr unsigned long long kScanFlagPre = 2ull << 62;
constexpr unsigned long long kScanValMask = (1ull << 62) - 1;
constexpr int kScanSpinLimit = 1 << 20;
constexpr int kScanErrBit = 2;  // the engine's probe-limit error bit

__device__ __forceinline__ unsigned long long scan_ld(const unsigned long long *p)
{
    unsigned long long v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void scan_st(unsigned long long *p, unsigned long long v)
{
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// status: nb + 2 words, zero on entry; status[nb] is the tile counter.
// With dlen, the length is min(*dlen, n), read on the device (n bounds the
// grid): items past it are not written, tiles wholly past it leave at once
// (tiles look back only at tiles of lower id, and ids follow launch order),
// and the tile of the last item writes the total.
template <typename Tin, typename Tout, typename Op, typename Tlen>
__global__ void __launch_bounds__(kScanThreads) k_scan_onepass(const Tin *__restrict__ in, Tout *__restrict__ out,
                                                               long long n, Op op, unsigned long long *status, int nb,
                                                               long long *total_out, int *err, const Tlen *dlen)
{
    __shared__ long long wt[32];
    __shared__ long long tot;
    __shared__ int s_tile;
    __shared__ long long s_excl;
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(&status[nb], 1ull);
    if (dlen) {
        const long long d = (long long)*dlen;
        n = d < 0 ? 0 : (d < n ? d : n);
    }
    __syncthreads();
    const int tile = s_tile;
    const int last_tile = dlen ? (n > 0 ? (int)((n - 1) / kScanTile) : 0) : nb - 1;
    if (tile > last_tile) return;  // block-uniform
    const long long base = (long long)tile * kScanTile + (long long)threadIdx.x * kScanItems;
    long long v[kScanItems];
    long long s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const long long idx = base + i;
        v[i] = idx < n ? op(in[idx], idx) : 0;
        s += v[i];
    }
    long long pre = block_exclusive_scan<long long>(s, wt, &tot);
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        const unsigned long long agg = (unsigned long long)tot & kScanValMask;
        long long excl = 0;
        if (tile == 0) {
            if (lane == 0) scan_st(&status[0], kScanFlagPre | agg);
        } else {
            if (lane == 0) scan_st(&status[tile], kScanFlagAgg | agg);
            int p = tile - 1;  // lane k looks at tile p - k
            bool timed_out = false;
            for (;;) {
                const int t = p - lane;
                unsigned long long w = kScanFlagPre;  // tiles before 0 count as prefix 0
                if (t >= 0) {
                    int it = 0;
                    for (;;) {
                        w = scan_ld(&status[t]);
                        if (w >> 62) break;
                        if (++it > kScanSpinLimit) {
                            timed_out = true;
                            w = kScanFlagPre;
                            break;
                        }
                        __nanosleep(32);
                    }
                }
                const unsigned pm = __ballot_sync(GALA_FULL_MASK, (w >> 62) == 2ull);
                const int kstar = pm ? __ffs(pm) - 1 : 32;
                long long c = lane <= kstar ? (long long)(w & kScanValMask) : 0;
#pragma unroll
                for (int o = 16; o >= 1; o >>= 1) c += __shfl_xor_sync(GALA_FULL_MASK, c, o);
                excl += c;
                if (pm) break;
                p -= 32;
            }
            if (__any_sync(GALA_FULL_MASK, timed_out) && lane == 0 && err) atomicOr(err, kScanErrBit);
            if (lane == 0) scan_st(&status[tile], kScanFlagPre | (((unsigned long long)excl + agg) & kScanValMask));
        }
        if (lane == 0) s_excl = excl;
    }
    __syncthreads();
    pre += s_excl;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const long long idx = base + i;
        if (idx < n) out[idx] = (Tout)pre;
        pre += v[i];
    }
    if (tile == last_tile && threadIdx.x == 0 && total_out) *total_out = s_excl + tot;
}

// Host wrapper: out[i] = sum_{j<i} op(in[j]); *total_out (device) = sum of all.
// partial needs ceil(n / kScanTile) + 2 slots (the tile status words and the
// counter).  err (device, may be null) receives kScanErrBit if a wait ran out.
void note_launch(int k);

template <typename Tin, typename Tout, typename Op>
void exclusive_scan(const Tin *in, Tout *out, long long n, Op op, long long *partial, long long *total_out,
                    cudaStream_t st, int *err = nullptr)
{
    int nb = (int)((n + kScanTile - 1) / kScanTile);
    if (nb < 1) nb = 1;
    unsigned long long *status = (unsigned long long *)partial;
    cudaMemsetAsync(status, 0, ((size_t)nb + 2) * sizeof(unsigned long long), st);
    k_scan_onepass<Tin, Tout, Op, int><<<nb, kScanThreads, 0, st>>>(in, out, n, op, status, nb, total_out, err,
                                                                    nullptr);
    note_launch(1);
}

// The same over the first min(*dlen, nmax) items, dlen on the device: the
// host needs no count, so nothing waits for the device.
template <typename Tin, typename Tout, typename Op, typename Tlen>
void exclusive_scan_dev(const Tin *in, Tout *out, long long nmax, const Tlen *dlen, Op op, long long *partial,
                        long long *total_out, cudaStream_t st, int *err = nullptr)
{
    int nb = (int)((nmax + kScanTile - 1) / kScanTile);
    if (nb < 1) nb = 1;
    unsigned long long *status = (unsigned long long *)partial;
    cudaMemsetAsync(status, 0, ((size_t)nb + 2) * sizeof(unsigned long long), st);
    k_scan_onepass<Tin, Tout, Op, Tlen><<<nb, kScanThreads, 0, st>>>(in, out, nmax, op, status, nb, total_out, err,
                                                                     dlen);
    note_launch(1);
}

}  // namespace gala
