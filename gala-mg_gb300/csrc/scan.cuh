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

// Exclusive scan in two launches over a resident grid (reduce, then scan):
// block b owns the tiles [b * per, (b + 1) * per) of kScanTile items.  The
// first launch writes each block's sum to partial[b]; the second gives every
// block its prefix (the sum of the partials before it) and scans its tiles in
// order with a running carry.  No block waits for another.  (A single-pass
// scan with decoupled look-back, Merrill & Garland 2016, measured 25 us for
// 2.7M items: its warps stalled at the block barrier while warp 0 waited for
// the look-back to reach back to a published prefix.)
//
// With dlen the length is min(*dlen, n), read on the device: items past it
// are not written.
template <typename Tlen>
__device__ __forceinline__ long long scan_len(long long n, const Tlen *dlen)
{
    if (!dlen) return n;
    const long long d = (long long)*dlen;
    return d < 0 ? 0 : (d < n ? d : n);
}

// Block-wide sum (every thread gets it); ws: 32 slots.
__device__ __forceinline__ long long scan_block_sum(long long x, long long *ws)
{
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) x += __shfl_xor_sync(GALA_FULL_MASK, x, o);
    if (lane == 0) ws[wid] = x;
    __syncthreads();
    long long t = lane < nw ? ws[lane] : 0;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) t += __shfl_xor_sync(GALA_FULL_MASK, t, o);
    __syncthreads();
    return t;
}

// A thread's kScanItems consecutive items from / to global memory: 16-byte
// accesses when the run is whole and aligned (a warp's scalar accesses at
// kScanItems-item strides queue in the load/store unit), else item by item.
template <typename T>
__device__ __forceinline__ void scan_load_items(const T *__restrict__ p, long long base, long long n,
                                                T (&x)[kScanItems])
{
    if constexpr (sizeof(T) == 4 || sizeof(T) == 8) {
        if (base + kScanItems <= n && (reinterpret_cast<uintptr_t>(p + base) & 15) == 0) {
            constexpr int kVec = 16 / sizeof(T);
#pragma unroll
            for (int j = 0; j < kScanItems; j += kVec) {
                const int4 q = *reinterpret_cast<const int4 *>(p + base + j);
                memcpy(&x[j], &q, 16);
            }
            return;
        }
    }
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) x[i] = base + i < n ? p[base + i] : T{};
}
template <typename T>
__device__ __forceinline__ void scan_store_items(T *__restrict__ p, long long base, long long n,
                                                 const T (&x)[kScanItems])
{
    if constexpr (sizeof(T) == 4 || sizeof(T) == 8) {
        if (base + kScanItems <= n && (reinterpret_cast<uintptr_t>(p + base) & 15) == 0) {
            constexpr int kVec = 16 / sizeof(T);
#pragma unroll
            for (int j = 0; j < kScanItems; j += kVec) {
                int4 q;
                memcpy(&q, &x[j], 16);
                *reinterpret_cast<int4 *>(p + base + j) = q;
            }
            return;
        }
    }
#pragma unroll
    for (int i = 0; i < kScanItems; ++i)
        if (base + i < n) p[base + i] = x[i];
}

template <typename Tin, typename Op, typename Tlen>
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const Tin *__restrict__ in, long long n, Op op,
                                                              long long *partial, const Tlen *dlen)
{
    __shared__ long long ws[32];
    n = scan_len(n, dlen);
    const long long ntiles = (n + kScanTile - 1) / kScanTile;
    const long long per = (ntiles + gridDim.x - 1) / gridDim.x;
    const long long i0 = blockIdx.x * per * kScanTile;
    long long i1 = i0 + per * kScanTile;
    if (i1 > n) i1 = n;
    long long s = 0;
    for (long long idx = i0 + threadIdx.x; idx < i1; idx += kScanThreads) s += op(in[idx], idx);  // coalesced
    s = scan_block_sum(s, ws);
    if (threadIdx.x == 0) partial[blockIdx.x] = s;
}

template <typename Tin, typename Tout, typename Op, typename Tlen>
__global__ void __launch_bounds__(kScanThreads) k_scan_apply(const Tin *__restrict__ in, Tout *__restrict__ out,
                                                             long long n, Op op, const long long *__restrict__ partial,
                                                             long long *total_out, const Tlen *dlen)
{
    __shared__ long long wt[32];
    __shared__ long long tot;
    n = scan_len(n, dlen);
    const long long ntiles = (n + kScanTile - 1) / kScanTile;
    const long long per = (ntiles + gridDim.x - 1) / gridDim.x;
    long long carry = 0;
    for (int q = threadIdx.x; q < (int)blockIdx.x; q += kScanThreads) carry += partial[q];
    carry = scan_block_sum(carry, wt);
    const long long t0 = blockIdx.x * per;
    const long long t1 = t0 + per < ntiles ? t0 + per : ntiles;
    for (long long t = t0; t < t1; ++t) {
        const long long base = t * kScanTile + (long long)threadIdx.x * kScanItems;
        Tin raw[kScanItems];
        scan_load_items(in, base, n, raw);
        long long v[kScanItems];
        long long s = 0;
#pragma unroll
        for (int i = 0; i < kScanItems; ++i) {
            const long long idx = base + i;
            v[i] = idx < n ? op(raw[i], idx) : 0;
            s += v[i];
        }
        long long pre = carry + block_exclusive_scan<long long>(s, wt, &tot);
        Tout o[kScanItems];
#pragma unroll
        for (int i = 0; i < kScanItems; ++i) {
            o[i] = (Tout)pre;
            pre += v[i];
        }
        scan_store_items(out, base, n, o);
        carry += tot;
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0 && total_out) *total_out = carry;
}

// Blocks of the scan grid: as many as are resident, at most one per tile.
inline int scan_blocks(long long n)
{
    static int cap = 0;
    if (cap == 0) {
        int dev = 0, sms = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cap = (sms > 0 ? sms : 148) * (2048 / kScanThreads);
    }
    long long nb = (n + kScanTile - 1) / kScanTile;
    if (nb > cap) nb = cap;
    if (nb < 1) nb = 1;
    return (int)nb;
}

// Host wrapper: out[i] = sum_{j<i} op(in[j]); *total_out (device) = sum of all.
// partial needs ceil(n / kScanTile) + 2 slots.  err is kept for the callers
// (the two launches never wait, so no error bit is set).
void note_launch(int k);

template <typename Tin, typename Tout, typename Op>
void exclusive_scan(const Tin *in, Tout *out, long long n, Op op, long long *partial, long long *total_out,
                    cudaStream_t st, int *err = nullptr)
{
    (void)err;
    const int nb = scan_blocks(n);
    k_scan_reduce<Tin, Op, int><<<nb, kScanThreads, 0, st>>>(in, n, op, partial, nullptr);
    k_scan_apply<Tin, Tout, Op, int><<<nb, kScanThreads, 0, st>>>(in, out, n, op, partial, total_out, nullptr);
    note_launch(2);
}

// The same over the first min(*dlen, nmax) items, dlen on the device: the
// host needs no count, so nothing waits for the device.
template <typename Tin, typename Tout, typename Op, typename Tlen>
void exclusive_scan_dev(const Tin *in, Tout *out, long long nmax, const Tlen *dlen, Op op, long long *partial,
                        long long *total_out, cudaStream_t st, int *err = nullptr)
{
    (void)err;
    const int nb = scan_blocks(nmax);
    k_scan_reduce<Tin, Op, Tlen><<<nb, kScanThreads, 0, st>>>(in, nmax, op, partial, dlen);
    k_scan_apply<Tin, Tout, Op, Tlen><<<nb, kScanThreads, 0, st>>>(in, out, nmax, op, partial, total_out, dlen);
    note_launch(2);
}

}  // namespace gala
