// scan.cuh - exclusive prefix sum over device arrays (three passes: block
// sums, scan of the block sums in one CTA, block-local rescan with offsets).
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

template <typename Tin, typename Op>
__global__ void __launch_bounds__(kScanThreads) k_scan_reduce(const Tin *__restrict__ in, long long n, Op op,
                                                              long long *__restrict__ partial)
{
    __shared__ long long wt[32];
    __shared__ long long tot;
    long long base = (long long)blockIdx.x * kScanTile;
    long long s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        long long idx = base + (long long)i * kScanThreads + threadIdx.x;
        if (idx < n) s += op(in[idx], idx);
    }
    block_exclusive_scan<long long>(s, wt, &tot);
    if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

// Exclusive scan of the block sums in one CTA (in place); writes the grand
// total to *total_out.
template <int kDummy = 0>
__global__ void __launch_bounds__(1024) k_scan_partials(long long *partial, int nb, long long *total_out)
{
    __shared__ long long wt[32];
    __shared__ long long tot;
    long long carry = 0;
    for (int base = 0; base < nb; base += 1024) {
        int i = base + threadIdx.x;
        long long v = i < nb ? partial[i] : 0;
        long long ex = block_exclusive_scan<long long>(v, wt, &tot);
        if (i < nb) partial[i] = ex + carry;
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[nb] = carry;
        if (total_out) *total_out = carry;
    }
}

template <typename Tin, typename Tout, typename Op>
__global__ void __launch_bounds__(kScanThreads) k_scan_down(const Tin *__restrict__ in, Tout *__restrict__ out,
                                                            long long n, Op op,
                                                            const long long *__restrict__ partial)
{
    __shared__ long long wt[32];
    __shared__ long long tot;
    long long base = (long long)blockIdx.x * kScanTile + (long long)threadIdx.x * kScanItems;
    long long v[kScanItems];
    long long s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        long long idx = base + i;
        v[i] = idx < n ? op(in[idx], idx) : 0;
        s += v[i];
    }
    long long pre = block_exclusive_scan<long long>(s, wt, &tot) + partial[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        long long idx = base + i;
        if (idx < n) out[idx] = (Tout)pre;
        pre += v[i];
    }
}

// Host wrapper: out[i] = sum_{j<i} op(in[j]); *total_out (device) = sum of all.
// partial needs ceil(n / kScanTile) + 1 slots.
void note_launch(int k);

template <typename Tin, typename Tout, typename Op>
void exclusive_scan(const Tin *in, Tout *out, long long n, Op op, long long *partial,
                    long long *total_out, cudaStream_t st)
{
    int nb = (int)((n + kScanTile - 1) / kScanTile);
    if (nb < 1) nb = 1;
    k_scan_reduce<Tin, Op><<<nb, kScanThreads, 0, st>>>(in, n, op, partial);
    k_scan_partials<0><<<1, 1024, 0, st>>>(partial, nb, total_out);
    k_scan_down<Tin, Tout, Op><<<nb, kScanThreads, 0, st>>>(in, out, n, op, partial);
    note_launch(3);
}

}  // namespace gala
