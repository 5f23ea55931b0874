// walk.cuh - warp walks over contiguous entry ranges of a CSR-like row list.
//
// A walk list holds rows that all have entries (row ends in offs_ll); a warp
// takes a range of consecutive entries and finds the row of each with a
// window of 32 row ends held one per lane.  Used by the contraction (stream
// fill, compaction) and by the incremental weight update (movers' rows).
#pragma once
#include <limits.h>

#include "common.cuh"

namespace gala {

// ---------------------------------------------------------------------------
// Row window: the 32 row ends offs[vbase+1 .. vbase+32] held one per lane.
// ---------------------------------------------------------------------------
struct RowWindow {
    const int64_t *offs;
    const long long *offs_ll;
    int n;
    int vbase;
    long long rowend;
    __device__ __forceinline__ long long at(int k) const
    {
        return offs ? (long long)offs[k] : offs_ll[k];
    }
    __device__ __forceinline__ void load()
    {
        const int k = vbase + 1 + (int)(threadIdx.x & 31);
        rowend = k <= n ? at(k) : LLONG_MAX;
    }
    // number of window rows that end at or before entry j (0..32)
    __device__ __forceinline__ int count_le(long long j) const
    {
        int cnt = 0;
#pragma unroll
        for (int s = 16; s >= 1; s >>= 1) {
            const long long r = __shfl_sync(GALA_FULL_MASK, rowend, cnt + s - 1);
            if (r <= j) cnt += s;
        }
        // every lane takes part in the shuffle (a full-mask shuffle behind a
        // lane-dependent condition is undefined)
        const long long last = __shfl_sync(GALA_FULL_MASK, rowend, 31);
        if (cnt == 31 && last <= j) cnt = 32;
        return cnt;
    }
};

// Owner row of entry j0 (the last v with offs_ll[v] <= j0), found by the
// whole warp: every round the 32 lanes probe 32 evenly spaced rows of
// [lo, hi] and the ballot keeps the interval of the last row starting at or
// before j0 (5 rounds for 2^25 rows instead of 25 dependent loads).
// offs_ll[0] <= j0 < offs_ll[n]; all lanes call.
__device__ __forceinline__ int warp_owner_row(const long long *offs_ll, int n, long long j0)
{
    const int lane = threadIdx.x & 31;
    int lo = 0, hi = n - 1;
    while (hi > lo) {
        const long long span = (long long)(hi - lo) + 1;
        const int p = lo + (int)((span * lane) >> 5);
        const unsigned m = __ballot_sync(GALA_FULL_MASK, offs_ll[p] <= j0);
        const int k = m ? 31 - __clz((int)m) : 0;
        const int nlo = lo + (int)((span * k) >> 5);
        hi = (k == 31) ? hi : lo + (int)((span * (k + 1)) >> 5) - 1;
        lo = nlo;
    }
    return lo;
}

// Cursor over a walk list (rows that all have entries, row ends in offs_ll):
// a window of 32 rows, one per lane, with their ends and two values per row
// (rowval(row, &pa, &pb), loaded when the window moves; rows past the list
// keep (-1, 0)).  32 consecutive entries span at most 32 such rows, so once
// the window starts at the owner of a batch's first entry it holds the whole
// batch.  The window moves only when a batch ends past it: with rows of a
// few dozen entries it is loaded once or twice per 1024-entry task, not once
// per batch.
template <typename RV>
struct RowCursor {
    RowWindow w;
    RV rowval;
    long long pa, pb;
    long long wend;  // end of the window's last row
    __device__ __forceinline__ void load()
    {
        w.load();
        wend = __shfl_sync(GALA_FULL_MASK, w.rowend, 31);
        const int r = w.vbase + (int)(threadIdx.x & 31);
        pa = -1;
        pb = 0;
        if (r < w.n) rowval(r, pa, pb);
    }
    __device__ __forceinline__ void start(long long j0)
    {
        w.vbase = warp_owner_row(w.offs_ll, w.n, j0);
        load();
    }
    // start at row r, the owner of the task's first entry (known)
    __device__ __forceinline__ void start_row(int r)
    {
        w.vbase = r;
        load();
    }
    // Batches are resolved in ascending order.  Entry j = jb + lane (this
    // lane's entry of the batch [jb, jl]) receives its row's values; returns
    // false when j lies outside the window, which a walk list never produces.
    // All lanes call.  The row of entry jb + k is the number of window rows
    // that end at or before it: the rows ending at or before jb (one ballot)
    // plus the row ends inside the batch, which are distinct (rows have
    // entries) and so form a bit mask over the batch (one OR-reduction).
    __device__ __forceinline__ bool resolve(long long jb, long long jl, long long j, long long &a, long long &b)
    {
        if (jl >= wend) {  // the batch ends past the window
            w.vbase += w.count_le(jb);
            load();
        }
        const int before = __popc(__ballot_sync(GALA_FULL_MASK, w.rowend <= jb));
        const long long q = w.rowend - jb;  // the row's end, relative to the batch
        const unsigned ends = __reduce_or_sync(GALA_FULL_MASK, (q >= 1 && q <= 31) ? (1u << (int)q) : 0u);
        const int k = (int)(j - jb);  // == lane
        const int idx = before + __popc(ends & ((2u << k) - 2u));
        a = __shfl_sync(GALA_FULL_MASK, pa, idx & 31);
        b = __shfl_sync(GALA_FULL_MASK, pb, idx & 31);
        return idx < 32;
    }
};

template <typename RV>
__device__ __forceinline__ RowCursor<RV> row_cursor(const long long *offs_ll, int n, RV rv)
{
    return RowCursor<RV>{RowWindow{nullptr, offs_ll, n, 0, 0}, rv, -1, 0};
}

// Batches of 32 entries a warp keeps in flight in the walk kernels (their
// loads are independent; one batch at a time leaves them latency-bound).
constexpr int kWalkUnroll = 4;

}  // namespace gala
