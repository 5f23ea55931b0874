// Leiden-style refinement of a level's phase-1 partition (no counterpart in
// the reference; gala_options.refine).  Deterministic synchronous rule,
// restated on the host by the oracle (refine_w64 in oracle/louvain_oracle.c):
//
//   every vertex starts as its own sub-community of its community C = P[v];
//   per sweep, a singleton v with 1..kRefineMaxDeg row entries that is well
//   connected, w(v, C - v) m2 >= K_v (Tot_C - K_v), targets among the well
//   connected sub-communities r of C next to it (ext(r) m2 >= K_r (Tot_C -
//   K_r), ext(r) = weight from r to the rest of C) the one of largest
//   X = w(v, r) m2 - K_v K_r (lowest id on ties), when X > 0;
//   a vertex moves to its target unless another vertex targets it, except
//   when exactly one does and that is its own target with a lower id;
//   sweeps repeat while vertices move, at most kRefineSweeps times.
//
// Integer weights (WT = int): every sum is below m2 < 2^31 and every product
// below 2^62, exact in int64.  Fixed-point float weights (WT = long long):
// sums below 2^62, products in 128 bits.  Passes walk the level's vertices
// with edges (the degree-bin order); candidates are decided one warp each,
// their candidate sub-communities summed in a per-warp shared-memory table.
#include "common.cuh"
#include "internal.h"

namespace gala {

namespace {

constexpr int kRefineMaxDeg = 256;  // rows longer than this stay singletons
constexpr int kRefineSweeps = 8;
constexpr int kRefTable = 512;      // per-warp slots (>= 2 x kRefineMaxDeg)
constexpr int kRefLog = 9;

// Exact products of the refinement's conditions and gains.
template <typename WT>
struct RefMath {
    using X = long long;
    static __device__ __forceinline__ X mul(long long a, long long b) { return a * b; }
    static __device__ __forceinline__ X shfl_xor(X v, int o) { return __shfl_xor_sync(GALA_FULL_MASK, v, o); }
};
template <>
struct RefMath<long long> {
    using X = __int128;
    static __device__ __forceinline__ X mul(long long a, long long b) { return (__int128)a * b; }
    static __device__ __forceinline__ X shfl_xor(X v, int o)
    {
        const unsigned long long lo = __shfl_xor_sync(GALA_FULL_MASK, (unsigned long long)v, o);
        const long long hi = __shfl_xor_sync(GALA_FULL_MASK, (long long)(v >> 64), o);
        return ((__int128)hi << 64) | (__int128)lo;
    }
};
// warps per decide block: the per-warp tables stay within 48 KB of static
// shared memory (10 bytes per slot for int weights, 14 for 64-bit ones)
template <typename WT>
__host__ __device__ constexpr int ref_warps()
{
    return sizeof(WT) == 4 ? 8 : 4;
}

template <typename WT>
__device__ __forceinline__ WT wt_of(const WT *w, long long j)
{
    return w ? w[j] : (WT)1;
}

// Per vertex with edges: wC = weight to the rest of its community.
template <typename WT>
__global__ void __launch_bounds__(256) k_ref_start(const int32_t *__restrict__ order, int nv,
                                                   const int64_t *__restrict__ offs,
                                                   const int32_t *__restrict__ nbr, const WT *__restrict__ w,
                                                   const int32_t *__restrict__ P, WT *wC)
{
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nv; i += nw) {
        const int v = order[i];
        const int p = P[v];
        WT s = 0;
        for (long long j = offs[v] + lane; j < offs[v + 1]; j += 32) {
            const int u = nbr[j];
            if (u != v && P[u] == p) s += wt_of(w, j);
        }
        s = warp_sum(s);
        if (lane == 0) wC[v] = s;
    }
}

__global__ void k_iota(int32_t *a, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = i;
}

// Per sweep: ext, Kr and sz of every sub-community (zeroed by the caller).
// One thread per vertex; rows longer than 32 entries are listed for the warp
// kernel below, which adds their ext share.
template <typename WT>
__global__ void __launch_bounds__(256) k_ref_sums(const int32_t *__restrict__ order, int n,
                                                  const int64_t *__restrict__ offs,
                                                  const int32_t *__restrict__ nbr, const WT *__restrict__ w,
                                                  const int32_t *__restrict__ P, const int32_t *__restrict__ R,
                                                  const WT *__restrict__ K, WT *ext, WT *Kr, int32_t *sz,
                                                  int32_t *big, int32_t *nbig)
{
    const int lane = threadIdx.x & 31;
    for (int i0 = blockIdx.x * blockDim.x + threadIdx.x - lane; i0 < n; i0 += gridDim.x * blockDim.x) {
        const int v = i0 + lane < n ? order[i0 + lane] : 0;
        bool is_big = false;
        if (i0 + lane < n) {
            const int p = P[v], r = R[v];
            const long long s0 = offs[v], e0 = offs[v + 1];
            is_big = e0 - s0 > 32;
            if (!is_big) {
                WT s = 0;
                for (long long j = s0; j < e0; ++j) {
                    const int u = nbr[j];
                    if (u != v && P[u] == p && R[u] != r) s += wt_of(w, j);
                }
                if (s) atomic_add_w(&ext[r], s);
            }
            atomic_add_w(&Kr[r], K[v]);
            atomicAdd(&sz[r], 1);
        }
        warp_append(is_big, v, big, nbig);
    }
}

template <typename WT>
__global__ void __launch_bounds__(256) k_ref_sums_big(const int32_t *__restrict__ big, const int32_t *__restrict__ nbig,
                                                      const int64_t *__restrict__ offs,
                                                      const int32_t *__restrict__ nbr, const WT *__restrict__ w,
                                                      const int32_t *__restrict__ P, const int32_t *__restrict__ R,
                                                      WT *ext)
{
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int cnt = *nbig;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < cnt; i += nw) {
        const int v = big[i];
        const int p = P[v], r = R[v];
        WT s = 0;
        for (long long j = offs[v] + lane; j < offs[v + 1]; j += 32) {
            const int u = nbr[j];
            if (u != v && P[u] == p && R[u] != r) s += wt_of(w, j);
        }
        s = warp_sum(s);
        if (lane == 0 && s) atomic_add_w(&ext[r], s);
    }
}

// Per sweep: the singletons that may move (listed; every target starts -1).
template <typename WT>
__global__ void __launch_bounds__(256) k_ref_cand(const int32_t *__restrict__ order, int n,
                                                  const int64_t *__restrict__ offs,
                                                  const int32_t *__restrict__ P, const int32_t *__restrict__ R,
                                                  const WT *__restrict__ K, const WT *__restrict__ wC,
                                                  const WT *__restrict__ TotC, const int32_t *__restrict__ sz,
                                                  long long m2, int32_t *target, int32_t *cand, int32_t *ncand)
{
    using M = RefMath<WT>;
    const int lane = threadIdx.x & 31;
    for (int i0 = blockIdx.x * blockDim.x + threadIdx.x - lane; i0 < n; i0 += gridDim.x * blockDim.x) {
        const int v = i0 + lane < n ? order[i0 + lane] : 0;
        bool ok = false;
        if (i0 + lane < n) {
            target[v] = -1;
            const long long deg = offs[v + 1] - offs[v];
            if (R[v] == v && sz[v] == 1 && deg >= 1 && deg <= kRefineMaxDeg) {
                const long long kv = K[v], tc = TotC[P[v]];
                ok = M::mul(wC[v], m2) >= M::mul(kv, tc - kv);
            }
        }
        warp_append(ok, v, cand, ncand);
    }
}

// Per sweep: the target of every listed candidate (or -1).
template <typename WT>
__global__ void __launch_bounds__(32 * ref_warps<WT>())
    k_ref_decide(const int32_t *__restrict__ cand, const int32_t *__restrict__ ncand,
                 const int64_t *__restrict__ offs, const int32_t *__restrict__ nbr, const WT *__restrict__ w,
                 const int32_t *__restrict__ P, const int32_t *__restrict__ R, const WT *__restrict__ K,
                 const WT *__restrict__ TotC, const WT *__restrict__ ext, const WT *__restrict__ Kr, long long m2,
                 int32_t *target, DevStats *st)
{
    using M = RefMath<WT>;
    using X = typename M::X;
    constexpr int NW = ref_warps<WT>();
    __shared__ int s_keys[NW][kRefTable];
    __shared__ WT s_vals[NW][kRefTable];
    __shared__ unsigned short s_occ[NW][kRefTable];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    int *keys = s_keys[wib];
    WT *vals = s_vals[wib];
    unsigned short *occ = s_occ[wib];
    for (int j = lane; j < kRefTable; j += 32) {
        keys[j] = -1;
        vals[j] = 0;
    }
    __syncwarp();
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int cnt = *ncand;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < cnt; i += nw) {
        const int v = cand[i];
        const long long s = offs[v];
        const int deg = (int)(offs[v + 1] - s);
        const int p = P[v];
        const long long kv = K[v], tc = TotC[p];
        int nocc = 0;
        for (int e0 = 0; e0 < deg; e0 += 32) {
            const int e = e0 + lane;
            int r = -1;
            WT wt = 0;
            if (e < deg) {
                const int u = nbr[s + e];
                if (u != v && P[u] == p) {
                    r = R[u];
                    wt = wt_of(w, s + e);
                    if (r == v) r = -1;
                }
            }
            bool created = false;
            int slot = -1;
            if (r >= 0) {
                unsigned h = hash_slot(r, kRefLog);
                for (int q = 0; q < kRefTable; ++q) {
                    const int k = atomicCAS(&keys[h], -1, r);
                    if (k == -1 || k == r) {
                        created = k == -1;
                        atomic_add_w(&vals[h], wt);
                        slot = (int)h;
                        break;
                    }
                    h = (h + 1) & (unsigned)(kRefTable - 1);
                }
                if (slot < 0) atomicOr(&st->err, kErrHashOverflow);
            }
            const unsigned cb = __ballot_sync(GALA_FULL_MASK, created);
            if (created) occ[nocc + __popc(cb & lanemask_lt())] = (unsigned short)slot;
            nocc += __popc(cb);
        }
        __syncwarp();
        // best well-connected candidate: largest X > 0, lowest id on ties
        X bx = 0;
        int best = -1;
        for (int q = lane; q < nocc; q += 32) {
            const int j = occ[q];
            const int r = keys[j];
            const long long kr = Kr[r];
            if (M::mul(ext[r], m2) >= M::mul(kr, tc - kr)) {
                const X x = M::mul(vals[j], m2) - M::mul(kv, kr);
                if (x > 0 && (best < 0 || x > bx || (x == bx && r < best))) {
                    bx = x;
                    best = r;
                }
            }
        }
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) {
            const X ox = M::shfl_xor(bx, o);
            const int ob = __shfl_xor_sync(GALA_FULL_MASK, best, o);
            if (ob >= 0 && (best < 0 || ox > bx || (ox == bx && ob < best))) {
                bx = ox;
                best = ob;
            }
        }
        if (lane == 0) target[v] = best;
        __syncwarp();
        for (int q = lane; q < nocc; q += 32) {
            const int j = occ[q];
            keys[j] = -1;
            vals[j] = 0;
        }
        __syncwarp();
    }
}

__global__ void k_ref_mark(const int32_t *__restrict__ cand, const int32_t *__restrict__ ncand,
                           const int32_t *__restrict__ target, int32_t *marks)
{
    const int n = *ncand;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int t = target[cand[i]];
        if (t >= 0) atomicAdd(&marks[t], 1);
    }
}

__global__ void k_ref_move(const int32_t *__restrict__ cand, const int32_t *__restrict__ ncand,
                           const int32_t *__restrict__ target, const int32_t *__restrict__ marks, int32_t *R,
                           int32_t *moved)
{
    int cnt = 0;
    const int n = *ncand;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int v = cand[i];
        const int t = target[v];
        if (t < 0) continue;
        const int m = marks[v];
        if (m == 0 || (m == 1 && target[t] == v && t < v)) {
            R[v] = t;
            cnt++;
        }
    }
    cnt = warp_sum(cnt);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(moved, cnt);
}

__global__ void k_ref_pmin(int n, const int32_t *__restrict__ P, const int32_t *__restrict__ lab, int32_t *pmin)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        atomicMin(&pmin[P[v]], lab[v]);
}

__global__ void k_ref_init_next(int n, const int32_t *__restrict__ P, const int32_t *__restrict__ lab,
                                const int32_t *__restrict__ pmin, int32_t *init)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x)
        init[lab[v]] = pmin[P[v]];
}

__global__ void k_fill(int32_t *a, int n, int32_t value)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) a[i] = value;
}

template <typename WT>
__global__ void k_start_partition(int n, const int32_t *__restrict__ init, const WT *__restrict__ K, int32_t *comm,
                                  WT *Tot, int32_t *size)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const int c = init[v];
        comm[v] = c;
        atomic_add_w(&Tot[c], K[v]);
        atomicAdd(&size[c], 1);
    }
}

int grid_for(long long items, int per_block)
{
    const long long cap = (long long)hub_grid_size() * 8;
    long long g = (items + per_block - 1) / per_block;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

template <typename WT>
int refine_t(const LevelGraph &g, const int32_t *P, const WT *K, const WT *TotC, long long m2, const int32_t *order,
             int nv, RefineBuffers &b, DevStats *stats, cudaStream_t st, gala_status *status)
{
    const int n = g.n;
    const WT *w = (const WT *)g.w;
    WT *wC = (WT *)b.wC, *ext = (WT *)b.ext, *Kr = (WT *)b.Kr;
    constexpr int kDecideBlock = 32 * ref_warps<WT>();
    const int gw = grid_for((long long)nv * 32, 256);  // one warp per vertex
    const int gd = grid_for((long long)nv * 32, kDecideBlock);
    const int gt = grid_for(nv, 256);
    k_iota<<<grid_for(n, 256), 256, 0, st>>>(b.R, n);
    k_ref_start<WT><<<gw, 256, 0, st>>>(order, nv, g.offs, g.nbr, w, P, wC);
    note_launch(2);
    int sweeps = 0;
    for (; sweeps < kRefineSweeps; ++sweeps) {
        cudaMemsetAsync(ext, 0, (size_t)n * sizeof(WT), st);
        cudaMemsetAsync(Kr, 0, (size_t)n * sizeof(WT), st);
        cudaMemsetAsync(b.sz, 0, (size_t)n * sizeof(int32_t), st);
        cudaMemsetAsync(b.marks, 0, (size_t)n * sizeof(int32_t), st);
        cudaMemsetAsync(b.moved, 0, 3 * sizeof(int32_t), st);
        k_ref_sums<WT><<<gt, 256, 0, st>>>(order, nv, g.offs, g.nbr, w, P, b.R, K, ext, Kr, b.sz, b.list,
                                           b.moved + 1);
        k_ref_sums_big<WT><<<gw, 256, 0, st>>>(b.list, b.moved + 1, g.offs, g.nbr, w, P, b.R, ext);
        k_ref_cand<WT><<<gt, 256, 0, st>>>(order, nv, g.offs, P, b.R, K, wC, TotC, b.sz, m2, b.target, b.list2,
                                           b.moved + 2);
        k_ref_decide<WT><<<gd, kDecideBlock, 0, st>>>(b.list2, b.moved + 2, g.offs, g.nbr, w, P, b.R, K, TotC, ext,
                                                      Kr, m2, b.target, stats);
        k_ref_mark<<<gt, 256, 0, st>>>(b.list2, b.moved + 2, b.target, b.marks);
        k_ref_move<<<gt, 256, 0, st>>>(b.list2, b.moved + 2, b.target, b.marks, b.R, b.moved);
        note_launch(6);
        int moved = 0, err = 0;
        cudaError_t ce = cudaGetLastError();
        if (ce == cudaSuccess) ce = cudaMemcpyAsync(&moved, b.moved, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (ce == cudaSuccess) ce = cudaMemcpyAsync(&err, &stats->err, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
        if (ce != cudaSuccess) {
            *status = cuda_fail(ce, "refinement");
            return -1;
        }
        if (err) {
            set_error("refinement: device error bits %d", err);
            *status = GALA_ERR_OVERFLOW;
            return -1;
        }
        if (moved == 0) break;
    }
    // totals of the final sub-communities (the next level's weighted degrees)
    cudaMemsetAsync(ext, 0, (size_t)n * sizeof(WT), st);
    cudaMemsetAsync(Kr, 0, (size_t)n * sizeof(WT), st);
    cudaMemsetAsync(b.sz, 0, (size_t)n * sizeof(int32_t), st);
    cudaMemsetAsync(b.moved + 1, 0, sizeof(int32_t), st);
    k_ref_sums<WT><<<gt, 256, 0, st>>>(order, nv, g.offs, g.nbr, w, P, b.R, K, ext, Kr, b.sz, b.list, b.moved + 1);
    note_launch(1);
    return sweeps;
}

}  // namespace

int refine_run(const LevelGraph &g, const int32_t *P, const void *K, const void *TotC, long long m2,
               const int32_t *order, int nv, RefineBuffers &b, DevStats *stats, cudaStream_t st,
               gala_status *status)
{
    if (g.wide)
        return refine_t<long long>(g, P, (const long long *)K, (const long long *)TotC, m2, order, nv, b, stats, st,
                                   status);
    return refine_t<int>(g, P, (const int *)K, (const int *)TotC, m2, order, nv, b, stats, st, status);
}

void p1_start_partition(Phase1Buffers &b, const int32_t *init, int n, cudaStream_t st)
{
    const size_t ws = b.wide ? sizeof(long long) : sizeof(int);
    cudaMemsetAsync(b.Tot, 0, (size_t)n * ws, st);
    cudaMemsetAsync(b.size, 0, (size_t)n * sizeof(int32_t), st);
    if (b.wide)
        k_start_partition<long long><<<grid_for(n, 256), 256, 0, st>>>(n, init, (const long long *)b.K, b.comm,
                                                                       (long long *)b.Tot, b.size);
    else
        k_start_partition<int><<<grid_for(n, 256), 256, 0, st>>>(n, init, b.K, b.comm, b.Tot, b.size);
    note_launch(1);
}

void refine_next_init(const int32_t *P, const int32_t *lab, int n, RefineBuffers &b, cudaStream_t st)
{
    const int gt = grid_for(n, 256);
    k_fill<<<gt, 256, 0, st>>>(b.pmin, n, 0x7fffffff);
    k_ref_pmin<<<gt, 256, 0, st>>>(n, P, lab, b.pmin);
    k_ref_init_next<<<gt, 256, 0, st>>>(n, P, lab, b.pmin, b.init);
    note_launch(3);
}

}  // namespace gala
