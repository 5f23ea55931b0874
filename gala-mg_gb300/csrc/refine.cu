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
// Integer weights only: every sum is below m2 < 2^31 and every product below
// 2^62, so int64 arithmetic is exact.  One warp per vertex; the candidate
// sub-communities of a vertex are summed in a per-warp shared-memory table.
#include "common.cuh"
#include "internal.h"

namespace gala {

namespace {

constexpr int kRefineMaxDeg = 256;  // rows longer than this stay singletons
constexpr int kRefineSweeps = 8;
constexpr int kRefTable = 512;      // per-warp slots (>= 2 x kRefineMaxDeg)
constexpr int kRefLog = 9;
constexpr int kRefWarps = 8;

// Per vertex: R = own id, wC = weight to the rest of its community.
__global__ void __launch_bounds__(256) k_ref_start(const int32_t *__restrict__ order, int nv,
                                                   const int64_t *__restrict__ offs,
                                                   const int32_t *__restrict__ nbr, const int32_t *__restrict__ w,
                                                   const int32_t *__restrict__ P, int32_t *wC)
{
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < nv; i += nw) {
        const int v = order[i];
        const int p = P[v];
        int s = 0;
        for (long long j = offs[v] + lane; j < offs[v + 1]; j += 32) {
            const int u = nbr[j];
            if (u != v && P[u] == p) s += w ? w[j] : 1;
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
__global__ void __launch_bounds__(256) k_ref_sums(const int32_t *__restrict__ order, int n,
                                                  const int64_t *__restrict__ offs,
                                                  const int32_t *__restrict__ nbr, const int32_t *__restrict__ w,
                                                  const int32_t *__restrict__ P, const int32_t *__restrict__ R,
                                                  const int32_t *__restrict__ K, int32_t *ext, int32_t *Kr,
                                                  int32_t *sz, int32_t *big, int32_t *nbig)
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
                int s = 0;
                for (long long j = s0; j < e0; ++j) {
                    const int u = nbr[j];
                    if (u != v && P[u] == p && R[u] != r) s += w ? w[j] : 1;
                }
                if (s) atomicAdd(&ext[r], s);
            }
            atomicAdd(&Kr[r], K[v]);
            atomicAdd(&sz[r], 1);
        }
        warp_append(is_big, v, big, nbig);
    }
}

__global__ void __launch_bounds__(256) k_ref_sums_big(const int32_t *__restrict__ big, const int32_t *__restrict__ nbig,
                                                      const int64_t *__restrict__ offs,
                                                      const int32_t *__restrict__ nbr, const int32_t *__restrict__ w,
                                                      const int32_t *__restrict__ P, const int32_t *__restrict__ R,
                                                      int32_t *ext)
{
    const int lane = threadIdx.x & 31;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    const int cnt = *nbig;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < cnt; i += nw) {
        const int v = big[i];
        const int p = P[v], r = R[v];
        int s = 0;
        for (long long j = offs[v] + lane; j < offs[v + 1]; j += 32) {
            const int u = nbr[j];
            if (u != v && P[u] == p && R[u] != r) s += w ? w[j] : 1;
        }
        s = warp_sum(s);
        if (lane == 0 && s) atomicAdd(&ext[r], s);
    }
}

// Per sweep: the singletons that may move (listed; every target starts -1).
__global__ void __launch_bounds__(256) k_ref_cand(const int32_t *__restrict__ order, int n,
                                                  const int64_t *__restrict__ offs,
                                                  const int32_t *__restrict__ P, const int32_t *__restrict__ R,
                                                  const int32_t *__restrict__ K, const int32_t *__restrict__ wC,
                                                  const int32_t *__restrict__ TotC, const int32_t *__restrict__ sz,
                                                  long long m2, int32_t *target, int32_t *cand, int32_t *ncand)
{
    const int lane = threadIdx.x & 31;
    for (int i0 = blockIdx.x * blockDim.x + threadIdx.x - lane; i0 < n; i0 += gridDim.x * blockDim.x) {
        const int v = i0 + lane < n ? order[i0 + lane] : 0;
        bool ok = false;
        if (i0 + lane < n) {
            target[v] = -1;
            const long long deg = offs[v + 1] - offs[v];
            if (R[v] == v && sz[v] == 1 && deg >= 1 && deg <= kRefineMaxDeg) {
                const long long kv = K[v], tc = TotC[P[v]];
                ok = (long long)wC[v] * m2 >= kv * (tc - kv);
            }
        }
        warp_append(ok, v, cand, ncand);
    }
}

// Per sweep: the target of every singleton (or -1).
__global__ void __launch_bounds__(256) k_ref_decide(const int32_t *__restrict__ cand, const int32_t *__restrict__ ncand,
                                                    const int64_t *__restrict__ offs,
                                                    const int32_t *__restrict__ nbr, const int32_t *__restrict__ w,
                                                    const int32_t *__restrict__ P, const int32_t *__restrict__ R,
                                                    const int32_t *__restrict__ K, const int32_t *__restrict__ wC,
                                                    const int32_t *__restrict__ TotC, const int32_t *__restrict__ ext,
                                                    const int32_t *__restrict__ Kr, const int32_t *__restrict__ sz,
                                                    long long m2, int32_t *target, DevStats *st)
{
    __shared__ int s_keys[kRefWarps][kRefTable];
    __shared__ int s_vals[kRefWarps][kRefTable];
    __shared__ unsigned short s_occ[kRefWarps][kRefTable];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    int *keys = s_keys[wib], *vals = s_vals[wib];
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
            int r = -1, wt = 0;
            if (e < deg) {
                const int u = nbr[s + e];
                if (u != v && P[u] == p) {
                    r = R[u];
                    wt = w ? w[s + e] : 1;
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
                        atomicAdd(&vals[h], wt);
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
        long long bx = 0;
        int best = -1;
        for (int q = lane; q < nocc; q += 32) {
            const int j = occ[q];
            const int r = keys[j];
            const long long kr = Kr[r];
            if ((long long)ext[r] * m2 >= kr * (tc - kr)) {
                const long long x = (long long)vals[j] * m2 - kv * kr;
                if (x > 0 && (best < 0 || x > bx || (x == bx && r < best))) {
                    bx = x;
                    best = r;
                }
            }
        }
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) {
            const long long ox = __shfl_xor_sync(GALA_FULL_MASK, bx, o);
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

int grid_for(long long items, int per_block)
{
    const long long cap = (long long)hub_grid_size() * 8;
    long long g = (items + per_block - 1) / per_block;
    return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace

int refine_run(const LevelGraph &g, const int32_t *P, const int32_t *K, const int32_t *TotC, long long m2,
               const int32_t *order, int nv, RefineBuffers &b, DevStats *stats, cudaStream_t st,
               gala_status *status)
{
    // vertices without edges stay singletons: the passes walk the level's
    // degree-bin order (every vertex with an edge), not all n ids
    const int n = g.n;
    const int32_t *w = (const int32_t *)g.w;
    const int gw = grid_for((long long)nv * 32, 256);  // one warp per vertex
    const int gt = grid_for(nv, 256);
    k_iota<<<grid_for(n, 256), 256, 0, st>>>(b.R, n);
    k_ref_start<<<gw, 256, 0, st>>>(order, nv, g.offs, g.nbr, w, P, b.wC);
    note_launch(2);
    int sweeps = 0;
    for (; sweeps < kRefineSweeps; ++sweeps) {
        cudaMemsetAsync(b.ext, 0, (size_t)n * sizeof(int32_t), st);
        cudaMemsetAsync(b.Kr, 0, (size_t)n * sizeof(int32_t), st);
        cudaMemsetAsync(b.sz, 0, (size_t)n * sizeof(int32_t), st);
        cudaMemsetAsync(b.marks, 0, (size_t)n * sizeof(int32_t), st);
        cudaMemsetAsync(b.moved, 0, 3 * sizeof(int32_t), st);
        k_ref_sums<<<gt, 256, 0, st>>>(order, nv, g.offs, g.nbr, w, P, b.R, K, b.ext, b.Kr, b.sz, b.list,
                                       b.moved + 1);
        k_ref_sums_big<<<gw, 256, 0, st>>>(b.list, b.moved + 1, g.offs, g.nbr, w, P, b.R, b.ext);
        k_ref_cand<<<gt, 256, 0, st>>>(order, nv, g.offs, P, b.R, K, b.wC, TotC, b.sz, m2, b.target, b.list2,
                                       b.moved + 2);
        k_ref_decide<<<gw, 256, 0, st>>>(b.list2, b.moved + 2, g.offs, g.nbr, w, P, b.R, K, b.wC, TotC, b.ext, b.Kr,
                                         b.sz, m2, b.target, stats);
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
    cudaMemsetAsync(b.ext, 0, (size_t)n * sizeof(int32_t), st);
    cudaMemsetAsync(b.Kr, 0, (size_t)n * sizeof(int32_t), st);
    cudaMemsetAsync(b.sz, 0, (size_t)n * sizeof(int32_t), st);
    cudaMemsetAsync(b.moved + 1, 0, sizeof(int32_t), st);
    k_ref_sums<<<gt, 256, 0, st>>>(order, nv, g.offs, g.nbr, w, P, b.R, K, b.ext, b.Kr, b.sz, b.list,
                                   b.moved + 1);
    note_launch(1);
    return sweeps;
}

namespace {
__global__ void k_start_partition(int n, const int32_t *__restrict__ init, const int32_t *__restrict__ K,
                                  int32_t *comm, int32_t *Tot, int32_t *size)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        const int c = init[v];
        comm[v] = c;
        atomicAdd(&Tot[c], K[v]);
        atomicAdd(&size[c], 1);
    }
}
}  // namespace

void p1_start_partition(Phase1Buffers &b, const int32_t *init, int n, cudaStream_t st)
{
    cudaMemsetAsync(b.Tot, 0, (size_t)n * sizeof(int32_t), st);
    cudaMemsetAsync(b.size, 0, (size_t)n * sizeof(int32_t), st);
    k_start_partition<<<grid_for(n, 256), 256, 0, st>>>(n, init, b.K, b.comm, b.Tot, b.size);
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
