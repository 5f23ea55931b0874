// batch.cu - per-graph reductions of a batch of graphs run as one union
// graph (block-diagonal CSR).  Batching has no counterpart in the reference;
// every graph follows the reference's single-graph rules with its own m2,
// min Tot, modularity and convergence.
//
// The vertices of graph g occupy the contiguous id range [goff[g], goff[g+1])
// at every level: contraction renumbers communities by ascending old id and a
// community never spans two graphs, so the ranges stay contiguous.
#include "common.cuh"
#include "internal.h"

namespace gala {

namespace {

__device__ __forceinline__ unsigned long long block_sum_u64(unsigned long long v, unsigned long long *red)
{
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    unsigned long long t = 0;
    if (wid == 0) {
        t = lane < (int)(blockDim.x >> 5) ? red[lane] : 0ull;
        t = warp_sum(t);
    }
    return t;  // valid in thread 0
}

__device__ __forceinline__ int block_min_i32(int v, int *red)
{
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) v = min(v, __shfl_xor_sync(GALA_FULL_MASK, v, o));
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) red[wid] = v;
    __syncthreads();
    int t = 0x7fffffff;
    if (wid == 0) {
        t = lane < (int)(blockDim.x >> 5) ? red[lane] : 0x7fffffff;
#pragma unroll
        for (int o = 16; o >= 1; o >>= 1) t = min(t, __shfl_xor_sync(GALA_FULL_MASK, t, o));
    }
    return t;
}

// One block per graph: the sums `what` asks for over the graph's range.
// Graphs with stop[g] set are left alone (their values are final).
__global__ void __launch_bounds__(256) k_graph_sums(int what, int G, const int64_t *__restrict__ goff,
                                                    const uint8_t *__restrict__ stop, const int32_t *__restrict__ In,
                                                    const int32_t *__restrict__ Tot, const int32_t *__restrict__ K,
                                                    const int32_t *__restrict__ size, GraphSums out)
{
    __shared__ unsigned long long red[32];
    __shared__ int redi[32];
    for (int g = blockIdx.x; g < G; g += gridDim.x) {
        if (stop && stop[g]) continue;
        const long long v0 = goff[g], v1 = goff[g + 1];
        unsigned long long si = 0, st2 = 0, sk = 0, nc = 0;
        int mn = 0x7fffffff;
        for (long long v = v0 + threadIdx.x; v < v1; v += blockDim.x) {
            if (what & kSumIn) si += (unsigned long long)In[v];
            if (what & (kSumTot2 | kMinTot)) {
                const int t = Tot[v];
                if (t != 0) {
                    st2 += (unsigned long long)((long long)t * t);
                    mn = min(mn, t);
                }
            }
            if (what & kSumK) sk += (unsigned long long)K[v];
            if (what & kCountComm) nc += size[v] > 0;
        }
        if (what & kSumIn) {
            si = block_sum_u64(si, red);
            if (threadIdx.x == 0) out.sum_in[g] = si;
        }
        if (what & kSumTot2) {
            st2 = block_sum_u64(st2, red);
            if (threadIdx.x == 0) out.sum_tot2[g] = st2;
        }
        if (what & kSumK) {
            sk = block_sum_u64(sk, red);
            if (threadIdx.x == 0) out.sum_k[g] = sk;
        }
        if (what & kCountComm) {
            nc = block_sum_u64(nc, red);
            if (threadIdx.x == 0) out.ncomm[g] = (int32_t)nc;
        }
        if (what & kMinTot) {
            mn = block_min_i32(mn, redi);
            if (threadIdx.x == 0) out.min_tot[g] = mn;
        }
        __syncthreads();
    }
}

// Undo this iteration's moves of the graphs flagged in `reject` (their Q
// did not grow by min_mod; louvain_main_process.cu:1004-1007 per graph).
__global__ void k_revert_graphs(const int32_t *__restrict__ mv_v, const int32_t *__restrict__ mv_old,
                                const int32_t *__restrict__ mv_new, const DevStats *__restrict__ stp,
                                const int32_t *__restrict__ gid, const uint8_t *__restrict__ reject, int32_t *comm,
                                int32_t *Tot, int32_t *size, const int32_t *__restrict__ K)
{
    const int nm = stp->n_movers;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nm; i += gridDim.x * blockDim.x) {
        const int v = mv_v[i];
        if (!reject[gid[v]]) continue;
        const int from = mv_new[i], to = mv_old[i];
        const int k = K[v];
        comm[v] = to;
        atomicAdd(&Tot[to], k);
        atomicSub(&Tot[from], k);
        atomicAdd(&size[to], 1);
        atomicSub(&size[from], 1);
    }
}

__global__ void k_gid_fill(int G, const int64_t *__restrict__ goff, int32_t *gid)
{
    for (int g = blockIdx.x; g < G; g += gridDim.x)
        for (long long v = goff[g] + threadIdx.x; v < goff[g + 1]; v += blockDim.x) gid[v] = g;
}

int grid_for(int G) { return G < 65535 ? G : 65535; }

// Union CSR of page-locked host graphs, read by the GPU through their
// device-mapped addresses: one block per graph shifts the graph's offsets by
// its first entry and its neighbour ids by its first vertex.  Four loads in
// flight per thread (host memory behind the chip-to-chip link has a long
// latency).
__global__ void __launch_bounds__(256) k_batch_gather(int G, BatchSrc s, int64_t *offs, int32_t *nbr, int32_t *w)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) offs[0] = 0;
    for (int g = blockIdx.x; g < G; g += gridDim.x) {
        const long long v0 = s.vstart[g], n = s.vstart[g + 1] - v0;
        const long long e0 = s.estart[g], E = s.estart[g + 1] - e0;
        const int64_t *so = s.offs[g];
        const int32_t *sn = s.nbr[g];
        const int32_t *sw = s.w[g];
        const int32_t shift = (int32_t)v0;
        for (long long v = threadIdx.x; v < n; v += blockDim.x) offs[v0 + v + 1] = e0 + so[v];
        constexpr int U = 4;
        for (long long j0 = 0; j0 < E; j0 += (long long)U * blockDim.x) {
            int32_t t[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const long long j = j0 + u * blockDim.x + threadIdx.x;
                t[u] = j < E ? sn[j] : 0;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const long long j = j0 + u * blockDim.x + threadIdx.x;
                if (j < E) nbr[e0 + j] = t[u] + shift;
            }
        }
        if (w) {
            for (long long j0 = 0; j0 < E; j0 += (long long)U * blockDim.x) {
                int32_t t[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const long long j = j0 + u * blockDim.x + threadIdx.x;
                    t[u] = (j < E && sw) ? sw[j] : 1;
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const long long j = j0 + u * blockDim.x + threadIdx.x;
                    if (j < E) w[e0 + j] = t[u];
                }
            }
        }
    }
}

// In-place shift of a union CSR whose per-graph parts were copied raw:
// graph g's inclusive offsets (at offs[vstart[g]+1 ...]) by its first entry,
// its neighbour ids by its first vertex.
__global__ void __launch_bounds__(256) k_batch_shift(int G, const int64_t *__restrict__ vstart,
                                                     const int64_t *__restrict__ estart, int64_t *offs, int32_t *nbr)
{
    if (blockIdx.x == 0 && threadIdx.x == 0) offs[0] = 0;
    for (int g = blockIdx.x; g < G; g += gridDim.x) {
        const long long v0 = vstart[g], v1 = vstart[g + 1], e0 = estart[g], e1 = estart[g + 1];
        const int32_t shift = (int32_t)v0;
        if (e0 != 0)
            for (long long v = v0 + threadIdx.x; v < v1; v += blockDim.x) offs[v + 1] += e0;
        if (shift != 0)
            for (long long j = e0 + threadIdx.x; j < e1; j += blockDim.x) nbr[j] += shift;
    }
}

// Union community ids -> ids local to each graph (graph g's vertices are
// [vstart[g], vstart[g+1]) of the input; its communities start at goff[g]).
__global__ void k_batch_local_labels(int G, const int64_t *__restrict__ vstart, const int64_t *__restrict__ goff,
                                     int32_t *labels)
{
    for (int g = blockIdx.x; g < G; g += gridDim.x) {
        const int32_t base = (int32_t)goff[g];
        for (long long v = vstart[g] + threadIdx.x; v < vstart[g + 1]; v += blockDim.x) labels[v] -= base;
    }
}

}  // namespace

void batch_gather(int G, const BatchSrc &src, int64_t *offs, int32_t *nbr, int32_t *w, cudaStream_t st)
{
    if (G <= 0) return;
    k_batch_gather<<<grid_for(G), 256, 0, st>>>(G, src, offs, nbr, w);
    note_launch(1);
}

void batch_shift(int G, const int64_t *vstart, const int64_t *estart, int64_t *offs, int32_t *nbr, cudaStream_t st)
{
    if (G <= 0) return;
    k_batch_shift<<<grid_for(G), 256, 0, st>>>(G, vstart, estart, offs, nbr);
    note_launch(1);
}

void batch_local_labels(int G, const int64_t *vstart, const int64_t *goff, int32_t *labels, cudaStream_t st)
{
    if (G <= 0) return;
    k_batch_local_labels<<<grid_for(G), 256, 0, st>>>(G, vstart, goff, labels);
    note_launch(1);
}

void batch_graph_sums(int what, int G, const int64_t *goff, const uint8_t *stop, const Phase1Buffers &b,
                      const GraphSums &out, cudaStream_t st)
{
    if (G <= 0) return;
    k_graph_sums<<<grid_for(G), 256, 0, st>>>(what, G, goff, stop, b.In, b.Tot, b.K, b.size, out);
    note_launch(1);
}

void batch_revert(Phase1Buffers &b, const int32_t *gid, const uint8_t *reject, int n, cudaStream_t st)
{
    int grid = (n + 255) / 256;
    if (grid > 1024) grid = 1024;
    if (grid < 1) grid = 1;
    k_revert_graphs<<<grid, 256, 0, st>>>(b.mv_v, b.mv_old, b.mv_new, b.stats, gid, reject, b.comm, b.Tot, b.size,
                                          b.K);
    note_launch(1);
}

void batch_gid_fill(int G, const int64_t *goff, int32_t *gid, cudaStream_t st)
{
    if (G <= 0) return;
    k_gid_fill<<<grid_for(G), 256, 0, st>>>(G, goff, gid);
    note_launch(1);
}

}  // namespace gala
