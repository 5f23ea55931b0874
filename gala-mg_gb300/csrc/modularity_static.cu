// modularity_static.cu - modularity of a partition on the device without any
// device allocation.
//
// Some callers of this library cannot call cudaMalloc: a host application
// that hands all device memory to its own pool allocator, or a latency-bound
// path where an allocation (and the synchronisation cudaMalloc/cudaFree can
// cause) is not allowed.  gala_modularity_device_static serves them: the
// caller passes the CSR and the labels (device) and gets Q back, and the
// scratch the computation needs - the total weight of every community and
// four sums - lives in the file-scope arrays below, sized for at most
// kStaticMaxVertices vertices.  Every GPU that loads this library holds that
// memory (8 MB + 36 B) until the process exits.
//
// The computation is the one phase 1 uses for Q: sum of In over vertices and
// total weight m2 as exact 64-bit integers, sum of Tot^2 over communities as
// an exact 128-bit integer (Tot^2 alone passes 2^64 once m2 > 2^32), then Q by
// one FP64 expression.
#include <stdio.h>
#include <string.h>

#include <mutex>

#include "common.cuh"
#include "internal.h"

namespace gala {

constexpr int kStaticMaxVertices = 1 << 20;
constexpr int kStaticMaxDevices = 64;

// Scratch shared by every call on a device: community totals and the sums.
static __device__ __align__(256) unsigned long long g_static_tot[kStaticMaxVertices];
// sum In, sum K, sum Tot^2 (low word), sum Tot^2 (high word)
static __device__ __align__(256) unsigned long long g_static_sums[4];
// bit 0: a label lies outside [0, n); bit 1: a weight is not positive
static __device__ __align__(256) int g_static_bad;

// Device addresses of the three arrays, looked up once per device (in host
// code the symbols are host-side stand-ins, not device addresses).
static unsigned long long *g_tot_ptr[kStaticMaxDevices];
static unsigned long long *g_sums_ptr[kStaticMaxDevices];
static int *g_bad_ptr[kStaticMaxDevices];
static std::mutex g_static_mu;

__global__ void k_static_zero(unsigned long long *tot, int n, unsigned long long *sums, int *bad)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) tot[i] = 0ull;
    if (blockIdx.x == 0 && threadIdx.x < 4) sums[threadIdx.x] = 0ull;
    if (blockIdx.x == 0 && threadIdx.x == 0) *bad = 0;
}

// One warp per vertex: K (row weight), In (weight to the own community);
// community totals by atomics, sums by warp then block reduction.
__global__ void __launch_bounds__(256) k_static_rows(int n, const int64_t *__restrict__ offs,
                                                     const int32_t *__restrict__ nbr, const int32_t *__restrict__ w,
                                                     const int32_t *__restrict__ comm, unsigned long long *tot,
                                                     unsigned long long *sums, int *bad)
{
    __shared__ unsigned long long s_in[8], s_k[8];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int wg = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nw = (gridDim.x * blockDim.x) >> 5;
    unsigned long long my_in = 0, my_k = 0;
    for (int v = wg; v < n; v += nw) {
        const int c = comm[v];
        unsigned long long k = 0, in = 0;
        for (long long j = offs[v] + lane; j < offs[v + 1]; j += 32) {
            const int32_t wi = w ? w[j] : 1;
            if (wi <= 0) atomicOr(bad, 2);
            const unsigned long long wt = wi > 0 ? (unsigned long long)wi : 0ull;
            k += wt;
            const int u = nbr[j];
            if (u >= 0 && u < n && comm[u] == c) in += wt;
        }
        k = warp_sum(k);
        in = warp_sum(in);
        if (lane == 0) {
            if (c >= 0 && c < n)
                atomicAdd(&tot[c], k);
            else
                atomicOr(bad, 1);
            my_in += in;
            my_k += k;
        }
    }
    if (lane == 0) {
        s_in[wid] = my_in;
        s_k[wid] = my_k;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long a = 0, b = 0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
            a += s_in[q];
            b += s_k[q];
        }
        if (a) atomicAdd(&sums[0], a);
        if (b) atomicAdd(&sums[1], b);
    }
}

// Sum of Tot^2 over communities, exact in 128 bits: Tot < 2^64, so a square
// needs up to 128 bits; each block adds its sum to the (lo, hi) pair, the
// carry taken from the low word's atomic result (order independent).
__global__ void __launch_bounds__(256) k_static_tot2(int n, const unsigned long long *__restrict__ tot,
                                                     unsigned long long *sums)
{
    __shared__ unsigned long long rlo[8], rhi[8];
    unsigned __int128 s = 0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x)
        s += (unsigned __int128)tot[c] * tot[c];
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) {
        const unsigned long long l = __shfl_xor_sync(GALA_FULL_MASK, (unsigned long long)s, o);
        const unsigned long long h = __shfl_xor_sync(GALA_FULL_MASK, (unsigned long long)(s >> 64), o);
        s += ((unsigned __int128)h << 64) | l;
    }
    if ((threadIdx.x & 31) == 0) {
        rlo[threadIdx.x >> 5] = (unsigned long long)s;
        rhi[threadIdx.x >> 5] = (unsigned long long)(s >> 64);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned __int128 t = 0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) t += ((unsigned __int128)rhi[q] << 64) | rlo[q];
        const unsigned long long l = (unsigned long long)t;
        unsigned long long h = (unsigned long long)(t >> 64);
        if (l) {
            const unsigned long long old = atomicAdd(&sums[2], l);
            if (old + l < old) h += 1;
        }
        if (h) atomicAdd(&sums[3], h);
    }
}

}  // namespace gala

using namespace gala;

extern "C" gala_status gala_modularity_device_static(int32_t n, const int64_t *d_offsets, const int32_t *d_neighbors,
                                                     const int32_t *d_weights, const int32_t *d_community,
                                                     double *modularity)
{
    clear_error();
    if (n <= 0 || !d_offsets || !d_neighbors || !d_community || !modularity) {
        set_error("gala_modularity_device_static: bad arguments");
        return GALA_ERR_INVALID;
    }
    if (n > kStaticMaxVertices) {
        set_error("gala_modularity_device_static: %d vertices exceed the static maximum of %d", n,
                  kStaticMaxVertices);
        return GALA_ERR_CAPACITY;
    }
    int dev = 0;
    cudaError_t ce = cudaGetDevice(&dev);
    if (ce != cudaSuccess) return cuda_fail(ce, "gala_modularity_device_static: no device");
    if (dev < 0 || dev >= kStaticMaxDevices) {
        set_error("gala_modularity_device_static: device %d out of range", dev);
        return GALA_ERR_INVALID;
    }
    unsigned long long *tot = nullptr, *sums = nullptr;
    int *bad = nullptr;
    {
        // first call on this device (with it current): look up the device
        // addresses of the static arrays
        std::lock_guard<std::mutex> lock(g_static_mu);
        if (!g_tot_ptr[dev]) {
            void *p = nullptr, *q = nullptr, *r = nullptr;
            if ((ce = cudaGetSymbolAddress(&p, g_static_tot)) != cudaSuccess ||
                (ce = cudaGetSymbolAddress(&q, g_static_sums)) != cudaSuccess ||
                (ce = cudaGetSymbolAddress(&r, g_static_bad)) != cudaSuccess)
                return cuda_fail(ce, "gala_modularity_device_static: symbol address");
            g_tot_ptr[dev] = (unsigned long long *)p;
            g_sums_ptr[dev] = (unsigned long long *)q;
            g_bad_ptr[dev] = (int *)r;
        }
        tot = g_tot_ptr[dev];
        sums = g_sums_ptr[dev];
        bad = g_bad_ptr[dev];
    }
    // the scratch keeps the previous call's contents: clear it first
    const int grid = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
    k_static_zero<<<grid, 256>>>(tot, n, sums, bad);
    const int rgrid = (int)(((long long)n * 32 + 255) / 256 < 2048 ? ((long long)n * 32 + 255) / 256 : 2048);
    k_static_rows<<<rgrid, 256>>>(n, d_offsets, d_neighbors, d_weights, d_community, tot, sums, bad);
    k_static_tot2<<<grid, 256>>>(n, tot, sums);
    note_launch(3);
    // a launch that failed for its configuration would leave the previous
    // call's sums in the scratch: report it instead of reading them
    if ((ce = cudaGetLastError()) != cudaSuccess) return cuda_fail(ce, "gala_modularity_device_static: launch");
    unsigned long long h[4] = {0, 0, 0, 0};
    int hbad = 0;
    if ((ce = cudaMemcpy(h, sums, sizeof(h), cudaMemcpyDeviceToHost)) != cudaSuccess ||
        (ce = cudaMemcpy(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda_fail(ce, "gala_modularity_device_static");
    if (hbad & 1) {
        set_error("gala_modularity_device_static: a community label lies outside [0, %d)", n);
        return GALA_ERR_INVALID;
    }
    if (hbad & 2) {
        set_error("gala_modularity_device_static: a weight is not positive");
        return GALA_ERR_INVALID;
    }
    if (h[1] == 0) {
        set_error("gala_modularity_device_static: graph has no edges");
        return GALA_ERR_INVALID;
    }
    // Q = sum In / m2 - sum Tot^2 / m2^2, the 128-bit sum converted as
    // hi * 2^64 + lo (the engine's expression)
    const double c = 1.0 / (double)h[1];
    const double t2 = (double)h[3] * 18446744073709551616.0 + (double)h[2];
    *modularity = (double)h[0] * c - t2 * c * c;
    return GALA_OK;
}
