// proposal.cu - the learned move-proposal network: an 8 -> 32 -> 32 -> 1 MLP
// that predicts, from per-vertex features, whether a vertex will move in the
// coming phase-1 iteration.  Vertices predicted to stay are not decided
// (learned mode of the engine); the engine certifies every convergence with
// a full plain sweep, so no reported partition rests on a skipped decision.
//
// Training data are traces of the plain method itself (features at decide
// time, label = the vertex moved).  Training runs on the GPU: one kernel
// computes the loss gradient of a mini-batch (forward + backward, FP32
// accumulation, per-block reduction of the gradient), one applies Adam; the
// inference weights are the master weights rounded to BF16, read back to FP32
// for the FMA chain (FP32 accumulate).
//
// Parameter layout (kParams floats): W1[32][8], b1[32], W2[32][32], b2[32],
// w3[32], b3.
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <random>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace gala {

constexpr int kIn = kPropFeatures;  // 8
constexpr int kH = 32;
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kH * kIn;
constexpr int kOffW2 = kOffB1 + kH;
constexpr int kOffB2 = kOffW2 + kH * kH;
constexpr int kOffW3 = kOffB2 + kH;
constexpr int kOffB3 = kOffW3 + kH;
static_assert(kOffB3 + 1 == kPropParams, "parameter layout");

// Forward pass of one sample with parameters P (FP32, shared memory).
__device__ __forceinline__ float mlp_forward(const float *P, const float *x, float *z1, float *z2)
{
#pragma unroll
    for (int o = 0; o < kH; ++o) {
        float s = P[kOffB1 + o];
#pragma unroll
        for (int i = 0; i < kIn; ++i) s = fmaf(P[kOffW1 + o * kIn + i], x[i], s);
        z1[o] = s;
    }
#pragma unroll 4
    for (int o = 0; o < kH; ++o) {
        float s = P[kOffB2 + o];
#pragma unroll
        for (int i = 0; i < kH; ++i) s = fmaf(P[kOffW2 + o * kH + i], fmaxf(z1[i], 0.f), s);
        z2[o] = s;
    }
    float out = P[kOffB3];
#pragma unroll
    for (int i = 0; i < kH; ++i) out = fmaf(P[kOffW3 + i], fmaxf(z2[i], 0.f), out);
    return out;
}

// Inference of one feature row (FP32 parameters in shared memory, FP32
// accumulation; the second layer is folded into the output sum).
__device__ __forceinline__ float mlp_infer(const float *P, const float *x)
{
    float h1[kH];
#pragma unroll
    for (int o = 0; o < kH; ++o) {
        float s = P[kOffB1 + o];
#pragma unroll
        for (int i = 0; i < kIn; ++i) s = fmaf(P[kOffW1 + o * kIn + i], x[i], s);
        h1[o] = fmaxf(s, 0.f);
    }
    float out = P[kOffB3];
#pragma unroll 8
    for (int o = 0; o < kH; ++o) {
        float s = P[kOffB2 + o];
#pragma unroll
        for (int i = 0; i < kH; ++i) s = fmaf(P[kOffW2 + o * kH + i], h1[i], s);
        out = fmaf(P[kOffW3 + o], fmaxf(s, 0.f), out);
    }
    return out;
}

__device__ __forceinline__ float sigmoidf_(float x) { return 1.f / (1.f + __expf(-x)); }

// Logits of n samples (feature rows of kIn floats) with the BF16 weights.
__global__ void __launch_bounds__(256) k_mlp_logits(const __nv_bfloat16 *__restrict__ wb, const float *__restrict__ X,
                                                    long long n, float *logits)
{
    __shared__ float P[kPropParams];
    for (int i = threadIdx.x; i < kPropParams; i += blockDim.x) P[i] = __bfloat162float(wb[i]);
    __syncthreads();
    for (long long s = blockIdx.x * (long long)blockDim.x + threadIdx.x; s < n; s += (long long)gridDim.x * blockDim.x) {
        float x[kIn];
#pragma unroll
        for (int i = 0; i < kIn; ++i) x[i] = X[s * kIn + i];
        logits[s] = mlp_infer(P, x);  // the engine's inference path
    }
}

// Gradient of the weighted binary cross-entropy over samples [0, n) with FP32
// master weights: loss = sum_s wt_s * BCE(sigmoid(out_s), y_s), wt = pos_weight
// for y = 1, else 1.  Per-sample gradients are summed over the warp by
// shuffles into the warp's own row of shared memory, the rows of a block in
// fixed order into the block's partial (global), and the partials of all
// blocks in fixed order by k_grad_sum: the gradient does not depend on
// scheduling, so training repeats bit-exactly.
constexpr int kGradBlock = 128;
constexpr int kGradWarps = kGradBlock / 32;
constexpr int kGradMaxBlocks = 128;
__global__ void __launch_bounds__(kGradBlock) k_mlp_grad(const float *__restrict__ Pm, const float *__restrict__ X,
                                                         const float *__restrict__ Y, long long n, float pos_weight,
                                                         float *grad_part, float *loss_part)
{
    __shared__ float P[kPropParams];
    __shared__ float Gw[kGradWarps][kPropParams];
    __shared__ float Lw[kGradWarps];
    for (int i = threadIdx.x; i < kPropParams; i += blockDim.x) {
        P[i] = Pm[i];
        for (int w = 0; w < kGradWarps; ++w) Gw[w][i] = 0.f;
    }
    if (threadIdx.x < kGradWarps) Lw[threadIdx.x] = 0.f;
    __syncthreads();
    float *G = Gw[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const long long stride = (long long)gridDim.x * blockDim.x;
    // all lanes of a warp run the same number of rounds (warp reductions inside)
    const long long base0 = blockIdx.x * (long long)blockDim.x + (threadIdx.x & ~31);
    for (long long base = base0; base < n; base += stride) {
        const long long s = base + lane;
        const bool valid = s < n;
        float x[kIn], z1[kH], z2[kH];
        float y = 0.f;
#pragma unroll
        for (int i = 0; i < kIn; ++i) x[i] = valid ? X[s * kIn + i] : 0.f;
        if (valid) y = Y[s];
        const float out = mlp_forward(P, x, z1, z2);
        const float p = sigmoidf_(out);
        const float wt = valid ? (y > 0.5f ? pos_weight : 1.f) : 0.f;
        // loss (stable form): wt * (softplus(out) - y*out)
        const float sp = out > 0.f ? out + log1pf(__expf(-out)) : log1pf(__expf(out));
        float l = wt * (sp - y * out);
        const float dout = wt * (p - y);
        // output layer
        float dh2[kH];
#pragma unroll
        for (int i = 0; i < kH; ++i) {
            const float h2 = fmaxf(z2[i], 0.f);
            float g = warp_sum(dout * h2);
            if (lane == 0) G[kOffW3 + i] += g;
            dh2[i] = z2[i] > 0.f ? dout * P[kOffW3 + i] : 0.f;
        }
        {
            float g = warp_sum(dout);
            if (lane == 0) G[kOffB3] += g;
            float lw = warp_sum(l);
            if (lane == 0) Lw[threadIdx.x >> 5] += lw;
        }
        // hidden layer 2: dW2[o][i] = dz2[o] * h1[i]
        float dh1[kH];
#pragma unroll
        for (int i = 0; i < kH; ++i) dh1[i] = 0.f;
        for (int o = 0; o < kH; ++o) {
            const float dz = dh2[o];
            float g = warp_sum(dz);
            if (lane == 0) G[kOffB2 + o] += g;
#pragma unroll
            for (int i = 0; i < kH; ++i) {
                const float h1 = fmaxf(z1[i], 0.f);
                float gg = warp_sum(dz * h1);
                if (lane == 0) G[kOffW2 + o * kH + i] += gg;
                dh1[i] = fmaf(dz, P[kOffW2 + o * kH + i], dh1[i]);
            }
        }
        // hidden layer 1
        for (int o = 0; o < kH; ++o) {
            const float dz = z1[o] > 0.f ? dh1[o] : 0.f;
            float g = warp_sum(dz);
            if (lane == 0) G[kOffB1 + o] += g;
#pragma unroll
            for (int i = 0; i < kIn; ++i) {
                float gg = warp_sum(dz * x[i]);
                if (lane == 0) G[kOffW1 + o * kIn + i] += gg;
            }
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < kPropParams; i += blockDim.x) {
        float t = 0.f;
        for (int w = 0; w < kGradWarps; ++w) t += Gw[w][i];
        grad_part[(long long)blockIdx.x * kPropParams + i] = t;
    }
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < kGradWarps; ++w) t += Lw[w];
        loss_part[blockIdx.x] = t;
    }
}

// grad = sum of the block partials in block order (and the loss likewise,
// added to *loss).
__global__ void k_grad_sum(const float *__restrict__ grad_part, const float *__restrict__ loss_part, int nblocks,
                           float *grad, float *loss)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kPropParams) {
        float t = 0.f;
        for (int b = 0; b < nblocks; ++b) t += grad_part[(long long)b * kPropParams + i];
        grad[i] = t;
    }
    if (i == kPropParams) {
        float t = 0.f;
        for (int b = 0; b < nblocks; ++b) t += loss_part[b];
        *loss += t;
    }
}

static int grad_blocks(long long n)
{
    long long g = (n + kGradBlock - 1) / kGradBlock;
    return (int)(g < kGradMaxBlocks ? (g < 1 ? 1 : g) : kGradMaxBlocks);
}

// Adam on the master weights (gradient divided by the batch size), then the
// BF16 inference copy.
__global__ void k_adam(float *Pm, float *m, float *v, const float *grad, float scale, float lr, float b1, float b2,
                       float eps, int t, __nv_bfloat16 *wb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kPropParams) return;
    const float g = grad[i] * scale;
    m[i] = b1 * m[i] + (1.f - b1) * g;
    v[i] = b2 * v[i] + (1.f - b2) * g * g;
    const float mh = m[i] / (1.f - powf(b1, (float)t));
    const float vh = v[i] / (1.f - powf(b2, (float)t));
    Pm[i] -= lr * mh / (sqrtf(vh) + eps);
    wb[i] = __float2bfloat16_rn(Pm[i]);
}

__global__ void k_to_bf16(const float *Pm, __nv_bfloat16 *wb)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < kPropParams) wb[i] = __float2bfloat16_rn(Pm[i]);
}

// Gather a mini-batch (indices idx) of the sample set into contiguous rows.
__global__ void k_gather_batch(const float *__restrict__ X, const float *__restrict__ Y, const int64_t *__restrict__ idx,
                               int nb, float *Xb, float *Yb)
{
    for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < nb; s += gridDim.x * blockDim.x) {
        const long long k = idx[s];
#pragma unroll
        for (int i = 0; i < kIn; ++i) Xb[(long long)s * kIn + i] = X[k * kIn + i];
        Yb[s] = Y[k];
    }
}

// ---------------------------------------------------------------------------
// Engine side: features, trace samples and proposals of one phase-1 sweep.
// ---------------------------------------------------------------------------
struct PropArgs {
    const int64_t *__restrict__ offs;
    const int32_t *__restrict__ comm;
    const int32_t *__restrict__ K;
    const int32_t *__restrict__ In;
    const int32_t *__restrict__ size;
    const float *__restrict__ feat_gain;
    const int32_t *__restrict__ feat_ndist;
    const int32_t *__restrict__ last_move;
    const int32_t *__restrict__ lists;  // active lists (bin segments)
    const int *__restrict__ counts;     // active count per bin
    int start[kNumBins];                // bin segment starts
    int32_t *prop_list;
    DevStats *st;
    const __nv_bfloat16 *__restrict__ wb;
    float *X;
    int32_t *V;
    long long cap;
    long long *count;
    float thr_logit;
    unsigned long long sample_mask;     // a vertex is sampled when hash & mask == 0
    int iteration, level;
};

// splitmix64 output function (Steele, Lea, Flood 2014): the sampling hash.
__device__ __forceinline__ unsigned long long mix64(unsigned long long z)
{
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
}

// The 8 features of vertex v before its decision in iteration a.iteration:
// log degree, weight fraction to the own community, last corrected gain,
// log distinct neighbour communities at the last decision, moved in the
// previous iteration, log iteration, level, log size of the own community.
__device__ __forceinline__ void vertex_features(const PropArgs &a, int v, float f[kIn])
{
    const long long deg = a.offs[v + 1] - a.offs[v];
    const int c = a.comm[v];
    const int k = a.K[v];
    f[0] = log1pf((float)deg);
    f[1] = k > 0 ? (float)a.In[v] / (float)k : 0.f;
    f[2] = fminf(fmaxf(a.feat_gain[v], -4.f), 4.f);
    f[3] = log1pf((float)max(a.feat_ndist[v], 0));
    f[4] = a.last_move[v] == a.iteration - 1 ? 1.f : 0.f;
    f[5] = log1pf((float)a.iteration);
    f[6] = (float)a.level;
    f[7] = log1pf((float)a.size[c]);
}

// MODE 1: append sampled feature rows (vertex ids in V, labelled after the
// sweep).  MODE 2: propose the vertices whose logit reaches the threshold.
template <int MODE>
__global__ void __launch_bounds__(256) k_prop_step(PropArgs a)
{
    __shared__ float P[MODE == 2 ? kPropParams : 1];
    if (MODE == 2) {
        for (int i = threadIdx.x; i < kPropParams; i += blockDim.x) P[i] = __bfloat162float(a.wb[i]);
        __syncthreads();
    }
    const int bin = blockIdx.y;
    const int cnt = a.counts[bin];
    const int32_t *list = a.lists + a.start[bin];
    const int lane = threadIdx.x & 31;
    unsigned long long sk = 0, ske = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long base = blockIdx.x * (long long)blockDim.x + (threadIdx.x & ~31); base < cnt; base += stride) {
        const long long i = base + lane;
        const bool has = i < cnt;
        int v = 0;
        float f[kIn];
        if (has) {
            v = list[i];
            vertex_features(a, v, f);
        }
        if (MODE == 1) {
            const unsigned long long h =
                mix64(((unsigned long long)a.level << 48) ^ ((unsigned long long)a.iteration << 32) ^ (unsigned)v);
            if (has && (h & a.sample_mask) == 0) {
                const long long k = atomicAdd((unsigned long long *)a.count, 1ull);
                if (k < a.cap) {
#pragma unroll
                    for (int j = 0; j < kIn; ++j) a.X[k * kIn + j] = f[j];
                    a.V[k] = v;
                }
            }
        } else {
            bool prop = false;
            if (has) {
                prop = mlp_infer(P, f) >= a.thr_logit;
                if (!prop) {
                    sk += 1;
                    ske += (unsigned long long)(a.offs[v + 1] - a.offs[v]);
                }
            }
            warp_append(prop, v, a.prop_list + a.start[bin], &a.st->prop_count[bin]);
        }
    }
    if (MODE == 2) {
        sk = warp_sum(sk);
        ske = warp_sum(ske);
        if (lane == 0 && sk) {
            atomicAdd(&a.st->skipped, sk);
            atomicAdd(&a.st->skipped_edges, ske);
        }
    }
}

__global__ void k_prop_mark(DevStats *st, const long long *count, int mode)
{
    st->trace_mark = *count;
    if (mode == 2)
        for (int i = 0; i < kNumBins; ++i) st->prop_count[i] = 0;
}

// Labels of the rows appended in this sweep: the vertex moved.
__global__ void k_trace_labels(const DevStats *__restrict__ st, const long long *__restrict__ count, long long cap,
                               const int32_t *__restrict__ V, const int32_t *__restrict__ last_move, int iteration,
                               float *Y)
{
    long long hi = *count;
    if (hi > cap) hi = cap;
    for (long long i = st->trace_mark + blockIdx.x * (long long)blockDim.x + threadIdx.x; i < hi;
         i += (long long)gridDim.x * blockDim.x)
        Y[i] = last_move[V[i]] == iteration ? 1.f : 0.f;
}

__global__ void k_features_init(int n, float *feat_gain, int32_t *feat_ndist, int32_t *last_move)
{
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < n; v += gridDim.x * blockDim.x) {
        feat_gain[v] = 0.f;
        feat_ndist[v] = -1;
        last_move[v] = -2;
    }
}

static int prop_num_sms()
{
    static int sms = 0;
    if (sms == 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 148;
    }
    return sms;
}

void p1_features_init(Phase1Buffers &b, int n, cudaStream_t st)
{
    if (n <= 0) return;
    int grid = (n + 255) / 256;
    if (grid > prop_num_sms() * 8) grid = prop_num_sms() * 8;
    k_features_init<<<grid, 256, 0, st>>>(n, b.feat_gain, b.feat_ndist, b.last_move);
    note_launch(1);
}

void p1_proposal_step(const LevelGraph &g, Phase1Buffers &b, const ProposalStep &ps, const int32_t *lists,
                      const int *counts, const int *bin_start, const int *level_cnt, cudaStream_t st)
{
    PropArgs a;
    a.offs = g.offs;
    a.comm = b.comm;
    a.K = b.K;
    a.In = b.In;
    a.size = b.size;
    a.feat_gain = b.feat_gain;
    a.feat_ndist = b.feat_ndist;
    a.last_move = b.last_move;
    a.lists = lists;
    a.counts = counts;
    int maxc = 0;
    for (int i = 0; i < kNumBins; ++i) {
        a.start[i] = bin_start[i];
        if (i < kNumBins - 1 && level_cnt[i] > maxc) maxc = level_cnt[i];
    }
    a.prop_list = b.prop_list;
    a.st = b.stats;
    a.wb = (const __nv_bfloat16 *)ps.pv.wb;
    a.X = ps.pv.X;
    a.V = ps.pv.V;
    a.cap = ps.pv.cap;
    a.count = ps.pv.count;
    const float t = ps.threshold;
    a.thr_logit = t <= 0.f ? -INFINITY : (t >= 1.f ? INFINITY : logf(t / (1.f - t)));
    a.sample_mask = (ps.sample_shift <= 0) ? 0ull : ((1ull << (ps.sample_shift > 62 ? 62 : ps.sample_shift)) - 1ull);
    a.iteration = ps.iteration;
    a.level = ps.level;
    k_prop_mark<<<1, 1, 0, st>>>(b.stats, ps.pv.count ? ps.pv.count : &b.stats->trace_mark, ps.mode);
    int gx = (maxc + 255) / 256;
    const int cap = prop_num_sms() * 4;
    if (gx > cap) gx = cap;
    if (gx < 1) gx = 1;
    dim3 grid(gx, kNumBins - 1);  // bins 0-6; hub vertices are always decided
    if (ps.mode == GALA_PROPOSAL_TRACE)
        k_prop_step<1><<<grid, 256, 0, st>>>(a);
    else
        k_prop_step<2><<<grid, 256, 0, st>>>(a);
    note_launch(2);
}

void p1_trace_labels(Phase1Buffers &b, const ProposalStep &ps, cudaStream_t st)
{
    k_trace_labels<<<prop_num_sms() * 2, 256, 0, st>>>(b.stats, ps.pv.count, ps.pv.cap, ps.pv.V, b.last_move,
                                                        ps.iteration, ps.pv.Y);
    note_launch(1);
}

}  // namespace gala

using namespace gala;

struct gala_proposal {
    int device = 0;
    cudaStream_t stream = nullptr;
    float *Pm = nullptr, *m = nullptr, *v = nullptr, *grad = nullptr, *loss = nullptr;
    float *grad_part = nullptr, *loss_part = nullptr;  // per-block gradient partials
    __nv_bfloat16 *wb = nullptr;
    int adam_t = 0;
    // samples: features (kIn per row), labels, row capacity
    long long cap = 0;
    float *X = nullptr, *Y = nullptr;
    int32_t *V = nullptr;        // vertex of each sample while its sweep runs
    long long *count = nullptr;  // device
    // mini-batch scratch
    int batch_cap = 0;
    float *Xb = nullptr, *Yb = nullptr;
    int64_t *idx = nullptr;
    std::vector<void *> allocs;
};

namespace {
template <typename T>
bool palloc(gala_proposal *p, T **ptr, size_t count)
{
    if (count == 0) count = 1;
    void *q = nullptr;
    if (cudaMalloc(&q, count * sizeof(T)) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    p->allocs.push_back(q);
    *ptr = (T *)q;
    return true;
}
}  // namespace

namespace gala {
// Sample buffer of a proposal (used by the engine's trace mode).
ProposalView proposal_view(gala_proposal *p)
{
    ProposalView v{};
    if (!p) return v;
    v.X = p->X;
    v.Y = p->Y;
    v.V = p->V;
    v.cap = p->cap;
    v.count = p->count;
    v.wb = p->wb;
    return v;
}
}  // namespace gala

extern "C" {

void gala_proposal_destroy(gala_proposal *p)
{
    if (!p) return;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(p->device);
    if (p->stream) cudaStreamSynchronize(p->stream);
    for (void *q : p->allocs) cudaFree(q);
    if (p->stream) cudaStreamDestroy(p->stream);
    cudaSetDevice(prev);
    delete p;
}

gala_status gala_proposal_create(int32_t device, int64_t max_samples, uint64_t seed, gala_proposal **out)
{
    clear_error();
    if (!out || max_samples < 0) {
        set_error("gala_proposal_create: bad arguments");
        return GALA_ERR_INVALID;
    }
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) {
        cudaGetLastError();
        set_error("no CUDA device visible");
        return GALA_ERR_NO_DEVICE;
    }
    cudaError_t ce;
    if ((ce = cudaSetDevice(device)) != cudaSuccess) return cuda_fail(ce, "cudaSetDevice");
    gala_proposal *p = new gala_proposal();
    p->device = device;
    p->cap = max_samples;
    p->batch_cap = 1 << 16;
    bool ok = cudaStreamCreateWithFlags(&p->stream, cudaStreamNonBlocking) == cudaSuccess;
    ok = ok && palloc(p, &p->grad_part, (size_t)kGradMaxBlocks * kPropParams) &&
         palloc(p, &p->loss_part, (size_t)kGradMaxBlocks);
    ok = ok && palloc(p, &p->Pm, kPropParams) && palloc(p, &p->m, kPropParams) && palloc(p, &p->v, kPropParams) &&
         palloc(p, &p->grad, kPropParams) && palloc(p, &p->loss, 1) && palloc(p, &p->wb, kPropParams) &&
         palloc(p, &p->X, (size_t)max_samples * kIn) && palloc(p, &p->Y, (size_t)max_samples) &&
         palloc(p, &p->V, (size_t)max_samples) &&
         palloc(p, &p->count, 1) && palloc(p, &p->Xb, (size_t)p->batch_cap * kIn) &&
         palloc(p, &p->Yb, (size_t)p->batch_cap) &&
         palloc(p, &p->idx, (size_t)std::max<long long>(p->batch_cap, max_samples));
    if (!ok) {
        gala_proposal_destroy(p);
        set_error("gala_proposal_create: device allocation failed");
        return GALA_ERR_OOM;
    }
    // He-style initialisation from a seeded host generator
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.f, 1.f);
    std::vector<float> h(kPropParams, 0.f);
    for (int i = 0; i < kH * kIn; ++i) h[kOffW1 + i] = nd(rng) * sqrtf(2.f / kIn);
    for (int i = 0; i < kH * kH; ++i) h[kOffW2 + i] = nd(rng) * sqrtf(2.f / kH);
    for (int i = 0; i < kH; ++i) h[kOffW3 + i] = nd(rng) * sqrtf(1.f / kH);
    cudaMemcpyAsync(p->Pm, h.data(), kPropParams * sizeof(float), cudaMemcpyHostToDevice, p->stream);
    cudaMemsetAsync(p->m, 0, kPropParams * sizeof(float), p->stream);
    cudaMemsetAsync(p->v, 0, kPropParams * sizeof(float), p->stream);
    cudaMemsetAsync(p->count, 0, sizeof(long long), p->stream);
    k_to_bf16<<<(kPropParams + 255) / 256, 256, 0, p->stream>>>(p->Pm, p->wb);
    note_launch(1);
    if ((ce = cudaStreamSynchronize(p->stream)) != cudaSuccess) {
        gala_proposal_destroy(p);
        return cuda_fail(ce, "gala_proposal_create");
    }
    *out = p;
    return GALA_OK;
}

gala_status gala_proposal_get_params(gala_proposal *p, float *params, int32_t capacity, int32_t *count)
{
    clear_error();
    if (!p) {
        set_error("gala_proposal_get_params: null proposal");
        return GALA_ERR_INVALID;
    }
    if (count) *count = kPropParams;
    if (!params) return GALA_OK;
    if (capacity < kPropParams) {
        set_error("gala_proposal_get_params: capacity %d < %d", capacity, kPropParams);
        return GALA_ERR_INVALID;
    }
    cudaSetDevice(p->device);
    cudaError_t ce = cudaMemcpy(params, p->Pm, kPropParams * sizeof(float), cudaMemcpyDeviceToHost);
    return ce == cudaSuccess ? GALA_OK : cuda_fail(ce, "gala_proposal_get_params");
}

gala_status gala_proposal_set_params(gala_proposal *p, const float *params, int32_t count)
{
    clear_error();
    if (!p || !params || count != kPropParams) {
        set_error("gala_proposal_set_params: bad arguments (need %d parameters)", kPropParams);
        return GALA_ERR_INVALID;
    }
    cudaSetDevice(p->device);
    cudaError_t ce = cudaMemcpy(p->Pm, params, kPropParams * sizeof(float), cudaMemcpyHostToDevice);
    if (ce != cudaSuccess) return cuda_fail(ce, "gala_proposal_set_params");
    k_to_bf16<<<(kPropParams + 255) / 256, 256, 0, p->stream>>>(p->Pm, p->wb);
    note_launch(1);
    ce = cudaStreamSynchronize(p->stream);
    return ce == cudaSuccess ? GALA_OK : cuda_fail(ce, "gala_proposal_set_params");
}

gala_status gala_proposal_samples(gala_proposal *p, int64_t *count, int64_t *positives)
{
    clear_error();
    if (!p) {
        set_error("gala_proposal_samples: null proposal");
        return GALA_ERR_INVALID;
    }
    cudaSetDevice(p->device);
    long long c = 0;
    cudaError_t ce = cudaMemcpy(&c, p->count, sizeof(long long), cudaMemcpyDeviceToHost);
    if (ce != cudaSuccess) return cuda_fail(ce, "gala_proposal_samples");
    if (c > p->cap) c = p->cap;
    if (count) *count = c;
    if (positives) {
        std::vector<float> y((size_t)c);
        if (c > 0 && (ce = cudaMemcpy(y.data(), p->Y, (size_t)c * sizeof(float), cudaMemcpyDeviceToHost)) !=
                         cudaSuccess)
            return cuda_fail(ce, "gala_proposal_samples");
        long long pos = 0;
        for (float f : y) pos += f > 0.5f;
        *positives = pos;
    }
    return GALA_OK;
}

gala_status gala_proposal_clear_samples(gala_proposal *p)
{
    clear_error();
    if (!p) {
        set_error("gala_proposal_clear_samples: null proposal");
        return GALA_ERR_INVALID;
    }
    cudaSetDevice(p->device);
    cudaError_t ce = cudaMemset(p->count, 0, sizeof(long long));
    return ce == cudaSuccess ? GALA_OK : cuda_fail(ce, "gala_proposal_clear_samples");
}

// Copy n samples (host) out of / into the sample set.
gala_status gala_proposal_read_samples(gala_proposal *p, int64_t first, int64_t n, float *features, float *labels)
{
    clear_error();
    if (!p || first < 0 || n < 0 || first + n > p->cap) {
        set_error("gala_proposal_read_samples: bad arguments");
        return GALA_ERR_INVALID;
    }
    cudaSetDevice(p->device);
    cudaError_t ce = cudaSuccess;
    if (features && n)
        ce = cudaMemcpy(features, p->X + first * kIn, (size_t)n * kIn * sizeof(float), cudaMemcpyDeviceToHost);
    if (ce == cudaSuccess && labels && n)
        ce = cudaMemcpy(labels, p->Y + first, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost);
    return ce == cudaSuccess ? GALA_OK : cuda_fail(ce, "gala_proposal_read_samples");
}

// Loss and gradient (summed over the samples) of caller-given samples with
// the current master weights: the check of the GPU backward pass.
gala_status gala_proposal_gradient(gala_proposal *p, const float *features, const float *labels, int32_t n,
                                   float pos_weight, float *grad_out, float *loss_out)
{
    clear_error();
    if (!p || !features || !labels || n <= 0 || n > p->batch_cap || !grad_out) {
        set_error("gala_proposal_gradient: bad arguments (n <= %d)", p ? p->batch_cap : 0);
        return GALA_ERR_INVALID;
    }
    cudaSetDevice(p->device);
    cudaStream_t st = p->stream;
    cudaMemcpyAsync(p->Xb, features, (size_t)n * kIn * sizeof(float), cudaMemcpyHostToDevice, st);
    cudaMemcpyAsync(p->Yb, labels, (size_t)n * sizeof(float), cudaMemcpyHostToDevice, st);
    cudaMemsetAsync(p->loss, 0, sizeof(float), st);
    const int gb = grad_blocks(n);
    k_mlp_grad<<<gb, kGradBlock, 0, st>>>(p->Pm, p->Xb, p->Yb, n, pos_weight, p->grad_part, p->loss_part);
    k_grad_sum<<<(kPropParams + 256) / 256, 256, 0, st>>>(p->grad_part, p->loss_part, gb, p->grad, p->loss);
    note_launch(2);
    cudaMemcpyAsync(grad_out, p->grad, kPropParams * sizeof(float), cudaMemcpyDeviceToHost, st);
    float l = 0.f;
    cudaMemcpyAsync(&l, p->loss, sizeof(float), cudaMemcpyDeviceToHost, st);
    cudaError_t ce = cudaGetLastError();  // a failed launch, else the stream's status
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return cuda_fail(ce, "gala_proposal_gradient");
    if (loss_out) *loss_out = l;
    return GALA_OK;
}

// Logits of caller-given samples with the BF16 inference weights.
gala_status gala_proposal_logits(gala_proposal *p, const float *features, int32_t n, float *logits)
{
    clear_error();
    if (!p || !features || !logits || n <= 0 || n > p->batch_cap) {
        set_error("gala_proposal_logits: bad arguments");
        return GALA_ERR_INVALID;
    }
    cudaSetDevice(p->device);
    cudaStream_t st = p->stream;
    cudaMemcpyAsync(p->Xb, features, (size_t)n * kIn * sizeof(float), cudaMemcpyHostToDevice, st);
    k_mlp_logits<<<(n + 255) / 256, 256, 0, st>>>(p->wb, p->Xb, n, p->Yb);
    note_launch(1);
    cudaMemcpyAsync(logits, p->Yb, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, st);
    cudaError_t ce = cudaGetLastError();  // a failed launch, else the stream's status
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    return ce == cudaSuccess ? GALA_OK : cuda_fail(ce, "gala_proposal_logits");
}

// Mini-batch Adam over the sample set: `epochs` passes of batches of
// batch_size samples drawn without replacement (seeded shuffle).
gala_status gala_proposal_train(gala_proposal *p, int32_t epochs, int32_t batch_size, float lr, float pos_weight,
                                uint64_t seed, float *final_loss)
{
    clear_error();
    if (!p || epochs <= 0 || batch_size <= 0 || batch_size > p->batch_cap) {
        set_error("gala_proposal_train: bad arguments (batch <= %d)", p ? p->batch_cap : 0);
        return GALA_ERR_INVALID;
    }
    int64_t n = 0;
    gala_status s = gala_proposal_samples(p, &n, nullptr);
    if (s) return s;
    if (n == 0) {
        set_error("gala_proposal_train: no samples");
        return GALA_ERR_INVALID;
    }
    cudaStream_t st = p->stream;
    // The sweeps append their samples with an atomic cursor, so the row order
    // of the sample set varies from run to run.  Training walks a canonical
    // order instead (rows sorted by vertex, features and label; equal rows
    // are interchangeable), shuffled by the seed: the same samples give the
    // same network.
    std::vector<int64_t> base((size_t)n);
    {
        std::vector<float> X((size_t)n * kIn), Y((size_t)n);
        std::vector<int32_t> V((size_t)n);
        cudaError_t ce = cudaMemcpyAsync(X.data(), p->X, X.size() * sizeof(float), cudaMemcpyDeviceToHost, st);
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(Y.data(), p->Y, Y.size() * sizeof(float), cudaMemcpyDeviceToHost, st);
        if (ce == cudaSuccess)
            ce = cudaMemcpyAsync(V.data(), p->V, V.size() * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
        if (ce != cudaSuccess) return cuda_fail(ce, "gala_proposal_train: samples");
        for (int64_t i = 0; i < n; ++i) base[i] = i;
        std::sort(base.begin(), base.end(), [&](int64_t a, int64_t b) {
            if (V[a] != V[b]) return V[a] < V[b];
            const int c = memcmp(&X[(size_t)a * kIn], &X[(size_t)b * kIn], kIn * sizeof(float));
            if (c != 0) return c < 0;
            return memcmp(&Y[a], &Y[b], sizeof(float)) < 0;
        });
    }
    std::mt19937_64 rng(seed);
    std::vector<int64_t> order((size_t)n), perm((size_t)n);
    for (int64_t i = 0; i < n; ++i) order[i] = i;
    float epoch_loss = 0.f;
    for (int e = 0; e < epochs; ++e) {
        std::shuffle(order.begin(), order.end(), rng);
        for (int64_t i = 0; i < n; ++i) perm[i] = base[order[i]];
        cudaMemsetAsync(p->loss, 0, sizeof(float), st);
        cudaMemcpyAsync(p->idx, perm.data(), (size_t)n * sizeof(int64_t), cudaMemcpyHostToDevice, st);
        for (int64_t b0 = 0; b0 < n; b0 += batch_size) {
            const int nb = (int)std::min<int64_t>(batch_size, n - b0);
            k_gather_batch<<<(nb + 255) / 256, 256, 0, st>>>(p->X, p->Y, p->idx + b0, nb, p->Xb, p->Yb);
            const int gb = grad_blocks(nb);
            k_mlp_grad<<<gb, kGradBlock, 0, st>>>(p->Pm, p->Xb, p->Yb, nb, pos_weight, p->grad_part, p->loss_part);
            k_grad_sum<<<(kPropParams + 256) / 256, 256, 0, st>>>(p->grad_part, p->loss_part, gb, p->grad, p->loss);
            p->adam_t++;
            k_adam<<<(kPropParams + 255) / 256, 256, 0, st>>>(p->Pm, p->m, p->v, p->grad, 1.f / nb, lr, 0.9f, 0.999f,
                                                             1e-8f, p->adam_t, p->wb);
            note_launch(4);
        }
        // synchronous read: the permutation is reshuffled only after the
        // epoch's copy and kernels are done
        cudaError_t ce = cudaMemcpyAsync(&epoch_loss, p->loss, sizeof(float), cudaMemcpyDeviceToHost, st);
        if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
        if (ce != cudaSuccess) return cuda_fail(ce, "gala_proposal_train");
        epoch_loss /= (float)n;
    }
    cudaError_t ce = cudaGetLastError();  // a failed launch, else the stream's status
    if (ce == cudaSuccess) ce = cudaStreamSynchronize(st);
    if (ce != cudaSuccess) return cuda_fail(ce, "gala_proposal_train");
    if (final_loss) *final_loss = epoch_loss;
    return GALA_OK;
}

}  // extern "C"
