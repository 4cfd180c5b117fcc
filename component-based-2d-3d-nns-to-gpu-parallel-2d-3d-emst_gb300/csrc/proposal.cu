// proposal.cu -- the learned proposal's data and training on the GPU:
//
//   * traces: while the plain method builds its round-1 neighbour lists,
//     sampled queries record their features and, once their list is
//     complete, the labels -- the K-th nearest distance relative to the own
//     leaf's bound, and whether that bound could be tightened at all
//     (written by k_knn_first, cnns_search.cuh);
//   * training: forward and backward of the 8-32-32-2 MLP with BF16 MMA
//     (m16n8k16, FP32 accumulate), FP32 master weights and Adam;
//   * packing: FP32 weights into the fragment order of the fused inference.
//
// None of this is in the reference (its search has no learned part); the
// proposal only sets the starting bound of the round-1 search, see
// proposal.cuh.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/emst.h"
#include "emst_ctx.h"
#include "emst_device.cuh"
#include "proposal.cuh"

namespace emst {

namespace {

using prop::kHid;
using prop::kIn;
using prop::kNumWeights;
using prop::kOut;
using prop::kRec;

__device__ __forceinline__ float bf16_val(__nv_bfloat16 b) { return __bfloat162float(b); }

__device__ __forceinline__ uint32_t pack2(__nv_bfloat16 lo, __nv_bfloat16 hi)
{
    return (uint32_t)*reinterpret_cast<const uint16_t*>(&lo) | ((uint32_t)*reinterpret_cast<const uint16_t*>(&hi) << 16);
}

// FP32 weights -> fragment order of prop::infer_warp (one warp).
__global__ void k_pack_frag(const float* __restrict__ w, prop::Frag* __restrict__ out)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    const float* W1 = w + prop::kOffW1;
    const float* W2 = w + prop::kOffW2;
    const float* W3 = w + prop::kOffW3;
    for (int j = 0; j < 4; ++j)
        out->w1[j][lane] = prop::pack_bf16(W1[(2 * t) * kHid + 8 * j + g], W1[(2 * t + 1) * kHid + 8 * j + g]);
    for (int j = 0; j < 4; ++j)
        for (int q = 0; q < 2; ++q) {
            const int n = 8 * j + g, k = 16 * q + 2 * t;
            out->w2[j][q][lane] = make_uint2(prop::pack_bf16(W2[k * kHid + n], W2[(k + 1) * kHid + n]),
                                             prop::pack_bf16(W2[(k + 8) * kHid + n], W2[(k + 9) * kHid + n]));
        }
    for (int q = 0; q < 2; ++q) {
        const int k = 16 * q + 2 * t;
        const bool live = g < kOut;
        out->w3[q][lane] = make_uint2(
            prop::pack_bf16(live ? W3[k * kOut + g] : 0.f, live ? W3[(k + 1) * kOut + g] : 0.f),
            prop::pack_bf16(live ? W3[(k + 8) * kOut + g] : 0.f, live ? W3[(k + 9) * kOut + g] : 0.f));
    }
    out->b1[lane] = w[prop::kOffB1 + lane];
    out->b2[lane] = w[prop::kOffB2 + lane];
    if (lane < 8) out->b3[lane] = lane < kOut ? w[prop::kOffB3 + lane] : 0.f;
}

// ----------------------------------------------------------------------------
// Training: one warp = 32 samples, all operands staged as BF16 in shared
// memory, every product an m16n8k16 MMA.
// ----------------------------------------------------------------------------
constexpr int kTrainWarps = 2;

// Operand fragments from a row-major BF16 matrix S (leading dimension ld).
// A tile element (i, k) = S[m0 + i][k0 + k], or S[k0 + k][m0 + i] when TRANS.
template <bool TRANS>
__device__ __forceinline__ void load_a(const __nv_bfloat16* S, int ld, int m0, int k0, uint32_t (&r)[4])
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    auto el = [&](int i, int k) { return TRANS ? S[(k0 + k) * ld + m0 + i] : S[(m0 + i) * ld + k0 + k]; };
    r[0] = pack2(el(g, 2 * t), el(g, 2 * t + 1));
    r[1] = pack2(el(g + 8, 2 * t), el(g + 8, 2 * t + 1));
    r[2] = pack2(el(g, 2 * t + 8), el(g, 2 * t + 9));
    r[3] = pack2(el(g + 8, 2 * t + 8), el(g + 8, 2 * t + 9));
}

// B tile element (k, j) = S[k0 + k][n0 + j], or S[n0 + j][k0 + k] when TRANS.
template <bool TRANS>
__device__ __forceinline__ void load_b(const __nv_bfloat16* S, int ld, int k0, int n0, uint32_t (&r)[2])
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    auto el = [&](int k, int j) { return TRANS ? S[(n0 + j) * ld + k0 + k] : S[(k0 + k) * ld + n0 + j]; };
    r[0] = pack2(el(2 * t, g), el(2 * t + 1, g));
    r[1] = pack2(el(2 * t + 8, g), el(2 * t + 9, g));
}

// C[M x N] = A[M x K] B[K x N] (+ bias per column), FP32 out to row-major C.
template <bool TA, bool TB>
__device__ void warp_gemm(const __nv_bfloat16* A, int lda, const __nv_bfloat16* B, int ldb, int M, int N, int K,
                          const float* bias, float* C, int ldc)
{
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    for (int m0 = 0; m0 < M; m0 += 16)
        for (int n0 = 0; n0 < N; n0 += 8) {
            float d[4];
            const float bl = bias ? bias[n0 + 2 * t] : 0.f, bh = bias ? bias[n0 + 2 * t + 1] : 0.f;
            d[0] = bl, d[1] = bh, d[2] = bl, d[3] = bh;
            for (int k0 = 0; k0 < K; k0 += 16) {
                uint32_t a[4], b[2];
                load_a<TA>(A, lda, m0, k0, a);
                load_b<TB>(B, ldb, k0, n0, b);
                prop::mma16816(d, a[0], a[1], a[2], a[3], b[0], b[1]);
            }
            C[(m0 + g) * ldc + n0 + 2 * t] = d[0];
            C[(m0 + g) * ldc + n0 + 2 * t + 1] = d[1];
            C[(m0 + g + 8) * ldc + n0 + 2 * t] = d[2];
            C[(m0 + g + 8) * ldc + n0 + 2 * t + 1] = d[3];
        }
    __syncwarp();
}

struct TrainSmem {
    __nv_bfloat16 w1[16 * kHid];  // rows 8..15 zero
    __nv_bfloat16 w2[kHid * kHid];
    __nv_bfloat16 w3[kHid * 16];  // columns 2..15 zero
    float b1[kHid], b2[kHid], b3[8];
    float gacc[kNumWeights];
    struct Warp {
        __nv_bfloat16 x[32 * 16], h1[32 * kHid], h2[32 * kHid], dO[32 * 16], dz2[32 * kHid], dz1[32 * kHid];
        float f[32 * kHid];  // FP32 GEMM output
        float dOf[32 * 2];
    } wp[kTrainWarps];
};

// Forward + backward over `count` samples, loss
//   (1/B) sum [ reg_w * m0 * (out0 - t0)^2 + softplus(out1) - y1 * out1 ],
// gradients accumulated into grad (FP32) and the loss sum into loss[0].
// Sample i of the step is record (mul * ((start + i) mod n) + add) mod n: an
// affine permutation of the records per epoch.
__global__ void __launch_bounds__(32 * kTrainWarps)
    k_train_step(const float* __restrict__ rec, uint64_t n, uint64_t start, uint64_t count, uint64_t mul,
                 uint64_t add, float inv_batch, float reg_w, const float* __restrict__ w, float* __restrict__ grad,
                 float* __restrict__ loss)
{
    __shared__ TrainSmem S;
    const int tid = threadIdx.x, lane = tid & 31, wi = tid >> 5;
    for (int i = tid; i < 16 * kHid; i += blockDim.x) {
        const int r = i / kHid, c = i % kHid;
        S.w1[i] = __float2bfloat16_rn(r < kIn ? w[prop::kOffW1 + r * kHid + c] : 0.f);
    }
    for (int i = tid; i < kHid * kHid; i += blockDim.x) S.w2[i] = __float2bfloat16_rn(w[prop::kOffW2 + i]);
    for (int i = tid; i < kHid * 16; i += blockDim.x) {
        const int r = i / 16, c = i % 16;
        S.w3[i] = __float2bfloat16_rn(c < kOut ? w[prop::kOffW3 + r * kOut + c] : 0.f);
    }
    for (int i = tid; i < kHid; i += blockDim.x) {
        S.b1[i] = w[prop::kOffB1 + i];
        S.b2[i] = w[prop::kOffB2 + i];
    }
    for (int i = tid; i < 8; i += blockDim.x) S.b3[i] = i < kOut ? w[prop::kOffB3 + i] : 0.f;
    for (int i = tid; i < kNumWeights; i += blockDim.x) S.gacc[i] = 0.f;
    __syncthreads();

    TrainSmem::Warp& P = S.wp[wi];
    const uint64_t s = (uint64_t)blockIdx.x * blockDim.x + tid;
    const bool live = s < count;
    float t0 = 0.f, y1 = 0.f, m0 = 0.f;
    {
        float f[kIn];
        if (live) {
            const uint64_t r = (mul * ((start + s) % n) + add) % n;
            const float* o = rec + r * kRec;
            for (int j = 0; j < kIn; ++j) f[j] = o[j];
            t0 = o[8];
            y1 = o[9];
            m0 = o[10] > 0.f ? 1.f : 0.f;
        } else {
            for (int j = 0; j < kIn; ++j) f[j] = 0.f;
        }
        for (int j = 0; j < 16; ++j) P.x[lane * 16 + j] = __float2bfloat16_rn(j < kIn ? f[j] : 0.f);
    }
    __syncwarp();
    // forward
    warp_gemm<false, false>(P.x, 16, S.w1, kHid, 32, kHid, 16, S.b1, P.f, kHid);
    for (int j = 0; j < kHid; ++j) P.h1[lane * kHid + j] = __float2bfloat16_rn(fmaxf(P.f[lane * kHid + j], 0.f));
    __syncwarp();
    warp_gemm<false, false>(P.h1, kHid, S.w2, kHid, 32, kHid, kHid, S.b2, P.f, kHid);
    for (int j = 0; j < kHid; ++j) P.h2[lane * kHid + j] = __float2bfloat16_rn(fmaxf(P.f[lane * kHid + j], 0.f));
    __syncwarp();
    warp_gemm<false, false>(P.h2, kHid, S.w3, 16, 32, 8, kHid, S.b3, P.f, 8);
    const float o0 = P.f[lane * 8], o1 = P.f[lane * 8 + 1];
    // loss and its gradient per output
    float l = 0.f, g0 = 0.f, g1 = 0.f;
    if (live) {
        const float e = o0 - t0;
        const float sp = fmaxf(o1, 0.f) + log1pf(expf(-fabsf(o1)));  // softplus
        l = reg_w * m0 * e * e + sp - y1 * o1;
        g0 = 2.f * reg_w * m0 * e * inv_batch;
        g1 = (1.f / (1.f + expf(-o1)) - y1) * inv_batch;
    }
    __syncwarp();
    P.dOf[lane * 2] = g0;
    P.dOf[lane * 2 + 1] = g1;
    for (int j = 0; j < 16; ++j) P.dO[lane * 16 + j] = __float2bfloat16_rn(j == 0 ? g0 : (j == 1 ? g1 : 0.f));
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if (lane == 0) atomicAdd(loss, l);
    __syncwarp();
    // layer 3: dW3 = H2^T dO, db3 = sum dO, dH2 = dO W3^T masked
    warp_gemm<true, false>(P.h2, kHid, P.dO, 16, kHid, 8, 32, nullptr, P.f, 8);
    for (int i = lane; i < kHid * kOut; i += 32) atomicAdd(&S.gacc[prop::kOffW3 + i], P.f[(i / kOut) * 8 + i % kOut]);
    if (lane < kOut) {
        float sb = 0.f;
        for (int r = 0; r < 32; ++r) sb += P.dOf[r * 2 + lane];
        atomicAdd(&S.gacc[prop::kOffB3 + lane], sb);
    }
    __syncwarp();
    warp_gemm<false, true>(P.dO, 16, S.w3, 16, 32, kHid, 16, nullptr, P.f, kHid);
    for (int j = 0; j < kHid; ++j) {
        const float v = bf16_val(P.h2[lane * kHid + j]) > 0.f ? P.f[lane * kHid + j] : 0.f;
        P.f[lane * kHid + j] = v;
        P.dz2[lane * kHid + j] = __float2bfloat16_rn(v);
    }
    __syncwarp();
    {
        float sb = 0.f;
        for (int r = 0; r < 32; ++r) sb += P.f[r * kHid + lane];
        atomicAdd(&S.gacc[prop::kOffB2 + lane], sb);
    }
    __syncwarp();
    // layer 2: dW2 = H1^T dZ2, dH1 = dZ2 W2^T masked
    warp_gemm<true, false>(P.h1, kHid, P.dz2, kHid, kHid, kHid, 32, nullptr, P.f, kHid);
    for (int i = lane; i < kHid * kHid; i += 32) atomicAdd(&S.gacc[prop::kOffW2 + i], P.f[i]);
    __syncwarp();
    warp_gemm<false, true>(P.dz2, kHid, S.w2, kHid, 32, kHid, kHid, nullptr, P.f, kHid);
    for (int j = 0; j < kHid; ++j) {
        const float v = bf16_val(P.h1[lane * kHid + j]) > 0.f ? P.f[lane * kHid + j] : 0.f;
        P.f[lane * kHid + j] = v;
        P.dz1[lane * kHid + j] = __float2bfloat16_rn(v);
    }
    __syncwarp();
    {
        float sb = 0.f;
        for (int r = 0; r < 32; ++r) sb += P.f[r * kHid + lane];
        atomicAdd(&S.gacc[prop::kOffB1 + lane], sb);
    }
    __syncwarp();
    // layer 1: dW1 = X^T dZ1 (rows 0..7)
    warp_gemm<true, false>(P.x, 16, P.dz1, kHid, 16, kHid, 32, nullptr, P.f, kHid);
    for (int i = lane; i < kIn * kHid; i += 32) atomicAdd(&S.gacc[prop::kOffW1 + i], P.f[i]);
    __syncthreads();
    for (int i = tid; i < kNumWeights; i += blockDim.x) atomicAdd(&grad[i], S.gacc[i]);
}

// Adam on the FP32 master weights; clears the gradient.
__global__ void k_adam(float* __restrict__ w, float* __restrict__ m, float* __restrict__ v, float* __restrict__ grad,
                       float lr_t, float b1, float b2, float eps)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kNumWeights) return;
    const float g = grad[i];
    grad[i] = 0.f;
    const float mi = b1 * m[i] + (1.f - b1) * g, vi = b2 * v[i] + (1.f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr_t * mi / (sqrtf(vi) + eps);
}

}  // namespace

uint64_t splitmix(uint64_t& s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static uint64_t gcd_u64(uint64_t a, uint64_t b)
{
    while (b) {
        const uint64_t t = a % b;
        a = b;
        b = t;
    }
    return a;
}

cudaError_t proposal_pack(const float* d_weights, void* d_frag, cudaStream_t s)
{
    k_pack_frag<<<1, 32, 0, s>>>(d_weights, reinterpret_cast<prop::Frag*>(d_frag));
    return cudaGetLastError();
}

size_t proposal_frag_bytes() { return sizeof(prop::Frag); }


// Adam steps over device records; weights in/out on the host.
static emst_status train_on_device(const float* d_rec, int64_t n, const emst_train_config* cfg, float* weights,
                                   float* loss_curve, cudaStream_t s)
{
    float *d_w = nullptr, *d_m = nullptr, *d_v = nullptr, *d_g = nullptr, *d_loss = nullptr;
    const int epochs = cfg->epochs > 0 ? cfg->epochs : 4;
    const int64_t batch = cfg->batch > 0 ? cfg->batch : 4096;
    const float lr = cfg->lr > 0.f ? cfg->lr : 2e-3f;
    const float reg_w = cfg->reg_weight > 0.f ? cfg->reg_weight : 1.f;
    uint64_t seed = cfg->seed;
    const int tpb = 32 * kTrainWarps;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    double b1t = 1.0, b2t = 1.0;
    float host_loss = 0.f;
    cudaError_t e = cudaMalloc(&d_w, sizeof(float) * kNumWeights);
    if (e == cudaSuccess) e = cudaMalloc(&d_m, sizeof(float) * kNumWeights);
    if (e == cudaSuccess) e = cudaMalloc(&d_v, sizeof(float) * kNumWeights);
    if (e == cudaSuccess) e = cudaMalloc(&d_g, sizeof(float) * kNumWeights);
    if (e == cudaSuccess) e = cudaMalloc(&d_loss, sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_w, weights, sizeof(float) * kNumWeights, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_m, 0, sizeof(float) * kNumWeights, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_v, 0, sizeof(float) * kNumWeights, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_g, 0, sizeof(float) * kNumWeights, s);
    for (int ep = 0; ep < epochs && e == cudaSuccess; ++ep) {
        // an affine permutation of the records for this epoch
        uint64_t mul = (splitmix(seed) % (uint64_t)n) | 1u;
        while (gcd_u64(mul, (uint64_t)n) != 1) mul = (mul + 2) % (uint64_t)n ? (mul + 2) % (uint64_t)n : 1;
        const uint64_t add = splitmix(seed) % (uint64_t)n;
        e = cudaMemsetAsync(d_loss, 0, sizeof(float), s);
        for (int64_t st = 0; st < n && e == cudaSuccess; st += batch) {
            const int64_t cnt = std::min<int64_t>(batch, n - st);
            const unsigned blocks = (unsigned)((cnt + tpb - 1) / tpb);
            k_train_step<<<blocks, tpb, 0, s>>>(d_rec, (uint64_t)n, (uint64_t)st, (uint64_t)cnt, mul, add,
                                                1.f / (float)cnt, reg_w, d_w, d_g, d_loss);
            b1t *= b1;
            b2t *= b2;
            const float lr_t = (float)(lr * std::sqrt(1.0 - b2t) / (1.0 - b1t));
            k_adam<<<(kNumWeights + 255) / 256, 256, 0, s>>>(d_w, d_m, d_v, d_g, lr_t, b1, b2, eps);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(&host_loss, d_loss, sizeof(float), cudaMemcpyDeviceToHost, s);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s);
        if (e == cudaSuccess && loss_curve) loss_curve[ep] = host_loss / (float)n;
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(weights, d_w, sizeof(float) * kNumWeights, cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(d_w);
    cudaFree(d_m);
    cudaFree(d_v);
    cudaFree(d_g);
    cudaFree(d_loss);
    if (e == cudaSuccess) return EMST_OK;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? EMST_ENOMEM : EMST_ECUDA;
}

}  // namespace emst

extern "C" {

emst_status emst_proposal_init(uint64_t seed, float* weights)
{
    using namespace emst::prop;
    if (!weights) return EMST_EINVAL;
    uint64_t s = seed;
    auto uni = [&]() { return (float)((emst::splitmix(s) >> 11) * (1.0 / 9007199254740992.0)) * 2.f - 1.f; };
    std::memset(weights, 0, sizeof(float) * kNumWeights);
    const float a1 = std::sqrt(6.f / kIn), a2 = std::sqrt(6.f / kHid);
    for (int i = 0; i < kIn * kHid; ++i) weights[kOffW1 + i] = a1 * uni();
    for (int i = 0; i < kHid * kHid; ++i) weights[kOffW2 + i] = a2 * uni();
    for (int i = 0; i < kHid * kOut; ++i) weights[kOffW3 + i] = 0.5f * a2 * uni();
    return EMST_OK;
}

emst_status emst_proposal_train(const float* records, int64_t n_records, int records_on_device,
                                const emst_train_config* cfg, float* weights, float* loss_curve)
{
    if (!records || n_records < 1 || !cfg || !weights) return EMST_EINVAL;
    if (cudaSetDevice(cfg->device) != cudaSuccess) {
        cudaGetLastError();
        return EMST_ECUDA;
    }
    cudaStream_t s = nullptr;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return EMST_ECUDA;
    const float* d_rec = records;
    float* own = nullptr;
    emst_status status = EMST_OK;
    if (!records_on_device) {
        const size_t bytes = sizeof(float) * emst::prop::kRec * (size_t)n_records;
        cudaError_t e = cudaMalloc(&own, bytes);
        if (e == cudaSuccess) e = cudaMemcpyAsync(own, records, bytes, cudaMemcpyHostToDevice, s);
        if (e != cudaSuccess) status = e == cudaErrorMemoryAllocation ? EMST_ENOMEM : EMST_ECUDA;
        d_rec = own;
    }
    if (status == EMST_OK) status = emst::train_on_device(d_rec, n_records, cfg, weights, loss_curve, s);
    cudaStreamSynchronize(s);
    cudaFree(own);
    cudaStreamDestroy(s);
    cudaGetLastError();
    return status;
}

emst_status emst_proposal_grad(const float* weights, const float* records, int64_t n_records, float reg_weight,
                               float* grad, float* loss)
{
    using namespace emst::prop;
    if (!weights || !records || n_records < 1 || !grad) return EMST_EINVAL;
    float *d_w = nullptr, *d_g = nullptr, *d_rec = nullptr, *d_loss = nullptr;
    const size_t rb = sizeof(float) * kRec * (size_t)n_records;
    const int tpb = 32 * emst::kTrainWarps;
    float host_loss = 0.f;
    cudaError_t e = cudaMalloc(&d_w, sizeof(float) * kNumWeights);
    if (e == cudaSuccess) e = cudaMalloc(&d_g, sizeof(float) * kNumWeights);
    if (e == cudaSuccess) e = cudaMalloc(&d_rec, rb);
    if (e == cudaSuccess) e = cudaMalloc(&d_loss, sizeof(float));
    if (e == cudaSuccess) e = cudaMemcpy(d_w, weights, sizeof(float) * kNumWeights, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(d_rec, records, rb, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(d_g, 0, sizeof(float) * kNumWeights);
    if (e == cudaSuccess) e = cudaMemset(d_loss, 0, sizeof(float));
    if (e == cudaSuccess) {
        emst::k_train_step<<<(unsigned)((n_records + tpb - 1) / tpb), tpb>>>(
            d_rec, (uint64_t)n_records, 0, (uint64_t)n_records, 1, 0, 1.f / (float)n_records,
            reg_weight > 0.f ? reg_weight : 1.f, d_w, d_g, d_loss);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(grad, d_g, sizeof(float) * kNumWeights, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(&host_loss, d_loss, sizeof(float), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && loss) *loss = host_loss / (float)n_records;
    cudaFree(d_w);
    cudaFree(d_g);
    cudaFree(d_rec);
    cudaFree(d_loss);
    if (e == cudaSuccess) return EMST_OK;
    cudaGetLastError();
    return e == cudaErrorMemoryAllocation ? EMST_ENOMEM : EMST_ECUDA;
}

}  // extern "C"
