// proposal.cuh -- the learned search proposal: features, the 8-32-32-2 MLP on
// BF16 tensor-core MMA (m16n8k16, FP32 accumulate), and the weight layouts
// shared by the fused inference (cnns_search.cuh) and the training kernels
// (proposal.cu).
//
// The proposal steers the round-1 neighbour-list build (k_knn_first), the
// dominant kernel of a solve.  There every point searches for its K nearest
// points; the warp's walk starts from a certified bound, the K-th smallest d2
// to the other points of the query's own leaf.  For each query the network
// predicts
//   out0: log2(d2 of its K-th nearest point / that certified bound) / 8, at
//         most 0 -- the search radius: the walk starts from the predicted
//         radius (times 2^margin), so fewer nodes and candidates fall within
//         the bound and fewer inserts run;
//   out1: logit of "the own leaf's bound can be tightened at all" (false when
//         the K nearest all lie in the own leaf) -- below the threshold the
//         query keeps the certified bound.
// Neither output changes what is found.  A query whose predicted radius held
// fewer than K points is searched again from the certified bound (a
// mispredict), so every list -- and the edge set -- is the plain method's.
#pragma once
#include <cstdint>

#include <cuda_bf16.h>

namespace emst {

namespace prop {

constexpr int kIn = 8, kHid = 32, kOut = 2;
// FP32 master weights, row-major [in][out]: W1 b1 W2 b2 W3 b3.
constexpr int kOffW1 = 0, kOffB1 = kOffW1 + kIn * kHid, kOffW2 = kOffB1 + kHid, kOffB2 = kOffW2 + kHid * kHid,
              kOffW3 = kOffB2 + kHid, kOffB3 = kOffW3 + kHid * kOut, kNumWeights = kOffB3 + kOut;  // 1410
// Trace record: 8 features, regression target, class label, regression mask,
// component label bits.
constexpr int kRec = 12;

// Fragment-ordered BF16 weights for the fused inference, one 32-bit register
// pair per lane and MMA: layer 1 (k 8 of 16 used: only register 0 of B is
// non-zero) 4 n-tiles; layer 2 4 n-tiles x 2 k-tiles; layer 3 1 n-tile x 2
// k-tiles; then the FP32 biases.
struct Frag {
    uint32_t w1[4][32];        // [ntile][lane]: B register 0 (rows 2t, 2t+1 of W1)
    uint2 w2[4][2][32];        // [ntile][ktile][lane]
    uint2 w3[2][32];           // [ktile][lane]
    float b1[kHid], b2[kHid], b3[8];
};

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);  // .x = lo (low half)
    return *reinterpret_cast<const uint32_t*>(&v);
}

// D = A(16x16, row) * B(16x8, col) + D, BF16 inputs, FP32 accumulate.
__device__ __forceinline__ void mma16816(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3,
                                         uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

__device__ __forceinline__ float lg8(float d2) { return log2f(fmaxf(d2, 1e-12f)) * 0.125f; }

// Features of one query of the round-1 neighbour-list build, after its warp
// scanned the query's own leaf:
//   t0, t2, tk  d2 of the nearest, third nearest and K-th nearest other point
//               of the own leaf (tk: the certified bound, finite);
//   ext2        squared diagonal of the leaf's box (the local spacing);
//   edge2       squared distance from the point to the surface of that box
//               (how far the leaf's points surround it);
//   pext2       squared diagonal of the parent node's box (density around);
//   occ         the leaf's points / 32 (cell occupancy);
//   round       the Boruvka round, comp the component's size (1 and 1 in the
//               round-1 build; both kept so that the inputs name the state).
// Distances enter as log2 ratios to tk, so the features do not depend on the
// cloud's scale.
__device__ __forceinline__ void knn_features(float t0, float t2, float tk, float ext2, float edge2, float pext2,
                                             float occ, int round, float comp, float (&f)[kIn])
{
    const float lk = lg8(tk);
    f[0] = lk - lg8(ext2);
    f[1] = lg8(t0) - lk;
    f[2] = lg8(t2) - lk;
    f[3] = lg8(edge2) - lk;
    f[4] = lg8(pext2) - lg8(ext2);
    f[5] = occ;
    f[6] = 0.125f * (float)round;
    f[7] = lg8(comp);
}

// Warp-wide inference: lane l's features (row l of a 32 x 8 batch) in, its
// two outputs out.  All 32 lanes must call it together.  W: the weights in
// global memory (read through the read-only cache).  No shared memory: rows
// move between lanes by shuffles, and layer outputs go from accumulator to
// operand registers directly (an m16n8 accumulator pair is the m16k16
// operand of the next layer).
__device__ __forceinline__ void infer_warp(const Frag* __restrict__ W, const float (&f)[kIn], float& o0, float& o1)
{
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
    uint32_t w[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) w[k] = pack_bf16(f[2 * k], f[2 * k + 1]);
    float out[2][4];
#pragma unroll
    for (int mt = 0; mt < 2; ++mt) {  // rows mt*16 + {g, g+8}, one m-tile through all layers
        // layer 1: word t (input columns 2t, 2t+1) of rows g and g+8; 8..15 are zero
        uint32_t x0 = 0, x1 = 0;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint32_t v0 = __shfl_sync(full, w[k], mt * 16 + g);
            const uint32_t v1 = __shfl_sync(full, w[k], mt * 16 + g + 8);
            if (k == t) x0 = v0, x1 = v1;
        }
        float h1[4][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float2 bb = __ldg(reinterpret_cast<const float2*>(&W->b1[8 * j + 2 * t]));
            h1[j][0] = bb.x, h1[j][1] = bb.y, h1[j][2] = bb.x, h1[j][3] = bb.y;
            mma16816(h1[j], x0, x1, 0u, 0u, __ldg(&W->w1[j][lane]), 0u);
        }
        // layer 2: the accumulator pair (2q, 2q+1) is the operand of k-tile q
        float h2[4][4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float2 bb = __ldg(reinterpret_cast<const float2*>(&W->b2[8 * j + 2 * t]));
            h2[j][0] = bb.x, h2[j][1] = bb.y, h2[j][2] = bb.x, h2[j][3] = bb.y;
        }
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const uint32_t a0 = pack_bf16(fmaxf(h1[2 * q][0], 0.f), fmaxf(h1[2 * q][1], 0.f));
            const uint32_t a1 = pack_bf16(fmaxf(h1[2 * q][2], 0.f), fmaxf(h1[2 * q][3], 0.f));
            const uint32_t a2 = pack_bf16(fmaxf(h1[2 * q + 1][0], 0.f), fmaxf(h1[2 * q + 1][1], 0.f));
            const uint32_t a3 = pack_bf16(fmaxf(h1[2 * q + 1][2], 0.f), fmaxf(h1[2 * q + 1][3], 0.f));
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint2 b = __ldg(&W->w2[j][q][lane]);
                mma16816(h2[j], a0, a1, a2, a3, b.x, b.y);
            }
        }
        // layer 3: 2 outputs in columns 0, 1 of one n-tile
        const float2 b3 = __ldg(reinterpret_cast<const float2*>(&W->b3[2 * t]));
        float o[4] = {b3.x, b3.y, b3.x, b3.y};
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const uint32_t a0 = pack_bf16(fmaxf(h2[2 * q][0], 0.f), fmaxf(h2[2 * q][1], 0.f));
            const uint32_t a1 = pack_bf16(fmaxf(h2[2 * q][2], 0.f), fmaxf(h2[2 * q][3], 0.f));
            const uint32_t a2 = pack_bf16(fmaxf(h2[2 * q + 1][0], 0.f), fmaxf(h2[2 * q + 1][1], 0.f));
            const uint32_t a3 = pack_bf16(fmaxf(h2[2 * q + 1][2], 0.f), fmaxf(h2[2 * q + 1][3], 0.f));
            const uint2 b = __ldg(&W->w3[q][lane]);
            mma16816(o, a0, a1, a2, a3, b.x, b.y);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i) out[mt][i] = o[i];
    }
    // row r's outputs sit in lane 4 * (r & 7) (t = 0): registers 0, 1 for
    // rows 0..7 of its m-tile, 2, 3 for rows 8..15
    const int src = 4 * (lane & 7), mt = lane >> 4, half = (lane >> 3) & 1;
    float r[2][4];
#pragma unroll
    for (int m = 0; m < 2; ++m)
#pragma unroll
        for (int i = 0; i < 4; ++i) r[m][i] = __shfl_sync(full, out[m][i], src);
    o0 = mt ? (half ? r[1][2] : r[1][0]) : (half ? r[0][2] : r[0][0]);
    o1 = mt ? (half ? r[1][3] : r[1][1]) : (half ? r[0][3] : r[0][1]);
}

}  // namespace prop

}  // namespace emst
