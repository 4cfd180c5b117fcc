// emst_device.cuh -- device-side arithmetic shared by the EMST kernels.
//
// The arithmetic here is the parity contract with the reference:
//   * squared distance: the float dot product of the float difference,
//     f = dx*dx; f += dy*dy; f += dz*dz (basic_components/include/Node.h:241-250),
//     with the accumulating steps fused (fma) as the reference's GPU build
//     contracts them; written with explicit _rn intrinsics so that no
//     compiler contraction can change it;
//   * regions: dominant axis (|d[dir]| >= max |d|) gives the face
//     2*dir + (d[dir] < 0); slab bit j (other axes in increasing order) is 0
//     for d >= 0 and 1 for d <= 0, so ties and zeros belong to several
//     regions (emst_coalition/include/NodeEMST.h:1207-1232);
//   * order between candidates of one query: (d2, original id), which is
//     EMST_isInf (basic_components/include/macros_cuda.h:37) restricted to a
//     fixed query point.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace emst {

constexpr int kLeaf = 32;  // points per spatial leaf = one warp of queries
constexpr uint64_t kNoKey = ~0ull;

template <int D>
struct Dim;
template <>
struct Dim<2> {
    static constexpr int K = 8;
    static constexpr int NSLAB = 2;
};
template <>
struct Dim<3> {
    static constexpr int K = 24;
    static constexpr int NSLAB = 4;
};

// Squared distance between two points given their float differences.
template <int D>
__device__ __forceinline__ float d2_of(float dx, float dy, float dz)
{
    float r = __fmul_rn(dx, dx);
    r = __fmaf_rn(dy, dy, r);
    if (D == 3) r = __fmaf_rn(dz, dz, r);
    return r;
}

// Packed FP32 pairs (sm_100 family: add/sub/mul/fma .rn.f32x2).  Each half is
// the IEEE round-to-nearest operation of the scalar instruction, denormals
// kept, so a pair gives bit for bit the two scalar results of d2_of: two
// candidates' distances for the price of one instruction per step.
using f32x2 = uint64_t;  // low word: the first value, high word: the second

__device__ __forceinline__ f32x2 f2_dup(float v)
{
    const uint64_t b = __float_as_uint(v);
    return b | (b << 32);
}
__device__ __forceinline__ f32x2 f2_sub(f32x2 a, f32x2 b)
{
    f32x2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 f2_mul(f32x2 a, f32x2 b)
{
    f32x2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f32x2 f2_fma(f32x2 a, f32x2 b, f32x2 c)
{
    f32x2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}

// d2_of for two candidates (x, y, z pairs) against one point (P duplicated).
template <int D>
__device__ __forceinline__ f32x2 d2_of2(f32x2 cx, f32x2 cy, f32x2 cz, f32x2 px, f32x2 py, f32x2 pz)
{
    const f32x2 dx = f2_sub(cx, px), dy = f2_sub(cy, py);
    f32x2 r = f2_fma(dy, dy, f2_mul(dx, dx));
    if (D == 3) {
        const f32x2 dz = f2_sub(cz, pz);
        r = f2_fma(dz, dz, r);
    }
    return r;
}

// Bits "d2 > bound" of two candidates, shifted into a mask from the bottom:
// the sign bit of bound - d2.  IEEE subtraction with denormals gives zero only
// for equal operands (+0 under round to nearest), so the sign is set exactly
// when d2 > bound, including d2 = +inf and a bound of -1.  The second value's
// bit goes in first, so after pairs 15, 14, ..., 0 bit j of the mask is
// candidate j; the candidates within the bound are the complement.
__device__ __forceinline__ uint32_t reject_append2(uint32_t mask, f32x2 bound2, f32x2 d2)
{
    const f32x2 s = f2_sub(bound2, d2);
    mask = __funnelshift_l((uint32_t)(s >> 32), mask, 1);
    return __funnelshift_l((uint32_t)s, mask, 1);
}

// Region bit mask of a candidate at offset d = q - p (general path: ties and zeros).
template <int D>
__device__ __forceinline__ uint32_t region_mask(float dx, float dy, float dz)
{
    constexpr int NS = Dim<D>::NSLAB;
    float a[3] = {fabsf(dx), fabsf(dy), fabsf(dz)};
    float d[3] = {dx, dy, dz};
    float m = fmaxf(a[0], a[1]);
    if (D == 3) m = fmaxf(m, a[2]);
    uint32_t mask = 0;
#pragma unroll
    for (int dir = 0; dir < D; ++dir) {
        if (!(a[dir] >= m)) continue;
        int face = 2 * dir + (d[dir] < 0.f ? 1 : 0);
#pragma unroll
        for (int s = 0; s < NS; ++s) {
            bool ok = true;
            int bit = 0;
#pragma unroll
            for (int i = 0; i < D; ++i) {
                if (i == dir) continue;
                bool neg = (s >> bit) & 1;
                ok = ok && (neg ? (d[i] <= 0.f) : (d[i] >= 0.f));
                ++bit;
            }
            if (ok) mask |= 1u << (face * NS + s);
        }
    }
    return mask;
}

// Fast path: the single region of a candidate with one dominant axis and no
// zero component on the other axes; returns -1 when the general path is needed.
// Branch-free (lanes of a warp hold different queries, so a dominant-axis
// if-chain would diverge); d = q - p never holds -0.0 (x - x = +0.0), so the
// sign bit is exactly d < 0.
template <int D>
__device__ __forceinline__ int region_fast(float dx, float dy, float dz)
{
    const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
    const int sx = __float_as_uint(dx) >> 31, sy = __float_as_uint(dy) >> 31;
    if (D == 2) {
        const bool gx = ax > ay, gy = ay > ax;
        const bool ok = (gx && dy != 0.f) || (gy && dx != 0.f);
        const int r = gx ? (sx * 2 + sy) : (4 + sy * 2 + sx);
        return ok ? r : -1;
    } else {
        const int sz = __float_as_uint(dz) >> 31;
        const bool gx = ax > ay && ax > az;
        const bool gy = ay > ax && ay > az;
        const bool gz = az > ax && az > ay;
        const bool nzx = dx != 0.f, nzy = dy != 0.f, nzz = dz != 0.f;
        const bool ok = (gx && nzy && nzz) || (gy && nzx && nzz) || (gz && nzx && nzy);
        // face * 4 + slab, slab bits over the other axes in increasing order
        const int rx = sx * 4 + sy + 2 * sz;
        const int ry = 8 + sy * 4 + sx + 2 * sz;
        const int rz = 16 + sz * 4 + sx + 2 * sy;
        const int r = gx ? rx : (gy ? ry : rz);
        return ok ? r : -1;
    }
}

// Does the relative box [a, b] (b >= a componentwise) meet the cone of region r?
// Exact on float offsets: a candidate's offset fl(q - p) lies in
// [fl(lo - p), fl(hi - p)] whenever q lies in [lo, hi].
template <int D>
__device__ __forceinline__ bool cone_hits(int r, const float* a, const float* b)
{
    constexpr int NS = Dim<D>::NSLAB;
    int face = r / NS, s = r % NS;
    int dir = face >> 1;
    bool negf = face & 1;
    float t = negf ? -a[dir] : b[dir];
    if (t < 0.f) return false;
    int bit = 0;
#pragma unroll
    for (int i = 0; i < D; ++i) {
        if (i == dir) continue;
        bool neg = (s >> bit) & 1;
        float lo = neg ? -b[i] : a[i];
        float hi = neg ? -a[i] : b[i];
        if (lo > t || hi < 0.f) return false;
        ++bit;
    }
    return true;
}

// Bit spreading: bit b of x moves to bit 2b (spread2) or 3b (spread3).
__device__ __forceinline__ uint64_t spread2(uint32_t x)
{
    uint64_t v = x;
    v = (v | (v << 16)) & 0x0000FFFF0000FFFFull;
    v = (v | (v << 8)) & 0x00FF00FF00FF00FFull;
    v = (v | (v << 4)) & 0x0F0F0F0F0F0F0F0Full;
    v = (v | (v << 2)) & 0x3333333333333333ull;
    v = (v | (v << 1)) & 0x5555555555555555ull;
    return v;
}
__device__ __forceinline__ uint64_t spread3(uint32_t x)
{
    uint64_t v = x & 0x1FFFFF;
    v = (v | (v << 32)) & 0x1F00000000FFFFull;
    v = (v | (v << 16)) & 0x1F0000FF0000FFull;
    v = (v | (v << 8)) & 0x100F00F00F00F00Full;
    v = (v | (v << 4)) & 0x10C30C30C30C30C3ull;
    v = (v | (v << 2)) & 0x1249249249249249ull;
    return v;
}

// Hilbert index of the cell x[0..D) on the order-kBits curve (by default 21
// in 3D, 31 in 2D: the widest that fit 64 bits), after J. Skilling, "Programming the Hilbert curve", AIP Conf. Proc.
// 707, 381 (2004): the coordinates are turned in place into the transposed
// index, whose bits, interleaved with axis 0 most significant in each group,
// form the index.  Cells with consecutive indices share a face, so a run of
// 32 consecutive points has a compact bounding box; a Z-order run can jump
// across the domain and leave a box that overlaps many others.  The curve
// starts at the origin and fills each origin sub-cube before leaving it, so
// cells below 2^b on every axis get indices below 2^(D*b).
template <int D, int kBits = (D == 3 ? 21 : 31)>
__device__ __forceinline__ uint64_t hilbert_index(uint32_t (&x)[3])
{
    static_assert(kBits >= 1 && kBits * D <= 63, "the index must fit 63 bits");
    constexpr uint32_t top = 1u << (kBits - 1);
#pragma unroll
    for (uint32_t q = top; q > 1; q >>= 1) {
        const uint32_t p = q - 1;
#pragma unroll
        for (int i = 0; i < D; ++i) {
            if (x[i] & q) {
                x[0] ^= p;  // invert the low bits
            } else {
                const uint32_t t = (x[0] ^ x[i]) & p;  // exchange the low bits
                x[0] ^= t;
                x[i] ^= t;
            }
        }
    }
#pragma unroll
    for (int i = 1; i < D; ++i) x[i] ^= x[i - 1];  // Gray encode
    uint32_t t = 0;
#pragma unroll
    for (uint32_t q = top; q > 1; q >>= 1)
        if (x[D - 1] & q) t ^= q - 1;
#pragma unroll
    for (int i = 0; i < D; ++i) x[i] ^= t;
    if (D == 3) return (spread3(x[0]) << 2) | (spread3(x[1]) << 1) | spread3(x[2]);
    return (spread2(x[0]) << 1) | spread2(x[1]);
}

// Block-aggregated slot reservation through counter *cnt: one atomic per
// block instead of one per warp.  A single counter taking an atomic from every
// warp of a pass over 10^7 points serialises at the L2 (round 1 hooks and
// keeps millions of roots).  Every thread of the block calls it (the callers'
// loops run the same trip count across the block, full warps); s_cnt has 33
// entries.  Returns the slot of a thread with pred.
__device__ __forceinline__ uint32_t block_reserve(bool pred, uint32_t* cnt, uint32_t* s_cnt)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
    const unsigned m = __ballot_sync(0xffffffffu, pred);
    if (lane == 0) s_cnt[w] = (uint32_t)__popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int i = 0; i < nw; ++i) {
            const uint32_t c = s_cnt[i];
            s_cnt[i] = t;
            t += c;
        }
        s_cnt[32] = t ? atomicAdd(cnt, t) : 0u;
    }
    __syncthreads();
    const uint32_t slot = s_cnt[32] + s_cnt[w] + (uint32_t)__popc(m & ((1u << lane) - 1u));
    __syncthreads();  // s_cnt is reused by the next call
    return slot;
}

}  // namespace emst
