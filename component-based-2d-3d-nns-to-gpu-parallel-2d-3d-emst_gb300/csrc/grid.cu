// grid.cu -- normalisation and spatial grid build.
//
// Replaces SolutionEMST::initialize (emst_coalition/src/SolutionEMST.cu:273-509)
// and the reference's cell matrix insertion (K_EMST_initializeSpiralSearch,
// EMSTOperators.h:80-110 -> CellBMD::insert, Cell.h:433-453) with:
//   1. a two-stage float min/max reduction (the readers' pMin/pMax,
//      InputRW.h:545-559) and the reference's unitX in double
//      (SolutionEMST.cu:305-341);
//   2. the rescale p' = float(float(p - pMin) * float(unitX)) (:361-364),
//      fused with a 39 / 40-bit Hilbert cell key per point (13 bits/axis in
//      3D, 20 in 2D: cells 2^-13 / 2^-20 of the extent, still finer than
//      the leaves of the densest clusters measured, and a 5-pass radix sort);
//   3. a radix sort of the cell keys, so points of one cell (and of
//      neighbouring cells) are contiguous: leaves of 32 consecutive points
//      have bounded occupancy whatever the density, unlike the reference's
//      fixed 32-slot cells (Cell.h:53) that overflow on clustered inputs;
//   4. per-leaf bounding boxes and an implicit binary tree over the leaves
//      (heap order, node i has children 2i and 2i+1, leaves at [L, 2L)),
//      each node also carrying its two smallest input ids, so that a node
//      whose points all coincide (exact duplicates) is searched as one point.
#include <cfloat>
#include <climits>
#include <cmath>

#include "emst_ctx.h"
#include "emst_device.cuh"
#include "radix.cuh"

namespace emst {

// bits per axis of the single-cloud cell key
template <int D>
constexpr int kCellBits = D == 3 ? 13 : 20;


namespace {

constexpr int kRedThreads = 256;
constexpr int kRedBlocksMax = 1024;

// Stage 1: per-block min/max per axis; also flags non-finite coordinates.
template <int D>
__global__ void k_minmax_part(const float* __restrict__ in, int64_t n, float* __restrict__ part,
                              DevCounters* __restrict__ ctr)
{
    __shared__ float smin[D][kRedThreads / 32];
    __shared__ float smax[D][kRedThreads / 32];
    float mn[D], mx[D];
    bool bad = false;
#pragma unroll
    for (int k = 0; k < D; ++k) {
        mn[k] = INFINITY;
        mx[k] = -INFINITY;
    }
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
#pragma unroll
        for (int k = 0; k < D; ++k) {
            float c = in[i * D + k];
            bad |= !isfinite(c);
            mn[k] = fminf(mn[k], c);
            mx[k] = fmaxf(mx[k], c);
        }
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(&ctr->err, 1u);
#pragma unroll
    for (int k = 0; k < D; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
            mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
        }
    }
    int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) {
#pragma unroll
        for (int k = 0; k < D; ++k) {
            smin[k][w] = mn[k];
            smax[k][w] = mx[k];
        }
    }
    __syncthreads();
    if (threadIdx.x < D) {
        int k = threadIdx.x;
        float a = INFINITY, b = -INFINITY;
        for (int j = 0; j < kRedThreads / 32; ++j) {
            a = fminf(a, smin[k][j]);
            b = fmaxf(b, smax[k][j]);
        }
        part[blockIdx.x * 6 + k] = a;
        part[blockIdx.x * 6 + 3 + k] = b;
    }
}

// Stage 2 (one block): final min/max, unitX (double, as SolutionEMST.cu:305-341),
// rescaled extents and the cell quantisation scale.
template <int D>
__global__ void k_minmax_final(const float* __restrict__ part, int nblk, int64_t n, NormParams* __restrict__ np)
{
    __shared__ float s[6][kRedThreads];
    float v[6];
    for (int k = 0; k < 3; ++k) {
        v[k] = INFINITY;
        v[3 + k] = -INFINITY;
    }
    for (int b = threadIdx.x; b < nblk; b += blockDim.x)
        for (int k = 0; k < D; ++k) {
            v[k] = fminf(v[k], part[b * 6 + k]);
            v[3 + k] = fmaxf(v[3 + k], part[b * 6 + 3 + k]);
        }
    for (int k = 0; k < 6; ++k) s[k][threadIdx.x] = v[k];
    __syncthreads();
    if (threadIdx.x != 0) return;
    float pmin[3] = {0, 0, 0}, pmax[3] = {0, 0, 0};
    for (int k = 0; k < D; ++k) {
        float a = INFINITY, b = -INFINITY;
        for (int t = 0; t < kRedThreads; ++t) {
            a = fminf(a, s[k][t]);
            b = fmaxf(b, s[3 + k][t]);
        }
        pmin[k] = a;
        pmax[k] = b;
    }
    double wg = (double)__fsub_rn(pmax[0], pmin[0]);
    double hg = (double)__fsub_rn(pmax[1], pmin[1]);
    double dg = 0.0;
    if (D >= 3) dg = (double)__fsub_rn(pmax[2], pmin[2]);
    if (wg == 0) wg = 1;
    if (hg == 0) hg = 1;
    double nn = (double)n;
    double wnd = sqrt(nn * wg / hg) * 2;
    if (D >= 3) {
        if (dg != 0)
            wnd = pow((nn * wg * wg) / (hg * dg), 0.333);
        else
            dg = 1;
    }
    double ux = (ceil(wnd) + 1) / wg;
    float uxf = __double2float_rn(ux);
    float smax = 0.f;
    for (int k = 0; k < 3; ++k) {
        np->pmin[k] = pmin[k];
        np->pmax[k] = pmax[k];
        float e = k < D ? __fmul_rn(__fsub_rn(pmax[k], pmin[k]), uxf) : 0.f;
        np->smax[k] = e;
        smax = fmaxf(smax, e);
    }
    np->unitx = ux;
    np->uxf = uxf;
    const float qmax = (float)((1u << kCellBits<D>) - 1u);  // 2^13-1 / 2^20-1: exact in float
    np->qscale = smax > 0.f ? qmax / smax : 0.f;
}

// Rescale (SolutionEMST.cu:361-364) + Hilbert cell key.
template <int D>
__global__ void k_rescale_key(const float* __restrict__ in, int64_t n, const NormParams* __restrict__ np,
                              float* __restrict__ scaled, uint64_t* __restrict__ key, uint32_t* __restrict__ idx,
                              int pack)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float uxf = np->uxf, qs = np->qscale;
    uint32_t cell[3] = {0u, 0u, 0u};
#pragma unroll
    for (int c = 0; c < D; ++c) {
        float s = __fmul_rn(__fsub_rn(in[i * D + c], np->pmin[c]), uxf);
        scaled[i * D + c] = s;
        float qf = fminf(fmaxf(__fmul_rn(s, qs), 0.f), (float)((1u << kCellBits<D>) - 1u));
        cell[c] = (uint32_t)qf;
    }
    const uint64_t h = hilbert_index<D, kCellBits<D>>(cell);
    if (pack > 0) {
        key[i] = (h << pack) | (uint64_t)i;  // the index rides in the low bits
    } else {
        key[i] = h;
        idx[i] = (uint32_t)i;
    }
}

// Gather rescaled points into leaf order; .w carries the input id.  With
// packed sorted keys (index in the low `pack` bits) the order is read from
// them and written to perm.
template <int D>
__global__ void k_gather(const float* __restrict__ scaled, const uint64_t* __restrict__ packed, int pack,
                         uint32_t* __restrict__ perm, int64_t n, float4* __restrict__ sp, uint32_t* __restrict__ pos0)
{
    int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= n) return;
    uint32_t i;
    if (packed) {
        i = (uint32_t)(packed[j] & ((1ull << pack) - 1ull));
        perm[j] = i;
    } else {
        i = perm[j];
    }
    if (i == 0) *pos0 = (uint32_t)j;
    float4 v;
    v.x = scaled[(int64_t)i * D + 0];
    v.y = scaled[(int64_t)i * D + 1];
    v.z = D == 3 ? scaled[(int64_t)i * D + 2] : 0.f;
    v.w = __int_as_float((int)i);
    sp[j] = v;
}

// Two smallest input ids (and their leaf positions) of a set of points:
// (id0, pos0, id1, pos1) with id0 < id1; INT_MAX / -1 when absent.  For a
// node whose box is a single point (all its points coincide) this is all the
// static-pruning search needs from it.
__device__ __forceinline__ int4 merge_ids(int4 a, int4 b)
{
    int4 r;
    if (a.x <= b.x) {
        r.x = a.x;
        r.y = a.y;
        if (b.x < a.z) {
            r.z = b.x;
            r.w = b.y;
        } else {
            r.z = a.z;
            r.w = a.w;
        }
    } else {
        r.x = b.x;
        r.y = b.y;
        if (a.x < b.z) {
            r.z = a.x;
            r.w = a.y;
        } else {
            r.z = b.z;
            r.w = b.w;
        }
    }
    return r;
}

// One warp per leaf: bounding box and two smallest ids of its (up to) 32
// points.  Leaf slots past the last leaf get empty boxes (lo = +inf, hi = -inf).
__global__ void k_leaf_boxes(const float4* __restrict__ sp, int64_t n, int64_t nchunk, int64_t L,
                             float4* __restrict__ nlo, float4* __restrict__ nhi, int4* __restrict__ nid)
{
    int64_t c = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    int lane = threadIdx.x & 31;
    if (c >= L) return;
    float lx = INFINITY, ly = INFINITY, lz = INFINITY, hx = -INFINITY, hy = -INFINITY, hz = -INFINITY;
    int4 id = make_int4(INT_MAX, -1, INT_MAX, -1);
    if (c < nchunk) {
        int64_t j = c * kLeaf + lane;
        if (j < n) {
            float4 v = sp[j];
            lx = hx = v.x;
            ly = hy = v.y;
            lz = hz = v.z;
            id.x = __float_as_int(v.w);
            id.y = (int)j;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        lx = fminf(lx, __shfl_xor_sync(0xffffffffu, lx, o));
        ly = fminf(ly, __shfl_xor_sync(0xffffffffu, ly, o));
        lz = fminf(lz, __shfl_xor_sync(0xffffffffu, lz, o));
        hx = fmaxf(hx, __shfl_xor_sync(0xffffffffu, hx, o));
        hy = fmaxf(hy, __shfl_xor_sync(0xffffffffu, hy, o));
        hz = fmaxf(hz, __shfl_xor_sync(0xffffffffu, hz, o));
        int4 other;
        other.x = __shfl_xor_sync(0xffffffffu, id.x, o);
        other.y = __shfl_xor_sync(0xffffffffu, id.y, o);
        other.z = __shfl_xor_sync(0xffffffffu, id.z, o);
        other.w = __shfl_xor_sync(0xffffffffu, id.w, o);
        id = merge_ids(id, other);
    }
    if (lane == 0) {
        nlo[L + c] = make_float4(lx, ly, lz, 0.f);
        nhi[L + c] = make_float4(hx, hy, hz, 0.f);
        nid[L + c] = id;
    }
}

// Internal nodes of one tree level: union of the children's boxes, merge of
// their smallest ids.
__global__ void k_tree_level(float4* __restrict__ nlo, float4* __restrict__ nhi, int4* __restrict__ nid,
                             int64_t first, int64_t count)
{
    int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (t >= count) return;
    int64_t i = first + t;
    float4 a = nlo[2 * i], b = nlo[2 * i + 1];
    float4 c = nhi[2 * i], d = nhi[2 * i + 1];
    nlo[i] = make_float4(fminf(a.x, b.x), fminf(a.y, b.y), fminf(a.z, b.z), 0.f);
    nhi[i] = make_float4(fmaxf(c.x, d.x), fmaxf(c.y, d.y), fmaxf(c.z, d.z), 0.f);
    nid[i] = merge_ids(nid[2 * i], nid[2 * i + 1]);
}

}  // namespace

int grid_sort_end_bit(int dim) { return dim * (dim == 3 ? kCellBits<3> : kCellBits<2>); }

int grid_reduce_blocks(int64_t n)
{
    const int64_t b = std::min<int64_t>(kRedBlocksMax, (n + kRedThreads * 8 - 1) / (kRedThreads * 8));
    return b < 1 ? 1 : (int)b;
}

cudaError_t grid_build(Ctx& c)
{
    const int64_t n = c.n;
    const int D = c.dim;
    cudaStream_t s = c.stream;
    cudaError_t e;
    const int nblk = grid_reduce_blocks(n);
    if ((e = c.ensure(c.part, (size_t)nblk * 6)) != cudaSuccess) return e;
    if ((e = c.ensure(c.norm, 1)) != cudaSuccess) return e;
    if ((e = c.ensure(c.scaled, (size_t)n * D)) != cudaSuccess) return e;
    if ((e = c.ensure(c.mkey, (size_t)n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.mkey_alt, (size_t)n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.perm, (size_t)n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.perm_alt, (size_t)n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.sp, (size_t)n)) != cudaSuccess) return e;
    c.nchunk = (n + kLeaf - 1) / kLeaf;
    c.L = 1;
    while (c.L < c.nchunk) c.L <<= 1;
    if ((e = c.ensure(c.nlo, (size_t)2 * c.L)) != cudaSuccess) return e;
    if ((e = c.ensure(c.nhi, (size_t)2 * c.L)) != cudaSuccess) return e;
    if ((e = c.ensure(c.nid, (size_t)2 * c.L)) != cudaSuccess) return e;

    // bits of a point index; with the cell key's they fit one 64-bit word up
    // to 2^24 points (2^25 in 3D)
    const int end_bit = grid_sort_end_bit(D);
    int ib = 0;
    while (ib < 32 && (1ll << ib) < n) ++ib;
    const int pack = ib > 0 && ib + end_bit <= 64 ? ib : 0;
    if (D == 2) {
        k_minmax_part<2><<<nblk, kRedThreads, 0, s>>>(c.in, n, c.part.p, c.ctr.p);
        k_minmax_final<2><<<1, kRedThreads, 0, s>>>(c.part.p, nblk, n, c.norm.p);
        k_rescale_key<2><<<blocks_for(n, 256), 256, 0, s>>>(c.in, n, c.norm.p, c.scaled.p, c.mkey.p, c.perm.p, pack);
    } else {
        k_minmax_part<3><<<nblk, kRedThreads, 0, s>>>(c.in, n, c.part.p, c.ctr.p);
        k_minmax_final<3><<<1, kRedThreads, 0, s>>>(c.part.p, nblk, n, c.norm.p);
        k_rescale_key<3><<<blocks_for(n, 256), 256, 0, s>>>(c.in, n, c.norm.p, c.scaled.p, c.mkey.p, c.perm.p, pack);
    }
    // Radix sort of the cell keys (only the significant bits): keys alone
    // when the index fits beside the key in 64 bits, else (key, index) pairs
    const size_t tmp = radix_scratch_bytes(n, end_bit);
    if ((e = c.ensure(c.sort_tmp, tmp)) != cudaSuccess) return e;
    bool in_alt = false;
    if (pack > 0)
        e = radix_sort_keys(c.mkey.p, c.mkey_alt.p, n, pack, end_bit, c.sort_tmp.p, tmp, &c.ctr.p->err, &in_alt, s);
    else
        e = radix_sort_pairs(c.mkey.p, c.mkey_alt.p, c.perm.p, c.perm_alt.p, n, end_bit, c.sort_tmp.p, tmp,
                             &c.ctr.p->err, &in_alt, s);
    if (e != cudaSuccess) return e;
    c.launches += 2 + radix_passes(end_bit);
    if (in_alt) {
        std::swap(c.mkey.p, c.mkey_alt.p);
        std::swap(c.mkey.cap, c.mkey_alt.cap);
        if (pack == 0) {
            std::swap(c.perm.p, c.perm_alt.p);
            std::swap(c.perm.cap, c.perm_alt.cap);
        }
    }
    const uint64_t* packed = pack > 0 ? c.mkey.p : nullptr;
    if (D == 2)
        k_gather<2><<<blocks_for(n, 256), 256, 0, s>>>(c.scaled.p, packed, pack, c.perm.p, n, c.sp.p, &c.ctr.p->pos0);
    else
        k_gather<3><<<blocks_for(n, 256), 256, 0, s>>>(c.scaled.p, packed, pack, c.perm.p, n, c.sp.p, &c.ctr.p->pos0);
    c.launches += 4;
    return leaf_tree(c);
}

// Leaf boxes (+ two smallest ids) and the implicit tree above them.
cudaError_t leaf_tree(Ctx& c)
{
    cudaStream_t s = c.stream;
    k_leaf_boxes<<<blocks_for(c.L * 32, 256), 256, 0, s>>>(c.sp.p, c.n, c.nchunk, c.L, c.nlo.p, c.nhi.p, c.nid.p);
    c.launches++;
    for (int64_t h = c.L >> 1; h >= 1; h >>= 1) {
        k_tree_level<<<blocks_for(h, 256), 256, 0, s>>>(c.nlo.p, c.nhi.p, c.nid.p, h, h);
        c.launches++;
    }
    return cudaGetLastError();
}

}  // namespace emst
