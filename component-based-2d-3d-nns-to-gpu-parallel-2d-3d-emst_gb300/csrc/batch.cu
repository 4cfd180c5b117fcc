// batch.cu -- many independent point clouds (2D and 3D mixed) in one solve.
//
// The clouds are concatenated and solved by ONE pipeline run: one sort, one
// leaf tree, one round loop (one CUDA graph), instead of one solve per cloud.
//   * every cloud is rescaled with its own pMin/pMax/unitX, exactly as a
//     single solve of that cloud would be (SolutionEMST.cu:273-379); 2D clouds
//     get z = 0, and fma(0, 0, r) == r, so their squared distances are the 2D
//     ones bit for bit;
//   * the cell key carries the cloud index (cb = ceil(log2 clouds) bits) above
//     a Hilbert index of the remaining 63 - cb bits (e.g. 18 bits/axis in 3D and
//     27 bits/axis in 2D for 512 clouds), so every cloud is a contiguous run of
//     leaves;
//   * every tree node records the cloud all its points belong to (or MIXED);
//     a search skips subtrees of other clouds, and checks the cloud of each
//     candidate only in the few leaves that straddle two clouds;
//   * input ids are global (concatenated) ids, monotone within a cloud, so
//     every tie-break is the one the single solve of that cloud makes;
//   * the loop ends when the number of components equals the number of
//     non-empty clouds.
#include <climits>
#include <cmath>


#include "emst_ctx.h"
#include "emst_device.cuh"
#include "radix.cuh"

namespace emst {

namespace {

constexpr int kThreads = 256;

// One block per cloud: min/max, unitX (the reference formula for that
// cloud's size and dimension) and the cell quantisation scale.
__global__ void k_batch_norm(const float* __restrict__ in, const int64_t* __restrict__ off,
                             const int64_t* __restrict__ foff, const int32_t* __restrict__ dims,
                             NormParams* __restrict__ np, DevCounters* __restrict__ ctr, int bits3, int bits2)
{
    __shared__ float s[6][kThreads];
    const int c = blockIdx.x;
    const int64_t n = off[c + 1] - off[c];
    const int D = dims[c];
    const float* p = in + foff[c];
    float v[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
    bool bad = false;
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x)
        for (int k = 0; k < D; ++k) {
            const float x = p[i * D + k];
            bad |= !isfinite(x);
            v[k] = fminf(v[k], x);
            v[3 + k] = fmaxf(v[3 + k], x);
        }
    if (bad) atomicOr(&ctr->err, 1u);
    for (int k = 0; k < 6; ++k) s[k][threadIdx.x] = v[k];
    __syncthreads();
    for (int h = kThreads / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h)
            for (int k = 0; k < 3; ++k) {
                s[k][threadIdx.x] = fminf(s[k][threadIdx.x], s[k][threadIdx.x + h]);
                s[3 + k][threadIdx.x] = fmaxf(s[3 + k][threadIdx.x], s[3 + k][threadIdx.x + h]);
            }
        __syncthreads();
    }
    if (threadIdx.x != 0 || n == 0) return;
    float pmin[3] = {0, 0, 0}, pmax[3] = {0, 0, 0};
    for (int k = 0; k < D; ++k) {
        pmin[k] = s[k][0];
        pmax[k] = s[3 + k][0];
    }
    double wg = (double)__fsub_rn(pmax[0], pmin[0]);
    double hg = (double)__fsub_rn(pmax[1], pmin[1]);
    double dg = 0.0;
    if (D >= 3) dg = (double)__fsub_rn(pmax[2], pmin[2]);
    if (wg == 0) wg = 1;
    if (hg == 0) hg = 1;
    const double nn = (double)n;
    double wnd = sqrt(nn * wg / hg) * 2;
    if (D >= 3) {
        if (dg != 0)
            wnd = pow((nn * wg * wg) / (hg * dg), 0.333);
        else
            dg = 1;
    }
    const double ux = (ceil(wnd) + 1) / wg;
    const float uxf = __double2float_rn(ux);
    float smax = 0.f;
    NormParams r;
    for (int k = 0; k < 3; ++k) {
        r.pmin[k] = pmin[k];
        r.pmax[k] = pmax[k];
        const float e = k < D ? __fmul_rn(__fsub_rn(pmax[k], pmin[k]), uxf) : 0.f;
        r.smax[k] = e;
        smax = fmaxf(smax, e);
    }
    r.unitx = ux;
    r.uxf = uxf;
    const float qmax = (float)((1u << (D == 3 ? bits3 : bits2)) - 1u);
    r.qscale = smax > 0.f ? qmax / smax : 0.f;
    r.pad = 0.f;
    np[c] = r;
}

// One block per cloud: rescale (float(float(p - pMin) * float(unitX))), key
// (cloud << shift | Hilbert index), staging float4 (x, y, z or 0, global id).
__global__ void k_batch_rescale_key(const float* __restrict__ in, const int64_t* __restrict__ off,
                                    const int64_t* __restrict__ foff, const int32_t* __restrict__ dims,
                                    const NormParams* __restrict__ np, float4* __restrict__ stage,
                                    uint64_t* __restrict__ key, uint32_t* __restrict__ idx,
                                    uint32_t* __restrict__ pcloud_in, int bits3, int bits2, int shift)
{
    const int c = blockIdx.x;
    const int64_t b = off[c], n = off[c + 1] - b;
    const int D = dims[c];
    const float* p = in + foff[c];
    const NormParams q = np[c];
    for (int64_t i = threadIdx.x; i < n; i += blockDim.x) {
        float s[3] = {0.f, 0.f, 0.f};
        uint32_t cell[3] = {0u, 0u, 0u};
        for (int k = 0; k < D; ++k) {
            s[k] = __fmul_rn(__fsub_rn(p[i * D + k], q.pmin[k]), q.uxf);
            const uint32_t qmax = (1u << (D == 3 ? bits3 : bits2)) - 1u;
            // float(qmax) may round up to 2^bits: clamp again after the conversion
            cell[k] = min((uint32_t)fminf(fmaxf(__fmul_rn(s[k], q.qscale), 0.f), (float)qmax), qmax);
        }
        // cells below 2^bits per axis: the index fits in D * bits <= shift bits
        const uint64_t m = D == 3 ? hilbert_index<3>(cell) : hilbert_index<2>(cell);
        const int64_t g = b + i;
        stage[g] = make_float4(s[0], s[1], s[2], __int_as_float((int)g));
        key[g] = ((uint64_t)c << shift) | m;
        idx[g] = (uint32_t)g;
        pcloud_in[g] = (uint32_t)c;
    }
}

__global__ void k_batch_gather(const float4* __restrict__ stage, const uint32_t* __restrict__ perm,
                               const uint32_t* __restrict__ pcloud_in, int64_t n, float4* __restrict__ sp,
                               uint32_t* __restrict__ pcloud)
{
    const int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (j >= n) return;
    const uint32_t g = perm[j];
    sp[j] = stage[g];
    pcloud[j] = pcloud_in[g];
}

// Edges of the solve (global ids) -> per cloud, local ids, at the cloud's
// expected row offset; counts checked against n_c - 1.
__global__ void k_batch_edges(const int32_t* __restrict__ edges, uint32_t ne, const uint32_t* __restrict__ pcloud_in,
                              const int64_t* __restrict__ off, const int64_t* __restrict__ eoff,
                              uint32_t* __restrict__ cursor, int32_t* __restrict__ out,
                              uint32_t* __restrict__ out_global, uint32_t* __restrict__ err)
{
    const uint32_t e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= ne) return;
    const int32_t u = edges[2 * (uint64_t)e], v = edges[2 * (uint64_t)e + 1];
    const uint32_t c = pcloud_in[u];
    if (pcloud_in[v] != c) {
        atomicOr(err, 16u);  // an edge across clouds: internal error
        return;
    }
    const uint32_t k = atomicAdd(&cursor[c], 1u);
    const int64_t cap = off[c + 1] - off[c] - 1;
    if ((int64_t)k >= cap) {
        atomicOr(err, 16u);
        return;
    }
    const int64_t row = eoff[c] + k;
    out[2 * row] = (int32_t)(u - off[c]);
    out[2 * row + 1] = (int32_t)(v - off[c]);
    out_global[2 * row] = (uint32_t)u;
    out_global[2 * row + 1] = (uint32_t)v;
}

// One block per cloud: tree length in the cloud's original coordinates,
// summed in a fixed order (rows of the cloud, strided by thread, then tree).
__global__ void k_batch_lengths(const uint32_t* __restrict__ eg, const int64_t* __restrict__ off,
                                const int64_t* __restrict__ eoff, const int64_t* __restrict__ foff,
                                const int32_t* __restrict__ dims, const float* __restrict__ in,
                                double* __restrict__ len)
{
    __shared__ double s[kThreads];
    const int c = blockIdx.x;
    const int64_t m = off[c + 1] - off[c] - 1;
    const int D = dims[c];
    const float* p = in + foff[c];
    double acc = 0.0;
    for (int64_t r = threadIdx.x; r < m; r += blockDim.x) {
        const int64_t u = eg[2 * (eoff[c] + r)] - off[c], v = eg[2 * (eoff[c] + r) + 1] - off[c];
        const float dx = __fsub_rn(p[u * D], p[v * D]);
        const float dy = __fsub_rn(p[u * D + 1], p[v * D + 1]);
        const float dz = D == 3 ? __fsub_rn(p[u * D + 2], p[v * D + 2]) : 0.f;
        acc += sqrt((double)(D == 3 ? d2_of<3>(dx, dy, dz) : d2_of<2>(dx, dy, dz)));
    }
    s[threadIdx.x] = acc;
    __syncthreads();
    for (int h = kThreads / 2; h > 0; h >>= 1) {
        if (threadIdx.x < h) s[threadIdx.x] += s[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) len[c] = m > 0 ? s[0] : 0.0;
}

// Cloud range of every tree node, (first cloud << 16) | last cloud: points
// are sorted cloud-major, so a node's points span a contiguous run of clouds
// read off its first and last point.  Nodes past the last point get the empty
// range (0xffff, 0), which no cloud falls in.
__global__ void k_node_cloud_range(const uint32_t* __restrict__ pcloud, uint32_t n, uint32_t L, uint32_t log2L,
                                   uint32_t* __restrict__ range)
{
    const uint32_t v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= 2 * L) return;
    if (v == 0) {
        range[0] = 0xffff0000u;
        return;
    }
    const uint32_t level = 31u - __clz(v);
    const uint64_t first = (uint64_t)(v - (1u << level)) << (log2L - level);  // first leaf
    const uint64_t span = (uint64_t)1 << (log2L - level);
    const uint64_t p0 = first * kLeaf, p1 = min((first + span) * (uint64_t)kLeaf, (uint64_t)n);
    range[v] = p0 < p1 ? (pcloud[p0] << 16) | pcloud[p1 - 1] : 0xffff0000u;
}

}  // namespace

// Batch grid: per-cloud normalisation, keys with the cloud index on top,
// one sort, leaf tree, per-node cloud ranges.
cudaError_t batch_grid_build(Ctx& c)
{
    const int64_t n = c.n;
    const int nc = c.n_clouds;
    cudaStream_t s = c.stream;
    cudaError_t e;
    if ((e = c.ensure(c.norm, (size_t)nc)) != cudaSuccess) return e;
    if ((e = c.ensure(c.stage, (size_t)n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.mkey, (size_t)n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.mkey_alt, (size_t)n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.perm, (size_t)n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.perm_alt, (size_t)n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.sp, (size_t)n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.pcloud_in, (size_t)n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.pcloud, (size_t)n)) != cudaSuccess) return e;
    c.nchunk = (n + kLeaf - 1) / kLeaf;
    c.L = 1;
    while (c.L < c.nchunk) c.L <<= 1;
    if ((e = c.ensure(c.nlo, (size_t)2 * c.L)) != cudaSuccess) return e;
    if ((e = c.ensure(c.nhi, (size_t)2 * c.L)) != cudaSuccess) return e;
    if ((e = c.ensure(c.nid, (size_t)2 * c.L)) != cudaSuccess) return e;
    if ((e = c.ensure(c.ncloud, (size_t)2 * c.L)) != cudaSuccess) return e;

    int cb = 1;
    while ((1 << cb) < nc) ++cb;
    const int shift = 63 - cb;
    const int bits3 = std::min(20, shift / 3), bits2 = std::min(30, shift / 2);
    k_batch_norm<<<nc, kThreads, 0, s>>>(c.in, c.d_off.p, c.d_foff.p, c.d_dims.p, c.norm.p, c.ctr.p, bits3, bits2);
    k_batch_rescale_key<<<nc, kThreads, 0, s>>>(c.in, c.d_off.p, c.d_foff.p, c.d_dims.p, c.norm.p, c.stage.p,
                                                c.mkey.p, c.perm.p, c.pcloud_in.p, bits3, bits2, shift);
    // (cloud << shift) | cell key: the cloud index takes the top bits of 63
    const size_t tmp = radix_scratch_bytes(n, 63);
    if ((e = c.ensure(c.sort_tmp, tmp)) != cudaSuccess) return e;
    bool in_alt = false;
    if ((e = radix_sort_pairs(c.mkey.p, c.mkey_alt.p, c.perm.p, c.perm_alt.p, n, 63, c.sort_tmp.p, tmp,
                              &c.ctr.p->err, &in_alt, s)) != cudaSuccess)
        return e;
    c.launches += 2 + radix_passes(63);
    if (in_alt) {
        std::swap(c.mkey.p, c.mkey_alt.p);
        std::swap(c.mkey.cap, c.mkey_alt.cap);
        std::swap(c.perm.p, c.perm_alt.p);
        std::swap(c.perm.cap, c.perm_alt.cap);
    }
    k_batch_gather<<<blocks_for(n, 256), 256, 0, s>>>(c.stage.p, c.perm.p, c.pcloud_in.p, n, c.sp.p, c.pcloud.p);
    c.launches += 3;
    if ((e = leaf_tree(c)) != cudaSuccess) return e;
    uint32_t log2L = 0;
    while ((1ll << log2L) < c.L) ++log2L;
    k_node_cloud_range<<<blocks_for(2 * c.L, 256), 256, 0, s>>>(c.pcloud.p, (uint32_t)n, (uint32_t)c.L, log2L,
                                                                c.ncloud.p);
    c.launches++;
    return cudaGetLastError();
}

cudaError_t batch_output(Ctx& c, int32_t* d_uv, double* d_len)
{
    cudaError_t e;
    const int nc = c.n_clouds;
    const int64_t rows = c.n - c.n_nonempty;  // sum over clouds of (n_c - 1)
    if ((e = c.ensure(c.bcursor, (size_t)nc)) != cudaSuccess) return e;
    if ((e = c.ensure(c.bedges, (size_t)2 * (rows > 0 ? rows : 1))) != cudaSuccess) return e;
    cudaMemsetAsync(c.bcursor.p, 0, sizeof(uint32_t) * nc, c.stream);
    if (c.n_edges)
        k_batch_edges<<<blocks_for(c.n_edges, 256), 256, 0, c.stream>>>(c.edges.p, c.n_edges, c.pcloud_in.p,
                                                                        c.d_off.p, c.d_eoff.p, c.bcursor.p, d_uv,
                                                                        c.bedges.p, &c.ctr.p->err);
    k_batch_lengths<<<nc, kThreads, 0, c.stream>>>(c.bedges.p, c.d_off.p, c.d_eoff.p, c.d_foff.p, c.d_dims.p, c.in,
                                                  d_len);
    c.launches += 2;
    return cudaGetLastError();
}

}  // namespace emst
