// dyn.cu -- dynamic-pruning search (search_mode 3): a per-round ring search
// over a uniform cell grid, without a static candidate table and without the
// leaf tree's node labels; optionally with the diffusion min-find.
//
// The reference's second pruning mode (NodeSpiralSearchMD::search,
// emst_coalition/include/NodeEMST.h:67-509, selected when
// EMST_SPIRAL_SEARCH_KD_SLAB_2 is off, SolutionEMST.h:55-56) searches, every
// round, rings of cells around each point for its nearest point outside its
// component, and keeps per region (face / slab) the nearest point of its own
// component it has met, closing a region for good once that point rules the
// rest of the region out.  This file restates that idea for the GPU with a
// closure rule that follows from the regions' geometry:
//
//   * cells: the reference's dual cells of side 2 in the rescaled frame
//     (ViewGridQuadMD with R = 1, emst_coalition/include/ViewGrid.h:241-359),
//     built by sorting the points' cell keys (radix.cu) into contiguous ranges
//     -- cells of any occupancy, the role of the reference's adaptive-size
//     linked-list cells (basic_components/include/CellAdaptiveSize.h:52-225)
//     instead of its 32-slot cells (Cell.h:53);
//   * regions: the K = 2D*2^(D-1) regions of the static table (dominant axis,
//     sign pattern; NodeEMST.h:1207-1232).  Any two offsets in one region are
//     at most 60 degrees apart, so for a point p of the query's component in
//     region r at squared distance dr, any candidate q of region r with
//     d2(ps, q) > dr is strictly nearer to p than to ps: the edge (p, q) beats
//     (ps, q), which cannot be the component's shortest outgoing edge.  A
//     margin of 2^-10 in d2 keeps that strict after float rounding, as long
//     as dr is not too small against d2(ps, q): with a = |p - ps| and
//     b = |q - ps| the exact gap d2(ps, q) - d2(p, q) is at least a (b - a),
//     which is (a/b)(1 - a/b) b^2, while a computed d2 is within 5 * 2^-24 of
//     itself.  So own-component points nearer than 2^-36 of the bounding
//     box's squared diagonal are not used (a coincident point, a = 0, proves
//     nothing: its edges tie with ps's and the ids decide); the ratio
//     d2(ps, q) / dr then stays below 2^36, the gap above 2^-18 b^2;
//   * per point and region, dp[r] = d2 of the nearest own-component point met
//     in r (components only grow, so it stays valid and only shrinks), and a
//     closed bit: once a search has covered region r out to dp[r] and met no
//     unpruned outside point there, none will ever appear (outside sets only
//     shrink), so region r never needs searching again.  A point whose K
//     regions are all closed is finished for the rest of the solve;
//   * a point whose previous partner is still outside its component keeps it
//     (NEMST_TEST_PREVIOUS, NodeEMST.h:160-170).
// The component minimum is exact: its endpoint ps never prunes its partner q
// (a pruning point p would give a shorter outgoing edge), so it reports the
// minimum, and every other point reports a real outgoing edge or nothing.
//
// Per-component minimum: by default each report goes to the component's
// 64-bit atomicMin slot (as in the component search).  With min_find 1 the
// diffusion alternative of the reference runs instead (k_diff_edges below).
#include <algorithm>
#include <cmath>
#include <cfloat>
#include <climits>

#include "emst_ctx.h"
#include "emst_device.cuh"
#include "radix.cuh"

namespace emst {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr uint32_t kNone = 0xffffffffu;
constexpr float kCell = 2.f;            // dual cell side (2R, R = 1) in the rescaled frame
constexpr float kPrune = 1.0009765625f;  // 1 + 2^-10: the strict margin of the region rule

struct GridDims {
    int nc[3];
};

__device__ __forceinline__ int cell_of(float x, int nc) { return min((int)(x * (1.f / kCell)), nc - 1); }

// Cell key of each point (leaf position order) and the identity values.
template <int D>
__global__ void k_dyn_keys(const float4* __restrict__ sp, uint32_t n, GridDims g, uint64_t* __restrict__ key,
                           uint32_t* __restrict__ val)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    const float4 p = sp[j];
    const int cx = cell_of(p.x, g.nc[0]), cy = cell_of(p.y, g.nc[1]);
    const int cz = D == 3 ? cell_of(p.z, g.nc[2]) : 0;
    key[j] = ((uint64_t)cz * g.nc[1] + cy) * g.nc[0] + cx;
    val[j] = j;
}

// First sorted entry of every cell (a cell without points: the next cell's).
__global__ void k_dyn_starts(const uint64_t* __restrict__ key, uint32_t n, uint64_t ncells,
                             uint32_t* __restrict__ start)
{
    const uint64_t c = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (c > ncells) return;
    uint32_t lo = 0, hi = n;  // lower bound of c
    while (lo < hi) {
        const uint32_t mid = (lo + hi) >> 1;
        if (key[mid] < c) lo = mid + 1;
        else hi = mid;
    }
    start[c] = lo;
}

__global__ void k_dyn_init(uint32_t n, int K, float* __restrict__ dp, uint32_t* __restrict__ closed,
                           uint32_t* __restrict__ selq)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    for (int r = 0; r < K; ++r) dp[(size_t)r * n + j] = INFINITY;
    closed[j] = 0u;
    selq[j] = kNone;
}

__global__ void k_dyn_iperm(uint32_t n, const uint32_t* __restrict__ perm, uint32_t* __restrict__ iperm)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) iperm[perm[j]] = j;
}

// Warp-aggregated append of `val` to list[] through counter *cnt (all lanes call).
__device__ __forceinline__ void append_warp(bool pred, uint32_t val, uint32_t* list, uint32_t* cnt)
{
    const unsigned m = __ballot_sync(kFull, pred);
    if (!m) return;
    const int lane = threadIdx.x & 31, leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(cnt, (uint32_t)__popc(m));
    base = __shfl_sync(kFull, base, leader);
    if (pred) list[base + __popc(m & ((1u << lane) - 1u))] = val;
}

// One thread per point: keep a partner still outside, else the ring search.
// rkey != null (diffusion min-find): the report goes to rkey[j] only.
template <int D>
__global__ void __launch_bounds__(256) k_dyn_search(const float4* __restrict__ sp, const uint32_t* __restrict__ lab,
                                                    uint32_t n, GridDims g, const uint32_t* __restrict__ cpos,
                                                    const uint32_t* __restrict__ cstart, float* __restrict__ dp,
                                                    uint32_t* __restrict__ closed, uint32_t* __restrict__ selq,
                                                    uint64_t* __restrict__ selkey, uint64_t* __restrict__ ckey,
                                                    uint32_t* __restrict__ prov, uint32_t* __restrict__ n_prov,
                                                    uint64_t* __restrict__ rkey, float dfloor,
                                                    unsigned long long* __restrict__ stats)
{
    constexpr int K = Dim<D>::K;
    constexpr uint32_t kAll = (1u << K) - 1u;
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    bool record = false;
    uint32_t st_cells = 0, st_cands = 0;
    bool searched = false;
    if (j < n) {
        const uint32_t lp = lab[j];
        uint32_t cl = closed[j];
        uint64_t key = kNoKey;
        const uint32_t q0 = selq[j];
        if (q0 != kNone && lab[q0] != lp) {
            key = selkey[j];  // previous partner still outside: still the best (outside sets only shrink)
        } else if (cl != kAll) {
            searched = true;
            // the component's best key so far bounds the search: beyond it no
            // point of this component can hold the minimum (read once; other
            // points only lower it)
            const uint64_t ck = rkey ? kNoKey : __ldcg(&ckey[lp]);
            const float cb = ck == kNoKey ? INFINITY : __uint_as_float((uint32_t)(ck >> 32));
            const float4 P = sp[j];
            const int op = __float_as_int(P.w);
            float d[K];
#pragma unroll
            for (int r = 0; r < K; ++r) d[r] = dp[(size_t)r * n + j];
            float bd = INFINITY;
            int bo = INT_MAX;
            uint32_t bs = kNone;
            uint32_t found = 0;  // regions where an unpruned outside point was met
            const int pc[3] = {cell_of(P.x, g.nc[0]), cell_of(P.y, g.nc[1]), D == 3 ? cell_of(P.z, g.nc[2]) : 0};
            const int maxr = max(max(g.nc[0], g.nc[1]), g.nc[2]);
            int rad = 0;
            for (; rad <= maxr; ++rad) {
                // every point of ring rad lies at least (rad - 1) cells away
                const float lbr = rad >= 1 ? (float)(rad - 1) * kCell : 0.f;
                const float lb2 = __fmul_rn(lbr, lbr) * 0.999f;
                // what the search still needs: its best so far, the
                // component's key, and every open region out to its
                // own-component bound
                float open_far = 0.f;
#pragma unroll
                for (int r = 0; r < K; ++r)
                    if (!((cl >> r) & 1u)) open_far = fmaxf(open_far, d[r]);
                const float need = fminf(fminf(bd, open_far), cb);
                if (rad > 0 && lb2 > need) break;
                // the cells at Chebyshev distance rad
                const int zr = D == 3 ? rad : 0;
                for (int dz = -zr; dz <= zr; ++dz)
                    for (int dy = -rad; dy <= rad; ++dy)
                        for (int dx = -rad; dx <= rad; ++dx) {
                            if (max(max(abs(dx), abs(dy)), abs(dz)) != rad) {
                                dx = rad - 1;  // the ring's interior: jump to its far side
                                continue;
                            }
                            const int cx = pc[0] + dx, cy = pc[1] + dy, cz = pc[2] + dz;
                            if (cx < 0 || cy < 0 || cz < 0 || cx >= g.nc[0] || cy >= g.nc[1] || cz >= g.nc[2])
                                continue;
                            const uint64_t c = ((uint64_t)cz * g.nc[1] + cy) * g.nc[0] + cx;
                            const uint32_t a = cstart[c], b = cstart[c + 1];
                            ++st_cells;
                            for (uint32_t t = a; t < b; ++t) {
                                const uint32_t q = cpos[t];
                                if (q == j) continue;
                                const float4 Q = sp[q];
                                const float ex = __fsub_rn(Q.x, P.x), ey = __fsub_rn(Q.y, P.y);
                                const float ez = D == 3 ? __fsub_rn(Q.z, P.z) : 0.f;
                                const float d2 = d2_of<D>(ex, ey, ez);
                                const uint32_t rm = region_mask<D>(ex, ey, ez);
                                ++st_cands;
                                if (lab[q] == lp) {
                                    if (d2 >= dfloor) {
#pragma unroll
                                        for (int r = 0; r < K; ++r)
                                            if ((rm >> r) & 1u) d[r] = fminf(d[r], d2);
                                    }
                                    continue;
                                }
                                // pruned: beyond an own-component point of one of its regions
                                bool pruned = false;
#pragma unroll
                                for (int r = 0; r < K; ++r)
                                    if ((rm >> r) & 1u) pruned = pruned || d2 > d[r] * kPrune;
                                if (pruned) continue;
                                found |= rm;
                                const int oq = __float_as_int(Q.w);
                                if (d2 < bd || (d2 == bd && oq < bo)) {
                                    bd = d2;
                                    bo = oq;
                                    bs = q;
                                }
                            }
                        }
            }
            // Every point nearer than `covered` was seen (the rings left out
            // start beyond it).  A region whose own-component bound lies
            // within it and where no unpruned outside point was met is closed.
            const float lbr = rad >= 1 ? (float)(rad - 1) * kCell : 0.f;
            const float covered = rad > maxr ? INFINITY : __fmul_rn(lbr, lbr) * 0.999f;
#pragma unroll
            for (int r = 0; r < K; ++r) {
                const bool all_seen = covered == INFINITY || d[r] * kPrune <= covered;
                if (!((found >> r) & 1u) && all_seen) cl |= 1u << r;
                dp[(size_t)r * n + j] = d[r];
            }
            closed[j] = cl;
            if (bs != kNone) {
                key = ((uint64_t)__float_as_uint(bd) << 32) | (uint32_t)min(op, bo);
                // every point as near as the best was seen: it is this point's
                // best unpruned partner, reusable while it stays outside; one
                // cut short by the component's key cannot be its winner
                selq[j] = bd <= covered ? bs : kNone;
                selkey[j] = key;
            } else {
                selq[j] = kNone;
            }
        }
        if (rkey) {
            rkey[j] = key;
        } else if (key != kNoKey && key <= __ldcg(&ckey[lp])) {
            const uint64_t old = atomicMin((unsigned long long*)&ckey[lp], (unsigned long long)key);
            record = old >= key;
        }
    }
    append_warp(record, j, prov, n_prov);
    if (stats) {
        unsigned long long sc = st_cells, sq = st_cands, s = searched ? 1ull : 0ull;
        for (int o = 16; o > 0; o >>= 1) {
            sc += __shfl_xor_sync(kFull, sc, o);
            sq += __shfl_xor_sync(kFull, sq, o);
            s += __shfl_xor_sync(kFull, s, o);
        }
        if ((threadIdx.x & 31) == 0) {
            atomicAdd(&stats[0], sc);
            atomicAdd(&stats[2], sq);
            atomicAdd(&stats[3], 1ull);
            atomicAdd(&stats[4], s);
        }
    }
}

// Diffusion min-find (the reference's alternative to a list walk from the
// root, K_EMST_findMinInComponentDB / K_EMST_findMinDB_1/_2,
// emst_coalition/include/EMSTOperators.h:454-915): every point starts from
// the key it reported this round and the minimum diffuses along the forest's
// edges -- each sweep gives both ends of every edge the smaller of their two
// values -- until no value changes; then every point holds its component's
// minimum.  No root slot, a sweep per unit of tree depth.  The reference
// orients each tree from its root and reduces bottom-up with threads waiting
// on their children; here each sweep is one launch and the host reads a
// changed flag after it.
__global__ void k_diff_edges(const int32_t* __restrict__ edges, const uint32_t* __restrict__ n_edges,
                             const uint32_t* __restrict__ iperm, uint64_t* __restrict__ best,
                             uint32_t* __restrict__ changed)
{
    const uint32_t ne = *n_edges;
    bool ch = false;
    for (uint32_t base = blockIdx.x * blockDim.x; base < ne; base += gridDim.x * blockDim.x) {
        const uint32_t e = base + threadIdx.x;
        if (e < ne) {
            const uint32_t u = iperm[edges[2 * (uint64_t)e]], v = iperm[edges[2 * (uint64_t)e + 1]];
            const uint64_t bu = __ldcg(&best[u]), bv = __ldcg(&best[v]);
            if (bu < bv) {
                atomicMin((unsigned long long*)&best[v], (unsigned long long)bu);
                ch = true;
            } else if (bv < bu) {
                atomicMin((unsigned long long*)&best[u], (unsigned long long)bv);
                ch = true;
            }
        }
    }
    if (__any_sync(kFull, ch) && (threadIdx.x & 31) == 0) atomicOr(changed, 1u);
}

// After the sweeps: the component's slot takes the diffused minimum, and the
// points whose own report equals it are the provisional winners.
__global__ void k_diff_finish(uint32_t n, const uint32_t* __restrict__ lab, const uint64_t* __restrict__ rkey,
                              const uint64_t* __restrict__ best, uint64_t* __restrict__ ckey,
                              uint32_t* __restrict__ prov, uint32_t* __restrict__ n_prov)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    bool record = false;
    if (j < n) {
        const uint64_t b = best[j];
        if (b != kNoKey) ckey[lab[j]] = b;  // every point of a component holds the same value
        record = rkey[j] != kNoKey && rkey[j] == b;
    }
    append_warp(record, j, prov, n_prov);
}

GridDims dims_of(const Ctx& c, const NormParams& np)
{
    GridDims g;
    for (int a = 0; a < 3; ++a) g.nc[a] = 1;
    for (int a = 0; a < c.dim; ++a) g.nc[a] = (int)(np.smax[a] / kCell) + 1;
    return g;
}

}  // namespace

// Cell index over the leaf-ordered points and the per-point region state.
cudaError_t dyn_init(Ctx& c)
{
    cudaError_t e;
    const size_t n = (size_t)c.n;
    NormParams np;
    if ((e = cudaMemcpyAsync(&np, c.norm.p, sizeof(np), cudaMemcpyDeviceToHost, c.stream)) != cudaSuccess) return e;
    if ((e = cudaStreamSynchronize(c.stream)) != cudaSuccess) return e;
    const GridDims g = dims_of(c, np);
    const uint64_t ncells = (uint64_t)g.nc[0] * g.nc[1] * g.nc[2];
    if (ncells > (1ull << 40)) return cudaErrorInvalidValue;
    int bits = 1;
    while ((1ull << bits) < ncells + 1) ++bits;
    if ((e = c.ensure(c.dyn_pos, n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.dyn_start, ncells + 1)) != cudaSuccess) return e;
    if ((e = c.ensure(c.dyn_dp, n * c.K)) != cudaSuccess) return e;
    if ((e = c.ensure(c.dyn_closed, n)) != cudaSuccess) return e;
    const size_t tmp = radix_scratch_bytes(c.n, bits);
    if ((e = c.ensure(c.sort_tmp, tmp)) != cudaSuccess) return e;
    // cell keys of the leaf positions, sorted with the grid build's sort (its
    // key and permutation buffers are free again once the points are gathered)
    if (c.dim == 2)
        k_dyn_keys<2><<<blocks_for(c.n, 256), 256, 0, c.stream>>>(c.sp.p, (uint32_t)c.n, g, c.mkey.p, c.perm_alt.p);
    else
        k_dyn_keys<3><<<blocks_for(c.n, 256), 256, 0, c.stream>>>(c.sp.p, (uint32_t)c.n, g, c.mkey.p, c.perm_alt.p);
    bool in_alt = false;
    if ((e = radix_sort_pairs(c.mkey.p, c.mkey_alt.p, c.perm_alt.p, c.dyn_pos.p, c.n, bits, c.sort_tmp.p, tmp,
                              &c.ctr.p->err, &in_alt, c.stream)) != cudaSuccess)
        return e;
    const uint64_t* skey = in_alt ? c.mkey_alt.p : c.mkey.p;
    if (!in_alt) {  // an even pass count (or no sort at all) leaves the positions in perm_alt
        if ((e = cudaMemcpyAsync(c.dyn_pos.p, c.perm_alt.p, n * sizeof(uint32_t), cudaMemcpyDeviceToDevice,
                                 c.stream)) != cudaSuccess)
            return e;
    }
    k_dyn_starts<<<(unsigned)((ncells + 1 + 255) / 256), 256, 0, c.stream>>>(skey, (uint32_t)c.n, ncells,
                                                                               c.dyn_start.p);
    k_dyn_init<<<blocks_for(c.n, 256), 256, 0, c.stream>>>((uint32_t)c.n, c.K, c.dyn_dp.p, c.dyn_closed.p,
                                                            c.selq.p);
    c.launches += 4 + radix_passes(bits);
    if (c.min_find == 1) {
        if ((e = c.ensure(c.iperm, n)) != cudaSuccess) return e;
        if ((e = c.ensure(c.dyn_rkey, n)) != cudaSuccess) return e;
        if ((e = c.ensure(c.dyn_best, n)) != cudaSuccess) return e;
        if ((e = c.ensure(c.dyn_flag, 1)) != cudaSuccess) return e;
        k_dyn_iperm<<<blocks_for(c.n, 256), 256, 0, c.stream>>>((uint32_t)c.n, c.perm.p, c.iperm.p);
        c.launches++;
    }
    c.dyn_dims[0] = g.nc[0];
    c.dyn_dims[1] = g.nc[1];
    c.dyn_dims[2] = g.nc[2];
    return cudaGetLastError();
}

// One round's search and per-component minimum (find_next_closest of
// search_mode 3).
cudaError_t dyn_select(Ctx& c)
{
    DevCounters* d = c.ctr.p;  // n_prov was zeroed by the round tick
    GridDims g;
    for (int a = 0; a < 3; ++a) g.nc[a] = c.dyn_dims[a];
    unsigned long long* st = c.profile ? c.nstats.p : nullptr;
    uint64_t* rk = c.min_find == 1 ? c.dyn_rkey.p : nullptr;
    // the pruning floor: 2^-36 of the cells' box squared diagonal
    double diag2 = 0.0;
    for (int a = 0; a < c.dim; ++a) diag2 += (double)g.nc[a] * kCell * (double)g.nc[a] * kCell;
    const float dfloor = (float)std::ldexp(diag2, -36);
    if (c.dim == 2)
        k_dyn_search<2><<<blocks_for(c.n, 256), 256, 0, c.stream>>>(
            c.sp.p, c.lab.p, (uint32_t)c.n, g, c.dyn_pos.p, c.dyn_start.p, c.dyn_dp.p, c.dyn_closed.p, c.selq.p,
            c.selkey.p, c.ckey.p, c.prov.p, &d->n_prov, rk, dfloor, st);
    else
        k_dyn_search<3><<<blocks_for(c.n, 256), 256, 0, c.stream>>>(
            c.sp.p, c.lab.p, (uint32_t)c.n, g, c.dyn_pos.p, c.dyn_start.p, c.dyn_dp.p, c.dyn_closed.p, c.selq.p,
            c.selkey.p, c.ckey.p, c.prov.p, &d->n_prov, rk, dfloor, st);
    c.launches++;
    c.nns_launches++;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !rk) return e;
    // diffusion min-find: sweeps over the forest's edges until nothing changes
    // (at most one sweep per point: a tree's depth is below its size)
    if ((e = cudaMemcpyAsync(c.dyn_best.p, rk, (size_t)c.n * sizeof(uint64_t), cudaMemcpyDeviceToDevice,
                             c.stream)) != cudaSuccess)
        return e;
    const unsigned eg = (unsigned)std::max<int64_t>(1, std::min<int64_t>(blocks_for(c.n, 256), (int64_t)c.sms * 8));
    for (int64_t it = 0; it <= c.n; ++it) {
        if ((e = cudaMemsetAsync(c.dyn_flag.p, 0, sizeof(uint32_t), c.stream)) != cudaSuccess) return e;
        k_diff_edges<<<eg, 256, 0, c.stream>>>(c.edges.p, &d->n_edges, c.iperm.p, c.dyn_best.p, c.dyn_flag.p);
        c.launches++;
        uint32_t changed = 0;
        if ((e = cudaMemcpyAsync(&changed, c.dyn_flag.p, sizeof(uint32_t), cudaMemcpyDeviceToHost, c.stream)) !=
            cudaSuccess)
            return e;
        if ((e = cudaStreamSynchronize(c.stream)) != cudaSuccess) return e;
        if (!changed) break;
    }
    k_diff_finish<<<blocks_for(c.n, 256), 256, 0, c.stream>>>((uint32_t)c.n, c.lab.p, rk, c.dyn_best.p, c.ckey.p,
                                                              c.prov.p, &d->n_prov);
    c.launches++;
    return cudaGetLastError();
}

}  // namespace emst
