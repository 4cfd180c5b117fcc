// nns.cu -- static-pruning region nearest neighbours ("computeOctants").
//
// Replaces NodeComputeOctantMD::computeOctants (emst_coalition/include/
// NodeEMST.h:1018-1296; kernel EMSTOperators.h:115-140): for every point p
// and every region R (K = 8 in 2D, 24 in 3D: dominant axis x sign x sign
// pattern of the other axes) the nearest point of R under (d2, input id).
//
// Design: one warp per query tile.  A tile is one leaf of 32 consecutive
// points in Hilbert order, so the 32 lanes hold 32 spatially close queries.
// The warp walks the implicit leaf tree depth-first (near child first); a
// node is opened when any lane may still improve a region from it:
//   * lower bound lb2 of d2 from the lane's query to the node's box, computed
//     with the same rounded operations as d2 itself, so lb2 <= d2(q) for every
//     q inside (monotonicity of rounding) -- pruning needs no epsilon;
//   * a region with a candidate only needs the node if lb2 <= its best d2;
//     a region still empty only needs it if the box meets the region's cone,
//     tested exactly on the float offsets.
// Candidate leaves are staged through shared memory (one float4 per point,
// broadcast reads), each lane folds the 32 candidates into its K region
// minima kept in shared memory ([region][lane], conflict-free).
//
// Output per point: the K minima deduplicated and sorted by (d2, input id),
// stored as (d2 bits << 32) | leaf position; a zero-distance entry marks the
// point for recomputation in later rounds (NodeEMST.h:1051-1077), where the
// same kernel runs in list mode with the reference's filter: a zero-distance
// candidate counts only when it lies in another component (:1204).
#include <climits>

#include "emst_ctx.h"
#include "emst_device.cuh"

namespace emst {

namespace {

constexpr int kStack = 64;
constexpr unsigned kFull = 0xffffffffu;

template <int D, int WPB, bool LIST>
__global__ void __launch_bounds__(WPB * 32)
    k_nns(const float4* __restrict__ sp, const float4* __restrict__ nlo, const float4* __restrict__ nhi,
          const int4* __restrict__ nid, uint32_t n, uint32_t L, uint32_t nchunk, const uint32_t* __restrict__ qlist,
          uint32_t nq, const uint32_t* __restrict__ lab, uint64_t* __restrict__ cand, unsigned char* __restrict__ cnt,
          unsigned char* __restrict__ cur, unsigned char* __restrict__ zflag, uint32_t* __restrict__ zero_out,
          uint32_t* __restrict__ zero_count, int32_t* __restrict__ tab_id, float* __restrict__ tab_d2,
          unsigned long long* __restrict__ stats)
{
    constexpr int K = Dim<D>::K;
    constexpr int NS = Dim<D>::NSLAB;
    __shared__ float s_bd[WPB][K][32];
    __shared__ int s_bo[WPB][K][32];
    __shared__ int s_bs[WPB][K][32];
    __shared__ float4 s_tile[WPB][32];
    __shared__ uint32_t s_stack[WPB][kStack];

    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t task = blockIdx.x * WPB + w;
    constexpr bool listmode = LIST;
    if (listmode ? (uint64_t)task * 32 >= nq : task >= nchunk) return;  // warp-uniform

    uint32_t me;
    bool valid;
    if (listmode) {
        uint32_t qi = task * 32 + lane;
        valid = qi < nq;
        me = valid ? qlist[qi] : 0;
    } else {
        me = task * 32 + lane;
        valid = me < n;
    }
    const float4 P = valid ? sp[me] : make_float4(0.f, 0.f, 0.f, 0.f);
    const int op = __float_as_int(P.w);
    const uint32_t labp = (listmode && valid) ? lab[me] : 0u;

    float(*bd)[32] = s_bd[w];
    int(*bo)[32] = s_bo[w];
    int(*bs)[32] = s_bs[w];
    // Register snapshot of the region minima (INFINITY = empty region) and
    // their maximum, refreshed after every fold; used only for pruning.
    float snap[K];
#pragma unroll
    for (int r = 0; r < K; ++r) {
        bd[r][lane] = INFINITY;
        bo[r][lane] = INT_MAX;
        bs[r][lane] = -1;
        snap[r] = INFINITY;
    }
    float maxall = valid ? INFINITY : -1.f;
    // search statistics (only accumulated when stats != nullptr)
    uint32_t st_leaves = 0, st_nodes = 0, st_cands = 0;

    auto refresh = [&]() {
        maxall = -1.f;
#pragma unroll
        for (int r = 0; r < K; ++r) {
            snap[r] = bs[r][lane] < 0 ? INFINITY : bd[r][lane];
            maxall = fmaxf(maxall, snap[r]);
        }
    };

    auto upd = [&](int r, float d2, int oq, int sq) {
        float b = bd[r][lane];
        if (d2 < b || (d2 == b && oq < bo[r][lane])) {
            bd[r][lane] = d2;
            bo[r][lane] = oq;
            bs[r][lane] = sq;
        }
    };

    // Fold one candidate (position c, input id oq, leaf position sq).
    auto fold = [&](float cx_, float cy_, float cz_, int oq, int sq) {
        const float dx = __fsub_rn(cx_, P.x);
        const float dy = __fsub_rn(cy_, P.y);
        const float dz = __fsub_rn(cz_, P.z);
        const float d2 = d2_of<D>(dx, dy, dz);
        if (d2 > maxall) return;  // cannot improve any region (all non-empty)
        if (listmode && d2 == 0.f && lab[sq] == labp) return;
        int r = region_fast<D>(dx, dy, dz);
        if (r >= 0) {
            upd(r, d2, oq, sq);
        } else {
            uint32_t mk = region_mask<D>(dx, dy, dz);
            while (mk) {
                int rr = __ffs(mk) - 1;
                mk &= mk - 1;
                upd(rr, d2, oq, sq);
            }
        }
    };

    auto leaf = [&](uint32_t chunk, bool need) {
        const uint32_t base = chunk * 32;
        const uint32_t m = min(32u, n - base);
        float4 t = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
        if ((uint32_t)lane < m) t = sp[base + lane];
        s_tile[w][lane] = t;
        __syncwarp();
        ++st_leaves;
        if (need) {
            st_cands += m;
            for (uint32_t j = 0; j < m; ++j) {
                const float4 c = s_tile[w][j];
                const int oq = __float_as_int(c.w);
                if (oq == op) continue;
                fold(c.x, c.y, c.z, oq, (int)(base + j));
            }
            refresh();
        }
        __syncwarp();
    };

    // May the box [lo, hi] hold a point that improves one of this lane's
    // regions?  For region R (dominant axis dir with sign, slab signs on the
    // other axes) every point q of box and cone has |d_i| >= L_i on the other
    // axes (the box's distance from 0 on the slab's side) and
    // |d_dir| >= T = max(L_dir, L_i) (dominance), so d2(q) >= d2_of(T, L_i)
    // evaluated with the same rounded operations (monotone): an exact lower
    // bound on the float offsets, compared with the region's minimum
    // (<=, because an equal d2 with a smaller id still improves it).
    auto needs = [&](const float4& lo, const float4& hi) -> bool {
        if (!valid) return false;
        const float a[3] = {__fsub_rn(lo.x, P.x), __fsub_rn(lo.y, P.y), __fsub_rn(lo.z, P.z)};
        const float b[3] = {__fsub_rn(hi.x, P.x), __fsub_rn(hi.y, P.y), __fsub_rn(hi.z, P.z)};
        {
            const float gx = fmaxf(fmaxf(a[0], -b[0]), 0.f);
            const float gy = fmaxf(fmaxf(a[1], -b[1]), 0.f);
            const float gz = D == 3 ? fmaxf(fmaxf(a[2], -b[2]), 0.f) : 0.f;
            if (d2_of<D>(gx, gy, gz) > maxall) return false;
        }
        // per axis, per side: lower bound of |d| and feasibility
        float Lp[3], Ln[3];
        bool fp[3], fn[3];
#pragma unroll
        for (int i = 0; i < D; ++i) {
            Lp[i] = fmaxf(a[i], 0.f);
            Ln[i] = fmaxf(-b[i], 0.f);
            fp[i] = b[i] >= 0.f;
            fn[i] = a[i] <= 0.f;
        }
        bool hit = false;
#pragma unroll
        for (int f = 0; f < 2 * D; ++f) {
            const int dir = f >> 1;
            const bool neg = f & 1;
            const float Ld = neg ? Ln[dir] : Lp[dir];
            const float Hd = neg ? -a[dir] : b[dir];
            const bool fd = neg ? fn[dir] : fp[dir];
#pragma unroll
            for (int s = 0; s < NS; ++s) {
                float l[3] = {0.f, 0.f, 0.f};
                float T = Ld;
                bool ok = fd;
                int bit = 0;
#pragma unroll
                for (int i = 0; i < D; ++i) {
                    if (i == dir) continue;
                    const bool sn = (s >> bit) & 1;
                    l[i] = sn ? Ln[i] : Lp[i];
                    ok = ok && (sn ? fn[i] : fp[i]);
                    T = fmaxf(T, l[i]);
                    ++bit;
                }
                l[dir] = T;
                ok = ok && T <= Hd;
                hit |= ok && d2_of<D>(l[0], l[1], l[2]) <= snap[f * NS + s];
            }
        }
        return hit;
    };

    // Warp reference point for near-first ordering.
    const float cx = __shfl_sync(kFull, P.x, 0), cy = __shfl_sync(kFull, P.y, 0), cz = __shfl_sync(kFull, P.z, 0);
    auto box_d2 = [&](uint32_t node) -> float {
        const float4 lo = nlo[node], hi = nhi[node];
        if (lo.x > hi.x) return INFINITY;
        const float gx = fmaxf(fmaxf(lo.x - cx, cx - hi.x), 0.f);
        const float gy = fmaxf(fmaxf(lo.y - cy, cy - hi.y), 0.f);
        const float gz = fmaxf(fmaxf(lo.z - cz, cz - hi.z), 0.f);
        return gx * gx + gy * gy + gz * gz;
    };

    const uint32_t own = listmode ? 0xffffffffu : L + task;
    if (!listmode) leaf(task, valid);

    int top = 0;
    if (lane == 0) s_stack[w][0] = 1u;
    top = 1;
    __syncwarp();
    while (top > 0) {
        const uint32_t node = s_stack[w][--top];
        __syncwarp();
        if (node == own) continue;
        const float4 lo = nlo[node], hi = nhi[node];
        if (lo.x > hi.x) continue;
        ++st_nodes;
        const bool need = needs(lo, hi);
        if (!__any_sync(kFull, need)) continue;
        if (lo.x == hi.x && lo.y == hi.y && lo.z == hi.z) {
            // All points of this subtree coincide: the smallest input id other
            // than the query's own is the only candidate that can matter.
            if (need) {
                const int4 id = nid[node];
                int oq = id.x, sq = id.y;
                if (oq == op) {
                    oq = id.z;
                    sq = id.w;
                }
                if (oq != INT_MAX) {
                    fold(lo.x, lo.y, lo.z, oq, sq);
                    refresh();
                }
            }
            continue;
        }
        if (node >= L) {
            leaf(node - L, need);
        } else {
            const uint32_t c0 = 2 * node, c1 = 2 * node + 1;
            const float d0 = box_d2(c0), d1 = box_d2(c1);
            const uint32_t nearc = d0 <= d1 ? c0 : c1, farc = d0 <= d1 ? c1 : c0;
            if (top + 2 > kStack) break;  // cannot happen for trees of depth < 62
            if (lane == 0) {
                s_stack[w][top] = farc;
                s_stack[w][top + 1] = nearc;
            }
            top += 2;
            __syncwarp();
        }
    }

    if (stats) {
        unsigned long long cands = st_cands;
        for (int o = 16; o > 0; o >>= 1) cands += __shfl_xor_sync(kFull, cands, o);
        if (lane == 0) {
            atomicAdd(&stats[0], (unsigned long long)st_leaves);
            atomicAdd(&stats[1], (unsigned long long)st_nodes);
            atomicAdd(&stats[2], cands);
            atomicAdd(&stats[3], 1ull);
        }
    }
    if (!valid) return;
    // Region-order table (round 1 only; optional).
    if (tab_id) {
        for (int r = 0; r < K; ++r) {
            tab_id[(int64_t)op * K + r] = bs[r][lane] >= 0 ? bo[r][lane] : -1;
            tab_d2[(int64_t)op * K + r] = bd[r][lane];
        }
    }
    // Compact, sort by (d2, input id), deduplicate.
    int m = 0;
    for (int r = 0; r < K; ++r) {
        if (bs[r][lane] >= 0) {
            bd[m][lane] = bd[r][lane];
            bo[m][lane] = bo[r][lane];
            bs[m][lane] = bs[r][lane];
            ++m;
        }
    }
    for (int i = 1; i < m; ++i) {
        float kd = bd[i][lane];
        int ko = bo[i][lane], ks = bs[i][lane];
        int j = i - 1;
        while (j >= 0 && (bd[j][lane] > kd || (bd[j][lane] == kd && bo[j][lane] > ko))) {
            bd[j + 1][lane] = bd[j][lane];
            bo[j + 1][lane] = bo[j][lane];
            bs[j + 1][lane] = bs[j][lane];
            --j;
        }
        bd[j + 1][lane] = kd;
        bo[j + 1][lane] = ko;
        bs[j + 1][lane] = ks;
    }
    uint64_t* out = cand + (uint64_t)me * K;
    int u = 0;
    bool zero = false;
    for (int i = 0; i < m; ++i) {
        if (i > 0 && bs[i][lane] == bs[i - 1][lane]) continue;
        const float d2 = bd[i][lane];
        zero |= d2 == 0.f;
        out[u++] = ((uint64_t)__float_as_uint(d2) << 32) | (uint32_t)bs[i][lane];
    }
    cnt[me] = (unsigned char)u;
    cur[me] = 0;
    zflag[me] = zero ? 1 : 0;
    if (zero) {
        uint32_t slot = atomicAdd(zero_count, 1u);
        zero_out[slot] = me;
    }
}

template <int D>
cudaError_t launch(Ctx& c, const uint32_t* qlist, uint32_t nq, uint32_t* zero_out, uint32_t* zero_count,
                   bool table)
{
    constexpr int WPB = 4;
    unsigned tasks = qlist ? (unsigned)((nq + 31) / 32) : (unsigned)c.nchunk;
    if (tasks == 0) return cudaSuccess;
    unsigned blocks = (tasks + WPB - 1) / WPB;
    auto kern = qlist ? k_nns<D, WPB, true> : k_nns<D, WPB, false>;
    kern<<<blocks, WPB * 32, 0, c.stream>>>(
        c.sp.p, c.nlo.p, c.nhi.p, c.nid.p, (uint32_t)c.n, (uint32_t)c.L, (uint32_t)c.nchunk, qlist, nq,
        qlist ? c.lab.p : nullptr, c.cand.p, c.cnt.p, c.cur.p, c.zflag.p, zero_out, zero_count,
        table ? c.tab_id.p : nullptr, table ? c.tab_d2.p : nullptr, c.profile ? c.nstats.p : nullptr);
    c.launches++;
    c.nns_launches++;
    return cudaGetLastError();
}

}  // namespace

// Round-1 table for every point (all components distinct, no filter).
cudaError_t nns_full(Ctx& c)
{
    cudaError_t e;
    const size_t n = (size_t)c.n;
    if ((e = c.ensure(c.cand, n * c.K)) != cudaSuccess) return e;
    if ((e = c.ensure(c.cnt, n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.cur, n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.zflag, n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.zero, n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.zero2, n)) != cudaSuccess) return e;
    if (c.keep_table) {
        if ((e = c.ensure(c.tab_id, n * c.K)) != cudaSuccess) return e;
        if ((e = c.ensure(c.tab_d2, n * c.K)) != cudaSuccess) return e;
    }
    uint32_t* zc = &c.ctr.p->n_zero_next;
    if ((e = cudaMemsetAsync(zc, 0, sizeof(uint32_t), c.stream)) != cudaSuccess) return e;
    return c.dim == 2 ? launch<2>(c, nullptr, 0, c.zero.p, zc, c.keep_table)
                      : launch<3>(c, nullptr, 0, c.zero.p, zc, c.keep_table);
}

// Later rounds: recompute the points whose table holds a zero distance, with
// the zero-distance / same-component filter.  c.n_zero is the host count of
// the current zero list; the refreshed list goes to zero2 (then swapped).
cudaError_t nns_recompute_zero(Ctx& c)
{
    cudaError_t e;
    if (c.n_zero == 0) return cudaSuccess;
    uint32_t* zc = &c.ctr.p->n_zero_next;
    if ((e = cudaMemsetAsync(zc, 0, sizeof(uint32_t), c.stream)) != cudaSuccess) return e;
    e = c.dim == 2 ? launch<2>(c, c.zero.p, c.n_zero, c.zero2.p, zc, false)
                   : launch<3>(c, c.zero.p, c.n_zero, c.zero2.p, zc, false);
    std::swap(c.zero.p, c.zero2.p);
    return e;
}

}  // namespace emst
