// cnns.cu -- component nearest-neighbour search (the default solver mode).
//
// Each Boruvka round needs, per component, its shortest outgoing edge under
// the order (d2, min id, max id) (EMST_isInf, macros_cuda.h:37).  The
// reference reaches it through a static region table (NodeEMST.h:1018-1384);
// this mode searches for it directly, per point, in the same leaf tree:
//
//   * node labels: after the labels are flattened, every tree node records
//     the component all its points share (or MIXED); a point's search skips
//     subtrees of its own component entirely;
//   * shared bound: a point prunes with min(its own best, the best key its
//     component holds so far in the 64-bit atomicMin slot) -- the slot is an
//     upper bound of the component's minimum, so the minimum is never pruned;
//   * reuse: a point whose previous partner is still outside its component
//     keeps it (the outside set only shrinks, so the minimum stands); only
//     the others ("dirty" points) search.  A result is kept for reuse only if
//     the shared bound did not cut the search short of it;
//   * lower bounds: every search leaves lbp[p] <= d2 of p's nearest point
//     outside its component, which stays valid in later rounds (components
//     only grow).  Dirty points search in two passes: first those with the
//     smallest bounds in their component (likely to hold its minimum), then
//     the rest, each skipped outright when its bound exceeds the best key its
//     component already holds (it cannot hold the minimum).
//
// For a fixed query the candidate order is (d2, input id), which is the
// reference order restricted to that query, so each component's minimum --
// and with it every round's edge set -- equals the static-table method's.
#include <climits>
#include <cmath>


#include "cnns_search.cuh"

namespace emst {

namespace {

constexpr int kStack = 64;
constexpr int kLeavesPerBlock = 1024;

__device__ __forceinline__ uint32_t merge_label(uint32_t a, uint32_t b)
{
    if (a == kEmpty) return b;
    if (b == kEmpty) return a;
    return a == b ? a : kMixed;
}

// Leaves of one block (a subtree of kLeavesPerBlock leaf slots, or all of L
// when smaller) and the levels above them inside that subtree.  With `par`
// (the flatten step) every point's label is first replaced by its root's
// root, lab[j] = par[lab[j]] (K_EMST_flatten_DST_1, EMSTOperators.h:412-433),
// so the relabel and the next round's node labels take one pass over lab.
// Warp w takes the block's leaves [32 w, 32 w + 32), lane i keeps leaf
// 32 w + i's label, and the subtree is merged by warp shuffles: five levels in
// every warp, then the levels above across the block's warps in warp 0 (one
// barrier instead of two per level).
__global__ void __launch_bounds__(1024)
    k_node_labels_sub(uint32_t* __restrict__ lab, const uint32_t* __restrict__ par, uint32_t n, uint32_t nchunk,
                      uint32_t L, uint32_t span, uint32_t* __restrict__ nlab)
{
    __shared__ uint32_t s_w[32];
    const uint32_t first = blockIdx.x * span;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t wl0 = 32u * (uint32_t)w;
    // four leaves per warp and step, their loads issued together (each leaf
    // is a chain of two dependent loads: the label, then its root)
    constexpr int kU = 4;
    uint32_t v = kEmpty;  // lane i: the label of leaf wl0 + i
    for (uint32_t s0 = 0; s0 < 32u && wl0 + s0 < span; s0 += kU) {
        uint32_t my[kU];
        bool ok[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const uint32_t l = wl0 + s0 + (uint32_t)u, c = first + l;
            const uint32_t j = c * 32 + lane;
            ok[u] = l < span && c < nchunk && j < n;
            my[u] = ok[u] ? lab[j] : 0u;
        }
        if (par) {
#pragma unroll
            for (int u = 0; u < kU; ++u)
                if (ok[u]) my[u] = __ldcg(&par[my[u]]);
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const uint32_t l = wl0 + s0 + (uint32_t)u, c = first + l;
            if (l >= span) break;  // warp-uniform
            if (par && ok[u]) lab[c * 32 + lane] = my[u];
            uint32_t out = kEmpty;
            if (c < nchunk) {
                const uint32_t f = __shfl_sync(kFull, my[u], 0);
                out = __all_sync(kFull, !ok[u] || my[u] == f) ? f : kMixed;
            }
            if (lane == 0) nlab[L + c] = out;
            if ((uint32_t)lane == s0 + (uint32_t)u) v = out;
        }
    }
    // level k node of block leaf i: (L + first) / 2^k + i / 2^k (L + first is a
    // multiple of span)
    const uint32_t base = L + first;
    for (int k = 1; k <= 5 && (1u << k) <= span; ++k) {
        v = merge_label(v, __shfl_down_sync(kFull, v, 1u << (k - 1)));
        const uint32_t i = wl0 + (uint32_t)lane;
        if ((lane & ((1 << k) - 1)) == 0 && i < span) nlab[(base >> k) + (i >> k)] = v;
    }
    if (span <= 32u) return;  // block-uniform
    if (lane == 0) s_w[w] = v;
    __syncthreads();
    if (w == 0) {
        const uint32_t nw = span >> 5;  // warps holding leaves
        v = (uint32_t)lane < nw ? s_w[lane] : kEmpty;
        for (int k = 6; (1u << k) <= span; ++k) {
            v = merge_label(v, __shfl_down_sync(kFull, v, 1u << (k - 6)));
            if ((lane & ((1 << (k - 5)) - 1)) == 0 && (uint32_t)lane < nw) nlab[(base >> k) + ((uint32_t)lane >> (k - 5))] = v;
        }
    }
}

// Levels above the per-block subtrees (nodes [1, top)), one block.
__global__ void __launch_bounds__(1024) k_node_labels_top(uint32_t top, uint32_t* __restrict__ nlab)
{
    for (uint32_t h = top >> 1; h >= 1; h >>= 1) {
        for (uint32_t t = threadIdx.x; t < h; t += blockDim.x)
            nlab[h + t] = merge_label(nlab[2 * (h + t)], nlab[2 * (h + t) + 1]);
        __syncthreads();
    }
}

// Points whose previous partner is still outside their component re-submit
// it; the others go to the dirty list and fold their lower bound into their
// component's minimum bound clb (when a first-pass rule reads it: clb set).
__global__ void k_reuse(uint32_t n, const uint32_t* __restrict__ lab, uint32_t* __restrict__ selq,
                        uint64_t* __restrict__ selkey, float* __restrict__ lbp, uint64_t* __restrict__ ckey,
                        uint32_t* __restrict__ clb, unsigned char* __restrict__ dflag, uint32_t* __restrict__ prov,
                        uint32_t* __restrict__ n_prov, const int* __restrict__ round,
                        const uint64_t* __restrict__ klist, unsigned char* __restrict__ kcur,
                        const uint32_t* __restrict__ perm, int knn_k)
{
    const int r = *round;
    // round 1 with neighbour lists: the list build searches every point and
    // writes every result this pass would, so the pass has nothing to do
    if (klist && r == 1) return;
    const bool lists = klist && r >= 2;
    __shared__ uint32_t s_cnt[33];
    const uint32_t stride = gridDim.x * blockDim.x;
    // The pass is bound by chains of dependent loads.  The next iteration's
    // partner, label, bound and list cursor are loaded one iteration ahead;
    // then the partner's label, the list entry at the cursor, the point's own
    // input id and its key are loaded together (the last three only where
    // they may be used), so a point waits on four levels of loads, not six.
    uint32_t p_next = blockIdx.x * blockDim.x + threadIdx.x;
    uint32_t q_next = kNone, lp_next = 0u, lb_next = 0u, j0_next = 0u;
    if (p_next < n) {
        q_next = selq[p_next];
        lp_next = lab[p_next];
        lb_next = __float_as_uint(lbp[p_next]);
        if (lists) j0_next = kcur[p_next];
    }
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride) {
        const uint32_t p = base + threadIdx.x;
        const uint32_t q = q_next, lp0 = lp_next, lb0 = lb_next, j0 = j0_next;
        p_next = p + stride;
        if (p_next < n) {
            q_next = selq[p_next];
            lp_next = lab[p_next];
            lb_next = __float_as_uint(lbp[p_next]);
            if (lists) j0_next = kcur[p_next];
        }
        bool is_dirty = false, record = false;
        uint64_t key = kNoKey;
        uint32_t lp = 0;
        if (p < n) {
            lp = lp0;
            // round 2 with lists: the partner is list entry 0, the round-1
            // edge, inside the component for certain (k_knn_first set the
            // cursor past it)
            const bool has_q = !(lists && r == 2) && q != kNone;
            const bool walk = lists && lb0 != 0x7f800000u && (int)j0 < knn_k;
            const uint32_t lq = has_q ? lab[q] : lp;
            const uint64_t sk = has_q ? selkey[p] : kNoKey;
            const uint64_t k0 = walk ? klist[(size_t)j0 * n + p] : ~0ull;
            const uint32_t op = walk ? perm[p] : 0u;
            if (has_q && lq != lp) {
                key = sk;
            } else {
                uint32_t lb = lb0;
                if (lists && lb != 0x7f800000u) {
                    // the first neighbour outside the component is the exact
                    // nearest outside point: every closer point precedes it.
                    // Entries before the cursor were found inside the
                    // component in an earlier round and stay inside
                    // (components only grow); their d2 is already in lbp.
                    bool full = true;
                    int j = (int)j0;
                    for (; j < knn_k; ++j) {
                        // d2 bits << 32 | position
                        const uint64_t kj = j == (int)j0 ? k0 : klist[(size_t)j * n + p];
                        const uint32_t qj = (uint32_t)kj;
                        if (qj == kNone) {
                            full = false;
                            break;
                        }
                        if (lab[qj] != lp) {
                            const uint32_t mn = min(op, perm[qj]);
                            key = (kj & 0xffffffff00000000ull) | mn;
                            selq[p] = qj;
                            selkey[p] = key;
                            lbp[p] = __uint_as_float((uint32_t)(kj >> 32));
                            break;
                        }
                        lb = max(lb, (uint32_t)(kj >> 32));  // non-negative floats order as their bits
                    }
                    if (j != (int)j0) kcur[p] = (unsigned char)j;
                    if (key == kNoKey && (j != (int)j0 || !full)) {
                        // none outside: a full list bounds the distance from below;
                        // a short one held every other point of the cloud
                        // (an exhausted list, j0 == knn_k, adds nothing new)
                        lb = full ? lb : 0x7f800000u;
                        lbp[p] = __uint_as_float(lb);
                    }
                }
                if (key == kNoKey) {
                    // lbp = +inf: no point outside the component exists (in a batch,
                    // the cloud is one component), and components only grow
                    is_dirty = lb != 0x7f800000u;
                    if (is_dirty && clb && lb < __ldcg(&clb[lp])) atomicMin(&clb[lp], lb);
                }
            }
        }
        // Fold the keys into the components' slots.  When every keyed lane of
        // the warp is in one component (most warps once components are
        // large), only the lanes holding the warp's smallest key go to the
        // slot: the others cannot be the component's minimum.
        const bool has = key != kNoKey;
        const unsigned hm = __ballot_sync(kFull, has);
        if (hm) {
            const uint32_t l0 = __shfl_sync(kFull, lp, __ffs(hm) - 1);
            bool go = has;
            if (__all_sync(kFull, !has || lp == l0)) {
                const uint32_t hi = __reduce_min_sync(kFull, has ? (uint32_t)(key >> 32) : ~0u);
                const uint32_t lo = __reduce_min_sync(kFull, has && (uint32_t)(key >> 32) == hi ? (uint32_t)key : ~0u);
                go = has && key == (((uint64_t)hi << 32) | lo);
            }
            if (go && key <= __ldcg(&ckey[lp])) {
                const uint64_t old = atomicMin((unsigned long long*)&ckey[lp], (unsigned long long)key);
                record = old >= key;
            }
        }
        if (p < n) dflag[p] = is_dirty ? 1 : 0;
        // late rounds record few points: one vote skips the reservation
        if (__syncthreads_or(record)) {
            const uint32_t slot = block_reserve(record, n_prov, s_cnt);
            if (record) prov[slot] = p;
        }
    }
}

// One warp per 32 dirty points: nearest point outside the query's component.
template <int D, int WPB>
__global__ void __launch_bounds__(WPB * 32)
    k_cnns(const float4* __restrict__ sp, const float4* __restrict__ nlo, const float4* __restrict__ nhi,
           const uint32_t* __restrict__ nlab, uint32_t n, uint32_t L, const uint32_t* __restrict__ dirty,
           const uint32_t* __restrict__ n_dirty, const uint32_t* __restrict__ lab, uint64_t* __restrict__ ckey,
           uint32_t* __restrict__ selq, uint64_t* __restrict__ selkey, uint32_t* __restrict__ prov,
           uint32_t* __restrict__ n_prov, float* __restrict__ lbp, const uint32_t* __restrict__ clb, int pass,
           uint32_t* __restrict__ defer, uint32_t* __restrict__ n_defer, unsigned long long* __restrict__ stats)
{
    __shared__ float4 s_tile[WPB][32];
    __shared__ uint32_t s_tlab[WPB][32];
    __shared__ uint32_t s_stack[WPB][kStack];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t total = *n_dirty;

    for (uint32_t task = blockIdx.x * WPB + w; (uint64_t)task * 32 < total; task += gridDim.x * WPB) {
        const uint32_t qi = task * 32 + lane;
        const bool listed = qi < total;
        const uint32_t me = listed ? dirty[qi] : 0u;
        const uint32_t labp0 = listed ? lab[me] : kEmpty;
        const float lb0 = listed ? lbp[me] : 0.f;
        bool valid = listed, deferred = false;
        if (listed) {
            const uint64_t k = __ldcg(&ckey[labp0]);
            const float cb0 = k == kNoKey ? INFINITY : __uint_as_float((uint32_t)(k >> 32));
            if (lb0 > cb0) {
                valid = false;  // cannot hold its component's minimum this round
            } else if (pass == 1 && lb0 > 4.f * __uint_as_float(__ldcg(&clb[labp0]))) {
                valid = false;  // not among its component's most promising points: second pass
                deferred = true;
            }
        }
        warp_append(deferred, me, defer, n_defer);
        const float4 P = valid ? sp[me] : make_float4(0.f, 0.f, 0.f, 0.f);
        const int op = __float_as_int(P.w);
        const uint32_t labp = valid ? labp0 : kEmpty;

        float bd = INFINITY;  // best d2
        int bo = INT_MAX;     // its input id
        int bs = -1;          // its leaf position
        float cut = INFINITY; // smallest lower bound pruned only because of the shared bound
        uint32_t st_leaves = 0, st_nodes = 0, st_cands = 0;
        const uint32_t st_queries = __popc(__ballot_sync(kFull, valid));

        auto shared_bound = [&]() -> float {
            if (!valid) return -1.f;
            const uint64_t k = __ldcg(&ckey[labp]);
            return k == kNoKey ? INFINITY : __uint_as_float((uint32_t)(k >> 32));
        };
        float cb = shared_bound();

        // Is the node worth opening for this lane?  lb2 <= d2(q) for every
        // point q in the box (same rounded operations, monotone).
        auto needs = [&](uint32_t node, const float4& lo, const float4& hi) -> bool {
            if (!valid) return false;
            if (nlab[node] == labp) return false;  // all points in the query's component
            const float gx = fmaxf(fmaxf(__fsub_rn(lo.x, P.x), __fsub_rn(P.x, hi.x)), 0.f);
            const float gy = fmaxf(fmaxf(__fsub_rn(lo.y, P.y), __fsub_rn(P.y, hi.y)), 0.f);
            const float gz = D == 3 ? fmaxf(fmaxf(__fsub_rn(lo.z, P.z), __fsub_rn(P.z, hi.z)), 0.f) : 0.f;
            const float lb2 = d2_of<D>(gx, gy, gz);
            if (lb2 > bd) return false;
            if (lb2 > cb) {
                cut = fminf(cut, lb2);
                return false;
            }
            return true;
        };

        const float cx = __shfl_sync(kFull, P.x, 0), cy = __shfl_sync(kFull, P.y, 0),
                    cz = __shfl_sync(kFull, P.z, 0);
        auto box_d2 = [&](uint32_t node) -> float {
            const float4 lo = nlo[node], hi = nhi[node];
            if (lo.x > hi.x) return INFINITY;
            const float gx = fmaxf(fmaxf(lo.x - cx, cx - hi.x), 0.f);
            const float gy = fmaxf(fmaxf(lo.y - cy, cy - hi.y), 0.f);
            const float gz = fmaxf(fmaxf(lo.z - cz, cz - hi.z), 0.f);
            return gx * gx + gy * gy + gz * gz;
        };

        int top = 0;
        if (lane == 0) s_stack[w][0] = 1u;
        top = 1;
        __syncwarp();
        while (top > 0) {
            const uint32_t node = s_stack[w][--top];
            __syncwarp();
            const float4 lo = nlo[node], hi = nhi[node];
            if (lo.x > hi.x) continue;
            ++st_nodes;
            const bool need = needs(node, lo, hi);
            if (!__any_sync(kFull, need)) continue;
            if (node >= L) {
                const uint32_t base = (node - L) * 32;
                const uint32_t m = min(32u, n - base);
                float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
                uint32_t tl = kEmpty;
                if ((uint32_t)lane < m) {
                    t = sp[base + lane];
                    tl = lab[base + lane];
                }
                s_tile[w][lane] = t;
                s_tlab[w][lane] = tl;
                __syncwarp();
                ++st_leaves;
                if (need) {
                    st_cands += m;
                    for (uint32_t j = 0; j < m; ++j) {
                        if (s_tlab[w][j] == labp) continue;
                        const float4 c = s_tile[w][j];
                        const float dx = __fsub_rn(c.x, P.x);
                        const float dy = __fsub_rn(c.y, P.y);
                        const float dz = __fsub_rn(c.z, P.z);
                        const float d2 = d2_of<D>(dx, dy, dz);
                        const int oq = __float_as_int(c.w);
                        if (d2 < bd || (d2 == bd && oq < bo)) {
                            bd = d2;
                            bo = oq;
                            bs = (int)(base + j);
                        }
                    }
                    cb = shared_bound();
                }
                __syncwarp();
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

        bool record = false;
        if (valid) {
            // nothing closer than min(cut, bd) lies outside the component
            const bool exact = bs >= 0 && bd < cut;
            lbp[me] = exact ? bd : fmaxf(lb0, fminf(cut, bd));
            if (bs >= 0) {
                const uint32_t mn = (uint32_t)min(op, bo);
                const uint64_t key = ((uint64_t)__float_as_uint(bd) << 32) | mn;
                // keep for reuse only if nothing cut off could still be as close
                selq[me] = exact ? (uint32_t)bs : kNone;
                selkey[me] = key;
                if (key <= __ldcg(&ckey[labp])) {
                    const uint64_t old = atomicMin((unsigned long long*)&ckey[labp], (unsigned long long)key);
                    record = old >= key;
                }
            } else {
                selq[me] = kNone;
            }
        }
        warp_append(record, me, prov, n_prov);
        if (stats) {
            unsigned long long cands = st_cands;
            for (int o = 16; o > 0; o >>= 1) cands += __shfl_xor_sync(kFull, cands, o);
            if (lane == 0) {
                atomicAdd(&stats[0], (unsigned long long)st_leaves);
                atomicAdd(&stats[1], (unsigned long long)st_nodes);
                atomicAdd(&stats[2], cands);
                atomicAdd(&stats[3], 1ull);
                atomicAdd(&stats[4], (unsigned long long)st_queries);
            }
        }
    }
}

// Query lists of a search pass, compacted in leaf order (a warp's 32
// queries are neighbours, so their traversals share nodes and cache lines;
// in round 1 every warp's queries are exactly one leaf).  Three launches:
// k_sel_count decides each point's list and counts per tile of kSelTile
// consecutive points, k_sel_scan turns the tile counts into offsets (one
// block), k_sel_write writes every tile's points at its offset in order.
//   stage 0 (first pass): a dirty point (flag != 0) whose lower bound exceeds
//     its component's key (set by the reused partners) cannot hold the
//     component's minimum and leaves the round (flag 0); one whose bound
//     exceeds `factor` times its component's smallest waits for the second
//     pass (flag 2, written to list2 when one is given); the others search
//     now (flag 1, list1).
//   stage 1 (second pass): a waiting point (flag 2) whose bound the first
//     pass did not rule out searches (list1); every flag ends at 0.
//   stage 2: every flagged point, unfiltered (list1); flags unchanged.
constexpr int kSelThreads = 256, kSelItems = 8, kSelTile = kSelThreads * kSelItems;
constexpr int kScanThreads = 1024;
constexpr unsigned char kSelPicked = 3;  // stage 1: selected, cleared by k_sel_write

__device__ __forceinline__ void load_flags(const unsigned char* __restrict__ flag, uint32_t p0, uint32_t n,
                                           unsigned char (&f)[kSelItems])
{
    if (p0 + kSelItems <= n) {
        const uint2 v = *reinterpret_cast<const uint2*>(flag + p0);  // p0 is a multiple of 8
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            f[k] = (unsigned char)(v.x >> (8 * k));
            f[4 + k] = (unsigned char)(v.y >> (8 * k));
        }
    } else {
#pragma unroll
        for (int k = 0; k < kSelItems; ++k) f[k] = p0 + k < n ? flag[p0 + k] : 0;
    }
}

// Which list a point's (new) flag puts it on: 0 none, 1 list1, 2 list2.
__device__ __forceinline__ int list_of(int stage, unsigned char f, bool two)
{
    if (stage == 0) return f == 1 ? 1 : (f == 2 && two ? 2 : 0);
    if (stage == 1) return f == kSelPicked ? 1 : 0;
    return f ? 1 : 0;
}

// Block-wide exclusive scan of a packed (list1 count | list2 count << 16).
__device__ __forceinline__ uint32_t block_exclusive(uint32_t v, uint32_t* s_warp, uint32_t& total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    uint32_t incl = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) s_warp[w] = incl;
    __syncthreads();
    if (w == 0) {
        const uint32_t x = lane < (int)(blockDim.x >> 5) ? s_warp[lane] : 0u;
        uint32_t in = x;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(kFull, in, o);
            if (lane >= o) in += t;
        }
        if (lane < (int)(blockDim.x >> 5)) s_warp[lane] = in - x;
        if (lane == (int)(blockDim.x >> 5) - 1) s_warp[32] = in;
    }
    __syncthreads();
    const uint32_t ex = s_warp[w] + incl - v;
    total = s_warp[32];
    __syncthreads();  // s_warp is reused by the caller's next scan
    return ex;
}

__global__ void __launch_bounds__(kSelThreads)
    k_sel_count(const int* __restrict__ skip_round, uint32_t n, int stage, unsigned char* __restrict__ flag,
                const uint32_t* __restrict__ lab,
                const float* __restrict__ lbp, const uint64_t* __restrict__ ckey, const uint32_t* __restrict__ clb,
                float factor, bool two, uint32_t* __restrict__ tile_cnt, unsigned long long* __restrict__ stats)
{
    if (skip_round && *skip_round == 1) return;  // round 1: the list build takes every point
    __shared__ uint32_t s_warp[33];
    const uint32_t tile = blockIdx.x;
    const uint32_t p0 = tile * kSelTile + threadIdx.x * kSelItems;
    unsigned char f[kSelItems];
    load_flags(flag, p0, n, f);
    uint32_t mine = 0, later = 0;
    bool changed = false;
    bool any = false;
#pragma unroll
    for (int k = 0; k < kSelItems; ++k) any |= f[k] != 0;
    if (any && stage != 2) {
        // labels and bounds in two 16-byte loads each (p0 is a multiple of 8),
        // then every flagged point's component key and bound at once: the
        // gathers of the eight points overlap instead of queueing
        uint32_t l[kSelItems];
        float lb[kSelItems];
        if (p0 + kSelItems <= n) {
            const uint4 a = *reinterpret_cast<const uint4*>(lab + p0), b = *reinterpret_cast<const uint4*>(lab + p0 + 4);
            const float4 c = *reinterpret_cast<const float4*>(lbp + p0), d = *reinterpret_cast<const float4*>(lbp + p0 + 4);
            l[0] = a.x; l[1] = a.y; l[2] = a.z; l[3] = a.w; l[4] = b.x; l[5] = b.y; l[6] = b.z; l[7] = b.w;
            lb[0] = c.x; lb[1] = c.y; lb[2] = c.z; lb[3] = c.w; lb[4] = d.x; lb[5] = d.y; lb[6] = d.z; lb[7] = d.w;
        } else {
#pragma unroll
            for (int k = 0; k < kSelItems; ++k) {
                l[k] = f[k] ? lab[p0 + k] : 0u;
                lb[k] = f[k] ? lbp[p0 + k] : 0.f;
            }
        }
        uint64_t key[kSelItems];
        uint32_t cl[kSelItems];
#pragma unroll
        for (int k = 0; k < kSelItems; ++k) {
            key[k] = f[k] ? __ldcg(&ckey[l[k]]) : kNoKey;
            cl[k] = f[k] && stage == 0 && clb ? __ldcg(&clb[l[k]]) : 0u;
        }
#pragma unroll
        for (int k = 0; k < kSelItems; ++k) {
            if (!f[k]) continue;
            const float cb = key[k] == kNoKey ? INFINITY : __uint_as_float((uint32_t)(key[k] >> 32));
            unsigned char nf;
            if (stage == 0) {
                nf = 0;
                if (!(lb[k] > cb)) nf = clb && lb[k] > factor * __uint_as_float(cl[k]) ? 2 : 1;
                later += nf == 2;
            } else {
                nf = (f[k] == 2 && !(lb[k] > cb)) ? kSelPicked : 0;
            }
            changed |= nf != f[k];
            f[k] = nf;
        }
    }
#pragma unroll
    for (int k = 0; k < kSelItems; ++k) {
        const int o = list_of(stage, f[k], two);
        mine += o == 1 ? 1u : (o == 2 ? 0x10000u : 0u);
    }
    if (changed) {
#pragma unroll
        for (int k = 0; k < kSelItems; ++k)
            if (p0 + k < n) flag[p0 + k] = f[k];
    }
    uint32_t total = 0;
    block_exclusive(mine, s_warp, total);
    if (threadIdx.x == 0) tile_cnt[tile] = total;
    if (stats && stage == 0) {
        for (int o = 16; o > 0; o >>= 1) later += __shfl_xor_sync(kFull, later, o);
        if ((threadIdx.x & 31) == 0 && later) atomicAdd(&stats[7], (unsigned long long)later);
    }
}

// Exclusive offsets of the tiles' packed counts, in place; the totals go to
// the list counters.  One block; each thread scans a run of tiles.
__global__ void __launch_bounds__(kScanThreads)
    k_sel_scan(const int* __restrict__ skip_round, uint32_t tiles, uint32_t* __restrict__ tile_cnt,
               uint32_t* __restrict__ cnt1, uint32_t* __restrict__ cnt2)
{
    if (skip_round && *skip_round == 1) return;  // round 1: the list build takes every point
    __shared__ uint32_t s_warp[33];
    const uint32_t per = (tiles + kScanThreads - 1) / kScanThreads;
    const uint32_t t0 = threadIdx.x * per;
    // packed sums: a run holds at most per * kSelTile points per list, and the
    // whole list at most n < 2^31; the two halves are kept apart in 64 bits
    uint64_t run1 = 0, run2 = 0;
    for (uint32_t t = t0; t < t0 + per && t < tiles; ++t) {
        run1 += tile_cnt[t] & 0xffffu;
        run2 += tile_cnt[t] >> 16;
    }
    // two block scans (32-bit each: list lengths are below 2^31)
    uint32_t tot1 = 0, tot2 = 0;
    uint32_t ex1 = block_exclusive((uint32_t)run1, s_warp, tot1);
    uint32_t ex2 = block_exclusive((uint32_t)run2, s_warp, tot2);
    for (uint32_t t = t0; t < t0 + per && t < tiles; ++t) {
        const uint32_t v = tile_cnt[t];
        // offsets do not fit 16 bits: list1 offsets in tile_cnt, list2 offsets
        // in the second half of the array
        tile_cnt[t] = ex1;
        tile_cnt[tiles + t] = ex2;
        ex1 += v & 0xffffu;
        ex2 += v >> 16;
    }
    if (threadIdx.x == 0) {
        *cnt1 = tot1;
        if (cnt2) *cnt2 = tot2;
    }
}

__global__ void __launch_bounds__(kSelThreads)
    k_sel_write(const int* __restrict__ skip_round, uint32_t n, int stage, unsigned char* __restrict__ flag, bool two,
                const uint32_t* __restrict__ tile_off,
                uint32_t tiles, uint32_t* __restrict__ list1, uint32_t* __restrict__ list2)
{
    if (skip_round && *skip_round == 1) return;  // round 1: the list build takes every point
    __shared__ uint32_t s_warp[33];
    const uint32_t tile = blockIdx.x;
    const uint32_t p0 = tile * kSelTile + threadIdx.x * kSelItems;
    unsigned char f[kSelItems];
    load_flags(flag, p0, n, f);
    uint32_t mine = 0;
#pragma unroll
    for (int k = 0; k < kSelItems; ++k) {
        const int o = list_of(stage, f[k], two);
        mine += o == 1 ? 1u : (o == 2 ? 0x10000u : 0u);
    }
    uint32_t total = 0;
    const uint32_t ex = block_exclusive(mine, s_warp, total);
    if (total == 0) return;
    uint32_t o1 = tile_off[tile] + (ex & 0xffffu);
    uint32_t o2 = two ? tile_off[tiles + tile] + (ex >> 16) : 0u;
    bool clear = false;
#pragma unroll
    for (int k = 0; k < kSelItems; ++k) {
        const uint32_t p = p0 + k;
        const int o = list_of(stage, f[k], two);
        if (o == 1) list1[o1++] = p;
        else if (o == 2) list2[o2++] = p;
        clear |= stage == 1 && f[k] == kSelPicked;
    }
    if (clear) {
#pragma unroll
        for (int k = 0; k < kSelItems; ++k)
            if (p0 + k < n && f[k] == kSelPicked) flag[p0 + k] = 0;
    }
}

// A search pass's list (see k_sel_count).  Three launches.
cudaError_t select_list(Ctx& c, int stage, float factor, uint32_t* list1, uint32_t* cnt1, uint32_t* list2,
                        uint32_t* cnt2, unsigned long long* stats)
{
    // with round-1 neighbour lists the list build searches every point in round 1
    const int* skip = (c.knn_seed && !c.cnns_warp && stage == 0) ? &c.ctr.p->round : nullptr;
    const uint32_t tiles = (uint32_t)((c.n + kSelTile - 1) / kSelTile);
    const bool two = list2 != nullptr;
    k_sel_count<<<tiles, kSelThreads, 0, c.stream>>>(skip, (uint32_t)c.n, stage, c.dflag.p, c.lab.p, c.lbp.p, c.ckey.p,
                                                     c.clb_used() ? c.clb.p : nullptr, factor, two, c.sel_tiles.p,
                                                     stats);
    k_sel_scan<<<1, kScanThreads, 0, c.stream>>>(skip, tiles, c.sel_tiles.p, cnt1, two ? cnt2 : nullptr);
    k_sel_write<<<tiles, kSelThreads, 0, c.stream>>>(skip, (uint32_t)c.n, stage, c.dflag.p, two, c.sel_tiles.p, tiles,
                                                     list1, list2);
    c.launches += 3;
    return cudaGetLastError();
}

// input id -> leaf position (perm maps leaf position -> input id)
__global__ void k_inverse_perm(uint32_t n, const uint32_t* __restrict__ perm, uint32_t* __restrict__ iperm)
{
    const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) iperm[perm[j]] = j;
}

__global__ void k_fill_u32(uint32_t* __restrict__ p, uint32_t n, uint32_t v)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

unsigned list_grid(uint64_t upper)
{
    uint64_t b = (upper + 255) / 256;
    if (b < 1) b = 1;
    if (b > 152ull * 16) b = 152ull * 16;
    return (unsigned)b;
}

}  // namespace

// Tree-node labels: the value (component, or cloud) shared by all points of
// a subtree, MIXED when they differ.
cudaError_t node_labels_of(Ctx& c, uint32_t* labels, uint32_t* out, const uint32_t* par)
{
    const uint32_t L = (uint32_t)c.L;
    const uint32_t span = L < (uint32_t)kLeavesPerBlock ? L : (uint32_t)kLeavesPerBlock;
    k_node_labels_sub<<<L / span, 1024, 0, c.stream>>>(labels, par, (uint32_t)c.n, (uint32_t)c.nchunk, L, span,
                                                       out);
    c.launches++;
    if (L / span >= 2) {
        k_node_labels_top<<<1, 1024, 0, c.stream>>>(L / span, out);
        c.launches++;
    }
    return cudaGetLastError();
}

// Node labels of the initial forest (every point its own component); the
// flatten step of every round refreshes them (boruvka.cu).
cudaError_t cnns_node_labels(Ctx& c)
{
    cudaError_t e;
    if ((e = c.ensure(c.nlab, (size_t)2 * c.L)) != cudaSuccess) return e;  // no-op after cnns_init
    if ((e = node_labels_of(c, c.lab.p, c.nlab.p)) != cudaSuccess) return e;
    return cudaGetLastError();
}

cudaError_t cnns_init(Ctx& c)
{
    cudaError_t e;
    const size_t n = (size_t)c.n;
    if ((e = c.ensure(c.dirty, n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.dirty2, n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.lbp, n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.clb, n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.nlab, (size_t)2 * c.L)) != cudaSuccess) return e;
    if ((e = c.ensure(c.dflag, n)) != cudaSuccess) return e;
    // per tile of the list compaction: counts, then list1 and list2 offsets
    if ((e = c.ensure(c.sel_tiles, 2 * ((n + kSelTile - 1) / kSelTile))) != cudaSuccess) return e;
    if (c.knn_seed && !c.cnns_warp) {
        if ((e = c.ensure(c.klist, n * c.knn_k)) != cudaSuccess) return e;
        if ((e = c.ensure(c.kcur, n)) != cudaSuccess) return e;
        if ((e = c.ensure(c.iperm, n)) != cudaSuccess) return e;
        k_inverse_perm<<<blocks_for(c.n, 256), 256, 0, c.stream>>>((uint32_t)c.n, c.perm.p, c.iperm.p);
        c.launches++;
    }
    k_fill_u32<<<blocks_for(c.n, 256), 256, 0, c.stream>>>(c.selq.p, (uint32_t)c.n, kNone);
    if (c.clb_used()) {
        k_fill_u32<<<blocks_for(c.n, 256), 256, 0, c.stream>>>(c.clb.p, (uint32_t)c.n, 0x7f800000u);
        c.launches++;
    }
    cudaMemsetAsync(c.lbp.p, 0, n * sizeof(float), c.stream);
    c.launches++;
    // node labels of the initial forest; each round's flatten refreshes them
    return cnns_node_labels(c);
}

// Reuse pass + two search passes over the dirty points; fills ckey and the
// provisional winner list exactly like the static-table selection does.
cudaError_t cnns_select(Ctx& c)
{
    DevCounters* d = c.ctr.p;  // n_dirty, n_dirty2, n_prov were zeroed by the round tick
    const bool knn = c.knn_seed && !c.cnns_warp;
    k_reuse<<<list_grid(c.n), 256, 0, c.stream>>>((uint32_t)c.n, c.lab.p, c.selq.p, c.selkey.p, c.lbp.p, c.ckey.p,
                                                  c.clb_used() ? c.clb.p : nullptr, c.dflag.p, c.prov.p, &d->n_prov,
                                                  &d->round,
                                                  knn ? c.klist.p : nullptr, c.kcur.p, c.perm.p, c.knn_k);
    c.launches++;
    // query lists in leaf order: a warp's 32 queries are neighbours, so their
    // traversals share nodes and cache lines
    unsigned long long* st = c.profile ? c.nstats.p : nullptr;
    cudaError_t e;
    if (c.cnns_warp) {
        e = select_list(c, 2, INFINITY, c.dirty.p, &d->n_dirty, nullptr, nullptr, st);
    } else {
        const bool ordered = c.first_pass_ordered;
        e = select_list(c, 0, c.first_pass_factor, c.dirty.p, &d->n_dirty, ordered ? c.dirty2.p : nullptr,
                        ordered ? &d->n_dirty2 : nullptr, st);
    }
    if (e != cudaSuccess) return e;
    constexpr int WPB = 4;
    const unsigned blocks = (unsigned)std::min<int64_t>((c.n + 32 * WPB - 1) / (32 * WPB), 152 * 32);
    const uint32_t* pc = c.n_clouds ? c.pcloud.p : nullptr;
    const uint32_t* nc = c.n_clouds ? c.ncloud.p : nullptr;
    // A second pass has work only if something can defer a point: a finite
    // first-pass factor or the warp search's defer list.  Otherwise it is
    // left out of the round.
    const bool two_passes = c.cnns_warp || !std::isinf(c.first_pass_factor);
    for (int pass = 1; pass <= (two_passes ? 2 : 1); ++pass) {
        const uint32_t* list = pass == 1 ? c.dirty.p : c.dirty2.p;
        const uint32_t* cnt = pass == 1 ? &d->n_dirty : &d->n_dirty2;
        if (c.cnns_warp) {
            if (c.dim == 2)
                k_cnns<2, WPB><<<blocks, WPB * 32, 0, c.stream>>>(
                    c.sp.p, c.nlo.p, c.nhi.p, c.nlab.p, (uint32_t)c.n, (uint32_t)c.L, list, cnt, c.lab.p, c.ckey.p,
                    c.selq.p, c.selkey.p, c.prov.p, &d->n_prov, c.lbp.p, c.clb.p, pass, c.dirty2.p, &d->n_dirty2,
                    st);
            else
                k_cnns<3, WPB><<<blocks, WPB * 32, 0, c.stream>>>(
                    c.sp.p, c.nlo.p, c.nhi.p, c.nlab.p, (uint32_t)c.n, (uint32_t)c.L, list, cnt, c.lab.p, c.ckey.p,
                    c.selq.p, c.selkey.p, c.prov.p, &d->n_prov, c.lbp.p, c.clb.p, pass, c.dirty2.p, &d->n_dirty2,
                    st);
        } else {
            CnnsArgs a{c.sp.p,   c.perm.p, c.nlo.p,   c.nhi.p, c.nlab.p, (uint32_t)c.n, (uint32_t)c.L, list,
                       cnt,      c.lab.p,  c.ckey.p,  c.selq.p, c.selkey.p, c.prov.p, &d->n_prov,  c.lbp.p,
                       c.clb.p,  pass,     c.dflag.p, pc,      nc,        st,       c.pfrag.p, c.margin,
                       c.threshold, &d->round,   nullptr,  nullptr,   knn};
            a.wide_limit = 0u;
            a.coop_min = kNoCoop;
            switch (c.search_split) {
            case 0: a.wide_limit = c.wide_limit; a.coop_min = c.coop_min; break;
            case 1: a.wide_limit = 0xffffffffu; break;
            case 2: a.coop_min = 0u; break;
            default: break;
            }
            const bool ordered = c.first_pass_ordered;
            if (ordered) {  // both segments in this one launch; no second pass
                if (pass == 2) continue;
                a.list2 = c.dirty2.p;
                a.n_list2 = &d->n_dirty2;
            }
            const int shape = search_shape_of(c);
            a.knn_k = c.knn_k;
            a.cmax = c.cmax.p;
            if (knn && pass == 1) {  // round 1 only (decided on the device)
                // the learned proposal steers the list build's starting bound
                // (single clouds); traces record the plain build
                const bool learned = c.learned && !pc && c.knn_k == kKnn;
                if (c.trace_cap > 0 && !learned && !pc && c.knn_k == kKnn) {
                    a.trace = c.trace.p;
                    a.trace_ctl = c.trace_ctl.p;
                    a.trace_cap = (uint64_t)c.trace_cap;
                    a.trace_mask = (1u << c.trace_shift) - 1u;
                }
                // host-driven rounds (profile mode) know the round: time the working launch
                const bool timed = c.kernel_timer && c.round == 1;
                if (timed) c.kernel_timer(c.timer_owner, 0, true);
                cudaError_t ek = c.dim == 2 ? launch_knn_first2(a, pc != nullptr, learned, c.klist.p, c.kcur.p,
                                                                c.iperm.p, c.sms, c.stream)
                                            : launch_knn_first3(a, pc != nullptr, learned, c.klist.p, c.kcur.p,
                                                                c.iperm.p, c.sms, c.stream);
                a.trace = nullptr;
                if (ek != cudaSuccess) return ek;
                if (timed) {
                    c.kernel_timer(c.timer_owner, 0, false);
                    c.knn_timed++;
                }
                c.launches++;
            }
            // the component search has no work in round 1 when the lists ran
            const bool timed = c.kernel_timer && !(knn && c.round == 1);
            if (timed) c.kernel_timer(c.timer_owner, 1, true);
            cudaError_t e1 = c.dim == 2 ? launch_cnns_t2(a, pc != nullptr, shape, c.sms, c.stream)
                                        : launch_cnns_t3(a, pc != nullptr, shape, c.sms, c.stream);
            if (e1 != cudaSuccess) return e1;
            if (a.wide_limit > 0) c.launches++;         // k_cnns_w beside k_cnns_t
            if (a.coop_min != kNoCoop) c.launches++;  // k_cnns_c beside them
            if (timed) {
                c.kernel_timer(c.timer_owner, 1, false);
                c.search_timed++;
            }
            if (pass == 1 && !ordered && two_passes) {
                cudaError_t e2 = select_list(c, 1, INFINITY, c.dirty2.p, &d->n_dirty2, nullptr, nullptr, nullptr);
                if (e2 != cudaSuccess) return e2;
            }
        }
        c.nns_launches++;
        c.launches++;
    }
    return cudaGetLastError();
}

}  // namespace emst
