// cnns_search.cuh -- the component search kernels, shared by the
// per-dimension translation units that instantiate them (cnns_t2.cu,
// cnns_t3.cu): per searching point, its nearest point outside its component
// under (d2, input id), folded into the component's key.  Together they take
// the place of the reference's per-round search, the static region table
// (K_computeOctants, NodeEMST.h:1018-1296) read by K_findNextClosestPoint
// (NodeEMST.h:1303-1384), with the same per-component result (cnns.cu).
//   k_knn_first  round 1: every point's kKnn nearest, warp per 32 queries
//                (the learned proposal steers its starting bound)
//   k_cnns_w     later rounds, short query lists: warp per query
//   k_cnns_t     later rounds, middle lists: thread per query (every launch
//                shape of the table)
//   k_cnns_c     later rounds, long lists: warp per 32 queries walking together
#pragma once
#include <cfloat>
#include <climits>

#include "emst_ctx.h"
#include "emst_device.cuh"
#include "proposal.cuh"

namespace emst {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr uint32_t kMixed = 0xffffffffu;
constexpr uint32_t kEmpty = 0xfffffffeu;
constexpr uint32_t kNone = 0xffffffffu;

// Warp-aggregated append of `val` to list[] through counter *cnt.
__device__ __forceinline__ void warp_append(bool pred, uint32_t val, uint32_t* list, uint32_t* cnt)
{
    const unsigned act = __activemask();
    const unsigned m = __ballot_sync(act, pred);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(cnt, (uint32_t)__popc(m));
    base = __shfl_sync(act, base, leader);
    if (pred) list[base + __popc(m & ((1u << lane) - 1u))] = val;
}

// Training-trace sampling: a fixed hash of the point's leaf position.
__device__ __forceinline__ uint32_t knn_sample_hash(uint32_t me)
{
    uint32_t h = me * 0x9E3779B1u ^ 0x27d4eb2fu;
    h ^= h >> 15;
    h *= 0x2c1b3c6du;
    h ^= h >> 12;
    return h;
}

// One thread per dirty point, each with its own traversal order: its own
// leaf first, then a depth-first walk from the root pushing the nearer child
// last, so every query sees good bounds early (queries of later rounds are
// sparse, and one warp-wide order would serve only some of them).
// CL: batched clouds (pcloud / ncloud given); a candidate must share the
// query's cloud.
// TPB threads per block, at least MINB blocks resident per SM (the launch
// shape; kSearchShapes lists the instantiated pairs).
template <int D, bool CL, int TPB, int MINB>
__global__ void __launch_bounds__(TPB, MINB) k_cnns_t(const CnnsArgs a)
{
    const float4* __restrict__ sp = a.sp;
    const float4* __restrict__ nlo = a.nlo;
    const float4* __restrict__ nhi = a.nhi;
    const uint32_t* __restrict__ nlab = a.nlab;
    const uint32_t n = a.n, L = a.L;
    const uint32_t* __restrict__ list = a.list;
    const uint32_t* __restrict__ n_list = a.n_list;
    const uint32_t* __restrict__ lab = a.lab;
    uint64_t* __restrict__ ckey = a.ckey;
    uint32_t* __restrict__ selq = a.selq;
    uint64_t* __restrict__ selkey = a.selkey;
    uint32_t* __restrict__ prov = a.prov;
    uint32_t* __restrict__ n_prov = a.n_prov;
    float* __restrict__ lbp = a.lbp;
    const int pass = a.pass;
    unsigned char* __restrict__ dflag = a.dflag;
    const uint32_t* __restrict__ pcloud = a.pcloud;
    const uint32_t* __restrict__ ncloud = a.ncloud;
    unsigned long long* __restrict__ stats = a.stats;
    constexpr int kTStack = 48;
    if (a.knn_round1 && *a.round == 1) return;  // round 1 is k_knn_first's
    // the queries: list, then (one launch, second segment) list2
    const uint32_t n1 = *n_list;
    const uint32_t total = n1 + (a.list2 ? *a.n_list2 : 0u);
    if (total <= a.wide_limit) return;  // a short list: k_cnns_w's (warp per query)
    if (total > a.coop_min) return;     // a long list: k_cnns_c's (warp per 32 queries, walking together)
    for (uint32_t base0 = blockIdx.x * blockDim.x; base0 < total; base0 += gridDim.x * blockDim.x) {
        const uint32_t qi = base0 + threadIdx.x;
        const bool listed = qi < total;
        const uint32_t me = listed ? (qi < n1 ? list[qi] : a.list2[qi - n1]) : 0u;
        const uint32_t labp = listed ? lab[me] : kEmpty;
        const float lb0 = listed ? lbp[me] : 0.f;
        bool valid = listed;
        float cb = INFINITY;
        if (listed) {
            const uint64_t k = __ldcg(&ckey[labp]);
            cb = k == kNoKey ? INFINITY : __uint_as_float((uint32_t)(k >> 32));
            if (lb0 > cb) valid = false;  // cannot hold its component's minimum this round
        }

        bool record = false;
        uint32_t st_leaves = 0, st_nodes = 0, st_cands = 0;
        if (valid) {
            const float4 P = sp[me];
            const int op = __float_as_int(P.w);
            const uint32_t qc = CL ? __ldg(&pcloud[me]) : 0u;  // the query's cloud (batches)
            float bd = INFINITY, cut = INFINITY;
            int bo = INT_MAX;  // input id of the best
            int bs = -1;       // leaf position of the best

            // sp holds (x, y, z, input id bits); the component labels are
            // read beside it from lab
            auto scan_leaf = [&](uint32_t leaf) {
                const uint32_t b = leaf * 32;
                if (b >= n) return;  // padding leaf (never reached: its bound is +inf)
                const uint32_t m = min(32u, n - b);
                ++st_leaves;
                st_cands += m;
                // a leaf straddling clouds: check every candidate's cloud
                bool mixed = false;
                if constexpr (CL) {
                    const uint32_t r = __ldg(&ncloud[L + leaf]);
                    mixed = (r >> 16) != (r & 0xffffu);
                }
                for (uint32_t j = 0; j < m; j += 4) {
                    float4 c[4];
                    uint32_t cl[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        c[k] = j + k < m ? __ldg(&sp[b + j + k]) : make_float4(0.f, 0.f, 0.f, 0.f);
                        cl[k] = j + k < m ? __ldg(&lab[b + j + k]) : labp;
                    }
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        if (cl[k] == labp) continue;
                        if (CL && mixed && j + k < m && __ldg(&pcloud[b + j + k]) != qc) continue;
                        const float d2 =
                            d2_of<D>(__fsub_rn(c[k].x, P.x), __fsub_rn(c[k].y, P.y), __fsub_rn(c[k].z, P.z));
                        const int oq = __float_as_int(c[k].w);
                        if (d2 < bd || (d2 == bd && oq < bo)) {
                            bd = d2;
                            bo = oq;
                            bs = (int)(b + j + k);
                        }
                    }
                }
            };
            // lower bound of d2 over a node's box, or +inf when the node cannot
            // help (empty, all in the query's component, all in another cloud);
            // +inf is tested explicitly: best and shared bound may be +inf too
            auto node_lb = [&](uint32_t node) -> float {
                const float4 lo = __ldg(&nlo[node]), hi = __ldg(&nhi[node]);
                if (lo.x > hi.x) return INFINITY;
                if (__ldg(&nlab[node]) == labp) return INFINITY;  // all in the query's component
                if constexpr (CL) {
                    // (first cloud << 16) | last cloud of the node's points
                    const uint32_t r = __ldg(&ncloud[node]);
                    if (qc < (r >> 16) || qc > (r & 0xffffu)) return INFINITY;  // all in other clouds
                }
                const float gx = fmaxf(fmaxf(__fsub_rn(lo.x, P.x), __fsub_rn(P.x, hi.x)), 0.f);
                const float gy = fmaxf(fmaxf(__fsub_rn(lo.y, P.y), __fsub_rn(P.y, hi.y)), 0.f);
                const float gz = D == 3 ? fmaxf(fmaxf(__fsub_rn(lo.z, P.z), __fsub_rn(P.z, hi.z)), 0.f) : 0.f;
                return d2_of<D>(gx, gy, gz);
            };

            // Own leaf first, then bottom-up: the sibling subtree of each
            // ancestor, nearest levels first, each searched depth-first with
            // the nearer child next.  Sibling addresses are known up front,
            // so no descent from the root is needed.
            const uint32_t own = me >> 5;
            if (__ldg(&nlab[L + own]) != labp) scan_leaf(own);
            uint32_t stack[kTStack];
            for (uint32_t v = L + own; v > 1; v >>= 1) {
                const uint32_t sib = v ^ 1u;
                ++st_nodes;
                const float ls = node_lb(sib);
                if (!(ls < INFINITY)) continue;
                if (ls > fminf(bd, cb)) {
                    if (ls <= bd) cut = fminf(cut, ls);
                    continue;
                }
                int top = 0;
                stack[top++] = sib;
                while (top > 0) {
                    // Traverse until this lane holds a leaf to scan, then scan
                    // it together with the other lanes that hold one: leaf
                    // scans of different lanes run side by side instead of
                    // alternating with node expansions.
                    uint32_t leaf = kNone;
                    while (top > 0) {
                        const uint32_t node = stack[--top];
                        ++st_nodes;
                        if (node >= L) {
                            // bound re-checked: bd may have shrunk since the push
                            const float lb = node_lb(node);
                            if (!(lb < INFINITY) || lb > bd) continue;
                            if (lb > cb) {
                                cut = fminf(cut, lb);
                                continue;
                            }
                            leaf = node - L;
                            break;
                        }
                        const uint32_t c0 = 2 * node, c1 = c0 + 1;
                        const float l0 = node_lb(c0), l1 = node_lb(c1);
                        const float lim = fminf(bd, cb);
                        // push the farther child first so the nearer one is searched next
                        const bool near0 = l0 <= l1;
                        const uint32_t cn = near0 ? c0 : c1, cf = near0 ? c1 : c0;
                        const float ln = near0 ? l0 : l1, lf = near0 ? l1 : l0;
                        if (top + 2 > kTStack) {  // cannot happen for trees of depth < 46
                            top = 0;
                            break;
                        }
                        if (lf < INFINITY && lf <= lim) stack[top++] = cf;
                        else if (lf <= bd && lf < INFINITY) cut = fminf(cut, lf);
                        if (ln < INFINITY && ln <= lim) stack[top++] = cn;
                        else if (ln <= bd && ln < INFINITY) cut = fminf(cut, ln);
                    }
                    if (leaf != kNone) {
                        scan_leaf(leaf);
                        const uint64_t k = __ldcg(&ckey[labp]);
                        cb = k == kNoKey ? INFINITY : __uint_as_float((uint32_t)(k >> 32));
                    }
                }
            }
            const bool exact = bs >= 0 && bd < cut;
            lbp[me] = exact ? bd : fmaxf(lb0, fminf(cut, bd));
            if (bs >= 0) {
                const uint32_t mn = (uint32_t)min(op, bo);
                const uint64_t key = ((uint64_t)__float_as_uint(bd) << 32) | mn;
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
        // Reconverge the warp before its next 32 queries: without this the
        // lanes of a diverged warp drift into different iterations and the
        // next traversals run with a fraction of the warp active.
        __syncwarp();
        if (listed && pass == 1) dflag[me] = 0;
        warp_append(record, me, prov, n_prov);
        if (stats) {
            unsigned long long sl = st_leaves, sn = st_nodes, sc = st_cands, q = valid ? 1ull : 0ull;
            for (int o = 16; o > 0; o >>= 1) {
                sl += __shfl_xor_sync(kFull, sl, o);
                sn += __shfl_xor_sync(kFull, sn, o);
                sc += __shfl_xor_sync(kFull, sc, o);
                q += __shfl_xor_sync(kFull, q, o);
            }
            const unsigned first = __ballot_sync(kFull, valid && pass == 1);
            if ((threadIdx.x & 31) == 0) {
                atomicAdd(&stats[0], sl);
                atomicAdd(&stats[1], sn);
                atomicAdd(&stats[2], sc);
                atomicAdd(&stats[3], 1ull);
                atomicAdd(&stats[4], q);
                atomicAdd(&stats[5], (unsigned long long)__popc(first));
            }
        }
    }
}

// Component search for short query lists: one warp per query.
//
// With few searching points (rounds after the neighbour lists settled most of
// them) thread-per-query warps are too few to fill the GPU and each runs 32
// divergent traversals of dependent loads: the round waits on the slowest
// warp.  Here a query owns a warp.  Its traversal is k_cnns_t's (own leaf,
// then the sibling subtree of each ancestor, same bounds and pruning: the
// query's best, its component's shared key, the per-node component labels and
// cloud ranges), but each step tests 32 nodes at once -- the descendants
// kWideFan levels below the popped node, one per lane -- and a leaf is scanned
// 32 points at a time, the (d2, input id) minimum taken across the warp.
// Leaves of a step are scanned nearest first, each re-tested against the
// bounds; internal descendants are pushed with the nearest on top.  The
// result, lower bound and provisional-winner record are k_cnns_t's.
template <int D, bool CL>
__global__ void __launch_bounds__(kWideWarps * 32) k_cnns_w(const CnnsArgs a)
{
    if (a.knn_round1 && *a.round == 1) return;  // round 1 is k_knn_first's
    const uint32_t n1 = *a.n_list;
    const uint32_t total = n1 + (a.list2 ? *a.n_list2 : 0u);
    if (total > a.wide_limit) return;  // a long list: k_cnns_t's
    const float4* __restrict__ sp = a.sp;
    const uint32_t* __restrict__ lab = a.lab;
    const float4* __restrict__ nlo = a.nlo;
    const float4* __restrict__ nhi = a.nhi;
    const uint32_t* __restrict__ nlab = a.nlab;
    const uint32_t n = a.n, L = a.L;
    const uint32_t* __restrict__ pcloud = a.pcloud;
    const uint32_t* __restrict__ ncloud = a.ncloud;
    uint64_t* __restrict__ ckey = a.ckey;
    // stack: each step pushes at most 2^kWideFan entries and each node on the
    // current path (at most ceil(27 / kWideFan) steps below a sibling root for
    // 32-bit point counts) leaves at most 2^kWideFan - 1 unpopped
    constexpr int kWStack = 256;
    static_assert((27 + kWideFan - 1) / kWideFan * ((1 << kWideFan) - 1) + 1 <= kWStack, "traversal stack bound");
    __shared__ uint32_t s_node[kWideWarps][kWStack];
    __shared__ float s_lb[kWideWarps][kWStack];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t* const stack = s_node[w];
    float* const stack_lb = s_lb[w];
    const uint32_t below = (1u << lane) - 1u;
    const int leaf_level = 31 - __clz(L);  // L is a power of two; node v sits on level 31 - clz(v)
    for (uint32_t qi = blockIdx.x * kWideWarps + w; qi < total; qi += gridDim.x * kWideWarps) {
        const uint32_t me = qi < n1 ? a.list[qi] : a.list2[qi - n1];
        const uint32_t labp = a.lab[me];
        const float lb0 = a.lbp[me];
        float cb;
        // other warps lower the key meanwhile: one lane reads it, every lane
        // takes that value, so the warp's decisions stay uniform
        auto refresh_cb = [&]() {
            uint64_t k = lane == 0 ? __ldcg(&ckey[labp]) : 0ull;
            k = __shfl_sync(kFull, k, 0);
            cb = k == kNoKey ? INFINITY : __uint_as_float((uint32_t)(k >> 32));
        };
        refresh_cb();
        const bool valid = !(lb0 > cb);  // else it cannot hold its component's minimum this round
        uint32_t st_leaves = 0, st_nodes = 0;
        bool record = false;
        if (valid) {
            const float4 P = sp[me];
            const uint32_t op = __float_as_uint(P.w);
            const uint32_t qc = CL ? __ldg(&pcloud[me]) : 0u;
            float bd = INFINITY, cut = INFINITY;
            uint64_t bkey = ~0ull;  // best: d2 bits << 32 | input id
            uint32_t bs = kNone;     // its leaf position
            // lower bound of d2 over a node's box, or +inf when the node
            // cannot help (empty, all in the query's component, all in
            // another cloud)
            auto node_lb = [&](uint32_t node) -> float {
                const float4 lo = __ldg(&nlo[node]), hi = __ldg(&nhi[node]);
                if (lo.x > hi.x) return INFINITY;
                if (__ldg(&nlab[node]) == labp) return INFINITY;
                if constexpr (CL) {
                    const uint32_t r = __ldg(&ncloud[node]);
                    if (qc < (r >> 16) || qc > (r & 0xffffu)) return INFINITY;
                }
                const float gx = fmaxf(fmaxf(__fsub_rn(lo.x, P.x), __fsub_rn(P.x, hi.x)), 0.f);
                const float gy = fmaxf(fmaxf(__fsub_rn(lo.y, P.y), __fsub_rn(P.y, hi.y)), 0.f);
                const float gz = D == 3 ? fmaxf(fmaxf(__fsub_rn(lo.z, P.z), __fsub_rn(P.z, hi.z)), 0.f) : 0.f;
                return d2_of<D>(gx, gy, gz);
            };
            // one leaf, one point per lane; the (d2, input id) minimum across the warp
            auto scan_leaf = [&](uint32_t leaf) {
                const uint32_t b = leaf * 32;
                const uint32_t m = min(32u, n - b);
                ++st_leaves;
                uint32_t kd = ~0u, ki = ~0u;
                if ((uint32_t)lane < m) {
                    const float4 c = __ldg(&sp[b + lane]);
                    bool ok = __ldg(&lab[b + lane]) != labp;
                    if constexpr (CL) ok = ok && __ldg(&pcloud[b + lane]) == qc;
                    if (ok) {
                        kd = __float_as_uint(
                            d2_of<D>(__fsub_rn(c.x, P.x), __fsub_rn(c.y, P.y), __fsub_rn(c.z, P.z)));
                        ki = __float_as_uint(c.w);
                    }
                }
                // non-negative floats order as their bits
                const uint32_t md = __reduce_min_sync(kFull, kd);
                const uint32_t mi = __reduce_min_sync(kFull, kd == md ? ki : ~0u);
                const uint64_t mk = ((uint64_t)md << 32) | mi;
                if (mk < bkey) {
                    const uint32_t src = __ffs(__ballot_sync(kFull, kd == md && ki == mi)) - 1;
                    bkey = mk;
                    bd = __uint_as_float(md);
                    bs = b + src;
                }
                refresh_cb();
            };

            const uint32_t own = me >> 5;
            if (__ldg(&nlab[L + own]) != labp) scan_leaf(own);
            for (uint32_t v = L + own; v > 1; v >>= 1) {
                const uint32_t sib = v ^ 1u;
                ++st_nodes;
                const float ls = node_lb(sib);
                if (!(ls < INFINITY) || ls > bd) continue;
                if (ls > cb) {  // ruled out by the component's key only: bounds this point's distance
                    cut = fminf(cut, ls);
                    continue;
                }
                __syncwarp();
                if (lane == 0) {
                    stack[0] = sib;
                    stack_lb[0] = ls;
                }
                int top = 1;
                __syncwarp();
                while (top > 0) {
                    --top;
                    const uint32_t node = stack[top];
                    const float lnode = stack_lb[top];
                    // bounds re-checked: they may have shrunk since the push
                    if (lnode > bd) continue;
                    if (lnode > cb) {
                        cut = fminf(cut, lnode);
                        continue;
                    }
                    const int lev = leaf_level - (31 - __clz(node));  // levels down to the leaves
                    const int e = min(lev, kWideFan);
                    const uint32_t cnt = 1u << e;
                    const uint32_t d = (node << e) + (uint32_t)lane;
                    const float lb = (uint32_t)lane < cnt ? node_lb(d) : INFINITY;
                    st_nodes += cnt;
                    {
                        // descendants only the component's key rules out bound the distance
                        const float lim = fminf(bd, cb);
                        const bool cutc = lb < INFINITY && lb > lim && lb <= bd;
                        cut = fminf(cut, __uint_as_float(
                                             __reduce_min_sync(kFull, cutc ? __float_as_uint(lb) : 0x7f800000u)));
                    }
                    uint32_t want = __ballot_sync(kFull, lb < INFINITY && lb <= fminf(bd, cb));
                    if (e == lev) {
                        // leaves, nearest first, each against the current bounds
                        while (want) {
                            const uint32_t mlb =
                                __reduce_min_sync(kFull, (want >> lane & 1u) ? __float_as_uint(lb) : ~0u);
                            const int j =
                                __ffs(__ballot_sync(kFull, (want >> lane & 1u) && __float_as_uint(lb) == mlb)) - 1;
                            want &= ~(1u << j);
                            const float lj = __uint_as_float(mlb);
                            if (lj > bd) break;  // this and the rest: farther than the best
                            if (lj > cb) {       // this and the rest: ruled out by the component's key only
                                cut = fminf(cut, lj);
                                break;
                            }
                            scan_leaf((node << e) + (uint32_t)j - L);
                        }
                    } else if (want) {
                        // internal descendants: the nearest pushed last, searched next
                        const uint32_t mlb = __reduce_min_sync(kFull, (want >> lane & 1u) ? __float_as_uint(lb) : ~0u);
                        const int jn =
                            __ffs(__ballot_sync(kFull, (want >> lane & 1u) && __float_as_uint(lb) == mlb)) - 1;
                        const uint32_t rest = want & ~(1u << jn);
                        const int nr = __popc(rest);
                        if (top + nr + 1 > kWStack) break;  // unreachable: see kWStack
                        __syncwarp();  // every lane has read the popped entry
                        if (rest >> lane & 1u) {
                            const int at = top + __popc(rest & below);
                            stack[at] = d;
                            stack_lb[at] = lb;
                        }
                        if (lane == jn) {
                            stack[top + nr] = d;
                            stack_lb[top + nr] = lb;
                        }
                        top += nr + 1;
                        __syncwarp();
                    }
                }
            }
            const bool exact = bs != kNone && bd < cut;
            if (lane == 0) {
                a.lbp[me] = exact ? bd : fmaxf(lb0, fminf(cut, bd));
                if (bs != kNone) {
                    const uint32_t mn = min(op, (uint32_t)bkey);
                    const uint64_t key = (bkey & 0xffffffff00000000ull) | mn;
                    a.selq[me] = exact ? bs : kNone;
                    a.selkey[me] = key;
                    if (key <= __ldcg(&ckey[labp])) {
                        const uint64_t old = atomicMin((unsigned long long*)&ckey[labp], (unsigned long long)key);
                        record = old >= key;
                    }
                } else {
                    a.selq[me] = kNone;
                }
            }
        }
        if (lane == 0) {
            if (a.pass == 1) a.dflag[me] = 0;
            if (record) a.prov[atomicAdd(a.n_prov, 1u)] = me;
            if (a.stats) {
                atomicAdd(&a.stats[0], (unsigned long long)st_leaves);
                atomicAdd(&a.stats[1], (unsigned long long)st_nodes);
                atomicAdd(&a.stats[2], (unsigned long long)st_leaves * 32ull);
                atomicAdd(&a.stats[3], 1ull);
                atomicAdd(&a.stats[4], valid ? 1ull : 0ull);
                atomicAdd(&a.stats[5], valid && a.pass == 1 ? 1ull : 0ull);
            }
        }
        __syncwarp();
    }
}

// Gathers of k_cnns_c and k_knn_first: nodes the frontier may hold, leaves a
// gather may collect.
constexpr int kWideFront = 128;
constexpr int kWideLeaves = 64;

// Ascending bitonic sort of 32 keys, one per lane.
__device__ __forceinline__ uint32_t bitonic_sort32(uint32_t v, int lane)
{
#pragma unroll 1
    for (int k = 2; k <= 32; k <<= 1)
#pragma unroll 1
        for (int j = k >> 1; j > 0; j >>= 1) {
            const uint32_t o = __shfl_xor_sync(kFull, v, j);
            const bool keep_min = ((lane & j) == 0) == ((lane & k) == 0);
            v = keep_min ? min(v, o) : max(v, o);
        }
    return v;
}

// Ascending bitonic sort of 64 keys: element e is v0 of lane e (e < 32) or
// v1 of lane e - 32.
__device__ __forceinline__ void bitonic_sort64(uint32_t& v0, uint32_t& v1, int lane)
{
#pragma unroll 1
    for (int k = 2; k <= 64; k <<= 1)
#pragma unroll 1
        for (int j = k >> 1; j > 0; j >>= 1) {
            if (j == 32) {  // k == 64: the halves of each lane, ascending
                const uint32_t lo = min(v0, v1), hi = max(v0, v1);
                v0 = lo;
                v1 = hi;
            } else {
                const uint32_t o0 = __shfl_xor_sync(kFull, v0, j), o1 = __shfl_xor_sync(kFull, v1, j);
                const bool lower = (lane & j) == 0;
                // e & k for e = lane and e = lane + 32 (they differ only for k == 32)
                const bool up0 = (lane & k) == 0, up1 = ((lane + 32) & k) == 0;
                v0 = lower == up0 ? min(v0, o0) : max(v0, o0);
                v1 = lower == up1 ? min(v1, o1) : max(v1, o1);
            }
        }
}

// Component search for long query lists: one warp per 32 consecutive
// queries, walking the tree together (k_knn_first's traversal), each lane
// keeping its own nearest point outside its component.
//
// In late rounds most points of most leaves search, so a warp's 32 queries
// are a leaf's points, in one component, and their bottom-up walks visit the
// same nodes; thread per query runs those walks as 32 divergent copies.  Per
// lane this is k_cnns_t's search: the bound is the lane's best and its
// component's key, nodes holding only its component or only other clouds are
// skipped, and nodes only the component's key rules out bound its distance
// from below (cut).  A node is entered when any lane wants it, so a lane may
// test points beyond its bound: those only lower its best to a real
// candidate, never past its true nearest.  A lane adds a node's bound to its
// cut whenever the key rules the node out for it, even if the warp enters the
// node for another lane: cut stays a lower bound of every point it skipped,
// so a result it calls exact is exact.
template <int D, bool CL>
__global__ void __launch_bounds__(kKnnWarps * 32, 4) k_cnns_c(const CnnsArgs a)
{
    if (a.knn_round1 && *a.round == 1) return;  // round 1 is k_knn_first's
    const uint32_t n1 = *a.n_list;
    const uint32_t total = n1 + (a.list2 ? *a.n_list2 : 0u);
    if (total <= a.wide_limit || total <= a.coop_min) return;  // shorter lists: k_cnns_w, k_cnns_t
    const float4* __restrict__ sp = a.sp;
    const uint32_t* __restrict__ lab = a.lab;
    const float4* __restrict__ nlo = a.nlo;
    const float4* __restrict__ nhi = a.nhi;
    const uint32_t* __restrict__ nlab = a.nlab;
    const uint32_t n = a.n, L = a.L;
    const uint32_t* __restrict__ pcloud = a.pcloud;
    const uint32_t* __restrict__ ncloud = a.ncloud;
    uint64_t* __restrict__ ckey = a.ckey;
    constexpr int kWStack = 64;  // a tree of 32-bit node ids is < 33 levels deep
    __shared__ float4 s_pt[kKnnWarps][32];
    // the staged leaf's coordinates again, one row per axis (packed d2)
    __shared__ __align__(16) float s_ax[kKnnWarps][D][32];
    __shared__ uint32_t s_lab[kKnnWarps][32];
    __shared__ uint32_t s_cl[kKnnWarps][CL ? 32 : 1];
    __shared__ uint32_t s_stack[kKnnWarps][kWStack];
    // the gather's frontier and its leaves' sort keys; none for point batches
    __shared__ uint32_t s_fr[kKnnWarps][CL ? 1 : kWideFront];
    __shared__ uint32_t s_lk[kKnnWarps][CL ? 1 : kWideLeaves];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4* const pt = s_pt[w];
    uint32_t* const labs = s_lab[w];
    uint32_t* const stack = s_stack[w];
    const uint32_t stride = gridDim.x * kKnnWarps * 32;
    // the list entry of the next iteration is loaded one iteration ahead
    auto entry = [&](uint32_t b) -> uint32_t {
        const uint32_t qi = b + lane;
        const uint32_t qs = qi < total ? qi : b;
        return qs < n1 ? a.list[qs] : a.list2[qs - n1];
    };
    uint32_t me_next = 0;
    if ((blockIdx.x * kKnnWarps + w) * 32 < total) me_next = entry((blockIdx.x * kKnnWarps + w) * 32);
    for (uint32_t base0 = (blockIdx.x * kKnnWarps + w) * 32; base0 < total; base0 += stride) {
        const uint32_t qi = base0 + lane;
        const bool listed = qi < total;
        const uint32_t me = me_next;
        if (base0 + stride < total) me_next = entry(base0 + stride);
        const uint32_t labp = listed ? a.lab[me] : kEmpty;
        const float lb0 = listed ? a.lbp[me] : 0.f;
        float cb = INFINITY;
        auto refresh_cb = [&]() {
            if (listed) {
                const uint64_t k = __ldcg(&ckey[labp]);
                cb = k == kNoKey ? INFINITY : __uint_as_float((uint32_t)(k >> 32));
            }
        };
        refresh_cb();
        const bool valid = listed && !(lb0 > cb);  // else it cannot hold its component's minimum this round
        const float4 P = sp[me];
        const uint32_t op = __float_as_uint(P.w);
        const uint32_t qc = CL ? __ldg(&pcloud[me]) : 0u;
        // best d2 so far (+inf: none); -1 for lanes with no search, so that
        // no node and no candidate is ever theirs
        float bd = valid ? INFINITY : -1.f;
        float cut = INFINITY;
        uint32_t bo = ~0u, bs = kNone;  // best's input id and leaf position
        uint32_t st_leaves = 0, st_nodes = 0;

        // this lane's lower bound of d2 over a node's box, or +inf when the
        // node cannot help it (empty, all in its component, all in other clouds)
        auto node_lb = [&](uint32_t node) -> float {
            const float4 lo = __ldg(&nlo[node]), hi = __ldg(&nhi[node]);
            if (__ldg(&nlab[node]) == labp) return INFINITY;
            if constexpr (CL) {
                const uint32_t r = __ldg(&ncloud[node]);
                if (qc < (r >> 16) || qc > (r & 0xffffu)) return INFINITY;
            }
            const float gx = fmaxf(fmaxf(__fsub_rn(lo.x, P.x), __fsub_rn(P.x, hi.x)), 0.f);
            const float gy = fmaxf(fmaxf(__fsub_rn(lo.y, P.y), __fsub_rn(P.y, hi.y)), 0.f);
            const float gz = D == 3 ? fmaxf(fmaxf(__fsub_rn(lo.z, P.z), __fsub_rn(P.z, hi.z)), 0.f) : 0.f;
            return d2_of<D>(gx, gy, gz);
        };
        auto wanted = [&](float lb) { return lb < INFINITY && lb <= fminf(bd, cb); };
        // a node the component's key (not the best) rules out bounds the distance
        auto note = [&](float lb) {
            if (lb < INFINITY && lb > fminf(bd, cb) && lb <= bd) cut = fminf(cut, lb);
        };
        // the whole warp scans one leaf for the lanes in `need` (as
        // k_knn_first: staged in shared memory; every lane tests all points
        // when many lanes want the leaf, else one ballot-free minimum per
        // wanting lane), each lane keeping its (d2, input id) minimum
        auto scan_leaf = [&](uint32_t leaf, uint32_t need) {
            const uint32_t b = leaf * 32;
            const uint32_t m = min(32u, n - b);
            ++st_leaves;
            __syncwarp();  // the previous leaf's reads are done
            if ((uint32_t)lane < m) {
                const float4 c = __ldg(&sp[b + lane]);
                pt[lane] = c;
                s_ax[w][0][lane] = c.x;
                s_ax[w][1][lane] = c.y;
                if constexpr (D == 3) s_ax[w][2][lane] = c.z;
                labs[lane] = __ldg(&lab[b + lane]);
                if constexpr (CL) s_cl[w][lane] = __ldg(&pcloud[b + lane]);
            } else {
                // past the last point: NaN coordinates fail every d2 <= bound
                // test, and so does the +inf of the rows (d2 = +inf)
                pt[lane] = make_float4(__int_as_float(0x7fffffff), 0.f, 0.f, __uint_as_float(~0u));
                s_ax[w][0][lane] = INFINITY;
                s_ax[w][1][lane] = 0.f;
                if constexpr (D == 3) s_ax[w][2][lane] = 0.f;
                labs[lane] = kEmpty;
                if constexpr (CL) s_cl[w][lane] = ~0u;
            }
            __syncwarp();
            if (__popc(need) > kKnnDense) {
                // two candidates' d2 per packed step (bit for bit d2_of),
                // then each in turn against the lane's best
#pragma unroll 4
                for (int h = 0; h < 16; ++h) {
                    const f32x2 cx = reinterpret_cast<const f32x2*>(s_ax[w][0])[h];
                    const f32x2 cy = reinterpret_cast<const f32x2*>(s_ax[w][1])[h];
                    const f32x2 cz = D == 3 ? reinterpret_cast<const f32x2*>(s_ax[w][D - 1])[h] : 0ull;
                    const f32x2 d2p =
                        d2_of2<D>(cx, cy, cz, f2_dup(P.x), f2_dup(P.y), f2_dup(D == 3 ? P.z : 0.f));
#pragma unroll
                    for (int u = 0; u < 2; ++u) {
                        const int j = 2 * h + u;
                        const float d2 = __uint_as_float(u ? (uint32_t)(d2p >> 32) : (uint32_t)d2p);
                        bool ok = d2 <= bd && labs[j] != labp;
                        if constexpr (CL) ok = ok && s_cl[w][j] == qc;
                        const uint32_t id = __float_as_uint(pt[j].w);
                        const bool better = ok && (d2 < bd || id < bo);  // (d2, id) order; ok has d2 <= bd
                        bd = better ? d2 : bd;
                        bo = better ? id : bo;
                        bs = better ? b + (uint32_t)j : bs;
                    }
                }
            } else {
                const float4 c = pt[lane];
                const uint32_t cid = __float_as_uint(c.w);
                const uint32_t clab = labs[lane];
                const uint32_t cc = CL ? s_cl[w][lane] : 0u;
                while (need) {
                    const int q = __ffs(need) - 1;
                    need &= need - 1u;
                    // every lane takes part in every shuffle and reduction
                    const float qx = __shfl_sync(kFull, P.x, q), qy = __shfl_sync(kFull, P.y, q);
                    const float qz = D == 3 ? __shfl_sync(kFull, P.z, q) : 0.f;
                    const float qb = __shfl_sync(kFull, bd, q);
                    const uint32_t ql = __shfl_sync(kFull, labp, q);
                    const uint32_t qq = CL ? __shfl_sync(kFull, qc, q) : 0u;
                    const float d2 = d2_of<D>(__fsub_rn(c.x, qx), __fsub_rn(c.y, qy), __fsub_rn(c.z, qz));
                    bool ok = d2 <= qb && clab != ql;
                    if constexpr (CL) ok = ok && cc == qq;
                    const uint32_t kd = ok ? __float_as_uint(d2) : ~0u;  // non-negative floats order as bits
                    const uint32_t md = __reduce_min_sync(kFull, kd);
                    const uint32_t mi = __reduce_min_sync(kFull, kd == md ? cid : ~0u);
                    const uint32_t src = __ffs(__ballot_sync(kFull, kd == md && cid == mi)) - 1;
                    if (lane == q && md != ~0u) {
                        const float d = __uint_as_float(md);
                        if (d < bd || mi < bo) {
                            bd = d;
                            bo = mi;
                            bs = b + src;
                        }
                    }
                }
            }
            refresh_cb();
        };

        // Leaves come from a warp-uniform state machine, so that every one
        // goes through the single scan below.  Default: the warp's own leaf
        // (lane 0's query's) first, then bottom-up -- every other leaf lies in
        // exactly one sibling subtree of its ancestors -- a node entered when
        // any lane wants it.
        //
        // Single-component warps (in late rounds most warps: 32 points of one
        // big component) gather first, as k_knn_first does: the own leaf and
        // the ancestors' siblings are tested one per lane in one step, then 32
        // nodes a step, against the queries' box grown by B (the largest
        // bound of any lane; here every lane's bound is its component's key)
        // and the shared label (a node holding only the component is
        // skipped).  The box-to-box bound never exceeds a lane's node_lb, so
        // nothing a lane wants is dropped, and a node it drops is beyond every
        // lane's key: its bound joins every lane's cut.  Often nothing is
        // gathered at all: a point deep inside its component learns in one
        // step that no outside point is nearer than the key, where the
        // depth-first walk tests the ancestors' siblings one by one.
        // Gathered leaves are scanned nearest first.  A frontier or leaf list
        // that overflows falls back to the depth-first walk.
        const uint32_t own = __shfl_sync(kFull, me, 0) >> 5;
        enum { kOwn, kGathered, kWalk, kDone };
        int phase = kOwn;
        int li = 0, nl = 0;
        uint32_t v0 = ~0u, v1 = ~0u;  // the gathered leaves' sorted keys
        const unsigned vmask = __ballot_sync(kFull, valid);
        if (!vmask) phase = kDone;  // no lane can hold its component's minimum
        if constexpr (!CL) {
            const uint32_t lab0 = __shfl_sync(kFull, labp, vmask ? __ffs(vmask) - 1 : 0);
            // rescaled coordinates are >= +0: their bits order as the values
            const uint32_t sx = __float_as_uint(P.x), sy = __float_as_uint(P.y), sz = __float_as_uint(P.z);
            const bool neg = ((sx | sy | sz) >> 31) != 0u;
            const float B = __uint_as_float(__reduce_max_sync(kFull, __float_as_uint(fmaxf(fminf(bd, cb), 0.f))));
            if (vmask && B < INFINITY && __all_sync(kFull, !valid || (labp == lab0 && !neg))) {
                float4 qlo, qhi;
                qlo.x = __uint_as_float(__reduce_min_sync(kFull, valid ? sx : 0x7f800000u));
                qlo.y = __uint_as_float(__reduce_min_sync(kFull, valid ? sy : 0x7f800000u));
                qlo.z = __uint_as_float(__reduce_min_sync(kFull, valid ? sz : 0x7f800000u));
                qhi.x = __uint_as_float(__reduce_max_sync(kFull, valid ? sx : 0u));
                qhi.y = __uint_as_float(__reduce_max_sync(kFull, valid ? sy : 0u));
                qhi.z = __uint_as_float(__reduce_max_sync(kFull, valid ? sz : 0u));
                uint32_t* const fr = s_fr[w];
                uint32_t* const lk = s_lk[w];
                const unsigned below = (1u << lane) - 1u;
                const int depth = 31 - __clz(L);  // levels under the root (L is a power of two)
                __syncwarp();
                if (lane < depth) fr[lane] = ((L + own) >> lane) ^ 1u;
                if (lane == depth) fr[lane] = L + own;
                __syncwarp();
                int top = depth + 1;
                float dropped = INFINITY;  // smallest bound of a node dropped by distance (this lane's tests)
                bool ok = true;
                while (top > 0) {
                    const int take = min(top, 32);
                    top -= take;
                    ++st_nodes;
                    uint32_t node = 0;
                    float lb = INFINITY;
                    if (lane < take) {
                        // label and box loaded together (one wait per step,
                        // not two); a node holding only the component is
                        // skipped
                        node = fr[top + lane];
                        const uint32_t nlb = __ldg(&nlab[node]);
                        const float4 lo = __ldg(&nlo[node]), hi = __ldg(&nhi[node]);
                        const float gx = fmaxf(fmaxf(__fsub_rn(lo.x, qhi.x), __fsub_rn(qlo.x, hi.x)), 0.f);
                        const float gy = fmaxf(fmaxf(__fsub_rn(lo.y, qhi.y), __fsub_rn(qlo.y, hi.y)), 0.f);
                        const float gz =
                            D == 3 ? fmaxf(fmaxf(__fsub_rn(lo.z, qhi.z), __fsub_rn(qlo.z, hi.z)), 0.f) : 0.f;
                        lb = nlb != lab0 ? d2_of<D>(gx, gy, gz) : INFINITY;
                    }
                    const bool want = lb <= B, is_leaf = node >= L;
                    if (!want) dropped = fminf(dropped, lb);  // +inf: empty or the component's own
                    const unsigned ml = __ballot_sync(kFull, want && is_leaf);
                    const unsigned mi = __ballot_sync(kFull, want && !is_leaf);
                    const int nlf = __popc(ml), nin = __popc(mi);
                    if (nl + nlf > kWideLeaves || top + 2 * nin > kWideFront) {
                        ok = false;
                        break;
                    }
                    __syncwarp();  // every lane has read its entry: the pushes may overwrite it
                    if (want && is_leaf) {
                        const int e = nl + __popc(ml & below);
                        stack[e] = node - L;
                        lk[e] = (__float_as_uint(lb) & ~(uint32_t)(kWideLeaves - 1)) | (uint32_t)e;
                    }
                    if (want && !is_leaf) {
                        const int e = top + 2 * __popc(mi & below);
                        fr[e] = 2u * node;
                        fr[e + 1] = 2u * node + 1u;
                    }
                    nl += nlf;
                    top += 2 * nin;
                    __syncwarp();
                }
                if (ok) {
                    // every lane's cut takes the nodes dropped by distance
                    const float dmin = __uint_as_float(__reduce_min_sync(kFull, __float_as_uint(dropped)));
                    if (valid) cut = fminf(cut, dmin);
                    v0 = lane < nl ? lk[lane] : ~0u;
                    v1 = lane + 32 < nl ? lk[lane + 32] : ~0u;
                    if (nl > 32) bitonic_sort64(v0, v1, lane);
                    else if (nl > 1) v0 = bitonic_sort32(v0, lane);
                    phase = kGathered;
                } else {
                    nl = 0;
                }
            }
        }
        uint32_t dv = L + own;  // the walk: the ancestor whose sibling comes next
        int top = 0;            // the walk's stack depth
        while (phase != kDone) {
            uint32_t leaf = 0, need = 0;
            if (phase == kOwn) {
                const float lo = node_lb(L + own);
                note(lo);
                leaf = own;
                need = __ballot_sync(kFull, wanted(lo));
                phase = kWalk;
            } else if (phase == kGathered) {
                if (li >= nl) {
                    phase = kDone;
                    continue;
                }
                const uint32_t e = __shfl_sync(kFull, li < 32 ? v0 : v1, li & 31) & (uint32_t)(kWideLeaves - 1);
                ++li;
                leaf = stack[e];
                ++st_nodes;
                const float lb = node_lb(L + leaf);
                note(lb);
                need = __ballot_sync(kFull, wanted(lb));
            } else {
                // the walk, up to the next leaf some lane wants
                for (;;) {
                    if (top == 0) {
                        if (dv <= 1) {
                            phase = kDone;
                            break;
                        }
                        const uint32_t sib = dv ^ 1u;
                        dv >>= 1;
                        ++st_nodes;
                        const float ls = node_lb(sib);
                        note(ls);
                        if (!__any_sync(kFull, wanted(ls))) continue;
                        __syncwarp();
                        stack[0] = sib;
                        top = 1;
                        __syncwarp();
                    }
                    const uint32_t node = stack[--top];
                    ++st_nodes;
                    if (node >= L) {
                        // bounds re-checked: they may have shrunk since the push
                        const float lb = node_lb(node);
                        note(lb);
                        need = __ballot_sync(kFull, wanted(lb));
                        if (need) {
                            leaf = node - L;
                            break;
                        }
                        continue;
                    }
                    const uint32_t c0 = 2 * node, c1 = c0 + 1;
                    const float l0 = node_lb(c0), l1 = node_lb(c1);
                    note(l0);
                    note(l1);
                    const bool w0 = __any_sync(kFull, wanted(l0)), w1 = __any_sync(kFull, wanted(l1));
                    // the child nearer to the warp's nearest lane is searched next
                    const uint32_t m0 = __reduce_min_sync(kFull, __float_as_uint(l0));
                    const uint32_t m1 = __reduce_min_sync(kFull, __float_as_uint(l1));
                    const bool near0 = m0 <= m1;
                    const bool wn = near0 ? w0 : w1, wf = near0 ? w1 : w0;
                    __syncwarp();  // every lane has read the popped entry
                    if (wf) stack[top++] = near0 ? c1 : c0;
                    if (wn) stack[top++] = near0 ? c0 : c1;
                    __syncwarp();
                }
            }
            if (need) scan_leaf(leaf, need);
        }
        bool record = false;
        if (valid) {
            const bool exact = bs != kNone && bd < cut;
            a.lbp[me] = exact ? bd : fmaxf(lb0, fminf(cut, bd));
            if (bs != kNone) {
                const uint32_t mn = min(op, bo);
                const uint64_t key = ((uint64_t)__float_as_uint(bd) << 32) | mn;
                a.selq[me] = exact ? bs : kNone;
                a.selkey[me] = key;
                if (key <= __ldcg(&ckey[labp])) {
                    const uint64_t old = atomicMin((unsigned long long*)&ckey[labp], (unsigned long long)key);
                    record = old >= key;
                }
            } else {
                a.selq[me] = kNone;
            }
        }
        if (listed && a.pass == 1) a.dflag[me] = 0;
        __syncwarp();
        warp_append(record, me, a.prov, a.n_prov);
        if (a.stats) {
            const uint32_t q = __popc(__ballot_sync(kFull, valid));
            const uint32_t f = __popc(__ballot_sync(kFull, valid && a.pass == 1));
            if (lane == 0) {
                atomicAdd(&a.stats[0], (unsigned long long)st_leaves);
                atomicAdd(&a.stats[1], (unsigned long long)st_nodes * 2ull * q);
                atomicAdd(&a.stats[2], (unsigned long long)st_leaves * 32ull * q);
                atomicAdd(&a.stats[3], 1ull);
                atomicAdd(&a.stats[4], (unsigned long long)q);
                atomicAdd(&a.stats[5], (unsigned long long)f);
            }
        }
    }
}

// Round 1 with neighbour lists: each point's kKnn nearest other points (its
// component is itself), sorted by (d2, input id) and kept for later rounds:
// there, the first entry outside the point's component is its exact nearest
// outside point -- every closer point is earlier in the list -- so most
// points of rounds 2-4 need no search (k_reuse).  Entry 0 is the round-1
// result, written like k_cnns_t's.  Runs only when the device round is 1.
//
// One warp per 32 consecutive queries of the list (in round 1 the list is
// every point in leaf order, so a warp's queries are one leaf).  The warp
// walks the tree together: its queries' own leaf first, then the sibling
// subtree of each ancestor, a node entered when any lane's lower bound
// reaches it.  A leaf is staged once in shared memory and every lane tests
// all its points (broadcast reads), so all 32 lanes compute distances on
// every candidate instead of diverging over per-lane traversals.  Each leaf
// reaches every lane at most once, and a lane's bound only shrinks, so every
// lane still sees every point within its final K-th distance: the lists are
// the exact K nearest, as with one traversal per lane.  During the search a
// list holds only its (d2 bits, input id) keys; each entry's leaf position is
// read from iperm (input id -> position) once, when the list is written.
template <int D, bool CL, bool LEARN, int K>
__global__ void __launch_bounds__(kKnnWarps * 32, 4) k_knn_first(const CnnsArgs a, uint64_t* __restrict__ klist,
                                                                unsigned char* __restrict__ kcur,
                                                                const uint32_t* __restrict__ iperm)
{
    if (*a.round != 1) return;
    const float4* __restrict__ sp = a.sp;
    const float4* __restrict__ nlo = a.nlo;
    const float4* __restrict__ nhi = a.nhi;
    const uint32_t n = a.n, L = a.L;
    const uint32_t* __restrict__ pcloud = a.pcloud;
    const uint32_t* __restrict__ ncloud = a.ncloud;
    constexpr int kWStack = 64;  // a tree of 32-bit node ids is < 33 levels deep
    static_assert(kWideLeaves <= kWStack && kWideFront >= 32, "the wide walk's leaf list and frontier");
    __shared__ float4 s_pt[kKnnWarps][32];
    // the staged leaf's coordinates again, one row per axis, read two
    // candidates at a time by the packed marking (x of a missing point +inf)
    __shared__ __align__(16) float s_ax[kKnnWarps][D][32];
    __shared__ uint32_t s_cl[kKnnWarps][CL ? 32 : 1];
    __shared__ uint32_t s_stack[kKnnWarps][kWStack];
    // the wide walk's frontier, its leaves' sort keys and boxes (lo then hi
    // per axis); none for point batches
    __shared__ uint32_t s_fr[kKnnWarps][CL ? 1 : kWideFront];
    __shared__ uint32_t s_lk[kKnnWarps][CL ? 1 : kWideLeaves];
    __shared__ float s_bx[kKnnWarps][CL ? 1 : 2 * D][kWideLeaves];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float4* const pt = s_pt[w];
    uint32_t* const stack = s_stack[w];
    // round 1: every point, in leaf order (the reuse pass and the list
    // compaction leave round 1 to this kernel)
    const uint32_t total = n;
    const uint32_t stride = gridDim.x * kKnnWarps * 32;
    for (uint32_t base0 = (blockIdx.x * kKnnWarps + w) * 32; base0 < total; base0 += stride) {
        const uint32_t qi = base0 + lane;
        const bool listed = qi < total;
        const uint32_t me = listed ? qi : base0;
        const float4 P = sp[me];
        const uint32_t qc = CL ? __ldg(&pcloud[me]) : 0u;
        // the list: (d2 bits << 32 | input id), sorted; positions are looked
        // up from the ids once at the end
        uint64_t kk[K];
#pragma unroll
        for (int j = 0; j < K; ++j) kk[j] = kNoKey;
        // d2 of the K-th entry once the list is full, FLT_MAX before (every
        // finite bound and distance passes, an empty box's +inf does not);
        // lanes past the list's end take -1 so that no node and no candidate
        // is ever theirs
        float bd = listed ? FLT_MAX : -1.f;
        uint32_t st_leaves = 0, st_nodes = 0, st_marked = 0, st_steps = 0;

        // This lane's lower bound of d2 over a node's box.  An empty box
        // (lo = +inf, hi = -inf) gives +inf through the arithmetic.  Node
        // labels are not checked: in round 1 a node holding only the query's
        // component holds only the query, and scanning it finds no candidate.
        auto node_lb = [&](uint32_t node) -> float {
            const float4 lo = __ldg(&nlo[node]), hi = __ldg(&nhi[node]);
            if constexpr (CL) {
                const uint32_t r = __ldg(&ncloud[node]);
                if (qc < (r >> 16) || qc > (r & 0xffffu)) return INFINITY;
            }
            const float gx = fmaxf(fmaxf(__fsub_rn(lo.x, P.x), __fsub_rn(P.x, hi.x)), 0.f);
            const float gy = fmaxf(fmaxf(__fsub_rn(lo.y, P.y), __fsub_rn(P.y, hi.y)), 0.f);
            const float gz = D == 3 ? fmaxf(fmaxf(__fsub_rn(lo.z, P.z), __fsub_rn(P.z, hi.z)), 0.f) : 0.f;
            return d2_of<D>(gx, gy, gz);
        };
        auto wanted = [&](float lb) { return lb <= bd; };
        // the whole warp scans one leaf, wanted by the lanes in `need`: stage
        // it in shared memory, mark each wanting lane's points within its
        // bound, then insert each lane's marked points -- the warp runs as
        // many insert steps as its busiest lane needs, not one per point that
        // any lane wants.  Marking: with many wanting lanes, every lane tests
        // all 32 points (broadcast reads); with few, the points sit one per
        // lane and each wanting query is tested against all of them at once
        // (one ballot per query).  A lane that does not want the leaf has no
        // point in it within its bound (the box bound never exceeds a
        // point's d2: both round the same differences the same way).
        auto stage_leaf = [&](uint32_t b, uint32_t m) {
            __syncwarp();  // the previous leaf's reads are done
            if ((uint32_t)lane < m) {
                const float4 c = __ldg(&sp[b + lane]);
                pt[lane] = c;
                s_ax[w][0][lane] = c.x;
                s_ax[w][1][lane] = c.y;
                if constexpr (D == 3) s_ax[w][2][lane] = c.z;
                if constexpr (CL) s_cl[w][lane] = __ldg(&pcloud[b + lane]);
            } else {
                // past the last point: NaN coordinates fail every d2 <= bound
                // test; +inf in the rows gives d2 = +inf, beyond every bound
                pt[lane] = make_float4(__int_as_float(0x7fffffff), 0.f, 0.f, 0.f);
                s_ax[w][0][lane] = INFINITY;
                s_ax[w][1][lane] = 0.f;
                if constexpr (D == 3) s_ax[w][2][lane] = 0.f;
                if constexpr (CL) s_cl[w][lane] = ~0u;
            }
            __syncwarp();
        };
        // d2 of candidates 2h and 2h + 1 of the staged leaf (packed, bit for
        // bit d2_of)
        auto pair_d2 = [&](int h) -> f32x2 {
            const f32x2 cx = reinterpret_cast<const f32x2*>(s_ax[w][0])[h];
            const f32x2 cy = reinterpret_cast<const f32x2*>(s_ax[w][1])[h];
            const f32x2 cz = D == 3 ? reinterpret_cast<const f32x2*>(s_ax[w][D - 1])[h] : 0ull;
            return d2_of2<D>(cx, cy, cz, f2_dup(P.x), f2_dup(P.y), f2_dup(D == 3 ? P.z : 0.f));
        };
        auto scan_leaf = [&](uint32_t leaf, uint32_t need, bool staged) {
            const uint32_t b = leaf * 32;
            const uint32_t m = min(32u, n - b);
            ++st_leaves;
            if (!staged) stage_leaf(b, m);
            uint32_t mask = 0;
            if (__popc(need) > kKnnDenseFirst) {
                if constexpr (CL) {
#pragma unroll 8
                    for (int j = 0; j < 32; ++j) {
                        const float4 c = pt[j];
                        const float d2 = d2_of<D>(__fsub_rn(c.x, P.x), __fsub_rn(c.y, P.y), __fsub_rn(c.z, P.z));
                        // in a batch, a point of another cloud is no candidate
                        // (lanes may hold different clouds)
                        const bool ok = d2 <= bd && s_cl[w][j] == qc;
                        mask |= (ok ? 1u : 0u) << j;
                    }
                } else {
                    // two candidates per packed step; the sign of bd - d2
                    // marks the rejected ones
                    const f32x2 b2 = f2_dup(bd);
                    uint32_t rej = 0;
#pragma unroll 8
                    for (int h = 15; h >= 0; --h) rej = reject_append2(rej, b2, pair_d2(h));
                    mask = ~rej;
                }
                // round 1: the query's component is the query alone
                if (leaf == (me >> 5)) mask &= ~(1u << (me & 31u));
            } else {
                const float4 c = pt[lane];
                const uint32_t cc = CL ? s_cl[w][lane] : 0u;
                while (need) {
                    const int q = __ffs(need) - 1;
                    need &= need - 1u;
                    const float qx = __shfl_sync(kFull, P.x, q), qy = __shfl_sync(kFull, P.y, q);
                    const float qz = D == 3 ? __shfl_sync(kFull, P.z, q) : 0.f;
                    const float qb = __shfl_sync(kFull, bd, q);
                    // round 1: the query's component is the query alone
                    const uint32_t qme = __shfl_sync(kFull, me, q);
                    // every lane takes part in every shuffle (none under a condition)
                    const uint32_t qq = CL ? __shfl_sync(kFull, qc, q) : 0u;
                    const float d2 = d2_of<D>(__fsub_rn(c.x, qx), __fsub_rn(c.y, qy), __fsub_rn(c.z, qz));
                    bool ok = d2 <= qb && b + (uint32_t)lane != qme;
                    if constexpr (CL) ok = ok && cc == qq;
                    const uint32_t mb = __ballot_sync(kFull, ok);
                    if (lane == q) mask = mb;
                }
            }
            st_marked += __popc(mask);
            while (mask) {
                const int j = __ffs(mask) - 1;
                mask &= mask - 1u;
                ++st_steps;
                const float4 c = pt[j];
                const float d2 = d2_of<D>(__fsub_rn(c.x, P.x), __fsub_rn(c.y, P.y), __fsub_rn(c.z, P.z));
                if (d2 > bd) continue;
                const uint64_t key = ((uint64_t)__float_as_uint(d2) << 32) | __float_as_uint(c.w);
                // sorted insert, all in registers and without a chain: every
                // entry is compared with the key at once (the list is sorted,
                // so the entries below it are a prefix; keys are distinct:
                // ids differ), then each slot keeps its entry, takes the key
                // or takes its predecessor
                bool below[K];
#pragma unroll
                for (int t = 0; t < K; ++t) below[t] = kk[t] < key;
                if (below[K - 1]) continue;
#pragma unroll
                for (int t = K - 1; t > 0; --t) kk[t] = below[t] ? kk[t] : (below[t - 1] ? key : kk[t - 1]);
                kk[0] = below[0] ? kk[0] : key;
                if (kk[K - 1] != kNoKey) bd = __uint_as_float((uint32_t)(kk[K - 1] >> 32));
            }
        };

        // the warp's own leaf (lane 0's query's) first, then bottom-up: every
        // other leaf lies in exactly one sibling subtree of its ancestors
        const uint32_t own = __shfl_sync(kFull, me, 0) >> 5;
        float tk = INFINITY;   // the own leaf's certified bound
        bool guessed = false;  // the walk starts from the learned radius, below tk
        float f[prop::kIn];    // proposal features (learned bound, traces)
        const bool tracing = a.trace != nullptr;
        {
            // Each lane's bound before the walk: the K-th smallest d2 to the
            // other points of the warp's own leaf (a min/max network over K
            // floats, no ids), an upper bound of its K-th nearest distance.
            // Marked with it instead of FLT_MAX, the own leaf and the leaves
            // after it offer only points that can still make the list, so
            // far fewer inserts run; a leaf of fewer than K + 1 points leaves
            // FLT_MAX.
            const uint32_t m_own = min(32u, n - own * 32);
            stage_leaf(own * 32, m_own);
            const int self = (me >> 5) == own ? (int)(me & 31u) : -1;
            float t[K];
#pragma unroll
            for (int i = 0; i < K; ++i) t[i] = INFINITY;
#pragma unroll 2
            for (int h = 0; h < 16; ++h) {
                const f32x2 d2 = pair_d2(h);
#pragma unroll
                for (int u = 0; u < 2; ++u) {
                    const int j = 2 * h + u;
                    float d = __uint_as_float(u ? (uint32_t)(d2 >> 32) : (uint32_t)d2);
                    bool ok = j != self && d <= FLT_MAX;  // padding (+inf) and the query itself are out
                    if constexpr (CL) ok = ok && s_cl[w][j] == qc;
                    d = ok ? d : INFINITY;
#pragma unroll
                    for (int i = 0; i < K; ++i) {
                        const float lo = fminf(t[i], d);
                        d = fmaxf(t[i], d);
                        t[i] = lo;
                    }
                }
            }
            tk = t[K - 1];
            if (listed && tk < bd) bd = tk;
            if (LEARN || tracing) {
                const bool fin = listed && tk < INFINITY;
                const uint32_t ol = L + (me >> 5);
                const float4 lo = __ldg(&nlo[ol]), hi = __ldg(&nhi[ol]);
                const float4 plo = __ldg(&nlo[ol >> 1]), phi = __ldg(&nhi[ol >> 1]);
                const float ex = hi.x - lo.x, ey = hi.y - lo.y, ez = D == 3 ? hi.z - lo.z : 0.f;
                const float px = phi.x - plo.x, py = phi.y - plo.y, pz = D == 3 ? phi.z - plo.z : 0.f;
                float e = fminf(fminf(P.x - lo.x, hi.x - P.x), fminf(P.y - lo.y, hi.y - P.y));
                if (D == 3) e = fminf(e, fminf(P.z - lo.z, hi.z - P.z));
                if (fin) {
                    prop::knn_features(t[0], t[2], tk, ex * ex + ey * ey + ez * ez, e * e,
                                       px * px + py * py + pz * pz, (float)min(32u, n - (me >> 5) * 32) * (1.f / 32.f),
                                       1, 1.f, f);
                } else {
#pragma unroll
                    for (int i = 0; i < prop::kIn; ++i) f[i] = 0.f;
                }
                if constexpr (LEARN) {
                    // one tensor-core inference for the warp's 32 queries
                    float o0, o1;
                    prop::infer_warp(reinterpret_cast<const prop::Frag*>(a.frag), f, o0, o1);
                    if (fin && o1 >= a.threshold) {
                        const float r = tk * exp2f(fminf(fmaf(8.f, o0, a.margin), 0.f));
                        if (r < bd) {
                            bd = r;
                            guessed = true;
                        }
                    }
                }
            }
        }
        const bool learned_lane = guessed;
        bool resumed = false;
        const uint32_t nleaves = (n + 31u) >> 5;
        // Gather (single point sets), run once the own leaf and its Hilbert
        // neighbours are scanned (spatially close, they tighten every lane's
        // bound): each lane tests another node against the own leaf's box
        // grown by B, the largest bound of any lane.  That box-to-box bound
        // never exceeds a lane's node_lb (the lane's point lies in the box;
        // rounded differences are monotone), so no node a lane still wants is
        // dropped.  It starts from the siblings of the own leaf's ancestors
        // (every other leaf lies under exactly one), all tested in one step,
        // and descends 32 nodes a step.  The gathered leaves keep their boxes
        // in shared memory and their ids in the stack's slots; their sort keys
        // (the bound's bits over the slot) come back sorted in v0 / v1, nearest
        // first.  Returns the number of leaves, or -1 when the frontier or the
        // leaf list overflows (degenerate boxes, e.g. many duplicates, or a
        // bound that reaches far): the depth-first walk then runs instead.
        auto gather = [&](uint32_t& v0, uint32_t& v1) -> int {
            // bd is -1 on lanes without a query; a bound is never negative
            const float B = __uint_as_float(__reduce_max_sync(kFull, __float_as_uint(fmaxf(bd, 0.f))));
            const float4 qlo = __ldg(&nlo[L + own]), qhi = __ldg(&nhi[L + own]);
            uint32_t* const fr = s_fr[w];
            uint32_t* const lk = s_lk[w];
            float(*const bx)[kWideLeaves] = s_bx[w];
            const unsigned below = (1u << lane) - 1u;
            const int depth = 31 - __clz(L);  // levels under the root (L is a power of two)
            __syncwarp();
            if (lane < depth) fr[lane] = ((L + own) >> lane) ^ 1u;
            __syncwarp();
            int top = depth, nl = 0;
            while (top > 0) {
                const int take = min(top, 32);
                top -= take;
                ++st_nodes;
                uint32_t node = 0;
                float lb = INFINITY;
                float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo;
                if (lane < take) {
                    node = fr[top + lane];
                    lo = __ldg(&nlo[node]);
                    hi = __ldg(&nhi[node]);
                    const float gx = fmaxf(fmaxf(__fsub_rn(lo.x, qhi.x), __fsub_rn(qlo.x, hi.x)), 0.f);
                    const float gy = fmaxf(fmaxf(__fsub_rn(lo.y, qhi.y), __fsub_rn(qlo.y, hi.y)), 0.f);
                    const float gz =
                        D == 3 ? fmaxf(fmaxf(__fsub_rn(lo.z, qhi.z), __fsub_rn(qlo.z, hi.z)), 0.f) : 0.f;
                    lb = d2_of<D>(gx, gy, gz);
                }
                const bool want = lb <= B, is_leaf = node >= L;
                const unsigned ml = __ballot_sync(kFull, want && is_leaf);
                const unsigned mi = __ballot_sync(kFull, want && !is_leaf);
                const int nlf = __popc(ml), nin = __popc(mi);
                if (nl + nlf > kWideLeaves || top + 2 * nin > kWideFront) return -1;
                __syncwarp();  // every lane has read its entry: the pushes may overwrite it
                if (want && is_leaf) {
                    const int e = nl + __popc(ml & below);
                    stack[e] = node - L;
                    lk[e] = (__float_as_uint(lb) & ~(uint32_t)(kWideLeaves - 1)) | (uint32_t)e;
                    bx[0][e] = lo.x;
                    bx[1][e] = lo.y;
                    bx[D][e] = hi.x;
                    bx[D + 1][e] = hi.y;
                    if constexpr (D == 3) {
                        bx[2][e] = lo.z;
                        bx[5][e] = hi.z;
                    }
                }
                if (want && !is_leaf) {
                    const int e = top + 2 * __popc(mi & below);
                    fr[e] = 2u * node;
                    fr[e + 1] = 2u * node + 1u;
                }
                nl += nlf;
                top += 2 * nin;
                __syncwarp();
            }
            v0 = lane < nl ? lk[lane] : ~0u;
            v1 = lane + 32 < nl ? lk[lane + 32] : ~0u;
            if (nl > 32) bitonic_sort64(v0, v1, lane);
            else if (nl > 1) v0 = bitonic_sort32(v0, lane);
            return nl;
        };
        for (int attempt = 0;; ++attempt) {
            // The leaves to scan come from a warp-uniform state machine, so
            // that every one goes through the single scan below (one copy of
            // its code): the own leaf; for single point sets its Hilbert
            // neighbours and then the gathered leaves, nearest first; the
            // depth-first walk (the own leaf's ancestors' sibling subtrees, a
            // node entered when any lane's lower bound reaches it) when the
            // gather gives up, and for point batches.
            enum { kOwn, kNext, kPrev, kGathered, kWalk, kDone };
            int phase = kOwn;
            int li = 0, nl = -2;        // gathered leaves: next index, count (-2: not gathered yet)
            uint32_t v0 = ~0u, v1 = ~0u;  // their sorted keys
            uint32_t dv = L + own;      // the walk: the ancestor whose sibling comes next
            int top = 0;                // the walk's stack depth
            while (phase != kDone) {
                uint32_t leaf = 0, need = 0;
                bool staged = false;
                if (phase == kOwn) {
                    leaf = own;
                    need = __ballot_sync(kFull, bd >= 0.f);
                    staged = attempt == 0;  // the bound above left it in shared memory
                    phase = CL ? kWalk : kNext;
                } else if (phase == kNext) {
                    phase = kPrev;
                    if (own + 1 < nleaves) {
                        leaf = own + 1;
                        need = __ballot_sync(kFull, wanted(node_lb(L + leaf)));
                    }
                } else if (phase == kPrev) {
                    phase = kGathered;
                    if (own > 0) {
                        leaf = own - 1;
                        need = __ballot_sync(kFull, wanted(node_lb(L + leaf)));
                    }
                } else if (phase == kGathered) {
                    if (nl == -2) {
                        nl = gather(v0, v1);
                        if (nl < 0) {
                            phase = kWalk;
                            continue;
                        }
                    }
                    if (li >= nl) {
                        phase = kDone;
                        continue;
                    }
                    const uint32_t e = __shfl_sync(kFull, li < 32 ? v0 : v1, li & 31) & (uint32_t)(kWideLeaves - 1);
                    ++li;
                    leaf = stack[e];
                    if (leaf + 1u == own || leaf == own + 1u) continue;  // scanned already
                    ++st_nodes;
                    // the lane's node_lb of the leaf, from the kept box
                    const float(*const bx)[kWideLeaves] = s_bx[w];
                    const float gx = fmaxf(fmaxf(__fsub_rn(bx[0][e], P.x), __fsub_rn(P.x, bx[D][e])), 0.f);
                    const float gy = fmaxf(fmaxf(__fsub_rn(bx[1][e], P.y), __fsub_rn(P.y, bx[D + 1][e])), 0.f);
                    float gz = 0.f;
                    if constexpr (D == 3) gz = fmaxf(fmaxf(__fsub_rn(bx[2][e], P.z), __fsub_rn(P.z, bx[5][e])), 0.f);
                    need = __ballot_sync(kFull, wanted(d2_of<D>(gx, gy, gz)));
                } else {
                    // the walk, up to the next leaf some lane wants
                    for (;;) {
                        if (top == 0) {
                            if (dv <= 1) {
                                phase = kDone;
                                break;
                            }
                            const uint32_t sib = dv ^ 1u;
                            dv >>= 1;
                            ++st_nodes;
                            if (!__any_sync(kFull, wanted(node_lb(sib)))) continue;
                            __syncwarp();
                            stack[0] = sib;
                            top = 1;
                            __syncwarp();
                        }
                        const uint32_t node = stack[--top];
                        ++st_nodes;
                        if (node >= L) {
                            const uint32_t lf = node - L;
                            // single point sets reach the walk after the neighbours
                            if (!CL && (lf + 1u == own || lf == own + 1u)) continue;
                            // bounds re-checked: they may have shrunk since the push
                            need = __ballot_sync(kFull, wanted(node_lb(node)));
                            if (need) {
                                leaf = lf;
                                break;
                            }
                            continue;
                        }
                        const uint32_t c0 = 2 * node, c1 = c0 + 1;
                        const float l0 = node_lb(c0), l1 = node_lb(c1);
                        const bool w0 = __any_sync(kFull, wanted(l0)), w1 = __any_sync(kFull, wanted(l1));
                        // the child nearer to the warp's nearest lane is searched next
                        const uint32_t m0 = __reduce_min_sync(kFull, __float_as_uint(l0));
                        const uint32_t m1 = __reduce_min_sync(kFull, __float_as_uint(l1));
                        const bool near0 = m0 <= m1;
                        const bool wn = near0 ? w0 : w1, wf = near0 ? w1 : w0;
                        __syncwarp();  // every lane has read the popped entry
                        if (wf) stack[top++] = near0 ? c1 : c0;
                        if (wn) stack[top++] = near0 ? c0 : c1;
                        __syncwarp();
                    }
                }
                if (need) scan_leaf(leaf, need, staged);
            }
            if constexpr (!LEARN) break;
            // A learned radius that held fewer than K points: the list is not
            // the K nearest.  Those lanes start over from the certified
            // bound; the others sit the walk out (bound -1: they want nothing).
            const bool miss = guessed && kk[K - 1] == kNoKey;
            if (attempt > 0 || !__any_sync(kFull, miss)) break;
            if (miss) {
#pragma unroll
                for (int j = 0; j < K; ++j) kk[j] = kNoKey;
                bd = tk;
                resumed = true;
            } else {
                bd = -1.f;
            }
            guessed = false;
        }
        if (tracing && listed && tk < INFINITY && (knn_sample_hash(me) & a.trace_mask) == 0) {
            // training record: features, the target radius log2(d2 of the
            // K-th nearest / tk) / 8, whether tk could be tightened at all,
            // the regression mask (the list is full)
            const uint32_t at = atomicAdd(a.trace_ctl, 1u);
            if (at < a.trace_cap) {
                float* o = a.trace + (uint64_t)at * prop::kRec;
                const bool full = kk[K - 1] != kNoKey;
                const float rk = full ? __uint_as_float((uint32_t)(kk[K - 1] >> 32)) : tk;
#pragma unroll
                for (int i = 0; i < prop::kIn; ++i) o[i] = f[i];
                o[8] = full ? prop::lg8(rk) - prop::lg8(tk) : 0.f;
                o[9] = full && rk < tk ? 1.f : 0.f;
                o[10] = full ? 1.f : 0.f;
                o[11] = 0.f;
            }
        }
        uint32_t p0 = kNone;  // entry 0's leaf position
        if (listed) {
#pragma unroll
            for (int j = 0; j < K; ++j) {
                const uint32_t pos = kk[j] == kNoKey ? kNone : __ldg(&iperm[(uint32_t)kk[j]]);
                if (j == 0) p0 = pos;
                klist[(size_t)j * n + me] = kk[j] == kNoKey ? ~0ull : ((kk[j] >> 32) << 32) | pos;
            }
            // entry 0 is this round's edge: inside the component from round 2 on
            kcur[me] = kk[0] == kNoKey ? 0 : 1;
        }
        // round-1 result: entry 0 (exact: every node within the K-th
        // distance was searched)
        if (listed) {
            const int op = __float_as_int(P.w);
            if (kk[0] != kNoKey) {
                const float d0 = __uint_as_float((uint32_t)(kk[0] >> 32));
                const uint32_t mn = (uint32_t)min(op, (int)(uint32_t)kk[0]);
                const uint64_t key = ((uint64_t)__float_as_uint(d0) << 32) | mn;
                a.lbp[me] = d0;
                a.selq[me] = p0;
                a.selkey[me] = key;
                // round 1: every point is its own component, the only writer
                // of its key, and its own winner; its winner slot holds what
                // k_resolve would write: (larger input id of the edge) << 32
                // | position
                a.ckey[me] = key;
                a.cmax[me] = ((uint64_t)max((uint32_t)op, (uint32_t)kk[0]) << 32) | me;
            } else {
                a.lbp[me] = INFINITY;  // alone in its cloud
                a.selq[me] = kNone;
            }
        }
        if (a.stats) {
            // leaves, nodes and insert steps are per warp; candidates per listed lane
            unsigned long long q = __popc(__ballot_sync(kFull, listed));
            const uint32_t marked = __reduce_add_sync(kFull, st_marked);
            const uint32_t steps = __reduce_max_sync(kFull, st_steps);
            const uint32_t nl = __popc(__ballot_sync(kFull, learned_lane));
            const uint32_t nr = __popc(__ballot_sync(kFull, resumed));
            if (lane == 0) {
                atomicAdd(&a.stats[0], (unsigned long long)st_leaves);
                atomicAdd(&a.stats[1], (unsigned long long)st_nodes * 32ull);
                atomicAdd(&a.stats[2], (unsigned long long)st_leaves * 32ull * q);
                atomicAdd(&a.stats[3], 1ull);
                atomicAdd(&a.stats[4], q);
                atomicAdd(&a.stats[5], q);
                atomicAdd(&a.stats[8], (unsigned long long)marked);
                atomicAdd(&a.stats[9], (unsigned long long)steps);
                atomicAdd(&a.stats[10], (unsigned long long)nl);
                atomicAdd(&a.stats[11], (unsigned long long)nr);
            }
        }
    }
}


// Launch of one shape; the grid covers the list's upper bound `a.n` with at
// most four waves of resident blocks (the kernel strides over the rest).
template <int D, bool CL, int I>
void launch_shape(const CnnsArgs& a, int sms, cudaStream_t s)
{
    constexpr int T = kSearchShapes[I].threads, M = kSearchShapes[I].min_blocks;
    uint64_t b = ((uint64_t)a.n + T - 1) / T;
    const uint64_t cap = (uint64_t)sms * M * 4;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    k_cnns_t<D, CL, T, M><<<(unsigned)b, T, 0, s>>>(a);
}

template <int D, bool CL, bool LEARN>
cudaError_t launch_knn(const CnnsArgs& a, uint64_t* klist, unsigned char* kcur, const uint32_t* iperm, int sms,
                       cudaStream_t s)
{
    constexpr int T = kKnnWarps * 32;
    uint64_t b = ((uint64_t)a.n + T - 1) / T;
    const uint64_t cap = (uint64_t)sms * 4 * 4;
    if (b > cap) b = cap;
    if (b < 1) b = 1;
    // list length: the context's choice (the learned proposal's network is trained for kKnn)
    static_assert(kKnn == 6, "the learned proposal is trained for lists of 6");
    switch (LEARN ? kKnn : a.knn_k) {
    case 4: k_knn_first<D, CL, false, 4><<<(unsigned)b, T, 0, s>>>(a, klist, kcur, iperm); break;
    case 5: k_knn_first<D, CL, false, 5><<<(unsigned)b, T, 0, s>>>(a, klist, kcur, iperm); break;
    case 8: k_knn_first<D, CL, false, 8><<<(unsigned)b, T, 0, s>>>(a, klist, kcur, iperm); break;
    case kKnn: k_knn_first<D, CL, LEARN, kKnn><<<(unsigned)b, T, 0, s>>>(a, klist, kcur, iperm); break;
    default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

template <int D, bool CL>
cudaError_t launch_dim(const CnnsArgs& a, int shape, int sms, cudaStream_t s)
{
    static_assert(kNumSearchShapes == 6, "one case per shape");
    switch (shape) {
    case 0: launch_shape<D, CL, 0>(a, sms, s); break;
    case 1: launch_shape<D, CL, 1>(a, sms, s); break;
    case 2: launch_shape<D, CL, 2>(a, sms, s); break;
    case 3: launch_shape<D, CL, 3>(a, sms, s); break;
    case 4: launch_shape<D, CL, 4>(a, sms, s); break;
    case 5: launch_shape<D, CL, 5>(a, sms, s); break;
    default: return cudaErrorInvalidValue;
    }
    if (a.wide_limit > 0) {
        // the warp-per-query kernel for short lists (each kernel reads the
        // list's length on the device and leaves the other's lists alone)
        uint64_t b = ((uint64_t)a.wide_limit + kWideWarps - 1) / kWideWarps;
        const uint64_t cap = (uint64_t)sms * 16;
        if (b > cap) b = cap;
        k_cnns_w<D, CL><<<(unsigned)b, kWideWarps * 32, 0, s>>>(a);
    }
    if (a.coop_min != kNoCoop) {
        // the cooperative kernel for long lists (grid: as k_knn_first's)
        constexpr int T = kKnnWarps * 32;
        uint64_t b = ((uint64_t)a.n + T - 1) / T;
        const uint64_t cap = (uint64_t)sms * 4 * 4;
        if (b > cap) b = cap;
        if (b < 1) b = 1;
        k_cnns_c<D, CL><<<(unsigned)b, T, 0, s>>>(a);
    }
    return cudaGetLastError();
}

}  // namespace

}  // namespace emst
