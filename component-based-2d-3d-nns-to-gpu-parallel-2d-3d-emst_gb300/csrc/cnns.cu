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

#include <cub/device/device_select.cuh>
#include <thrust/iterator/counting_iterator.h>

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
// when smaller) and the levels above them inside that subtree.
__global__ void __launch_bounds__(1024)
    k_node_labels_sub(const uint32_t* __restrict__ lab, uint32_t n, uint32_t nchunk, uint32_t L, uint32_t span,
                      uint32_t* __restrict__ nlab)
{
    __shared__ uint32_t s[kLeavesPerBlock];
    const uint32_t first = blockIdx.x * span;
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    for (uint32_t l = w; l < span; l += blockDim.x >> 5) {
        const uint32_t c = first + l;
        uint32_t out = kEmpty;
        if (c < nchunk) {
            const uint32_t j = c * 32 + lane;
            const bool v = j < n;
            const uint32_t my = v ? lab[j] : 0u;
            const uint32_t l0 = __shfl_sync(kFull, my, 0);
            out = __all_sync(kFull, !v || my == l0) ? l0 : kMixed;
        }
        if (lane == 0) {
            s[l] = out;
            nlab[L + c] = out;
        }
    }
    __syncthreads();
    uint32_t base = (L + first);
    for (uint32_t cnt = span >> 1; cnt >= 1; cnt >>= 1) {
        base >>= 1;
        uint32_t v = 0;
        const bool act = threadIdx.x < cnt;
        if (act) v = merge_label(s[2 * threadIdx.x], s[2 * threadIdx.x + 1]);
        __syncthreads();
        if (act) {
            s[threadIdx.x] = v;
            nlab[base + threadIdx.x] = v;
        }
        __syncthreads();
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
// component's minimum bound clb.
__global__ void k_reuse(uint32_t n, const uint32_t* __restrict__ lab, uint32_t* __restrict__ selq,
                        uint64_t* __restrict__ selkey, float* __restrict__ lbp, uint64_t* __restrict__ ckey,
                        uint32_t* __restrict__ clb, unsigned char* __restrict__ dflag, uint32_t* __restrict__ prov,
                        uint32_t* __restrict__ n_prov, const int* __restrict__ round,
                        const uint64_t* __restrict__ klist, unsigned char* __restrict__ kcur,
                        const uint32_t* __restrict__ perm)
{
    const bool lists = klist && *round >= 2;  // round 1 builds them
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t p = base + threadIdx.x;
        bool is_dirty = false, record = false;
        if (p < n) {
            const uint32_t q = selq[p];
            const uint32_t lp = lab[p];
            uint64_t key = kNoKey;
            if (q != kNone && lab[q] != lp) {
                key = selkey[p];
            } else {
                uint32_t lb = __float_as_uint(lbp[p]);
                if (lists && lb != 0x7f800000u) {
                    // the first neighbour outside the component is the exact
                    // nearest outside point: every closer point precedes it.
                    // Entries before the cursor were found inside the
                    // component in an earlier round and stay inside
                    // (components only grow); their d2 is already in lbp.
                    bool full = true;
                    const int j0 = kcur[p];
                    int j = j0;
                    for (; j < kKnn; ++j) {
                        const uint64_t kj = klist[(size_t)j * n + p];  // d2 bits << 32 | position
                        const uint32_t qj = (uint32_t)kj;
                        if (qj == kNone) {
                            full = false;
                            break;
                        }
                        if (lab[qj] != lp) {
                            const uint32_t mn = min(perm[p], perm[qj]);
                            key = (kj & 0xffffffff00000000ull) | mn;
                            selq[p] = qj;
                            selkey[p] = key;
                            lbp[p] = __uint_as_float((uint32_t)(kj >> 32));
                            break;
                        }
                        lb = max(lb, (uint32_t)(kj >> 32));  // non-negative floats order as their bits
                    }
                    if (j != j0) kcur[p] = (unsigned char)j;
                    if (key == kNoKey && (j != j0 || !full)) {
                        // none outside: a full list bounds the distance from below;
                        // a short one held every other point of the cloud
                        // (an exhausted list, j0 == kKnn, adds nothing new)
                        lb = full ? lb : 0x7f800000u;
                        lbp[p] = __uint_as_float(lb);
                    }
                }
                if (key == kNoKey) {
                    // lbp = +inf: no point outside the component exists (in a batch,
                    // the cloud is one component), and components only grow
                    is_dirty = lb != 0x7f800000u;
                    if (is_dirty && lb < __ldcg(&clb[lp])) atomicMin(&clb[lp], lb);
                }
            }
            if (key != kNoKey && key <= __ldcg(&ckey[lp])) {
                const uint64_t old = atomicMin((unsigned long long*)&ckey[lp], (unsigned long long)key);
                record = old >= key;
            }
        }
        if (p < n) dflag[p] = is_dirty ? 1 : 0;
        warp_append(record, p, prov, n_prov);
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

// Per round: each point's current component label into the .w word of its
// packed (x, y, z, label) record.  The coordinates are copied once per solve
// (cnns_init) and never change, so only 4 of the 16 bytes are written.
__global__ void k_pack_spl(uint32_t n, const uint32_t* __restrict__ lab, float4* __restrict__ spl)
{
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    reinterpret_cast<uint32_t*>(spl)[4 * (size_t)i + 3] = lab[i];
}

// Who searches in the first pass (flag 1), who waits for the second (2), who
// needs no search this round (0), decided before the search so that search
// warps carry only real searches.  A dirty point whose lower bound exceeds
// its component's key (set by reused partners) cannot hold the minimum; one
// whose bound exceeds `factor` times its component's smallest waits.
__global__ void k_filter_first(uint32_t n, unsigned char* __restrict__ flag, const uint32_t* __restrict__ lab,
                               const float* __restrict__ lbp, const uint64_t* __restrict__ ckey,
                               const uint32_t* __restrict__ clb, float factor, unsigned long long* __restrict__ stats)
{
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += gridDim.x * blockDim.x) {
        const uint32_t p = base + threadIdx.x;
        bool later = false;
        if (p < n && flag[p]) {
            const uint32_t l = lab[p];
            const float lb = lbp[p];
            const uint64_t k = __ldcg(&ckey[l]);
            const float cb = k == kNoKey ? INFINITY : __uint_as_float((uint32_t)(k >> 32));
            later = !(lb > cb) && lb > factor * __uint_as_float(__ldcg(&clb[l]));
            flag[p] = lb > cb ? 0 : (later ? 2 : 1);
        }
        if (stats) {
            const unsigned m = __ballot_sync(kFull, later);
            if ((threadIdx.x & 31) == 0 && m) atomicAdd(&stats[7], (unsigned long long)__popc(m));
        }
    }
}

// Second-pass searchers: waiting points (2) whose bound the first pass did
// not rule out.
__global__ void k_filter_second(uint32_t n, unsigned char* __restrict__ flag, const uint32_t* __restrict__ lab,
                                const float* __restrict__ lbp, const uint64_t* __restrict__ ckey)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    const unsigned char f = flag[p];
    if (!f) return;
    bool go = false;
    if (f == 2) {
        const uint64_t k = __ldcg(&ckey[lab[p]]);
        go = k == kNoKey || !(lbp[p] > __uint_as_float((uint32_t)(k >> 32)));
    }
    flag[p] = go ? 1 : 0;
}

struct FlagIsOne {
    const unsigned char* f;
    __host__ __device__ bool operator()(uint32_t i) const { return f[i] == 1; }
};

struct FlagIsTwo {
    const unsigned char* f;
    __host__ __device__ bool operator()(uint32_t i) const { return f[i] == 2; }
};

cudaError_t select_flagged_two(Ctx& c, uint32_t* out, uint32_t* count)
{
    size_t tb = c.sel_tmp.cap;
    return cub::DeviceSelect::If(c.sel_tmp.p, tb, thrust::counting_iterator<uint32_t>(0), out, count, (int)c.n,
                                 FlagIsTwo{c.dflag.p}, c.stream);
}

cudaError_t select_flagged_one(Ctx& c, uint32_t* out, uint32_t* count)
{
    size_t tb = c.sel_tmp.cap;
    return cub::DeviceSelect::If(c.sel_tmp.p, tb, thrust::counting_iterator<uint32_t>(0), out, count, (int)c.n,
                                 FlagIsOne{c.dflag.p}, c.stream);
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
cudaError_t node_labels_of(Ctx& c, const uint32_t* labels, uint32_t* out)
{
    const uint32_t L = (uint32_t)c.L;
    const uint32_t span = L < (uint32_t)kLeavesPerBlock ? L : (uint32_t)kLeavesPerBlock;
    k_node_labels_sub<<<L / span, 1024, 0, c.stream>>>(labels, (uint32_t)c.n, (uint32_t)c.nchunk, L, span, out);
    c.launches++;
    if (L / span >= 2) {
        k_node_labels_top<<<1, 1024, 0, c.stream>>>(L / span, out);
        c.launches++;
    }
    return cudaGetLastError();
}

// Per-round node labels (the component shared by all points of a subtree)
// and the packed (x, y, z, label) points of the thread-per-query search.
cudaError_t cnns_node_labels(Ctx& c)
{
    cudaError_t e;
    if ((e = ensure(c.nlab, (size_t)2 * c.L)) != cudaSuccess) return e;  // no-op after cnns_init
    if ((e = node_labels_of(c, c.lab.p, c.nlab.p)) != cudaSuccess) return e;
    if (!c.cnns_warp) {
        if ((e = ensure(c.spl, (size_t)c.n)) != cudaSuccess) return e;
        k_pack_spl<<<blocks_for(c.n, 256), 256, 0, c.stream>>>((uint32_t)c.n, c.lab.p, c.spl.p);
        c.launches++;
    }
    return cudaGetLastError();
}

cudaError_t cnns_init(Ctx& c)
{
    cudaError_t e;
    const size_t n = (size_t)c.n;
    if ((e = ensure(c.dirty, n)) != cudaSuccess) return e;
    if ((e = ensure(c.dirty2, n)) != cudaSuccess) return e;
    if ((e = ensure(c.lbp, n)) != cudaSuccess) return e;
    if ((e = ensure(c.clb, n)) != cudaSuccess) return e;
    if ((e = ensure(c.nlab, (size_t)2 * c.L)) != cudaSuccess) return e;
    if ((e = ensure(c.spl, n)) != cudaSuccess) return e;
    // the packed points' coordinates, once per solve (each round writes the labels)
    if ((e = cudaMemcpyAsync(c.spl.p, c.sp.p, n * sizeof(float4), cudaMemcpyDeviceToDevice, c.stream)) !=
        cudaSuccess)
        return e;
    if ((e = ensure(c.dflag, n)) != cudaSuccess) return e;
    if (c.knn_seed && !c.cnns_warp) {
        if ((e = ensure(c.klist, n * kKnn)) != cudaSuccess) return e;
        if ((e = ensure(c.kcur, n)) != cudaSuccess) return e;
        if ((e = ensure(c.iperm, n)) != cudaSuccess) return e;
        k_inverse_perm<<<blocks_for(c.n, 256), 256, 0, c.stream>>>((uint32_t)c.n, c.perm.p, c.iperm.p);
        c.launches++;
    }
    size_t tb = 0, tb2 = 0;
    if ((e = cub::DeviceSelect::Flagged(nullptr, tb, thrust::counting_iterator<uint32_t>(0), c.dflag.p, c.dirty.p,
                                        &c.ctr.p->n_dirty, (int)n, c.stream)) != cudaSuccess)
        return e;
    if ((e = cub::DeviceSelect::If(nullptr, tb2, thrust::counting_iterator<uint32_t>(0), c.dirty.p,
                                   &c.ctr.p->n_dirty, (int)n, FlagIsOne{c.dflag.p}, c.stream)) != cudaSuccess)
        return e;
    if ((e = ensure(c.sel_tmp, std::max(tb, tb2))) != cudaSuccess) return e;
    k_fill_u32<<<blocks_for(c.n, 256), 256, 0, c.stream>>>(c.selq.p, (uint32_t)c.n, kNone);
    k_fill_u32<<<blocks_for(c.n, 256), 256, 0, c.stream>>>(c.clb.p, (uint32_t)c.n, 0x7f800000u);
    cudaMemsetAsync(c.lbp.p, 0, n * sizeof(float), c.stream);
    c.launches += 2;
    return cudaGetLastError();
}

// Reuse pass + two search passes over the dirty points; fills ckey and the
// provisional winner list exactly like the static-table selection does.
cudaError_t cnns_select(Ctx& c)
{
    DevCounters* d = c.ctr.p;  // n_dirty, n_dirty2, n_prov were zeroed by the round tick
    const bool knn = c.knn_seed && !c.cnns_warp;
    k_reuse<<<list_grid(c.n), 256, 0, c.stream>>>((uint32_t)c.n, c.lab.p, c.selq.p, c.selkey.p, c.lbp.p, c.ckey.p,
                                                  c.clb.p, c.dflag.p, c.prov.p, &d->n_prov, &d->round,
                                                  knn ? c.klist.p : nullptr, c.kcur.p, c.perm.p);
    c.launches++;
    // query lists in leaf order: a warp's 32 queries are neighbours, so their
    // traversals share nodes and cache lines
    cudaError_t e;
    unsigned long long* st = c.profile ? c.nstats.p : nullptr;
    if (c.cnns_warp) {
        size_t tb = c.sel_tmp.cap;
        e = cub::DeviceSelect::Flagged(c.sel_tmp.p, tb, thrust::counting_iterator<uint32_t>(0), c.dflag.p, c.dirty.p,
                                       &d->n_dirty, (int)c.n, c.stream);
        c.launches += 2;  // a CUB selection is two kernels
    } else {
        // the learned proposal makes the first-pass choice itself
        const float first_factor = c.learned && !c.n_clouds ? INFINITY : c.first_pass_factor;
        k_filter_first<<<list_grid(c.n), 256, 0, c.stream>>>((uint32_t)c.n, c.dflag.p, c.lab.p, c.lbp.p, c.ckey.p,
                                                              c.clb.p, first_factor, st);
        c.launches++;
        e = select_flagged_one(c, c.dirty.p, &d->n_dirty);
        c.launches += 2;
        if (e == cudaSuccess && c.first_pass_ordered && !(c.learned && !c.n_clouds)) {
            e = select_flagged_two(c, c.dirty2.p, &d->n_dirty2);
            c.launches += 2;
        }
    }
    if (e != cudaSuccess) return e;
    constexpr int WPB = 4;
    const unsigned blocks = (unsigned)std::min<int64_t>((c.n + 32 * WPB - 1) / (32 * WPB), 152 * 32);
    const uint32_t* pc = c.n_clouds ? c.pcloud.p : nullptr;
    const uint32_t* nc = c.n_clouds ? c.ncloud.p : nullptr;
    // A second pass has work only if something can defer a point: a finite
    // first-pass factor, the learned proposal (single clouds), or the warp
    // search's defer list.  Otherwise it is left out of the round.
    const bool two_passes = c.cnns_warp || (c.learned && !pc) || !std::isinf(c.first_pass_factor);
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
            CnnsArgs a{c.spl.p,  c.perm.p, c.nlo.p,   c.nhi.p, c.nlab.p, (uint32_t)c.n, (uint32_t)c.L, list,
                       cnt,      c.lab.p,  c.ckey.p,  c.selq.p, c.selkey.p, c.prov.p, &d->n_prov,  c.lbp.p,
                       c.clb.p,  pass,     c.dflag.p, pc,      nc,        st,       c.pfrag.p, c.margin,
                       c.threshold, &d->round,   nullptr,  nullptr,   knn};
            // the learned first pass steers the lists k_cnns_t takes (its
            // inference runs there); the other kernels search theirs plainly
            // and defer nothing
            a.wide_limit = 0u;
            a.coop_min = kNoCoop;
            switch (c.search_split) {
            case 0: a.wide_limit = kWideLimit; a.coop_min = kCoopMin; break;
            case 1: a.wide_limit = 0xffffffffu; break;
            case 2: a.coop_min = 0u; break;
            default: break;
            }
            const bool ordered = c.first_pass_ordered && !(c.learned && !pc);
            if (ordered) {  // both segments in this one launch; no second pass
                if (pass == 2) continue;
                a.list2 = c.dirty2.p;
                a.n_list2 = &d->n_dirty2;
            }
            const int shape = search_shape_of(c);
            const bool learned = c.learned && pass == 1 && !pc;
            if (pass == 1 && c.trace_cap > 0 && !learned) {
                cudaError_t et = proposal_trace_begin(c);
                if (et != cudaSuccess) return et;
            }
            if (knn && pass == 1) {  // round 1 only (decided on the device)
                // host-driven rounds (profile mode) know the round: time the working launch
                const bool timed = c.kernel_timer && c.round == 1;
                if (timed) c.kernel_timer(c.timer_owner, 0, true);
                cudaError_t ek = c.dim == 2 ? launch_knn_first2(a, pc != nullptr, c.klist.p, c.kcur.p, c.iperm.p, c.sms, c.stream)
                                            : launch_knn_first3(a, pc != nullptr, c.klist.p, c.kcur.p, c.iperm.p, c.sms, c.stream);
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
            cudaError_t e1 = c.dim == 2 ? launch_cnns_t2(a, pc != nullptr, learned, shape, c.sms, c.stream)
                                        : launch_cnns_t3(a, pc != nullptr, learned, shape, c.sms, c.stream);
            if (e1 != cudaSuccess) return e1;
            if (a.wide_limit > 0) c.launches++;         // k_cnns_w beside k_cnns_t
            if (a.coop_min != kNoCoop) c.launches++;  // k_cnns_c beside them
            if (timed) {
                c.kernel_timer(c.timer_owner, 1, false);
                c.search_timed++;
            }
            if (pass == 1 && !ordered && two_passes) {
                k_filter_second<<<blocks_for(c.n, 256), 256, 0, c.stream>>>((uint32_t)c.n, c.dflag.p, c.lab.p,
                                                                             c.lbp.p, c.ckey.p);
                c.launches++;
                cudaError_t e2 = select_flagged_one(c, c.dirty2.p, &d->n_dirty2);
                if (e2 != cudaSuccess) return e2;
                c.launches += 2;
            }
        }
        c.nns_launches++;
        c.launches++;
    }
    if (c.trace_cap > 0 && !(c.learned && !pc)) {
        cudaError_t et = proposal_trace_end(c);
        if (et != cudaSuccess) return et;
    }
    return cudaGetLastError();
}

}  // namespace emst
