// boruvka.cu -- the per-round Boruvka operators.
//
//   select   (K_findNextClosestPoint, NodeEMST.h:1303-1384): each active point
//            advances a cursor over its sorted region list past entries that
//            are already in its component (they stay inside for good), takes
//            the first outside entry -- the minimum by (d2, input id) -- and
//            folds the edge key (d2 bits << 32 | min input id) into its root's
//            slot with one 64-bit atomicMin.  Points whose whole list is inside
//            leave the active list.
//   resolve  (K_createComponentList + K_findMinPair, NodeEMST.h:817-955):
//            the third key of the order (max input id) and the winner point
//            are settled by a second 64-bit atomicMin, only over points whose
//            atomicMin saw a value >= their own key (the final minimum is
//            always among them).
//   hook     (K_EMST_connectComponentAndUnion_2, EMSTOperators.h:1267-1303):
//            a root hooks onto the root across its edge; for a mutual pair
//            the root holding the lower input id stays root and that side
//            emits the edge once.
//   flatten  (K_EMST_flatten_DST_1, EMSTOperators.h:412-433): path-halving
//            walk of the hooked roots, then every point's label is replaced
//            by its root's root; surviving roots are compacted.
#include "emst_ctx.h"
#include "emst_device.cuh"

namespace emst {

namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr uint32_t kNoPartner = 0xffffffffu;  // selq of a point without a certified partner

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

__global__ void k_init(uint32_t n, uint32_t* __restrict__ lab, uint32_t* __restrict__ par,
                       uint32_t* __restrict__ roots, uint32_t* __restrict__ act, uint64_t* __restrict__ ckey,
                       uint64_t* __restrict__ cmax)
{
    // roots: first half holds the current roots (DevCounters::rpar = 0)
    uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    lab[i] = i;
    par[i] = i;
    roots[i] = i;
    act[i] = i;
    ckey[i] = kNoKey;
    cmax[i] = kNoKey;
}

template <int K>
__global__ void k_select(const uint32_t* __restrict__ act, const uint32_t* __restrict__ n_act,
                         const uint64_t* __restrict__ cand, const unsigned char* __restrict__ cnt,
                         unsigned char* __restrict__ cur, const unsigned char* __restrict__ zflag,
                         const uint32_t* __restrict__ lab, const uint32_t* __restrict__ perm,
                         uint64_t* __restrict__ ckey, uint32_t* __restrict__ selq, uint64_t* __restrict__ selkey,
                         uint32_t* __restrict__ act_next, uint32_t* __restrict__ n_act_next,
                         uint32_t* __restrict__ prov, uint32_t* __restrict__ n_prov)
{
    const uint32_t total = *n_act;
    for (uint32_t base = blockIdx.x * blockDim.x; base < total; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        bool keep = false, record = false;
        uint32_t p = 0;
        if (i < total) {
            p = act[i];
            const uint32_t lp = lab[p];
            unsigned c = cur[p];
            const unsigned m = cnt[p];
            const uint64_t* L = cand + (uint64_t)p * K;
            uint64_t e = 0;
            uint32_t q = 0;
            while (c < m) {
                e = L[c];
                q = (uint32_t)e;
                if (lab[q] != lp) break;
                ++c;
            }
            if (c != cur[p]) cur[p] = (unsigned char)c;
            const bool found = c < m;
            keep = found || zflag[p];
            if (found) {
                const uint32_t op = perm[p], oq = perm[q];
                const uint64_t key = (e & 0xFFFFFFFF00000000ull) | (uint64_t)min(op, oq);
                selq[p] = q;
                selkey[p] = key;
                if (key <= __ldcg(&ckey[lp])) {
                    const uint64_t old = atomicMin((unsigned long long*)&ckey[lp], (unsigned long long)key);
                    record = old >= key;
                }
            }
        }
        warp_append(keep, p, act_next, n_act_next);
        warp_append(record, p, prov, n_prov);
    }
}

// Per component, among its provisional winners (points whose key reached
// the component's slot), the one with the smallest (larger input id of the
// edge, position): the (d2, min id, max id) order's winner.  Four winners per
// thread and iteration, each level of their loads issued together (label,
// partner, key and input id; then the component's key and the partner's id).
__global__ void k_resolve(const uint32_t* __restrict__ prov, const uint32_t* __restrict__ n_prov,
                          const uint32_t* __restrict__ lab, const uint32_t* __restrict__ perm,
                          const uint64_t* __restrict__ ckey, const uint32_t* __restrict__ selq,
                          const uint64_t* __restrict__ selkey, uint64_t* __restrict__ cmax,
                          const int* __restrict__ skip_round)
{
    // round 1 with neighbour lists: the list build wrote every winner slot
    if (skip_round && *skip_round == 1) return;
    constexpr int kU = 4;
    const uint32_t total = *n_prov;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i0 = blockIdx.x * blockDim.x + threadIdx.x; i0 < total; i0 += kU * stride) {
        uint32_t p[kU], lp[kU], q[kU], op[kU], oq[kU];
        uint64_t sk[kU], ck[kU];
        bool v[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const uint32_t i = i0 + (uint32_t)u * stride;
            v[u] = i < total;
            p[u] = v[u] ? prov[i] : 0u;
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            lp[u] = v[u] ? lab[p[u]] : 0u;
            q[u] = v[u] ? selq[p[u]] : kNoPartner;
            sk[u] = v[u] ? selkey[p[u]] : kNoKey;
            op[u] = v[u] ? perm[p[u]] : 0u;
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            ck[u] = v[u] ? ckey[lp[u]] : 0ull;
            oq[u] = v[u] && q[u] != kNoPartner ? perm[q[u]] : 0u;
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            // a result without a partner (not certified) cannot be the winner; if
            // it held the component's key the hook reports it (no winner found)
            if (!v[u] || sk[u] != ck[u] || q[u] == kNoPartner) continue;
            const uint32_t mx = max(op[u], oq[u]);
            atomicMin((unsigned long long*)&cmax[lp[u]], (unsigned long long)(((uint64_t)mx << 32) | p[u]));
        }
    }
}

// Every root with an outgoing edge hooks onto the root across it (a mutual
// pair: the root holding the lower input id stays) and emits the edge once.
// Four roots per thread and iteration, each level of their chains of
// dependent loads issued together: the root's key and winner; the winner's
// partner and input id; the partner's root and input id; that root's key and
// winner.
__global__ void k_hook(const uint32_t* __restrict__ roots2, const DevCounters* dc,
                       const uint32_t* __restrict__ lab, const uint32_t* __restrict__ perm,
                       const uint64_t* __restrict__ ckey, const uint64_t* __restrict__ cmax,
                       const uint32_t* __restrict__ selq, uint32_t* __restrict__ par, int32_t* __restrict__ edges,
                       int32_t* __restrict__ eround, uint32_t* __restrict__ n_edges, uint32_t n,
                       uint32_t* __restrict__ err)
{
    __shared__ uint32_t s_cnt[33];
    constexpr int kU = 4;
    const uint32_t total = dc->n_roots;
    const int round = dc->round;
    const uint32_t* roots = roots2 + (size_t)dc->rpar * n;
    const uint32_t stride = gridDim.x * blockDim.x;
    // block-uniform trip count: block_reserve synchronises the block
    for (uint32_t base = blockIdx.x * blockDim.x; base < total; base += kU * stride) {
        uint32_t c[kU], w[kU], q[kU], ow[kU], cq[kU], oq[kU];
        uint64_t ck[kU], cm[kU], kq[kU], mq[kU];
        bool v[kU], go[kU];
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            const uint32_t i = base + (uint32_t)u * stride + threadIdx.x;
            v[u] = i < total;
            c[u] = v[u] ? roots[i] : 0u;
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            ck[u] = v[u] ? ckey[c[u]] : kNoKey;
            cm[u] = v[u] ? cmax[c[u]] : kNoKey;
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            go[u] = ck[u] != kNoKey && cm[u] != kNoKey && (uint32_t)cm[u] < n;
            w[u] = go[u] ? (uint32_t)cm[u] : 0u;
            q[u] = go[u] ? selq[w[u]] : 0u;
            ow[u] = go[u] ? perm[w[u]] : 0u;
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            cq[u] = go[u] ? lab[q[u]] : 0u;
            oq[u] = go[u] ? perm[q[u]] : 0u;
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            kq[u] = go[u] ? ckey[cq[u]] : kNoKey;
            mq[u] = go[u] ? cmax[cq[u]] : kNoKey;
        }
#pragma unroll
        for (int u = 0; u < kU; ++u) {
            bool emit = false;
            uint32_t a = 0, b = 0;
            if (v[u] && ck[u] != kNoKey && !go[u]) {
                atomicOr(err, 2u);  // a root with an edge key but no winner: internal error
            } else if (go[u]) {
                const bool mutual = kq[u] == ck[u] && (mq[u] >> 32) == (cm[u] >> 32);
                if (!mutual || ow[u] > oq[u]) par[c[u]] = cq[u];
                emit = !mutual || ow[u] < oq[u];
                a = min(ow[u], oq[u]);
                b = max(ow[u], oq[u]);
            }
            const uint32_t k = block_reserve(emit, n_edges, s_cnt);
            if (emit && k + 1 >= n) atomicOr(err, 4u);  // more than n - 1 edges: internal error
            if (emit && k + 1 < n) {
                edges[2 * (uint64_t)k] = (int32_t)a;
                edges[2 * (uint64_t)k + 1] = (int32_t)b;
                eround[k] = round;
            }
        }
    }
}

// Path-halving walk from every previous root to its new root.  The hook
// graph is acyclic, so a walk ends within n_roots steps; the step cap only
// turns an internal error into an error flag instead of an endless loop.
__global__ void k_jump(const uint32_t* __restrict__ roots2, const DevCounters* __restrict__ dc, uint32_t n,
                       uint32_t* __restrict__ par, uint32_t* __restrict__ err)
{
    const uint32_t total = dc->n_roots;
    const uint32_t* roots = roots2 + (size_t)dc->rpar * n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const uint32_t c = roots[i];
        uint32_t x = c;
        for (uint32_t step = 0;; ++step) {
            if (step > total) {
                atomicOr(err, 8u);
                break;
            }
            const uint32_t y = __ldcg(&par[x]);
            if (y == x) break;
            const uint32_t z = __ldcg(&par[y]);
            if (z == y) {
                x = y;
                break;
            }
            // Halve only if x still points at y: a plain store could overwrite
            // another thread's final par[x] = root with the stale ancestor z.
            atomicCAS(&par[x], y, z);
            x = z;
        }
        if (x != c) par[c] = x;
    }
}

__global__ void k_relabel(uint32_t n, uint32_t* __restrict__ lab, const uint32_t* __restrict__ par)
{
    uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) * 4;
    if (i + 3 < n) {
        uint4 l = *reinterpret_cast<uint4*>(lab + i);
        l.x = __ldcg(&par[l.x]);
        l.y = __ldcg(&par[l.y]);
        l.z = __ldcg(&par[l.z]);
        l.w = __ldcg(&par[l.w]);
        *reinterpret_cast<uint4*>(lab + i) = l;
    } else {
        for (; i < n; ++i) lab[i] = __ldcg(&par[lab[i]]);
    }
}

// Surviving roots of the current half go to the other half; the count
// of the current list was moved to s_roots by k_flatten_begin.
__global__ void k_compact_roots(uint32_t* __restrict__ roots2, DevCounters* dc, uint32_t n,
                                const uint32_t* __restrict__ par, uint64_t* __restrict__ ckey,
                                uint64_t* __restrict__ cmax, uint32_t* __restrict__ clb)
{
    const uint32_t total = dc->s_roots;
    const uint32_t* roots = roots2 + (size_t)dc->rpar * n;
    uint32_t* roots_next = roots2 + (size_t)(dc->rpar ^ 1u) * n;
    uint32_t* n_roots_next = &dc->n_roots;
    __shared__ uint32_t s_cnt[33];
    for (uint32_t base = blockIdx.x * blockDim.x; base < total; base += gridDim.x * blockDim.x) {
        const uint32_t i = base + threadIdx.x;
        bool keep = false;
        uint32_t c = 0;
        if (i < total) {
            c = roots[i];
            keep = par[c] == c;
            if (keep) {
                ckey[c] = kNoKey;
                cmax[c] = kNoKey;
                if (clb) clb[c] = 0x7f800000u;  // +inf
            }
        }
        const uint32_t slot = block_reserve(keep, n_roots_next, s_cnt);
        if (keep) roots_next[slot] = c;
    }
}

__global__ void k_count_other(uint32_t n, const uint32_t* __restrict__ lab, const uint32_t* __restrict__ pos0,
                              uint32_t* __restrict__ out)
{
    const uint32_t r0 = lab[*pos0];
    uint32_t cnt = 0;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) cnt += lab[i] != r0;
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(kFull, cnt, o);
    if ((threadIdx.x & 31) == 0 && cnt) atomicAdd(out, cnt);
}

template <int D>
__global__ void k_edge_len(const int32_t* __restrict__ edges, uint32_t ne, const float* __restrict__ in,
                           double* __restrict__ part)
{
    __shared__ double s[256 / 32];
    double acc = 0.0;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
        const int64_t u = edges[2 * (uint64_t)e], v = edges[2 * (uint64_t)e + 1];
        const float dx = __fsub_rn(in[u * D], in[v * D]);
        const float dy = __fsub_rn(in[u * D + 1], in[v * D + 1]);
        const float dz = D == 3 ? __fsub_rn(in[u * D + 2], in[v * D + 2]) : 0.f;
        acc += sqrt((double)d2_of<D>(dx, dy, dz));
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int j = 0; j < (int)(blockDim.x / 32); ++j) t += s[j];
        part[blockIdx.x] = t;
    }
}

// One block sums the per-block partials in a fixed order (deterministic).
__global__ void __launch_bounds__(1024) k_sum_parts(const double* __restrict__ part, int nb, double* __restrict__ out)
{
    __shared__ double s[32];
    double t = 0.0;
    for (int j = threadIdx.x; j < nb; j += blockDim.x) t += part[j];
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(kFull, t, o);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = t;
    __syncthreads();
    if (threadIdx.x < 32) {
        t = threadIdx.x < (blockDim.x >> 5) ? s[threadIdx.x] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(kFull, t, o);
        if (threadIdx.x == 0) *out = t;
    }
}

__global__ void k_labels_out(uint32_t n, const uint32_t* __restrict__ lab, const uint32_t* __restrict__ perm,
                             int32_t* __restrict__ out)
{
    uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    out[perm[p]] = (int32_t)perm[lab[p]];
}

unsigned list_grid(uint64_t upper)
{
    uint64_t b = (upper + 255) / 256;
    if (b < 1) b = 1;
    if (b > 152ull * 16) b = 152ull * 16;
    return (unsigned)b;
}

}  // namespace

__global__ void k_flatten_begin(DevCounters* dc)
{
    dc->s_roots = dc->n_roots;
    dc->n_roots = 0;
}

__global__ void k_flatten_end(DevCounters* dc) { dc->rpar ^= 1u; }

// Start of a round: per-round counters to zero, round number + 1.
__global__ void k_round_tick(DevCounters* dc)
{
    dc->round += 1;
    dc->n_dirty = 0;
    dc->n_dirty2 = 0;
    dc->n_prov = 0;
}

// End of a round (after the flatten): record the cumulative edge count and
// decide, on the device, whether another round runs.  The round cap bounds
// the loop whatever the data.
__global__ void k_round_end(DevCounters* dc, int64_t* cum, int max_rounds, cudaGraphConditionalHandle h)
{
    const int r = dc->round;
    if (r >= 1 && r <= 128) cum[r - 1] = dc->n_edges;
    const bool progress = dc->n_edges != dc->prev_edges;
    dc->prev_edges = dc->n_edges;
    const bool more = dc->err == 0 && dc->n_roots > dc->n_target && progress && r < max_rounds;
    cudaGraphSetConditional(h, more ? 1u : 0u);
}

cudaError_t boruvka_init(Ctx& c)
{
    cudaError_t e;
    const size_t n = (size_t)c.n;
    if ((e = c.ensure(c.lab, n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.par, n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.selq, n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.selkey, n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.ckey, n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.cmax, n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.act, n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.act2, n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.roots, 2 * n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.dcum, 128)) != cudaSuccess) return e;
    if ((e = c.ensure(c.prov, n)) != cudaSuccess) return e;
    if ((e = c.ensure(c.edges, 2 * (n > 1 ? n - 1 : 1))) != cudaSuccess) return e;
    if ((e = c.ensure(c.eround, n > 1 ? n - 1 : 1)) != cudaSuccess) return e;
    k_init<<<blocks_for(c.n, 256), 256, 0, c.stream>>>((uint32_t)c.n, c.lab.p, c.par.p, c.roots.p, c.act.p,
                                                        c.ckey.p, c.cmax.p);
    c.n_act = (uint32_t)c.n;
    c.n_roots = (uint32_t)c.n;
    c.launches++;
    return cudaGetLastError();
}

cudaError_t boruvka_flatten(Ctx& c)
{
    DevCounters* d = c.ctr.p;
    const uint32_t n = (uint32_t)c.n;
    k_jump<<<list_grid(c.n_roots), 256, 0, c.stream>>>(c.roots.p, d, n, c.par.p, &d->err);
    if (c.search_mode == 0) {
        // component search: the relabel also writes the next round's node labels
        cudaError_t e = node_labels_of(c, c.lab.p, c.nlab.p, c.par.p);
        if (e != cudaSuccess) return e;
        c.launches--;  // counted below with the relabel
    } else {
        k_relabel<<<blocks_for((c.n + 3) / 4, 256), 256, 0, c.stream>>>(n, c.lab.p, c.par.p);
    }
    k_flatten_begin<<<1, 1, 0, c.stream>>>(d);
    k_compact_roots<<<list_grid(c.n_roots), 256, 0, c.stream>>>(c.roots.p, d, n, c.par.p, c.ckey.p, c.cmax.p,
                                                                c.search_mode == 0 && c.clb_used() ? c.clb.p
                                                                                                    : nullptr);
    k_flatten_end<<<1, 1, 0, c.stream>>>(d);
    c.launches += 5;
    return cudaGetLastError();
}

cudaError_t round_tick(Ctx& c)
{
    k_round_tick<<<1, 1, 0, c.stream>>>(c.ctr.p);
    c.launches++;
    return cudaGetLastError();
}

cudaError_t round_end(Ctx& c, cudaGraphConditionalHandle h)
{
    k_round_end<<<1, 1, 0, c.stream>>>(c.ctr.p, c.dcum.p, c.max_rounds, h);
    c.launches++;
    return cudaGetLastError();
}

cudaError_t boruvka_select(Ctx& c)
{
    DevCounters* d = c.ctr.p;
    cudaMemcpyAsync(&d->s_act, &d->n_act, sizeof(uint32_t), cudaMemcpyDeviceToDevice, c.stream);
    cudaMemsetAsync(&d->n_act, 0, sizeof(uint32_t), c.stream);
    cudaMemsetAsync(&d->n_prov, 0, sizeof(uint32_t), c.stream);
    const unsigned g = list_grid(c.n_act);
    if (c.dim == 2)
        k_select<8><<<g, 256, 0, c.stream>>>(c.act.p, &d->s_act, c.cand.p, c.cnt.p, c.cur.p, c.zflag.p, c.lab.p,
                                             c.perm.p, c.ckey.p, c.selq.p, c.selkey.p, c.act2.p, &d->n_act,
                                             c.prov.p, &d->n_prov);
    else
        k_select<24><<<g, 256, 0, c.stream>>>(c.act.p, &d->s_act, c.cand.p, c.cnt.p, c.cur.p, c.zflag.p, c.lab.p,
                                              c.perm.p, c.ckey.p, c.selq.p, c.selkey.p, c.act2.p, &d->n_act,
                                              c.prov.p, &d->n_prov);
    std::swap(c.act.p, c.act2.p);
    c.launches++;
    return cudaGetLastError();
}

cudaError_t boruvka_resolve(Ctx& c)
{
    DevCounters* d = c.ctr.p;
    // the round-1 list build (component search) fills the winner slots itself
    const int* skip = (c.search_mode == 0 && c.knn_seed && !c.cnns_warp) ? &d->round : nullptr;
    k_resolve<<<list_grid(c.n_act), 256, 0, c.stream>>>(c.prov.p, &d->n_prov, c.lab.p, c.perm.p, c.ckey.p, c.selq.p,
                                                         c.selkey.p, c.cmax.p, skip);
    c.launches++;
    return cudaGetLastError();
}

cudaError_t boruvka_hook(Ctx& c)
{
    DevCounters* d = c.ctr.p;
    k_hook<<<list_grid(c.n_roots), 256, 0, c.stream>>>(c.roots.p, d, c.lab.p, c.perm.p, c.ckey.p, c.cmax.p, c.selq.p,
                                                       c.par.p, c.edges.p, c.eround.p, &d->n_edges, (uint32_t)c.n,
                                                       &d->err);
    c.launches++;
    return cudaGetLastError();
}

cudaError_t boruvka_count_other(Ctx& c)
{
    DevCounters* d = c.ctr.p;
    cudaMemsetAsync(&d->n_other, 0, sizeof(uint32_t), c.stream);
    k_count_other<<<list_grid(c.n), 256, 0, c.stream>>>((uint32_t)c.n, c.lab.p, &d->pos0, &d->n_other);
    c.launches++;
    return cudaGetLastError();
}

cudaError_t evaluate_length(Ctx& c, double* d_out)
{
    cudaError_t e;
    const unsigned nb = list_grid(c.n_edges ? c.n_edges : 1);
    if ((e = c.ensure(c.lpart, nb)) != cudaSuccess) return e;
    if (c.dim == 2)
        k_edge_len<2><<<nb, 256, 0, c.stream>>>(c.edges.p, c.n_edges, c.in, c.lpart.p);
    else
        k_edge_len<3><<<nb, 256, 0, c.stream>>>(c.edges.p, c.n_edges, c.in, c.lpart.p);
    k_sum_parts<<<1, 1024, 0, c.stream>>>(c.lpart.p, (int)nb, d_out);
    c.launches += 2;
    return cudaGetLastError();
}

cudaError_t labels_to_input_order(Ctx& c, int32_t* d_out, const uint32_t* src)
{
    k_labels_out<<<blocks_for(c.n, 256), 256, 0, c.stream>>>((uint32_t)c.n, src ? src : c.lab.p, c.perm.p, d_out);
    c.launches++;
    return cudaGetLastError();
}

// Labels after the round that just ended (rounds 1..cap), for the per-round
// forests (EMSF): snapshot r-1 holds the flattened roots after round r.
__global__ void k_snapshot(uint32_t n, const uint32_t* __restrict__ lab, const DevCounters* dc, uint32_t cap,
                           uint32_t* __restrict__ snaps)
{
    const int r = dc->round;
    if (r < 1 || (uint32_t)r > cap) return;
    uint32_t* out = snaps + (size_t)(r - 1) * n;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) out[i] = lab[i];
}

cudaError_t snapshot_labels(Ctx& c)
{
    if (!c.snap_cap) return cudaSuccess;
    const unsigned b = (unsigned)std::min<int64_t>(blocks_for(c.n, 256), (int64_t)c.sms * 8);
    k_snapshot<<<b ? b : 1, 256, 0, c.stream>>>((uint32_t)c.n, c.lab.p, c.ctr.p, (uint32_t)c.snap_cap, c.snaps.p);
    c.launches++;
    return cudaGetLastError();
}

}  // namespace emst
