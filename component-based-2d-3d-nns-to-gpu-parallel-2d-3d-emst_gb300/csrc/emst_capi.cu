// emst_capi.cu -- the C ABI (include/emst.h) and the host-side round driver.
//
// The operator sequence and its stage checks follow SolutionEMST::activate
// (emst_coalition/src/SolutionEMSTOperators.cu:156-422): flatten, termination
// test, iteration++, find-min-1 (computeOctants + findNextClosestPoint),
// find-min-2 (component min pair), connect-and-union; the loop stops when one
// component remains or at the 100-round cap (:210).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <utility>
#include <vector>

#include "../../include/emst.h"
#include "emst_ctx.h"
#include "proposal.cuh"

// timed phases: the operators, then the two search kernels
enum { PH_GRID = 0, PH_OCTANTS, PH_SELECT, PH_RESOLVE, PH_HOOK, PH_FLATTEN, PH_KNN, PH_SEARCH, PH_COUNT };

struct emst_ctx {
    emst::Ctx c;
    int stage = 0;  // 0: needs flatten, 1: flattened, 2: octants, 3: next-closest, 4: min-pair
    int64_t last_edges = 0;
    emst::DevBuf<int32_t> tmp_i32;
    emst::DevBuf<float> tmp_f32;
    // phase timing: (phase, start, end) event pairs recorded since the last sync
    struct Pending {
        int phase;
        cudaEvent_t a, b;
    };
    std::vector<Pending> pending;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> pool;
    double ms[PH_COUNT] = {};
    std::pair<cudaEvent_t, cudaEvent_t> open[2] = {};  // kernel timer: started, not yet ended
    // the whole round loop as one CUDA graph (conditional WHILE node)
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    std::vector<const void*> gkey;
    int64_t body_launches = 0;
    emst_tuning tuning = {};  // the last emst_autotune's stages
    // emst_solve: the edge list's copy to the host runs here beside the length kernel
    cudaStream_t side = nullptr;
    cudaEvent_t side_ev = nullptr;
};

namespace {

using emst::Ctx;


// An event pair from the context's pool (created on demand); {null, null} on failure.
std::pair<cudaEvent_t, cudaEvent_t> take_events(emst_ctx* x)
{
    if (x->pool.empty()) {
        cudaEvent_t e0, e1;
        if (cudaEventCreate(&e0) != cudaSuccess) return {nullptr, nullptr};
        if (cudaEventCreate(&e1) != cudaSuccess) {
            cudaEventDestroy(e0);
            return {nullptr, nullptr};
        }
        x->pool.push_back({e0, e1});
    }
    auto p = x->pool.back();
    x->pool.pop_back();
    return p;
}

// Records CUDA events around one operator on the context's stream.
struct Timed {
    emst_ctx* x;
    int ph;
    cudaEvent_t a = nullptr, b = nullptr;
    Timed(emst_ctx* x_, int ph_) : x(x_), ph(ph_)
    {
        if (!x->c.profile) return;
        auto p = take_events(x);
        a = p.first;
        b = p.second;
        if (a) cudaEventRecord(a, x->c.stream);
    }
    ~Timed()
    {
        if (!a) return;
        cudaEventRecord(b, x->c.stream);
        x->pending.push_back({ph, a, b});
    }
};

// Events around one search-kernel launch (Ctx::kernel_timer): which 0 = the
// round-1 neighbour-list kernel, 1 = the component search.
void kernel_timer_cb(void* owner, int which, bool begin)
{
    emst_ctx* x = static_cast<emst_ctx*>(owner);
    auto& o = x->open[which];
    if (begin) {
        o = take_events(x);
        if (o.first) cudaEventRecord(o.first, x->c.stream);
    } else if (o.first) {
        cudaEventRecord(o.second, x->c.stream);
        x->pending.push_back({PH_KNN + which, o.first, o.second});
        o = {nullptr, nullptr};
    }
}

// After a stream synchronisation: fold the recorded phase times in.
void harvest(emst_ctx* x)
{
    for (auto& p : x->pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) x->ms[p.phase] += ms;
        x->pool.push_back({p.a, p.b});
    }
    x->pending.clear();
    cudaGetLastError();
}

emst_status set_err(emst_ctx* x, emst_status st, const std::string& msg)
{
    if (x) x->c.err = msg;
    return st;
}

emst_status cuda_err(emst_ctx* x, cudaError_t e, const char* where)
{
    if (e == cudaSuccess) return EMST_OK;
    cudaGetLastError();  // clear a sticky launch error where possible
    return set_err(x, e == cudaErrorMemoryAllocation ? EMST_ENOMEM : EMST_ECUDA,
                   std::string(where) + ": " + cudaGetErrorString(e));
}

#define EMST_CUDA(x, call, where)                                  \
    do {                                                           \
        cudaError_t _e = (call);                                   \
        if (_e != cudaSuccess) return cuda_err((x), _e, (where));  \
    } while (0)

emst_status read_counters(emst_ctx* x)
{
    Ctx& c = x->c;
    EMST_CUDA(x, cudaMemcpyAsync(c.hctr, c.ctr.p, sizeof(emst::DevCounters), cudaMemcpyDeviceToHost, c.stream),
              "counters");
    EMST_CUDA(x, cudaStreamSynchronize(c.stream), "sync");
    harvest(x);
    c.n_act = c.hctr->n_act;
    c.n_roots = c.hctr->n_roots;
    c.n_zero = c.hctr->n_zero_next;
    c.n_edges = c.hctr->n_edges;
    if (c.hctr->err & 1u) return set_err(x, EMST_EINVAL, "non-finite input coordinate");
    if (c.hctr->err) return set_err(x, EMST_ECUDA, "internal consistency check failed (flags " +
                                               std::to_string(c.hctr->err) + ")");
    return EMST_OK;
}

emst_status check_ready(emst_ctx* x)
{
    if (!x) return EMST_EINVAL;
    if (x->c.phase == 0) return set_err(x, EMST_ESTATE, "emst_initialize has not been called");
    EMST_CUDA(x, cudaSetDevice(x->c.device), "cudaSetDevice");
    return EMST_OK;
}

emst_status do_flatten(emst_ctx* x)
{
    Ctx& c = x->c;
    if (x->stage != 0) return set_err(x, EMST_ESTATE, "flatten: previous round not finished");
    if (c.round > 0) {
        Timed t(x, PH_FLATTEN);
        EMST_CUDA(x, emst::boruvka_flatten(c), "flatten");
        EMST_CUDA(x, emst::snapshot_labels(c), "snapshot");
    }
    emst_status st = read_counters(x);
    if (st != EMST_OK) return st;
    if (c.round > (int)c.cum_edges.size()) c.cum_edges.push_back(c.n_edges);
    x->stage = 1;
    return EMST_OK;
}

emst_status do_octants(emst_ctx* x)
{
    Ctx& c = x->c;
    if (x->stage != 1) return set_err(x, EMST_ESTATE, "compute_octants: call flatten first");
    c.round++;
    Timed t(x, PH_OCTANTS);
    EMST_CUDA(x, emst::round_tick(c), "round tick");
    // (component search: nothing to do here -- the node labels it prunes with
    // were written by the last flatten, or by the initialisation before round 1)
    if (c.search_mode == 1) {
        if (c.round == 1)
            EMST_CUDA(x, emst::nns_full(c), "compute_octants");
        else
            EMST_CUDA(x, emst::nns_recompute_zero(c), "compute_octants (zero recompute)");
    }
    x->stage = 2;
    return EMST_OK;
}

emst_status do_select(emst_ctx* x)
{
    if (x->stage != 2) return set_err(x, EMST_ESTATE, "find_next_closest: call compute_octants first");
    Timed t(x, PH_SELECT);
    if (x->c.search_mode == 0)
        EMST_CUDA(x, emst::cnns_select(x->c), "find_next_closest");
    else if (x->c.search_mode == 3)
        EMST_CUDA(x, emst::dyn_select(x->c), "find_next_closest");
    else
        EMST_CUDA(x, emst::boruvka_select(x->c), "find_next_closest");
    x->stage = 3;
    return EMST_OK;
}

emst_status do_resolve(emst_ctx* x)
{
    if (x->stage != 3) return set_err(x, EMST_ESTATE, "find_min_pair: call find_next_closest first");
    Timed t(x, PH_RESOLVE);
    EMST_CUDA(x, emst::boruvka_resolve(x->c), "find_min_pair");
    x->stage = 4;
    return EMST_OK;
}

emst_status do_hook(emst_ctx* x)
{
    if (x->stage != 4) return set_err(x, EMST_ESTATE, "connect_union: call find_min_pair first");
    Timed t(x, PH_HOOK);
    EMST_CUDA(x, emst::boruvka_hook(x->c), "connect_union");
    x->stage = 0;
    return EMST_OK;
}

emst_status do_activate(emst_ctx* x, int* more)
{
    Ctx& c = x->c;
    *more = 0;
    if (c.finished) return EMST_OK;
    emst_status st = do_flatten(x);
    if (st != EMST_OK) return st;
    if (c.n_roots <= (uint32_t)c.n_nonempty) {
        c.finished = true;
        x->stage = 0;
        return EMST_OK;
    }
    if (c.round > 0 && (int64_t)c.n_edges == x->last_edges) {
        c.finished = true;
        x->stage = 0;
        return set_err(x, EMST_ENOCONVERGE, "a round added no edge while several components remain");
    }
    if (c.round == c.max_rounds) {
        c.finished = true;
        x->stage = 0;
        return set_err(x, EMST_ENOCONVERGE, "round cap reached");
    }
    x->last_edges = c.n_edges;
    if ((st = do_octants(x)) != EMST_OK) return st;
    if ((st = do_select(x)) != EMST_OK) return st;
    if ((st = do_resolve(x)) != EMST_OK) return st;
    if ((st = do_hook(x)) != EMST_OK) return st;
    *more = 1;
    return EMST_OK;
}

emst_status do_initialize(emst_ctx* x, const float* points, int64_t n, int dim, int is_device)
{
    Ctx& c = x->c;
    if (!points) return set_err(x, EMST_EINVAL, "points is NULL");
    if (dim != 2 && dim != 3) return set_err(x, EMST_EINVAL, "dim must be 2 or 3");
    if (n < 1) return set_err(x, EMST_EINVAL, "n must be >= 1");
    if (n >= (int64_t)0x7fffffff) return set_err(x, EMST_EOVERFLOW, "n must be < 2^31 - 1");
    EMST_CUDA(x, cudaSetDevice(c.device), "cudaSetDevice");
    if (!is_device) {
        EMST_CUDA(x, c.ensure(c.in_own, (size_t)n * dim), "alloc points");
        EMST_CUDA(x, cudaMemcpyAsync(c.in_own.p, points, sizeof(float) * n * dim, cudaMemcpyHostToDevice, c.stream),
                  "upload points");
        c.in = c.in_own.p;
    } else {
        c.in = points;
    }
    c.n = n;
    c.dim = dim;
    c.K = dim == 2 ? 8 : 24;
    std::memset(c.hctr, 0, sizeof(emst::DevCounters));
    c.hctr->n_act = (uint32_t)n;
    c.hctr->n_roots = (uint32_t)n;
    c.hctr->n_target = 1;
    c.n_clouds = 0;
    c.n_nonempty = 1;
    EMST_CUDA(x, cudaMemcpyAsync(c.ctr.p, c.hctr, sizeof(emst::DevCounters), cudaMemcpyHostToDevice, c.stream),
              "counters");
    c.launches = 0;
    c.nns_launches = 0;
    c.knn_timed = 0;
    c.search_timed = 0;
    if (c.profile) {
        EMST_CUDA(x, c.ensure(c.nstats, emst::kNumStats), "alloc");
        EMST_CUDA(x, cudaMemsetAsync(c.nstats.p, 0, emst::kNumStats * sizeof(unsigned long long), c.stream), "stats");
    }
    c.snap_cap = 0;
    if (c.snap_rounds > 0) {
        EMST_CUDA(x, c.ensure(c.snaps, (size_t)c.snap_rounds * n), "alloc snapshots");
        c.snap_cap = c.snap_rounds;
    }
    for (double& v : x->ms) v = 0.0;
    {
        Timed t(x, PH_GRID);
        EMST_CUDA(x, emst::grid_build(c), "grid build");
        EMST_CUDA(x, emst::boruvka_init(c), "init");
        if (c.search_mode == 0) EMST_CUDA(x, emst::cnns_init(c), "init");
        if (c.search_mode == 3) EMST_CUDA(x, emst::dyn_init(c), "init");
    }
    c.round = 0;
    c.finished = false;
    c.n_edges = 0;
    c.n_zero = 0;
    c.cum_edges.clear();
    c.phase = 1;
    x->stage = 0;
    x->last_edges = 0;
    return EMST_OK;
}

void drop_graph(emst_ctx* x)
{
    if (x->gexec) cudaGraphExecDestroy(x->gexec);
    if (x->graph) cudaGraphDestroy(x->graph);
    x->gexec = nullptr;
    x->graph = nullptr;
    x->gkey.clear();
}

// One round of the component search, in stream order (captured once).
emst_status enqueue_round(emst_ctx* x, cudaGraphConditionalHandle h)
{
    Ctx& c = x->c;
    EMST_CUDA(x, emst::round_tick(c), "round tick");
    EMST_CUDA(x, emst::cnns_select(c), "find_next_closest");
    EMST_CUDA(x, emst::boruvka_resolve(c), "find_min_pair");
    EMST_CUDA(x, emst::boruvka_hook(c), "connect_union");
    EMST_CUDA(x, emst::boruvka_flatten(c), "flatten");
    EMST_CUDA(x, emst::snapshot_labels(c), "snapshot");
    EMST_CUDA(x, emst::round_end(c, h), "round end");
    return EMST_OK;
}

// Build (or reuse) the graph: a WHILE node whose body is one round; the
// round-end kernel sets the condition on the device, so the whole loop runs
// without a host round trip.  The body is captured on the context's own
// stream (the caller's stream may be the legacy default stream).
emst_status build_graph(emst_ctx* x)
{
    Ctx& c = x->c;
    std::vector<const void*> key = {(const void*)(intptr_t)c.n, (const void*)(intptr_t)c.dim, c.in, c.sp.p,
                                    c.lab.p, c.roots.p, c.edges.p, c.nlab.p, c.lbp.p, c.prov.p,
                                    c.dirty.p, c.perm.p, c.selq.p, c.ckey.p, c.nlo.p, c.dflag.p,
                                    (const void*)(intptr_t)emst::search_shape_of(c), c.pfrag.p,
                                    (const void*)(intptr_t)(c.learned ? 1 : 0), c.trace.p,
                                    (const void*)(intptr_t)c.trace_cap, (const void*)(intptr_t)c.trace_shift,
                                    (const void*)(intptr_t)c.n_clouds, c.pcloud.p, c.ncloud.p, c.snaps.p,
                                    (const void*)(intptr_t)c.snap_cap, c.klist.p, c.kcur.p, c.iperm.p,
                                    (const void*)(intptr_t)(c.knn_seed ? 1 : 0), (const void*)(intptr_t)c.knn_k,
                                    (const void*)(intptr_t)c.wide_limit, (const void*)(intptr_t)c.coop_min};
    if (x->gexec && key == x->gkey) return EMST_OK;
    drop_graph(x);
    cudaGraph_t g = nullptr, body = nullptr;
    cudaGraphConditionalHandle h;
    cudaGraphNode_t node;
    EMST_CUDA(x, cudaGraphCreate(&g, 0), "graph");
    x->graph = g;
    EMST_CUDA(x, cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault), "graph handle");
    cudaGraphNodeParams cp = {};
    cp.type = cudaGraphNodeTypeConditional;
    cp.conditional.handle = h;
    cp.conditional.type = cudaGraphCondTypeWhile;
    cp.conditional.size = 1;
    EMST_CUDA(x, cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &cp), "graph node");
    body = cp.conditional.phGraph_out[0];
    cudaStream_t work = c.stream;
    const uint32_t save_roots = c.n_roots, save_act = c.n_act;
    const int64_t save_launches = c.launches;
    c.stream = c.own_stream;
    c.n_roots = (uint32_t)c.n;  // grid sizes: upper bounds (every kernel reads its count on the device)
    c.n_act = (uint32_t)c.n;
    cudaError_t e = cudaStreamBeginCaptureToGraph(c.stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeRelaxed);
    emst_status st = e == cudaSuccess ? enqueue_round(x, h) : cuda_err(x, e, "begin capture");
    cudaGraph_t captured = nullptr;
    cudaError_t e2 = cudaStreamEndCapture(c.stream, &captured);
    c.stream = work;
    c.n_roots = save_roots;
    c.n_act = save_act;
    x->body_launches = c.launches - save_launches;
    c.launches = save_launches;
    if (st != EMST_OK) return st;
    EMST_CUDA(x, e2, "end capture");
    EMST_CUDA(x, cudaGraphInstantiate(&x->gexec, g, 0), "graph instantiate");
    x->gkey = key;
    return EMST_OK;
}

emst_status run_graph(emst_ctx* x)
{
    Ctx& c = x->c;
    emst_status st = read_counters(x);
    if (st != EMST_OK) return st;
    if (c.n_roots > (uint32_t)c.n_nonempty) {
        if ((st = build_graph(x)) != EMST_OK) return st;
        EMST_CUDA(x, cudaGraphLaunch(x->gexec, c.stream), "graph launch");
        if ((st = read_counters(x)) != EMST_OK) return st;
        c.round = c.hctr->round;
        c.launches += (int64_t)c.round * x->body_launches;
        c.nns_launches += 2 * (int64_t)c.round;
        int64_t cum[128];
        const int r = c.round < 128 ? c.round : 128;
        if (r > 0) {
            EMST_CUDA(x, cudaMemcpyAsync(cum, c.dcum.p, sizeof(int64_t) * r, cudaMemcpyDeviceToHost, c.stream),
                      "round stats");
            EMST_CUDA(x, cudaStreamSynchronize(c.stream), "sync");
        }
        c.cum_edges.assign(cum, cum + r);
    }
    c.finished = true;
    x->stage = 0;
    if (c.n_roots > (uint32_t)c.n_nonempty) {
        if (c.round >= c.max_rounds) return set_err(x, EMST_ENOCONVERGE, "round cap reached");
        return set_err(x, EMST_ENOCONVERGE, "a round added no edge while several components remain");
    }
    return EMST_OK;
}

emst_status do_run(emst_ctx* x)
{
    Ctx& c = x->c;
    if (c.search_mode == 0 && !c.cnns_warp && c.use_graph && !c.profile && c.round == 0 && x->stage == 0)
        return run_graph(x);
    int more = 1;
    while (more) {
        emst_status st = do_activate(x, &more);
        if (st != EMST_OK) return st;
    }
    return EMST_OK;
}

}  // namespace

extern "C" {

emst_status emst_create(const emst_config* cfg, emst_ctx** out)
{
    if (!out) return EMST_EINVAL;
    *out = nullptr;
    emst_ctx* x = new (std::nothrow) emst_ctx();
    if (!x) return EMST_ENOMEM;
    Ctx& c = x->c;
    if (cfg) {
        c.device = cfg->device;
        if (cfg->max_rounds > 0) c.max_rounds = cfg->max_rounds;
        if (cfg->warps_per_block > 0) c.warps_per_block = cfg->warps_per_block;
        c.keep_table = cfg->keep_region_table != 0;
        c.profile = cfg->profile != 0;
        if (cfg->search_mode < 0 || cfg->search_mode > 3) {
            delete x;
            return EMST_EINVAL;
        }
        c.search_mode = (cfg->search_mode == 1 || c.keep_table) ? 1 : (cfg->search_mode == 3 ? 3 : 0);
        c.cnns_warp = cfg->search_mode == 2;
        c.use_graph = cfg->host_rounds == 0;
        if (cfg->search_shape > 0) c.search_shape = cfg->search_shape - 1;
        if (cfg->first_pass_factor > 0.f) c.first_pass_factor = cfg->first_pass_factor;
        c.first_pass_ordered = cfg->first_pass_ordered != 0;
        c.knn_seed = cfg->round1_neighbours >= 0;
        bool ok = cfg->round1_neighbours == 0 || cfg->round1_neighbours == -1;
        for (int k = 0; k < emst::kNumKnnLengths; ++k) ok = ok || cfg->round1_neighbours == emst::kKnnLengths[k];
        if (!ok || cfg->wide_search < -1 || cfg->wide_search > 2) {
            delete x;
            return EMST_EINVAL;
        }
        if (cfg->round1_neighbours > 0) c.knn_k = cfg->round1_neighbours;
        if (cfg->min_find < 0 || cfg->min_find > 1 || (cfg->min_find == 1 && c.search_mode != 3)) {
            delete x;
            return EMST_EINVAL;
        }
        c.min_find = cfg->min_find;
        c.search_split = cfg->wide_search;
        if (cfg->wide_max_list > 0) c.wide_limit = cfg->wide_max_list;
        if (cfg->coop_min_list > 0) c.coop_min = cfg->coop_min_list;
    }
    if (c.profile) {
        c.kernel_timer = kernel_timer_cb;
        c.timer_owner = x;
    }
    cudaError_t e = cudaSetDevice(c.device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&c.sms, cudaDevAttrMultiProcessorCount, c.device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c.own_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = c.ensure(c.ctr, 1);
    if (e == cudaSuccess) e = c.ensure(c.dlen, 1);
    if (e == cudaSuccess) e = cudaMallocHost(&c.hctr, sizeof(emst::DevCounters));
    if (e == cudaSuccess) e = cudaMallocHost(&c.hlen, sizeof(double));
    if (e != cudaSuccess) {
        emst_destroy(x);
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? EMST_ENOMEM : EMST_ECUDA;
    }
    c.stream = c.own_stream;
    *out = x;
    return EMST_OK;
}

emst_status emst_destroy(emst_ctx* x)
{
    if (!x) return EMST_OK;
    Ctx& c = x->c;
    cudaSetDevice(c.device);
    if (c.stream) cudaStreamSynchronize(c.stream);
    emst::release(c.in_own);
    emst::release(c.scaled);
    emst::release(c.sp);
    emst::release(c.perm);
    emst::release(c.perm_alt);
    emst::release(c.mkey);
    emst::release(c.mkey_alt);
    emst::release(c.sort_tmp);
    emst::release(c.part);
    emst::release(c.norm);
    emst::release(c.nlo);
    emst::release(c.nhi);
    emst::release(c.nid);
    emst::release(c.nstats);
    emst::release(c.nlab);
    emst::release(c.dirty);
    emst::release(c.dirty2);
    emst::release(c.dflag);
    emst::release(c.sel_tiles);
    emst::release(c.dyn_pos);
    emst::release(c.dyn_start);
    emst::release(c.dyn_closed);
    emst::release(c.dyn_flag);
    emst::release(c.dyn_dp);
    emst::release(c.dyn_rkey);
    emst::release(c.dyn_best);
    emst::release(c.pfrag);
    emst::release(c.trace);
    emst::release(c.trace_ctl);
    emst::release(c.snaps);
    emst::release(c.klist);
    emst::release(c.iperm);
    emst::release(c.kcur);
    emst::release(c.lbp);
    emst::release(c.clb);
    emst::release(c.d_off);
    emst::release(c.d_foff);
    emst::release(c.d_eoff);
    emst::release(c.d_dims);
    emst::release(c.stage);
    emst::release(c.pcloud_in);
    emst::release(c.pcloud);
    emst::release(c.ncloud);
    emst::release(c.bcursor);
    emst::release(c.bedges);
    emst::release(c.cand);
    emst::release(c.cnt);
    emst::release(c.cur);
    emst::release(c.zflag);
    emst::release(c.tab_id);
    emst::release(c.tab_d2);
    emst::release(c.lab);
    emst::release(c.par);
    emst::release(c.selq);
    emst::release(c.ckey);
    emst::release(c.cmax);
    emst::release(c.selkey);
    emst::release(c.act);
    emst::release(c.act2);
    emst::release(c.roots);
    emst::release(c.dcum);
    emst::release(c.prov);
    emst::release(c.zero);
    emst::release(c.zero2);
    emst::release(c.edges);
    emst::release(c.eround);
    emst::release(c.ctr);
    emst::release(c.lpart);
    emst::release(c.dlen);
    emst::release(x->tmp_i32);
    emst::release(x->tmp_f32);
    for (auto& p : x->pending) x->pool.push_back({p.a, p.b});
    for (auto& p : x->pool) {
        cudaEventDestroy(p.first);
        cudaEventDestroy(p.second);
    }
    if (c.hctr) cudaFreeHost(c.hctr);
    if (c.hlen) cudaFreeHost(c.hlen);
    drop_graph(x);
    if (x->side) cudaStreamDestroy(x->side);
    if (x->side_ev) cudaEventDestroy(x->side_ev);
    if (c.own_stream) cudaStreamDestroy(c.own_stream);
    delete x;
    return EMST_OK;
}

const char* emst_last_error(const emst_ctx* x) { return x ? x->c.err.c_str() : "null context"; }

emst_status emst_set_stream(emst_ctx* x, void* stream)
{
    if (!x) return EMST_EINVAL;
    x->c.stream = stream == EMST_OWN_STREAM ? x->c.own_stream : (cudaStream_t)stream;  // NULL: legacy default
    return EMST_OK;
}

emst_status emst_initialize(emst_ctx* x, const float* points, int64_t n, int dim, int points_are_device)
{
    if (!x) return EMST_EINVAL;
    return do_initialize(x, points, n, dim, points_are_device);
}

emst_status emst_compute_octants(emst_ctx* x)
{
    emst_status st = check_ready(x);
    return st != EMST_OK ? st : do_octants(x);
}

emst_status emst_find_next_closest(emst_ctx* x)
{
    emst_status st = check_ready(x);
    return st != EMST_OK ? st : do_select(x);
}

emst_status emst_find_min_pair(emst_ctx* x)
{
    emst_status st = check_ready(x);
    return st != EMST_OK ? st : do_resolve(x);
}

emst_status emst_connect_union(emst_ctx* x)
{
    emst_status st = check_ready(x);
    return st != EMST_OK ? st : do_hook(x);
}

emst_status emst_flatten(emst_ctx* x)
{
    emst_status st = check_ready(x);
    return st != EMST_OK ? st : do_flatten(x);
}

emst_status emst_test_termination(emst_ctx* x, int64_t* n_other)
{
    emst_status st = check_ready(x);
    if (st != EMST_OK) return st;
    if (!n_other) return set_err(x, EMST_EINVAL, "n_other is NULL");
    if (x->stage != 1) return set_err(x, EMST_ESTATE, "test_termination: call flatten first");
    EMST_CUDA(x, emst::boruvka_count_other(x->c), "test_termination");
    if ((st = read_counters(x)) != EMST_OK) return st;
    *n_other = x->c.hctr->n_other;
    return EMST_OK;
}

emst_status emst_activate(emst_ctx* x, int* more)
{
    emst_status st = check_ready(x);
    if (st != EMST_OK) return st;
    int m = 0;
    st = do_activate(x, &m);
    if (more) *more = m;
    return st;
}

emst_status emst_run(emst_ctx* x)
{
    emst_status st = check_ready(x);
    return st != EMST_OK ? st : do_run(x);
}

emst_status emst_evaluate(emst_ctx* x, int64_t* n_edges, double* length)
{
    emst_status st = check_ready(x);
    if (st != EMST_OK) return st;
    Ctx& c = x->c;
    if ((st = read_counters(x)) != EMST_OK) return st;
    EMST_CUDA(x, emst::evaluate_length(c, c.dlen.p), "evaluate");
    EMST_CUDA(x, cudaMemcpyAsync(c.hlen, c.dlen.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream), "evaluate");
    EMST_CUDA(x, cudaStreamSynchronize(c.stream), "evaluate");
    if (n_edges) *n_edges = c.n_edges;
    if (length) *length = *c.hlen;
    return EMST_OK;
}

emst_status emst_get_edges(emst_ctx* x, int32_t* uv, int32_t* round_of_edge, int64_t cap, int64_t* n_edges)
{
    emst_status st = check_ready(x);
    if (st != EMST_OK) return st;
    Ctx& c = x->c;
    if ((st = read_counters(x)) != EMST_OK) return st;
    if (n_edges) *n_edges = c.n_edges;
    int64_t m = c.n_edges < (uint64_t)cap ? (int64_t)c.n_edges : cap;
    if (m > 0 && uv)
        EMST_CUDA(x, cudaMemcpyAsync(uv, c.edges.p, sizeof(int32_t) * 2 * m, cudaMemcpyDeviceToHost, c.stream),
                  "get_edges");
    if (m > 0 && round_of_edge)
        EMST_CUDA(x, cudaMemcpyAsync(round_of_edge, c.eround.p, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, c.stream),
                  "get_edges");
    EMST_CUDA(x, cudaStreamSynchronize(c.stream), "get_edges");
    if (cap < (int64_t)c.n_edges) return set_err(x, EMST_EOVERFLOW, "edge buffer too small");
    return EMST_OK;
}

emst_status emst_get_labels(emst_ctx* x, int32_t* labels, int64_t cap)
{
    emst_status st = check_ready(x);
    if (st != EMST_OK) return st;
    Ctx& c = x->c;
    if (!labels || cap < c.n) return set_err(x, EMST_EOVERFLOW, "labels buffer too small");
    EMST_CUDA(x, x->c.ensure(x->tmp_i32, (size_t)c.n), "alloc");
    EMST_CUDA(x, emst::labels_to_input_order(c, x->tmp_i32.p), "labels");
    EMST_CUDA(x, cudaMemcpyAsync(labels, x->tmp_i32.p, sizeof(int32_t) * c.n, cudaMemcpyDeviceToHost, c.stream),
              "labels");
    EMST_CUDA(x, cudaStreamSynchronize(c.stream), "labels");
    return EMST_OK;
}

emst_status emst_get_round_stats(emst_ctx* x, int64_t* rounds, int64_t* cum_edges, int64_t cap)
{
    emst_status st = check_ready(x);
    if (st != EMST_OK) return st;
    const auto& v = x->c.cum_edges;
    if (rounds) *rounds = (int64_t)v.size();
    for (int64_t i = 0; cum_edges && i < cap && i < (int64_t)v.size(); ++i) cum_edges[i] = v[i];
    return EMST_OK;
}

emst_status emst_get_region_table(emst_ctx* x, int32_t* ids, float* d2, int64_t cap)
{
    emst_status st = check_ready(x);
    if (st != EMST_OK) return st;
    Ctx& c = x->c;
    if (!c.keep_table) return set_err(x, EMST_ESTATE, "context created without keep_region_table");
    if (c.round < 1) return set_err(x, EMST_ESTATE, "compute_octants has not run");
    const int64_t m = c.n * c.K;
    if (cap < m) return set_err(x, EMST_EOVERFLOW, "table buffer too small");
    if (ids) EMST_CUDA(x, cudaMemcpyAsync(ids, c.tab_id.p, sizeof(int32_t) * m, cudaMemcpyDeviceToHost, c.stream), "table");
    if (d2) EMST_CUDA(x, cudaMemcpyAsync(d2, c.tab_d2.p, sizeof(float) * m, cudaMemcpyDeviceToHost, c.stream), "table");
    EMST_CUDA(x, cudaStreamSynchronize(c.stream), "table");
    return EMST_OK;
}

emst_status emst_get_neighbour_lists(emst_ctx* x, int32_t* ids, float* d2, int64_t cap, int* k)
{
    emst_status st = check_ready(x);
    if (st != EMST_OK) return st;
    Ctx& c = x->c;
    if (c.search_mode != 0 || c.cnns_warp || !c.knn_seed || !c.klist.p)
        return set_err(x, EMST_ESTATE, "no neighbour lists: they come from the component search with round1_neighbours >= 0");
    if (c.round < 1) return set_err(x, EMST_ESTATE, "find_next_closest has not run");
    const int kk = c.knn_k;
    if (k) *k = kk;
    const int64_t n = c.n, m = n * kk;
    if (!ids && !d2) return EMST_OK;  // the list length only
    if (cap < m) return set_err(x, EMST_EOVERFLOW, "list buffer too small");
    // entries hold leaf positions; a position's input id is its point's w
    std::vector<uint64_t> lst((size_t)m);
    std::vector<float4> pts((size_t)n);
    EMST_CUDA(x, cudaMemcpyAsync(lst.data(), c.klist.p, sizeof(uint64_t) * m, cudaMemcpyDeviceToHost, c.stream), "lists");
    EMST_CUDA(x, cudaMemcpyAsync(pts.data(), c.sp.p, sizeof(float4) * n, cudaMemcpyDeviceToHost, c.stream), "lists");
    EMST_CUDA(x, cudaStreamSynchronize(c.stream), "lists");
    for (int64_t pos = 0; pos < n; ++pos) {
        int32_t id;
        std::memcpy(&id, &pts[(size_t)pos].w, sizeof(id));
        for (int j = 0; j < kk; ++j) {
            const uint64_t e = lst[(size_t)j * n + pos];
            const size_t o = (size_t)id * kk + j;
            if (e == ~0ull) {
                if (ids) ids[o] = -1;
                if (d2) d2[o] = INFINITY;
                continue;
            }
            const uint32_t q = (uint32_t)e, bits = (uint32_t)(e >> 32);
            if (ids) std::memcpy(&ids[o], &pts[q].w, sizeof(int32_t));
            if (d2) std::memcpy(&d2[o], &bits, sizeof(float));
        }
    }
    return EMST_OK;
}

emst_status emst_get_profile(emst_ctx* x, emst_profile* out)
{
    emst_status st = check_ready(x);
    if (st != EMST_OK) return st;
    if (!out) return set_err(x, EMST_EINVAL, "out is NULL");
    EMST_CUDA(x, cudaStreamSynchronize(x->c.stream), "sync");
    harvest(x);
    std::memset(out, 0, sizeof(*out));
    out->ms_grid = x->ms[PH_GRID];
    out->ms_octants = x->ms[PH_OCTANTS];
    out->ms_select = x->ms[PH_SELECT];
    out->ms_resolve = x->ms[PH_RESOLVE];
    out->ms_hook = x->ms[PH_HOOK];
    out->ms_flatten = x->ms[PH_FLATTEN];
    out->ms_knn = x->ms[PH_KNN];
    out->ms_search = x->ms[PH_SEARCH];
    out->knn_launches = x->c.knn_timed;
    out->search_launches = x->c.search_timed;
    out->launches = x->c.launches;
    out->octant_launches = x->c.nns_launches;
    out->rounds = x->c.round;
    if (x->c.profile && x->c.nstats.p) {
        unsigned long long st[emst::kNumStats];
        EMST_CUDA(x, cudaMemcpy(st, x->c.nstats.p, sizeof(st), cudaMemcpyDeviceToHost), "stats");
        out->knn_marked = (int64_t)st[8];
        out->knn_insert_steps = (int64_t)st[9];
        out->knn_learned = (int64_t)st[10];
        out->knn_resumed = (int64_t)st[11];
        out->first_pass_searches = (int64_t)st[5];
        out->first_pass_resumed = (int64_t)st[6];
        out->first_pass_deferred = (int64_t)st[7];
        out->leaf_visits = (int64_t)st[0];
        out->node_tests = (int64_t)st[1];
        out->candidates = (int64_t)st[2];
        out->search_warps = (int64_t)st[3];
        out->search_queries = (int64_t)st[4];
    }
    return EMST_OK;
}

emst_status emst_keep_round_labels(emst_ctx* x, int rounds)
{
    if (!x || rounds < 0 || rounds > 100) return EMST_EINVAL;
    x->c.snap_rounds = rounds;  // takes effect from the next initialize / solve
    return EMST_OK;
}

emst_status emst_get_round_labels(emst_ctx* x, int round, int32_t* labels, int64_t cap)
{
    emst_status st = check_ready(x);
    if (st != EMST_OK) return st;
    Ctx& c = x->c;
    if (c.n_clouds) return set_err(x, EMST_EINVAL, "the context holds a batch of clouds");
    if (round < 1 || round > (int)c.cum_edges.size()) return set_err(x, EMST_EINVAL, "no such round");
    if (round > c.snap_cap) return set_err(x, EMST_EINVAL, "round labels not kept (emst_keep_round_labels)");
    if (!labels || cap < c.n) return set_err(x, EMST_EOVERFLOW, "labels buffer too small");
    EMST_CUDA(x, x->c.ensure(x->tmp_i32, (size_t)c.n), "alloc");
    EMST_CUDA(x, emst::labels_to_input_order(c, x->tmp_i32.p, c.snaps.p + (size_t)(round - 1) * c.n), "labels");
    EMST_CUDA(x, cudaMemcpyAsync(labels, x->tmp_i32.p, sizeof(int32_t) * c.n, cudaMemcpyDeviceToHost, c.stream),
              "labels");
    EMST_CUDA(x, cudaStreamSynchronize(c.stream), "labels");
    return EMST_OK;
}

emst_status emst_get_size(emst_ctx* x, int64_t* n, int* dim)
{
    emst_status st = check_ready(x);
    if (st != EMST_OK) return st;
    if (x->c.n_clouds) return set_err(x, EMST_EINVAL, "the context holds a batch of clouds");
    if (n) *n = x->c.n;
    if (dim) *dim = x->c.dim;
    return EMST_OK;
}

emst_status emst_get_rescaled(emst_ctx* x, float* out, double* unit_x, int64_t cap)
{
    emst_status st = check_ready(x);
    if (st != EMST_OK) return st;
    Ctx& c = x->c;
    if (out) {
        if (cap < c.n * c.dim) return set_err(x, EMST_EOVERFLOW, "buffer too small");
        EMST_CUDA(x, cudaMemcpyAsync(out, c.scaled.p, sizeof(float) * c.n * c.dim, cudaMemcpyDeviceToHost, c.stream),
                  "rescaled");
    }
    emst::NormParams np;
    EMST_CUDA(x, cudaMemcpyAsync(&np, c.norm.p, sizeof(np), cudaMemcpyDeviceToHost, c.stream), "rescaled");
    EMST_CUDA(x, cudaStreamSynchronize(c.stream), "rescaled");
    if (unit_x) *unit_x = np.unitx;
    return EMST_OK;
}

emst_status emst_solve(emst_ctx* x, const float* points, int64_t n, int dim, int32_t* uv, int64_t* n_edges,
                       double* length)
{
    if (!x) return EMST_EINVAL;
    emst_status st = do_initialize(x, points, n, dim, 0);
    if (st != EMST_OK) return st;
    if ((st = do_run(x)) != EMST_OK) return st;
    if ((st = read_counters(x)) != EMST_OK) return st;
    Ctx& c = x->c;
    const int64_t ne = (int64_t)c.n_edges;
    if (n_edges) *n_edges = ne;
    if (uv && ne > (n > 1 ? n - 1 : 0)) return set_err(x, EMST_EOVERFLOW, "edge buffer too small");
    // The edge list goes to the host on a second stream while the length
    // kernel runs on the context's stream (both only read the edges); one
    // wait for both.
    const bool copy = uv && ne > 0;
    if (copy) {
        if (!x->side) EMST_CUDA(x, cudaStreamCreateWithFlags(&x->side, cudaStreamNonBlocking), "stream");
        if (!x->side_ev) EMST_CUDA(x, cudaEventCreateWithFlags(&x->side_ev, cudaEventDisableTiming), "event");
        EMST_CUDA(x, cudaEventRecord(x->side_ev, c.stream), "event");
        EMST_CUDA(x, cudaStreamWaitEvent(x->side, x->side_ev, 0), "event");
        EMST_CUDA(x, cudaMemcpyAsync(uv, c.edges.p, sizeof(int32_t) * 2 * ne, cudaMemcpyDeviceToHost, x->side),
                  "get_edges");
    }
    if (length) {
        EMST_CUDA(x, emst::evaluate_length(c, c.dlen.p), "evaluate");
        EMST_CUDA(x, cudaMemcpyAsync(c.hlen, c.dlen.p, sizeof(double), cudaMemcpyDeviceToHost, c.stream), "evaluate");
    }
    EMST_CUDA(x, cudaStreamSynchronize(c.stream), "sync");
    if (copy) EMST_CUDA(x, cudaStreamSynchronize(x->side), "sync");
    if (length) *length = *c.hlen;
    return EMST_OK;
}

emst_status emst_solve_batch(emst_ctx* x, const float* points, const int64_t* point_offsets, const int32_t* dims,
                             int32_t n_clouds, int32_t* uv, double* lengths, int64_t* n_edges)
{
    if (!x) return EMST_EINVAL;
    Ctx& c = x->c;
    if (!points || !point_offsets || !dims || n_clouds < 1) return set_err(x, EMST_EINVAL, "bad batch arguments");
    if (n_clouds > (1 << 16)) return set_err(x, EMST_EOVERFLOW, "at most 65536 clouds");
    if (c.search_mode != 0 || c.cnns_warp)
        return set_err(x, EMST_EINVAL, "batches run in the component search mode (search_mode 0)");
    std::vector<int64_t> foff(n_clouds + 1), eoff(n_clouds + 1);
    foff[0] = 0;
    eoff[0] = 0;
    int64_t nonempty = 0;
    if (point_offsets[0] != 0) return set_err(x, EMST_EINVAL, "point_offsets[0] must be 0");
    for (int i = 0; i < n_clouds; ++i) {
        const int64_t m = point_offsets[i + 1] - point_offsets[i];
        if (m < 0) return set_err(x, EMST_EINVAL, "point_offsets must not decrease");
        if (dims[i] != 2 && dims[i] != 3) return set_err(x, EMST_EINVAL, "dims must be 2 or 3");
        foff[i + 1] = foff[i] + m * dims[i];
        eoff[i + 1] = eoff[i] + (m > 0 ? m - 1 : 0);
        nonempty += m > 0;
    }
    const int64_t n = point_offsets[n_clouds];
    if (n >= (int64_t)0x7fffffff) return set_err(x, EMST_EOVERFLOW, "total points must be < 2^31 - 1");
    EMST_CUDA(x, cudaSetDevice(c.device), "cudaSetDevice");
    if (n_edges) *n_edges = eoff[n_clouds];
    if (n == 0) {
        for (int i = 0; lengths && i < n_clouds; ++i) lengths[i] = 0.0;
        return EMST_OK;
    }
    EMST_CUDA(x, c.ensure(c.in_own, (size_t)foff[n_clouds]), "alloc points");
    EMST_CUDA(x, c.ensure(c.d_off, (size_t)n_clouds + 1), "alloc");
    EMST_CUDA(x, c.ensure(c.d_foff, (size_t)n_clouds + 1), "alloc");
    EMST_CUDA(x, c.ensure(c.d_eoff, (size_t)n_clouds + 1), "alloc");
    EMST_CUDA(x, c.ensure(c.d_dims, (size_t)n_clouds), "alloc");
    EMST_CUDA(x, c.ensure(c.dlen, (size_t)n_clouds), "alloc");
    EMST_CUDA(x, x->c.ensure(x->tmp_i32, (size_t)2 * (eoff[n_clouds] > 0 ? eoff[n_clouds] : 1)), "alloc");
    cudaStream_t s = c.stream;
    EMST_CUDA(x, cudaMemcpyAsync(c.in_own.p, points, sizeof(float) * foff[n_clouds], cudaMemcpyHostToDevice, s),
              "upload");
    EMST_CUDA(x, cudaMemcpyAsync(c.d_off.p, point_offsets, sizeof(int64_t) * (n_clouds + 1), cudaMemcpyHostToDevice, s),
              "upload");
    EMST_CUDA(x, cudaMemcpyAsync(c.d_foff.p, foff.data(), sizeof(int64_t) * (n_clouds + 1), cudaMemcpyHostToDevice, s),
              "upload");
    EMST_CUDA(x, cudaMemcpyAsync(c.d_eoff.p, eoff.data(), sizeof(int64_t) * (n_clouds + 1), cudaMemcpyHostToDevice, s),
              "upload");
    EMST_CUDA(x, cudaMemcpyAsync(c.d_dims.p, dims, sizeof(int32_t) * n_clouds, cudaMemcpyHostToDevice, s), "upload");
    c.in = c.in_own.p;
    c.n = n;
    c.snap_cap = 0;  // per-round labels are kept for single-cloud solves only
    c.dim = 3;  // 2D clouds carry z = 0 (fma(0, 0, r) == r keeps their distances 2D)
    c.K = 24;
    c.n_clouds = n_clouds;
    c.n_nonempty = nonempty;
    std::memset(c.hctr, 0, sizeof(emst::DevCounters));
    c.hctr->n_act = (uint32_t)n;
    c.hctr->n_roots = (uint32_t)n;
    c.hctr->n_target = (uint32_t)nonempty;
    EMST_CUDA(x, cudaMemcpyAsync(c.ctr.p, c.hctr, sizeof(emst::DevCounters), cudaMemcpyHostToDevice, s), "counters");
    c.launches = 0;
    c.nns_launches = 0;
    c.knn_timed = 0;
    c.search_timed = 0;
    for (double& v : x->ms) v = 0.0;
    if (c.profile) {
        EMST_CUDA(x, c.ensure(c.nstats, emst::kNumStats), "alloc");
        EMST_CUDA(x, cudaMemsetAsync(c.nstats.p, 0, emst::kNumStats * sizeof(unsigned long long), s), "stats");
    }
    {
        Timed t(x, PH_GRID);
        EMST_CUDA(x, emst::batch_grid_build(c), "batch grid build");
        EMST_CUDA(x, emst::boruvka_init(c), "init");
        EMST_CUDA(x, emst::cnns_init(c), "init");
    }
    c.round = 0;
    c.finished = false;
    c.n_edges = 0;
    c.n_zero = 0;
    c.cum_edges.clear();
    c.phase = 1;
    x->stage = 0;
    x->last_edges = 0;
    emst_status st = do_run(x);
    if (st != EMST_OK) return st;
    if ((int64_t)c.n_edges != eoff[n_clouds])
        return set_err(x, EMST_ECUDA, "batch edge count mismatch: " + std::to_string(c.n_edges) + " edges, expected " +
                                          std::to_string(eoff[n_clouds]) + " after " + std::to_string(c.round) +
                                          " rounds, " + std::to_string(c.n_roots) + " components");
    EMST_CUDA(x, emst::batch_output(c, x->tmp_i32.p, c.dlen.p), "batch output");
    if (uv && eoff[n_clouds] > 0)
        EMST_CUDA(x, cudaMemcpyAsync(uv, x->tmp_i32.p, sizeof(int32_t) * 2 * eoff[n_clouds], cudaMemcpyDeviceToHost, s),
                  "download");
    if (lengths)
        EMST_CUDA(x, cudaMemcpyAsync(lengths, c.dlen.p, sizeof(double) * n_clouds, cudaMemcpyDeviceToHost, s),
                  "download");
    return read_counters(x);
}

emst_status emst_set_proposal(emst_ctx* x, const float* weights, float margin, float threshold)
{
    if (!x) return EMST_EINVAL;
    Ctx& c = x->c;
    if (!weights) {
        c.learned = false;
        return EMST_OK;
    }
    if (c.search_mode != 0 || c.cnns_warp)
        return set_err(x, EMST_EINVAL, "the learned proposal drives the component search (search_mode 0)");
    if (!(margin >= 0.f && margin <= 64.f)) return set_err(x, EMST_EINVAL, "margin must be in [0, 64]");
    if (!std::isfinite(threshold)) return set_err(x, EMST_EINVAL, "threshold must be finite");
    for (int i = 0; i < emst::prop::kNumWeights; ++i)
        if (!std::isfinite(weights[i])) return set_err(x, EMST_EINVAL, "non-finite proposal weight");
    EMST_CUDA(x, cudaSetDevice(c.device), "cudaSetDevice");
    EMST_CUDA(x, c.ensure(c.pfrag, emst::proposal_frag_bytes()), "alloc");
    EMST_CUDA(x, x->c.ensure(x->tmp_f32, (size_t)emst::prop::kNumWeights), "alloc");
    EMST_CUDA(x, cudaMemcpyAsync(x->tmp_f32.p, weights, sizeof(float) * emst::prop::kNumWeights,
                                 cudaMemcpyHostToDevice, c.stream), "upload");
    EMST_CUDA(x, emst::proposal_pack(x->tmp_f32.p, c.pfrag.p, c.stream), "pack");
    EMST_CUDA(x, cudaStreamSynchronize(c.stream), "sync");
    c.learned = true;
    c.margin = margin;
    c.threshold = threshold;
    return EMST_OK;
}

emst_status emst_trace_enable(emst_ctx* x, int64_t capacity, int sample_shift)
{
    if (!x || capacity < 0 || capacity > 0xfffffff0ll || sample_shift < 0 || sample_shift > 24) return EMST_EINVAL;
    Ctx& c = x->c;
    if (capacity > 0 && (c.search_mode != 0 || c.cnns_warp))
        return set_err(x, EMST_EINVAL, "traces come from the component search (search_mode 0)");
    EMST_CUDA(x, cudaSetDevice(c.device), "cudaSetDevice");
    c.trace_cap = capacity;
    c.trace_shift = sample_shift;
    if (capacity == 0) return EMST_OK;
    EMST_CUDA(x, c.ensure(c.trace, (size_t)capacity * emst::prop::kRec), "alloc trace");
    EMST_CUDA(x, c.ensure(c.trace_ctl, 2), "alloc");
    EMST_CUDA(x, cudaMemsetAsync(c.trace_ctl.p, 0, 2 * sizeof(uint32_t), c.stream), "trace reset");
    return EMST_OK;
}

emst_status emst_get_trace(emst_ctx* x, float* records, int64_t cap, int64_t* count)
{
    if (!x || !count) return EMST_EINVAL;
    Ctx& c = x->c;
    *count = 0;
    if (c.trace_cap == 0) return EMST_OK;
    uint32_t ctl[2] = {0, 0};
    EMST_CUDA(x, cudaMemcpyAsync(ctl, c.trace_ctl.p, sizeof(ctl), cudaMemcpyDeviceToHost, c.stream), "trace count");
    EMST_CUDA(x, cudaStreamSynchronize(c.stream), "sync");
    const int64_t have = std::min<int64_t>((int64_t)ctl[0], c.trace_cap);
    *count = have;
    if (records && cap > 0 && have > 0)
        EMST_CUDA(x, cudaMemcpy(records, c.trace.p, sizeof(float) * emst::prop::kRec * std::min(have, cap),
                                cudaMemcpyDeviceToHost), "trace download");
    return EMST_OK;
}

emst_status emst_get_trace_device(emst_ctx* x, const float** d_records, int64_t* count)
{
    if (!x || !d_records) return EMST_EINVAL;
    *d_records = x->c.trace.p;
    return emst_get_trace(x, nullptr, 0, count);
}

emst_status emst_search_shape_info(int* count, int* threads, int* min_blocks, int cap)
{
    if (count) *count = emst::kNumSearchShapes;
    for (int k = 0; k < emst::kNumSearchShapes && k < cap; ++k) {
        if (threads) threads[k] = emst::kSearchShapes[k].threads;
        if (min_blocks) min_blocks[k] = emst::kSearchShapes[k].min_blocks;
    }
    return EMST_OK;
}

emst_status emst_get_search_shape(emst_ctx* x, int* search_shape)
{
    if (!x || !search_shape) return EMST_EINVAL;
    *search_shape = x->c.search_shape >= 0 ? x->c.search_shape + 1 : 0;
    return EMST_OK;
}

// Candidate values of the autotuner's stages (emst_tuning).
constexpr uint32_t kTuneCoop[4] = {50000u, 150000u, 400000u, emst::kNoCoop};
constexpr uint32_t kTuneWide[3] = {16384u, 65536u, 150000u};

emst_status emst_autotune(emst_ctx* x, const float* points, int64_t n, int dim, int* best, double* ms, int cap)
{
    if (!x) return EMST_EINVAL;
    Ctx& c = x->c;
    if (c.search_mode != 0 || c.cnns_warp)
        return set_err(x, EMST_EINVAL, "the autotuner tunes the component search (search_mode 0)");
    if (!points || n < 2) return set_err(x, EMST_EINVAL, "the autotuner needs at least two host points");
    EMST_CUDA(x, cudaSetDevice(c.device), "cudaSetDevice");
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    EMST_CUDA(x, cudaEventCreate(&e0), "event");
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return set_err(x, EMST_ECUDA, "event");
    }
    emst_status st = EMST_OK;
    // best of two timed solves (after one warm-up solve, which also builds the
    // graph) with the context's current settings
    auto time_solve = [&](double& out) {
        double t = 1e300;
        for (int rep = 0; rep < 3 && st == EMST_OK; ++rep) {
            if ((st = do_initialize(x, points, n, dim, 0)) != EMST_OK) break;
            cudaEventRecord(e0, c.stream);
            if ((st = do_run(x)) != EMST_OK) break;
            cudaEventRecord(e1, c.stream);
            if (cudaEventSynchronize(e1) != cudaSuccess) {
                st = set_err(x, EMST_ECUDA, "autotune timing");
                break;
            }
            float el = 0.f;
            cudaEventElapsedTime(&el, e0, e1);
            if (rep > 0 && el < t) t = el;
        }
        out = t;
    };
    auto argmin = [](const double* v, int m) {
        int b = 0;
        for (int i = 1; i < m; ++i)
            if (v[i] < v[b]) b = i;
        return b;
    };
    emst_tuning& tu = x->tuning;
    std::memset(&tu, 0, sizeof(tu));
    for (int k = 0; k < emst::kNumKnnLengths; ++k) tu.knn_k_values[k] = emst::kKnnLengths[k];
    for (int k = 0; k < 4; ++k) tu.coop_min_values[k] = kTuneCoop[k];
    for (int k = 0; k < 3; ++k) tu.wide_max_values[k] = kTuneWide[k];
    // Coordinate descent, the stages that move a solve most first: the
    // round-1 list length (lists on, no learned proposal -- it is trained for
    // the default length), the list-length thresholds of the search kernels
    // (split by length only), the thread-per-query launch shape.
    if (c.knn_seed && !c.learned) {
        for (int k = 0; k < emst::kNumKnnLengths && st == EMST_OK; ++k) {
            c.knn_k = emst::kKnnLengths[k];
            time_solve(tu.ms_knn_k[k]);
        }
        if (st == EMST_OK) c.knn_k = emst::kKnnLengths[argmin(tu.ms_knn_k, emst::kNumKnnLengths)];
    }
    if (c.search_split == 0) {
        for (int k = 0; k < 4 && st == EMST_OK; ++k) {
            c.coop_min = kTuneCoop[k];
            time_solve(tu.ms_coop_min[k]);
        }
        if (st == EMST_OK) c.coop_min = kTuneCoop[argmin(tu.ms_coop_min, 4)];
        for (int k = 0; k < 3 && st == EMST_OK; ++k) {
            c.wide_limit = kTuneWide[k];
            time_solve(tu.ms_wide_max[k]);
        }
        if (st == EMST_OK) c.wide_limit = kTuneWide[argmin(tu.ms_wide_max, 3)];
    }
    for (int k = 0; k < emst::kNumSearchShapes && st == EMST_OK; ++k) {
        c.search_shape = k;
        time_solve(tu.ms_shape[k]);
        if (ms && k < cap) ms[k] = tu.ms_shape[k];
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st != EMST_OK) return st;
    const int best_k = argmin(tu.ms_shape, emst::kNumSearchShapes);
    c.search_shape = best_k;
    if (best) *best = best_k + 1;
    return EMST_OK;
}

emst_status emst_get_tuning(emst_ctx* x, emst_tuning* out)
{
    if (!x || !out) return EMST_EINVAL;
    *out = x->tuning;
    out->knn_k = x->c.knn_seed ? x->c.knn_k : 0;
    out->coop_min = x->c.coop_min;
    out->wide_max = x->c.wide_limit;
    out->search_shape = emst::search_shape_of(x->c) + 1;
    return EMST_OK;
}

emst_status emst_solve_device(emst_ctx* x, const float* d_points, int64_t n, int dim, int32_t* d_uv,
                              double* d_length, int64_t* n_edges)
{
    if (!x) return EMST_EINVAL;
    emst_status st = do_initialize(x, d_points, n, dim, 1);
    if (st != EMST_OK) return st;
    if ((st = do_run(x)) != EMST_OK) return st;
    Ctx& c = x->c;
    if (d_length) EMST_CUDA(x, emst::evaluate_length(c, d_length), "evaluate");
    if (x->c.profile) {
        EMST_CUDA(x, cudaStreamSynchronize(c.stream), "sync");
        harvest(x);
    }
    if (d_uv && c.n_edges)
        EMST_CUDA(x, cudaMemcpyAsync(d_uv, c.edges.p, sizeof(int32_t) * 2 * c.n_edges, cudaMemcpyDeviceToDevice,
                                     c.stream),
                  "edges");
    if (n_edges) *n_edges = c.n_edges;
    return EMST_OK;
}

}  // extern "C"
