// emst_ctx.h -- host-side context of the EMST library and the launchers that
// the C ABI (emst_capi.cu) drives.
//
// HBM layout (all arrays indexed by position in leaf order unless noted):
//   in        n*dim float   caller's points, input order (original frame)
//   scaled    n*dim float   rescaled points, input order
//   sp        n float4      rescaled points in leaf (Hilbert) order, .w = input id
//   perm      n uint32      leaf position -> input id
//   nlo/nhi   2L float4     bounding boxes of the implicit leaf tree (heap order)
//   nid       2L int4       per node: two smallest input ids and their leaf positions
//   cand      n*K uint64    per point: region nearest neighbours, deduplicated and
//                           sorted by (d2, input id); (d2 bits << 32) | leaf position
//   cnt/cur   n uint8       list length / first entry not yet known to be inside
//   zflag     n uint8       list holds a zero-distance entry (recompute next round)
//   lab       n uint32      component root (leaf position) of every point
//   par       n uint32      union-find parent, meaningful for roots
//   ckey      n uint64      per root: (d2 bits << 32) | min input id of its best edge
//   cmax      n uint64      per root: (max input id << 32) | winner leaf position
//   selq      n uint32      per point: selected partner this round
//   selkey    n uint64      per point: selected edge key this round
//   act/roots/prov/zero     work lists (leaf positions)
//   edges     2(n-1) int32  output edges (input ids, u < v); eround: round per edge
#pragma once
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/emst.h"

namespace emst {

// Neighbours kept per point by round 1 (k_knn_first) to answer later rounds:
// the default, and the lengths the list build is compiled for (the autotuner
// picks one per context).
constexpr int kKnn = EMST_ROUND1_NEIGHBOURS;
constexpr int kNumKnnLengths = 4;
constexpr int kKnnLengths[kNumKnnLengths] = {4, 5, 6, 8};
constexpr int kKnnWarps = 8;  // warps per block of k_knn_first
constexpr int kKnnDense = 16;  // k_cnns_c: lanes wanting a leaf above which all lanes test all its points
constexpr int kKnnDenseFirst = 11;  // the same for k_knn_first (packed marking; swept 8, 11, 16)
constexpr int kWideWarps = 8;  // warps per block of k_cnns_w
constexpr int kWideFan = 5;    // k_cnns_w: levels a traversal step descends (32 nodes, one per lane)
// longest query list k_cnns_w takes (warp per query); longer lists fill the GPU
// thread per query (k_cnns_t).  Measured at 10^7 points: 5.6k queries 0.06 vs
// 0.41 ms, 94k queries 0.42 vs 0.37 ms
constexpr uint32_t kWideLimit = 65536;
// shortest query list k_cnns_c takes: rounds where enough points of a leaf
// search that a warp's 32 queries walk mostly the same nodes.  Swept (profile
// solves of gauss3d_1e7 / bezier2d_1e7): 150k 18.30 / 13.37 ms, 400k 18.50 /
// 13.43, 10^6 18.57 / 13.51
constexpr uint32_t kCoopMin = 150000;
constexpr uint32_t kNoCoop = 0xffffffffu;

// Device-side counters.  n_act / n_roots hold the CURRENT list sizes between
// kernels; a kernel that rebuilds a list first has its input size copied to
// the matching s_* slot (stream-ordered), then appends into the live counter.
struct DevCounters {
    uint32_t n_act;
    uint32_t n_roots;
    uint32_t n_prov;
    uint32_t n_edges;
    uint32_t n_zero_next;
    uint32_t n_other;
    uint32_t err;
    uint32_t pos0;  // leaf position of input point 0
    uint32_t s_act;
    uint32_t s_roots;
    uint32_t n_dirty;
    uint32_t n_dirty2;
    uint32_t rpar;        // which half of the 2n roots buffer holds the current roots
    int32_t round;        // rounds started (device copy, read by k_hook)
    uint32_t prev_edges;  // edge count at the end of the previous round
    uint32_t n_target;    // components left when done (1, or the number of non-empty clouds)
};

struct NormParams {
    float pmin[3];
    float pmax[3];
    float uxf;       // float(unitX)
    float qscale;    // cell quantisation scale
    double unitx;    // unitX as the reference computes it (double)
    float smax[3];   // rescaled maxima
    float pad;
};

template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;  // elements
};

struct Ctx {
    int device = 0;
    int max_rounds = 100;
    int warps_per_block = 4;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string err;

    int64_t n = 0;
    int dim = 0;
    int K = 0;
    int64_t nchunk = 0;
    int64_t L = 0;  // leaf slots (power of two >= nchunk)

    const float* in = nullptr;  // bound input (device)
    DevBuf<float> in_own;
    DevBuf<float> scaled;
    DevBuf<float4> sp;
    DevBuf<uint32_t> perm, perm_alt;
    DevBuf<uint64_t> mkey, mkey_alt;
    DevBuf<unsigned char> sort_tmp;  // radix sort scratch (radix_scratch_bytes)
    DevBuf<float> part;  // reduction partials
    DevBuf<NormParams> norm;
    DevBuf<float4> nlo, nhi;
    DevBuf<int4> nid;  // per node: two smallest input ids + leaf positions

    DevBuf<uint64_t> cand;
    DevBuf<unsigned char> cnt, cur, zflag;
    DevBuf<int32_t> tab_id;
    DevBuf<float> tab_d2;
    bool keep_table = false;

    DevBuf<uint32_t> lab, par, selq;
    DevBuf<uint64_t> ckey, cmax, selkey;
    DevBuf<uint32_t> act, act2, roots, prov, zero, zero2;  // roots: 2n, halves by DevCounters::rpar
    DevBuf<int64_t> dcum;                                  // per round: cumulative edges (device)
    uint32_t n_act = 0, n_roots = 0, n_zero = 0;
    DevBuf<int32_t> edges, eround;
    DevBuf<DevCounters> ctr;
    DevCounters* hctr = nullptr;  // pinned mirror
    DevBuf<double> lpart;
    DevBuf<double> dlen;
    double* hlen = nullptr;  // pinned

    // launch accounting (hand-written kernels) and optional phase timing
    int64_t launches = 0;
    int64_t nns_launches = 0;
    // profile mode: CUDA events around the search kernels' launches (which 0:
    // the round-1 neighbour-list kernel, 1: the component search), set by the
    // C ABI layer; null when not profiling
    void (*kernel_timer)(void* owner, int which, bool begin) = nullptr;
    void* timer_owner = nullptr;
    int64_t knn_timed = 0, search_timed = 0;  // launches timed
    bool profile = false;
    int search_mode = 0;      // 0: component search (cnns.cu), 1: static region table (nns.cu), 3: dynamic pruning (dyn.cu)
    bool cnns_warp = false;   // component search: warp per 32 queries instead of thread per query
    bool use_graph = true;    // component search: run the round loop as one CUDA graph
    int search_shape = -1;    // component search launch shape (kSearchShapes); -1: default for the dimension
    int sms = 152;            // multiprocessors of the device
    DevBuf<uint32_t> nlab;    // per node: component shared by all its points, or MIXED
    DevBuf<uint32_t> dirty, dirty2;  // points that search this round (first / second pass)
    DevBuf<unsigned char> dflag;     // per point: dirty flag (search pass)
    DevBuf<uint32_t> sel_tiles;      // query-list compaction: per tile counts / offsets
    DevBuf<float> lbp;               // per point: lower bound of d2 to its nearest outside point

    // batch of clouds (batch.cu)
    int n_clouds = 0;                // 0: single cloud
    int64_t n_nonempty = 1;          // components left at the end
    DevBuf<int64_t> d_off, d_foff, d_eoff;  // per cloud: first point, first float, first output edge row
    DevBuf<int32_t> d_dims;
    DevBuf<float4> stage;            // rescaled points in input order before the sort
    DevBuf<uint32_t> pcloud_in, pcloud;  // cloud of each point (input / leaf order)
    DevBuf<uint32_t> ncloud;             // per node: (first cloud << 16) | last cloud of its points
    DevBuf<uint32_t> bcursor, bedges;            // output scatter cursors, edges with global ids
    DevBuf<uint32_t> clb;            // per root: min lbp over its dirty points (float bits)
    DevBuf<unsigned long long> nstats;  // search counters (emst_profile), kNumStats entries

    // learned proposal (proposal.cuh): packed weights, radius margin (log2)
    bool learned = false;
    float margin = 1.f;
    // plain first pass: a point whose lower bound exceeds this factor times
    // its component's smallest waits for the second pass.  Default: none waits
    // (one pass); with the query lists compacted before each pass, deferring
    // measured slower on GB300 for every factor tried (1.0001 .. 16)
    float first_pass_factor = INFINITY;
    // The per-root smallest bound clb is read only by a finite first-pass
    // factor and by the warp search's deferral; otherwise no pass keeps it.
    bool clb_used() const { return cnns_warp || !std::isinf(first_pass_factor); }
    // round 1 keeps each point's knn_k nearest (k_knn_first); later rounds take
    // the first entry outside the component without a search (k_reuse)
    bool knn_seed = true;
    int knn_k = kKnn;
    // list lengths at which the search switches kernel: up to wide_limit warp
    // per query, above coop_min (and wide_limit) warp per 32 queries, thread
    // per query between (search_split 0)
    uint32_t wide_limit = kWideLimit;
    uint32_t coop_min = kCoopMin;
    // which kernel searches a round's query list: 0 by its length (k_cnns_w
    // for short lists, k_cnns_c for long ones, k_cnns_t between), -1 k_cnns_t
    // only, 1 k_cnns_w only, 2 k_cnns_c only
    int search_split = 0;
    // knn_k entries per point, entry-major (entry j of point p at j * n + p):
    // d2 bits << 32 | leaf position, sorted by (d2, input id); ~0 = no entry
    DevBuf<uint64_t> klist;
    DevBuf<unsigned char> kcur;  // per point: leading list entries known to lie in its component
    DevBuf<uint32_t> iperm;      // input id -> leaf position (the list build keeps ids, writes positions)
    // one search launch per round: the points the factor keeps first, the
    // others after them (instead of a second pass)
    bool first_pass_ordered = false;
    float threshold = 0.f;
    DevBuf<unsigned char> pfrag;
    // search traces for training: records of prop::kRec floats, 1 in 2^shift
    // first-pass queries; ctl = {records written, first record of the round}
    DevBuf<float> trace;
    int64_t trace_cap = 0;
    int trace_shift = 0;
    DevBuf<uint32_t> trace_ctl;
    // dynamic-pruning search (search_mode 3, dyn.cu): leaf positions grouped
    // by grid cell, each cell's first entry, per point and region the d2 of
    // the nearest own-component point met, per point the closed regions
    DevBuf<uint32_t> dyn_pos, dyn_start, dyn_closed, dyn_flag;
    DevBuf<float> dyn_dp;
    int dyn_dims[3] = {1, 1, 1};
    // per-component minimum: 0 packed atomicMin on the root's slot, 1 diffusion
    // over the forest's edges (search_mode 3; per point the key it reported
    // this round and the diffused minimum)
    int min_find = 0;
    DevBuf<uint64_t> dyn_rkey, dyn_best;
    // per-round labels (EMSF snapshots): rounds kept, buffer of snap_cap * n roots
    int snap_rounds = 0;
    int64_t snap_cap = 0;
    DevBuf<uint32_t> snaps;

    // every buffer is carved from caller-provided memory: ensure() fails
    // instead of allocating (the allocation-free entry point)
    bool no_alloc = false;
    template <typename T>
    cudaError_t ensure(DevBuf<T>& b, size_t n);

    int round = 0;        // rounds started
    int phase = 0;        // 0 = not initialised, 1 = initialised
    bool finished = false;
    bool octants_done = false;
    uint32_t n_edges = 0;
    std::vector<int64_t> cum_edges;
};

// grid.cu
cudaError_t grid_build(Ctx& c);
int grid_sort_end_bit(int dim);       // significant bits of the single-cloud cell keys
int grid_reduce_blocks(int64_t n);    // blocks of the min/max reduction (partials: 6 floats each)
cudaError_t leaf_tree(Ctx& c);
// batch.cu
cudaError_t batch_grid_build(Ctx& c);
cudaError_t batch_output(Ctx& c, int32_t* d_uv, double* d_len);
// nns.cu
cudaError_t nns_full(Ctx& c);
cudaError_t nns_recompute_zero(Ctx& c);
// boruvka.cu
cudaError_t boruvka_init(Ctx& c);
cudaError_t boruvka_flatten(Ctx& c);
cudaError_t boruvka_select(Ctx& c);
cudaError_t boruvka_resolve(Ctx& c);
cudaError_t boruvka_hook(Ctx& c);
cudaError_t boruvka_count_other(Ctx& c);
cudaError_t round_tick(Ctx& c);
cudaError_t round_end(Ctx& c, cudaGraphConditionalHandle h);
cudaError_t evaluate_length(Ctx& c, double* d_out);
cudaError_t labels_to_input_order(Ctx& c, int32_t* d_out, const uint32_t* src = nullptr);
cudaError_t snapshot_labels(Ctx& c);
cudaError_t table_to_host_order(Ctx& c);
// dyn.cu
cudaError_t dyn_init(Ctx& c);
cudaError_t dyn_select(Ctx& c);
// cnns.cu
cudaError_t cnns_init(Ctx& c);
cudaError_t cnns_node_labels(Ctx& c);
cudaError_t cnns_select(Ctx& c);
cudaError_t node_labels_of(Ctx& c, uint32_t* labels, uint32_t* out, const uint32_t* par = nullptr);

// Arguments of one component-search launch (cnns_search.cuh).
struct CnnsArgs {
    const float4* sp;      // (x, y, z, input id bits) in leaf order
    const uint32_t* perm;
    const float4* nlo;
    const float4* nhi;
    const uint32_t* nlab;
    uint32_t n, L;
    const uint32_t* list;
    const uint32_t* n_list;
    const uint32_t* lab;
    uint64_t* ckey;
    uint32_t* selq;
    uint64_t* selkey;
    uint32_t* prov;
    uint32_t* n_prov;
    float* lbp;
    const uint32_t* clb;
    int pass;
    unsigned char* dflag;
    const uint32_t* pcloud;
    const uint32_t* ncloud;
    unsigned long long* stats;
    const void* frag;  // learned proposal: fragment-ordered weights (prop::Frag), or null
    float margin;      // learned proposal: log2 factor on the predicted radius (d2)
    float threshold;   // learned proposal: gate logit at or above which the radius is used
    const int* round;  // rounds started (device)
    const uint32_t* list2;    // second segment of the same launch (ordered first pass), or null
    const uint32_t* n_list2;
    bool knn_round1;          // round 1 runs k_knn_first (neighbour lists), not this kernel
    // lists of at most this many queries go to k_cnns_w (warp per query), longer
    // ones to k_cnns_t (thread per query); 0: k_cnns_t only
    uint32_t wide_limit;
    // lists longer than this (and than wide_limit) go to k_cnns_c (warp per
    // 32 queries walking together); kNoCoop: never
    uint32_t coop_min;
    // neighbours kept per point by the round-1 list build (kKnnLengths)
    int knn_k;
    // training traces of the round-1 list build (null: off): records of
    // prop::kRec floats, ctl[0] counts them, 1 in (mask + 1) queries sampled
    float* trace;
    uint32_t* trace_ctl;
    uint64_t trace_cap;
    uint32_t trace_mask;
    // round-1 list build: per point the winner slot k_resolve would fill (the
    // component is the point alone, so its own result is the winner)
    uint64_t* cmax;
};

// Search counters of profile contexts (emst_profile): 0 leaves, 1 node tests,
// 2 candidates, 3 warps, 4 queries, 5 first-pass searches, 6 resumed, 7
// deferred; round-1 list build: 8 candidates marked, 9 insert steps (warp),
// 10 queries given a learned radius, 11 of those searched again.
constexpr int kNumStats = 12;


// Launch shapes of the component search: threads per block and the minimum
// number of resident blocks per SM the compiler must fit (which caps the
// registers per thread).  emst_autotune times them; the defaults per
// dimension are the fastest measured on GB300.
struct SearchShape {
    int threads, min_blocks;
};
constexpr int kNumSearchShapes = 6;
constexpr SearchShape kSearchShapes[kNumSearchShapes] = {{256, 4}, {256, 5}, {256, 6}, {128, 8}, {128, 12}, {512, 3}};

// Shape used by a context: its own choice, else the default for the dimension.
constexpr int kDefaultShape2 = 1, kDefaultShape3 = 1;
inline int search_shape_of(const Ctx& c)
{
    if (c.search_shape >= 0 && c.search_shape < kNumSearchShapes) return c.search_shape;
    return c.dim == 2 ? kDefaultShape2 : kDefaultShape3;
}

cudaError_t proposal_pack(const float* d_weights, void* d_frag, cudaStream_t s);
size_t proposal_frag_bytes();
uint64_t splitmix(uint64_t& s);

cudaError_t launch_knn_first2(const CnnsArgs& a, bool clouds, bool learned, uint64_t* klist, unsigned char* kcur,
                             const uint32_t* iperm, int sms, cudaStream_t s);
cudaError_t launch_knn_first3(const CnnsArgs& a, bool clouds, bool learned, uint64_t* klist, unsigned char* kcur,
                             const uint32_t* iperm, int sms, cudaStream_t s);
cudaError_t launch_cnns_t2(const CnnsArgs& a, bool clouds, int shape, int sms, cudaStream_t s);
cudaError_t launch_cnns_t3(const CnnsArgs& a, bool clouds, int shape, int sms, cudaStream_t s);

// Grows a context buffer to n elements.  A context built over caller-owned
// memory (Ctx::no_alloc) never frees or allocates: a buffer that is too small
// is an error, never a silent cudaMalloc.
template <typename T>
cudaError_t ensure(DevBuf<T>& b, size_t n, bool no_alloc)
{
    if (b.cap >= n && b.p) return cudaSuccess;
    if (no_alloc) return cudaErrorMemoryAllocation;
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
    size_t want = n < 1 ? 1 : n;
    cudaError_t e = cudaMalloc(&b.p, want * sizeof(T));
    if (e == cudaSuccess) b.cap = want;
    return e;
}

template <typename T>
cudaError_t Ctx::ensure(DevBuf<T>& b, size_t n)
{
    return emst::ensure(b, n, no_alloc);
}

template <typename T>
void release(DevBuf<T>& b)
{
    if (b.p) cudaFree(b.p);
    b.p = nullptr;
    b.cap = 0;
}

inline unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace emst
