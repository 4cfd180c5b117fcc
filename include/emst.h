/*
 * emst.h -- C ABI of the GB300-native Boruvka 2D/3D EMST library.
 *
 * Drop-in for the reference's EMST operator path (emst_coalition): a caller
 * that drove SolutionEMST / EMSTOperators can drive the same sequence of
 * operators through these entry points (initialise -> per round: flatten,
 * termination test, find-next-closest, find-min-pair, connect-and-union ->
 * evaluate / links), or call emst_solve() for the whole loop.
 *
 * Conventions
 *   - Points are float, array-of-structs, n * dim values (dim 2 or 3), in the
 *     caller's original coordinates (the reference's Grid<PointE<Dim>>
 *     adaptiveMapOriginal).  Point ids are 0-based input positions.
 *   - Every entry point returns an emst_status; no exception crosses the ABI.
 *     emst_last_error() gives a message for the last failure on a context.
 *   - One context = one CUDA stream on one device.  A context is not
 *     thread-safe; distinct contexts may be used concurrently.
 *   - Device buffers are owned by the context and reused across calls.
 *
 * Reference citations are relative to the reference project root.
 */
#ifndef EMST_GB300_H
#define EMST_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
    EMST_OK = 0,
    EMST_EINVAL = 1,      /* bad argument (dim, n, null pointer, NaN / Inf coordinate) */
    EMST_ENOMEM = 2,      /* device or host allocation failed */
    EMST_EOVERFLOW = 3,   /* a size limit of the call was exceeded */
    EMST_ENOCONVERGE = 4, /* round cap (100) or an iteration cap was hit */
    EMST_ECUDA = 5,       /* CUDA runtime error (message in emst_last_error) */
    EMST_ESTATE = 6       /* operator called out of order */
} emst_status;

typedef struct emst_ctx emst_ctx;

typedef struct {
    int device;          /* CUDA device ordinal */
    int max_rounds;      /* Boruvka round cap; 0 = the reference's 100
                            (SolutionEMSTOperators.cu:210) */
    int warps_per_block; /* NNS launch shape; 0 = autotuned default */
    int keep_region_table; /* != 0: keep the round-1 region table for
                              emst_get_region_table (n * K * 8 bytes) */
    int profile;           /* != 0: time every phase with CUDA events */
    int search_mode;       /* 0: component nearest-neighbour search (default);
                              1: static-pruning region table, the reference's
                              computeOctants (implied by keep_region_table);
                              2: component search, one warp per 32 queries;
                              3: dynamic pruning, the reference's per-round
                              ring search over cells without a candidate
                              table (NodeSpiralSearchMD, NodeEMST.h:67-509):
                              per point and region the nearest own-component
                              point bounds the search, regions close for
                              good.  Rounds run host-driven.  Every mode
                              gives the same edges; other values: EINVAL */
    int host_rounds;       /* != 0: drive the component search's rounds from
                              the host instead of one CUDA graph */
    int search_shape;      /* component search launch shape: 0 = default for
                              the dimension, k = entry k-1 of the shape table
                              (emst_search_shape_info); see emst_autotune */
    float first_pass_factor; /* component search, first pass: a point whose
                              lower bound of d2 exceeds this factor times the
                              smallest in its component waits for the second
                              pass (searched only if the component's key does
                              not rule it out); 0 = default; INFINITY = one
                              pass */
    int first_pass_ordered; /* != 0: one search launch per round, the points
                              the factor keeps first and the others after
                              them, instead of a second pass */
    int round1_neighbours; /* 0 = default: round 1 keeps each point's
                              EMST_ROUND1_NEIGHBOURS nearest, and later
                              rounds take the first one outside the
                              component without a search (8 bytes per entry
                              + 1 per point); 4, 5, 6 or 8: that many
                              (emst_autotune picks one); -1 = off; other
                              values: EMST_EINVAL */
    int wide_search;       /* which kernel searches a round's query list:
                              0 = default, by its length: at most 65536
                              points one warp per query (k_cnns_w), more than
                              150000 one warp per 32 queries walking the tree
                              together (k_cnns_c), one thread per query
                              between (k_cnns_t); -1 = thread per query
                              only; 1 = warp per query only; 2 = warp per 32
                              queries only.  Every choice gives the same
                              edges; other values: EMST_EINVAL */
    uint32_t wide_max_list; /* wide_search 0: longest list searched warp
                              per query; 0 = default (65536) */
    uint32_t coop_min_list; /* wide_search 0: lists longer than this are
                              searched warp per 32 queries; 0 = default
                              (150000); 0xffffffff = never */
    int min_find;          /* per-component minimum outgoing edge: 0 =
                              packed 64-bit atomicMin on the component's root
                              slot (default); 1 = diffusion over the forest's
                              edges until every point holds its component's
                              minimum, the reference's tree-based alternative
                              (K_EMST_findMinInComponentDB,
                              EMSTOperators.h:454-915); search_mode 3 only
                              (other combinations: EMST_EINVAL).  Same edges */
} emst_config;

/* Per-phase device times (ms, accumulated since emst_initialize) and kernel
 * launch counts, as the reference's TspResultInfo per-phase timers
 * (emst_coalition/include/EMSTOperators.h:54-70, SolutionEMSTOperators.cu:167-373). */
typedef struct {
    double ms_grid;     /* initialise: rescale + cell keys + sort + leaf tree */
    double ms_octants;  /* compute_octants (static-pruning region table) */
    double ms_select;   /* find_next_closest */
    double ms_resolve;  /* find_min_pair */
    double ms_hook;     /* connect_union */
    double ms_flatten;  /* flatten */
    int64_t launches;          /* kernels launched by the library */
    int64_t octant_launches;   /* of which region-table kernels */
    int64_t rounds;
    /* region search work (static pruning), all launches: leaves (32-point
     * cells) visited per warp, tree nodes tested, candidate points folded
     * (summed over queries), warps (one per 32 queries) */
    int64_t leaf_visits;
    int64_t node_tests;
    int64_t candidates;
    int64_t search_warps;
    int64_t search_queries; /* component mode: point searches run (all rounds) */
    /* component mode, first search pass: searches run, of those the ones cut
     * short by the learned radius and searched again in the second pass (the
     * proposal's mispredictions), and points sent to the second pass
     * without a first search */
    int64_t first_pass_searches;
    int64_t first_pass_resumed;
    int64_t first_pass_deferred;
    /* component mode, profile contexts (host-driven rounds): CUDA-event time
     * of the search kernels' own launches -- the round-1 neighbour-list
     * kernel (its working launch) and the component search (rounds with
     * work) -- and how many launches each figure covers */
    double ms_knn;
    double ms_search;
    int64_t knn_launches;
    int64_t search_launches;
    /* round-1 neighbour-list build, profile contexts: candidates marked for
     * insertion (summed over queries), insert steps (summed over warps, the
     * busiest lane's count), queries that started from the learned radius,
     * and of those the ones searched again from the certified bound (the
     * proposal's mispredictions) */
    int64_t knn_marked;
    int64_t knn_insert_steps;
    int64_t knn_learned;
    int64_t knn_resumed;
} emst_profile;

/* Context lifetime.  Replaces CalculateurEMST::initialize / the static
 * SolutionEMST object (emst_coalition/src/CalculateurEMST.cu:52-169) without
 * global state.  cfg may be NULL for defaults. */
emst_status emst_create(const emst_config* cfg, emst_ctx** out);
emst_status emst_destroy(emst_ctx* ctx);
const char* emst_last_error(const emst_ctx* ctx);

/* Bind the context's work to an existing CUDA stream (cudaStream_t passed as
 * a void*).  NULL is the legacy default stream, as everywhere in CUDA: work
 * the caller queued there before the call runs first, and device outputs are
 * ready for work the caller queues there afterwards.  EMST_OWN_STREAM returns
 * to the context's own (non-blocking) stream, where a new context starts. */
#define EMST_OWN_STREAM ((void*)(intptr_t)-1)
emst_status emst_set_stream(emst_ctx* ctx, void* stream);

/* ---------------------------------------------------------------------------
 * Operator API (mirrors EMSTOperators, emst_coalition/include/EMSTOperators.h)
 * ------------------------------------------------------------------------- */

/* Upload / bind points, rescale them and build the spatial grid.
 * Replaces SolutionEMST::initialize(NetLink&, pMin, pMax)
 * (emst_coalition/src/SolutionEMST.cu:273-509: rescale :349-379, sizing
 * :305-341, cell grid :427-482) together with K_initializeSpiralSearch
 * (EMSTOperators.h:80-110, 1436-1446), K_initDisjointSet (:330-343) and
 * K_clearLinks (:374-387).
 * points_are_device != 0: `points` is a device pointer the caller keeps alive
 * until the next emst_initialize / emst_destroy. */
emst_status emst_initialize(emst_ctx* ctx, const float* points, int64_t n, int dim, int points_are_device);

/* Static-pruning region table: for every point the nearest point of each of
 * the K = 2D*2^(D-1) regions (8 in 2D, 24 in 3D).  Replaces K_computeOctants
 * (EMSTOperators.h:1466-1476 -> NodeComputeOctantMD::computeOctants,
 * NodeEMST.h:1018-1296).  On rounds > 1 only points whose table holds a
 * zero-distance entry are recomputed, as the reference does (:1051-1077).
 * Each entry is the exact nearest point of its region under (d2, input id).
 * The reference's ring search closes a face's slabs per ring and can leave a
 * region's entry at a farther point, or empty, when the nearest one lies in
 * a cell of a ring it already closed; a caller reading rows
 * (emst_get_region_table) can therefore see a different table from the
 * reference's in those rows.  The EMST edge set is the same: a point dropped
 * that way is never a tree edge (a nearer point of another region covers
 * it). */
emst_status emst_compute_octants(emst_ctx* ctx);

/* Per point: nearest table entry outside its component.  Replaces
 * K_findNextClosestPoint (EMSTOperators.h:1490-1500 ->
 * NodeComputeOctantMD::search, NodeEMST.h:1303-1384). */
emst_status emst_find_next_closest(emst_ctx* ctx);

/* Per component: shortest outgoing edge under the (d2, min id, max id)
 * order.  Replaces K_createComponentList + K_findMinPair
 * (NodeEMST.h:817-955). */
emst_status emst_find_min_pair(emst_ctx* ctx);

/* Hook components along their winning edges and append the edges.  Replaces
 * K_connectComponentAndUnion (EMSTOperators.h:1267-1303, 1802-1814). */
emst_status emst_connect_union(emst_ctx* ctx);

/* Compress the disjoint-set forest so every point holds its root.  Replaces
 * K_flatten_DST (EMSTOperators.h:412-433, 1586-1599). */
emst_status emst_flatten(emst_ctx* ctx);

/* Number of points whose root differs from point 0's root (0 = finished).
 * Replaces EMSTOperators::testTermination (EMSTOperators.h:1517-1536). */
emst_status emst_test_termination(emst_ctx* ctx, int64_t* n_other);

/* One Boruvka round = flatten, termination test, compute_octants,
 * find_next_closest, find_min_pair, connect_union.  *more = 0 once finished.
 * Replaces SolutionEMST::activate (SolutionEMSTOperators.cu:156-422). */
emst_status emst_activate(emst_ctx* ctx, int* more);

/* All rounds until one component remains (or the round cap).  Replaces
 * SolutionEMST::run (SolutionEMSTOperators.cu:145-153). */
emst_status emst_run(emst_ctx* ctx);

/* Tree size (edges) and length, the length in ORIGINAL coordinates as
 * sum of sqrt(double(float squared distance)).  Replaces SolutionEMST::evaluate
 * (SolutionEMST.cu:560-581 -> K_EMST_evaluate_ST, EMSTOperators.h:262-292). */
emst_status emst_evaluate(emst_ctx* ctx, int64_t* n_edges, double* length);

/* Copy results to host memory.
 * uv: 2 * cap int32 (u < v, original point ids); round_of_edge: cap int32
 * (1-based Boruvka round that added the edge; may be NULL).  Edges are in
 * the order the rounds produced them.  Replaces the per-point adjacency
 * BufferLink::operator<< / NeuralNetEMST::writeLinks (BufferLink.h:245-279,
 * NeuralNetEMST.h:275-326). */
emst_status emst_get_edges(emst_ctx* ctx, int32_t* uv, int32_t* round_of_edge, int64_t cap, int64_t* n_edges);

/* Root point id per point (the disjointSetMap, NeuralNetEMST.h:59-79). */
emst_status emst_get_labels(emst_ctx* ctx, int32_t* labels, int64_t cap);

/* Number of rounds run so far, and cumulative edge count after each round
 * (cap entries). */
emst_status emst_get_round_stats(emst_ctx* ctx, int64_t* rounds, int64_t* cum_edges, int64_t cap);

/* The round-1 region table: ids (original point ids, -1 = empty region) and
 * squared distances in the rescaled frame, n * K entries each, in region
 * order face * 2^(D-1) + slab (NodeEMST.h:966-972). */
emst_status emst_get_region_table(emst_ctx* ctx, int32_t* ids, float* d2, int64_t cap);

/* The round-1 neighbour lists of a solve that built them (search_mode 0 with
 * round1_neighbours >= 0): per point, in input order, its *k nearest other
 * points, ascending under (squared distance in the rescaled frame, id);
 * ids -1 and d2 +inf past the end when fewer than *k other points exist.
 * ids and d2 hold n * (*k) entries each (either may be NULL); *k is the list
 * length (may be NULL).  No reference counterpart: the reference keeps no
 * per-point lists. */
emst_status emst_get_neighbour_lists(emst_ctx* ctx, int32_t* ids, float* d2, int64_t cap, int* k);

/* Phase times and launch counts since the last emst_initialize (phase times
 * need emst_config.profile != 0). */
emst_status emst_get_profile(emst_ctx* ctx, emst_profile* out);

/* Rescaled coordinates (n * dim floats, input order) and unitX
 * (SolutionEMST.cu:305-364). */
emst_status emst_get_rescaled(emst_ctx* ctx, float* out, double* unit_x, int64_t cap);
/* Hierarchical EMSF (the reference reads the forest back after every round,
 * SolutionEMSTOperators.cu:145-153, 413-416): the forest after round k is
 * the edges whose round_of_edge (emst_get_edges) is <= k.  To also get each
 * point's union-find root after round k, ask the context to keep the labels
 * of the first `rounds` rounds (n * rounds * 4 bytes of device memory) before
 * solving; emst_get_round_labels then returns them in emst_get_labels' form. */
emst_status emst_keep_round_labels(emst_ctx* ctx, int rounds);
emst_status emst_get_round_labels(emst_ctx* ctx, int round, int32_t* labels, int64_t cap);

/* Point count and dimension of the context's (single-cloud) point set. */
emst_status emst_get_size(emst_ctx* ctx, int64_t* n, int* dim);

/* ---------------------------------------------------------------------------
 * One-shot solvers
 * ------------------------------------------------------------------------- */

/* Host buffers in, host buffers out: initialize + run + evaluate + get_edges.
 * The e2e path of CalculateurEMST::run (CalculateurEMST.cu:236-260). */
emst_status emst_solve(emst_ctx* ctx, const float* points, int64_t n, int dim, int32_t* uv, int64_t* n_edges,
                       double* length);

/* Many independent clouds, 2D and 3D mixed, in one solve (one sort, one
 * tree, one round loop): the batched form of CalculateurEMST::run.
 * points: the clouds' AoS floats back to back (cloud i: n_i * dims[i]);
 * point_offsets: n_clouds + 1 cumulative point counts (host);
 * uv: sum of max(n_i - 1, 0) pairs, cloud i's edges first at row
 *     sum_{j<i} max(n_j - 1, 0), local point ids (u < v);
 * lengths: per cloud, as emst_evaluate.  Each cloud's edge set is the one
 * emst_solve gives for that cloud alone.  Component search mode only. */
emst_status emst_solve_batch(emst_ctx* ctx, const float* points, const int64_t* point_offsets, const int32_t* dims,
                             int32_t n_clouds, int32_t* uv, double* lengths, int64_t* n_edges);

/* Device buffers in and out (points n*dim floats; uv 2*(n-1) int32;
 * length one double).  The component search runs its round loop as one CUDA
 * graph with the termination test on the device: the host synchronises once
 * after the loop (to read the edge count and round statistics) and once at
 * the end.  Host-driven contexts (emst_config.host_rounds or profile) read the
 * counters once per round. */
emst_status emst_solve_device(emst_ctx* ctx, const float* d_points, int64_t n, int dim, int32_t* d_uv,
                              double* d_length, int64_t* n_edges);

/* ---------------------------------------------------------------------------
 * The reference's files (host code; no GPU work)
 * ------------------------------------------------------------------------- */

/* Reads a point file the way InputRW::readFile does
 * (emst_coalition/include/InputRW.h:60-623): the suffix picks the format --
 * ".2d" (count, then x y per point), ".3d" (count, then x y z), ".points"
 * ("Width = W Height = H", then x y z per point), anything else TSPLIB
 * (DIMENSION, then "i x y" lines after NODE_COORD_SECTION).  Call with
 * points NULL for *n and *dim, then with cap >= *n points (n * dim floats). */
emst_status emst_read_points(const char* path, float* points, int64_t cap, int64_t* n, int* dim);

/* Writes <base>.links (per point: NumLinks and its tree neighbours as "j 0"),
 * <base>.disjointSetMap (final root of each point as a byte offset, 4 x id)
 * and <base>.points (rescaled coordinates, 6 significant digits), as
 * NeuralNetEMST::writeLinks and the grid writers do
 * (emst_coalition/include/NeuralNetEMST.h:275-326, BufferLink.h:266-279).
 * Neighbours are listed by round, then id.  The context must hold a finished
 * single-cloud solve. */
emst_status emst_write_results(emst_ctx* ctx, const char* base);

/* Reads a .links file into an edge list (each undirected edge once, u < v);
 * uv NULL returns the counts only. */
emst_status emst_read_links(const char* path, int32_t* uv, int64_t cap, int64_t* n_edges, int64_t* n_points);

/* ---------------------------------------------------------------------------
 * Learned search proposal (no counterpart in the reference; it stands beside
 * the plain search and leaves its results unchanged)
 *
 * It steers round 1, where every point builds its list of the
 * EMST_ROUND1_NEIGHBOURS nearest points (the dominant step of a solve).  The
 * plain search starts each query's walk from a certified bound: the K-th
 * smallest squared distance to the other points of its own 32-point leaf.  A
 * small network (8 inputs -- the own leaf's nearest, third and K-th
 * distances, the leaf's extent and occupancy, the parent node's extent, the
 * point's distance to its leaf's surface, the round and the component size --
 * two hidden layers of 32, 2 outputs; BF16 tensor-core inference fused into
 * the search kernel) predicts the ratio of the query's true K-th nearest
 * distance to that bound, and a gate: whether the bound can be tightened at
 * all.  Where the gate is at or above `threshold`, the walk starts from the
 * predicted radius times 2^margin (in d2, never above the certified bound):
 * fewer nodes and candidates fall within it.  A query whose radius held fewer
 * than K points walks again from the certified bound, so every list -- and
 * the edge set -- is the plain method's.
 * ------------------------------------------------------------------------- */

#define EMST_ROUND1_NEIGHBOURS 6    /* list length of emst_config.round1_neighbours */
#define EMST_PROPOSAL_WEIGHTS 1410 /* W1[8][32] b1[32] W2[32][32] b2[32] W3[32][2] b3[2], FP32 */
#define EMST_TRACE_RECORD 12       /* floats per trace record */

/* Turns the learned proposal on (weights: EMST_PROPOSAL_WEIGHTS floats) or
 * off (weights NULL).  margin: log2 factor on the predicted radius (d2), in
 * [0, 64]; threshold: gate logit at or above which a query starts from the
 * predicted radius.  Single-cloud solves with round-1 neighbour lists only
 * (batches keep the plain bound). */
emst_status emst_set_proposal(emst_ctx* ctx, const float* weights, float margin, float threshold);

/* Training traces: from now on, solves of this context (plain search)
 * record 1 in 2^sample_shift round-1 queries, up to `capacity` records in
 * total (capacity 0: off).  Record: the 8 features, log2(d2 of the K-th
 * nearest point / the own leaf's bound)/8, [that bound could be tightened],
 * 1 if the query has K neighbours (else both targets are void), 0. */
emst_status emst_trace_enable(emst_ctx* ctx, int64_t capacity, int sample_shift);
emst_status emst_get_trace(emst_ctx* ctx, float* records, int64_t cap, int64_t* count);
emst_status emst_get_trace_device(emst_ctx* ctx, const float** d_records, int64_t* count);

typedef struct {
    int epochs;       /* passes over the records (0: 4) */
    int batch;        /* records per Adam step (0: 4096) */
    float lr;         /* Adam step size (0: 2e-3) */
    float reg_weight; /* radius loss weight against the class loss (0: 1) */
    uint64_t seed;    /* record order */
    int device;
} emst_train_config;

/* Seeded initial weights (uniform, fan-in scaled). */
emst_status emst_proposal_init(uint64_t seed, float* weights);
/* Trains the proposal on trace records (host or device) with the library's
 * BF16 tensor-core forward/backward kernels and Adam; weights in (initial)
 * and out (trained); loss_curve (optional): mean loss per epoch. */
emst_status emst_proposal_train(const float* records, int64_t n_records, int records_on_device,
                                const emst_train_config* cfg, float* weights, float* loss_curve);
/* One forward/backward over host records: gradient of the mean loss
 * (EMST_PROPOSAL_WEIGHTS floats) and the loss, for checking. */
emst_status emst_proposal_grad(const float* weights, const float* records, int64_t n_records, float reg_weight,
                               float* grad, float* loss);

/* ---------------------------------------------------------------------------
 * Launch-shape autotuner (no counterpart in the reference, whose kernels use
 * fixed 4x4x4 / 8x8 thread blocks: EMSTOperators.h:1405-1416)
 * ------------------------------------------------------------------------- */

/* The component search's launch shapes: *count entries; per entry k
 * (emst_config.search_shape = k + 1) the threads per block and the minimum
 * resident blocks per SM it is compiled for (cap entries written). */
emst_status emst_search_shape_info(int* count, int* threads, int* min_blocks, int cap);

/* Tunes the component search on `points` (host, n x dim) by coordinate
 * descent, each candidate timed as the best of two solves after a warm-up
 * solve, and keeps the fastest setting of each stage for this context:
 *   1. the round-1 list length (4, 5, 6, 8; lists on and no learned
 *      proposal, which is trained for the default);
 *   2. the list length above which a round is searched warp per 32 queries
 *      (50k, 150k, 400k, never) and the one up to which warp per query
 *      (16k, 64k, 150k) -- with wide_search 0;
 *   3. the thread-per-query launch shape (emst_search_shape_info).
 * *best: the chosen emst_config.search_shape value; ms (optional, cap
 * entries): the time per shape of stage 3.  emst_get_tuning returns every
 * stage's candidates and times.  Afterwards the context holds a finished
 * solve of `points`.  Every setting gives the same edges.  Component search
 * mode only. */
emst_status emst_autotune(emst_ctx* ctx, const float* points, int64_t n, int dim, int* best, double* ms, int cap);
emst_status emst_get_search_shape(emst_ctx* ctx, int* search_shape);

typedef struct {
    int knn_k;                   /* round-1 list length in use (0: lists off) */
    uint32_t coop_min;           /* warp-per-32-queries threshold in use */
    uint32_t wide_max;           /* warp-per-query threshold in use */
    int search_shape;            /* emst_config.search_shape value in use */
    int knn_k_values[4];         /* stage 1 candidates and their times (ms; 0: stage skipped) */
    double ms_knn_k[4];
    uint32_t coop_min_values[4]; /* stage 2 candidates (0xffffffff: never) and times */
    double ms_coop_min[4];
    uint32_t wide_max_values[3];
    double ms_wide_max[3];
    double ms_shape[6];          /* stage 3: per launch shape */
} emst_tuning;

/* The context's search settings and the last emst_autotune's stage tables. */
emst_status emst_get_tuning(emst_ctx* ctx, emst_tuning* out);

/* ---------------------------------------------------------------------------
 * Allocation-free region table
 * ------------------------------------------------------------------------- */

/* Largest point set emst_region_table_noalloc accepts, and the size of the
 * device array it works in.  The array is a static device variable of the
 * library: under CUDA's default lazy module loading it is placed on a device
 * by the first emst_region_table_noalloc call there (which looks up its
 * address) and stays until the process exits; a caller that must not see
 * that reservation mid-run makes one call at start-up. */
#define EMST_NOALLOC_MAX_POINTS 32768
#define EMST_NOALLOC_SCRATCH_BYTES (12u << 20)

/* No counterpart in the reference.  The same region table as
 * emst_compute_octants + emst_get_region_table (ids as input point ids, -1 for
 * an empty region, and squared distances in the rescaled frame, n * K entries
 * each), for callers that must not allocate device memory once they are
 * running: a host whose device memory is owned by its own allocator, a
 * real-time pipeline where a cudaMalloc / cudaFree may stall or fail mid-run,
 * or a plugin whose processing callback forbids allocation.  The caller passes
 * device buffers for the points (n * dim floats) and both outputs; every
 * intermediate buffer lives in one fixed device array inside the library, so
 * nothing is allocated and n is limited to EMST_NOALLOC_MAX_POINTS (larger n
 * returns EMST_EOVERFLOW).  The first call on a device looks up that array's
 * device address (make it before any stream capture).  Calls share the array:
 * calls that may overlap on the GPU race and must be serialised by the caller.
 * Synchronises `stream` (a cudaStream_t, NULL = legacy default stream) before
 * returning; EMST_EINVAL for a non-finite coordinate. */
emst_status emst_region_table_noalloc(const float* d_points, int64_t n, int dim, int32_t* d_ids, float* d_d2,
                                      void* stream);

#ifdef __cplusplus
}
#endif

#endif /* EMST_GB300_H */
