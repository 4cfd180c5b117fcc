/*
 * emst_kd_oracle.c -- exact CPU EMST for full-size parity checks.
 *
 * TEST INFRASTRUCTURE ONLY (like emst_oracle.c, whose library it joins): only
 * tests/, __graft_entry__.smoke() and bench.py's CPU legs may load it, and
 * only as the checker.  The product library never links or calls it.
 *
 * The faithful restatement in emst_oracle.c walks the reference's cell rings
 * (emst_coalition/include/NodeEMST.h:1018-1296); on clustered sets its cells
 * hold thousands of points and a 10^7-point solve takes hours.  This file
 * computes the same Boruvka rounds with a different, independent search: a
 * median-split kd-tree, and per round each point's nearest point outside its
 * component.  The rounds, the tie-break and the union rule are the reference's:
 *   - distance: the float dot product of float differences with fused
 *     accumulation (basic_components/include/Node.h:241-250, the same d2 as
 *     emst_oracle.c's metric variant 0);
 *   - per component, the minimum outgoing edge under (d2, min id, max id)
 *     (EMST_isInf, basic_components/include/macros_cuda.h:37;
 *     K_NEMST_findMinPair, emst_coalition/include/NodeEMST.h:871-955);
 *   - hook rule: a winner's root hooks onto its partner's root unless the
 *     partner is a winner pointing back, in which case only the lower id's
 *     side stays root (K_EMST_connectComponentAndUnion_2,
 *     emst_coalition/include/EMSTOperators.h:1267-1303);
 *   - flatten / termination / round cap as SolutionEMST::activate
 *     (emst_coalition/src/SolutionEMSTOperators.cu:156-422).
 * For a fixed query point the order (d2, min id, max id) over candidates q is
 * the order (d2, q), so each point's nearest outside point under (d2, q) and
 * then the component minimum give exactly the reference's per-round edges.
 * Outputs match oracle_emst(): edges in round order (winners by increasing
 * point index), round of each edge, cumulative edges per round, final labels.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define KD_LEAF 8
#define KD_MAX_ROUNDS 100 /* SolutionEMSTOperators.cu:210 */
#define KD_NONE (-1)

static inline float kd_d2(const float* a, const float* b, int dim)
{
    float dx = a[0] - b[0], dy = a[1] - b[1];
    float r = dx * dx;
    r = fmaf(dy, dy, r);
    if (dim == 3) {
        float dz = a[2] - b[2];
        r = fmaf(dz, dz, r);
    }
    return r;
}

typedef struct {
    int64_t n;
    int dim;
    const float* sp;
    int64_t* idx;   /* point ids, leaf order */
    int64_t nnodes;
    int64_t* lo_i;  /* per node: [lo_i, hi_i) into idx */
    int64_t* hi_i;
    int64_t* child; /* per node: first child (second = first + 1), -1 for a leaf */
    float* box;     /* per node: lo[3], hi[3] */
    int64_t* nlab;  /* per node: label shared by all its points, or -2 (mixed) */
} kdtree_t;

static float coord(const kdtree_t* t, int64_t i, int a) { return t->sp[i * t->dim + a]; }

/* Quickselect on idx[lo, hi) so that idx[mid] holds the median by axis a
 * (ties broken by id so that the split is deterministic). */
static int kd_less(const kdtree_t* t, int64_t x, int64_t y, int a)
{
    float cx = coord(t, x, a), cy = coord(t, y, a);
    return cx < cy || (cx == cy && x < y);
}

static void kd_select(kdtree_t* t, int64_t lo, int64_t hi, int64_t mid, int a)
{
    int64_t* v = t->idx;
    while (hi - lo > 1) {
        /* median of three pivot */
        int64_t m = lo + (hi - lo) / 2;
        int64_t p0 = v[lo], p1 = v[m], p2 = v[hi - 1], piv;
        if (kd_less(t, p0, p1, a)) {
            if (kd_less(t, p1, p2, a)) piv = p1;
            else piv = kd_less(t, p0, p2, a) ? p2 : p0;
        } else {
            if (kd_less(t, p0, p2, a)) piv = p0;
            else piv = kd_less(t, p1, p2, a) ? p2 : p1;
        }
        /* three-way partition around piv */
        int64_t i = lo, lt = lo, gt = hi;
        while (i < gt) {
            if (kd_less(t, v[i], piv, a)) {
                int64_t s = v[i]; v[i] = v[lt]; v[lt] = s;
                ++i; ++lt;
            } else if (kd_less(t, piv, v[i], a)) {
                --gt;
                int64_t s = v[i]; v[i] = v[gt]; v[gt] = s;
            } else {
                ++i;
            }
        }
        if (mid < lt) hi = lt;
        else if (mid >= gt) lo = gt;
        else return;
    }
}

static void kd_box(kdtree_t* t, int64_t node)
{
    float* b = t->box + 6 * node;
    for (int a = 0; a < 3; ++a) {
        b[a] = INFINITY;
        b[3 + a] = -INFINITY;
    }
    for (int64_t k = t->lo_i[node]; k < t->hi_i[node]; ++k)
        for (int a = 0; a < t->dim; ++a) {
            float c = coord(t, t->idx[k], a);
            if (c < b[a]) b[a] = c;
            if (c > b[3 + a]) b[3 + a] = c;
        }
    if (t->dim == 2) {
        b[2] = 0.f;
        b[5] = 0.f;
    }
}

static int kd_build(kdtree_t* t, const float* sp, int64_t n, int dim)
{
    memset(t, 0, sizeof(*t));
    t->n = n;
    t->dim = dim;
    t->sp = sp;
    int64_t cap = 2 * (n / (KD_LEAF / 2) + 2);
    t->idx = (int64_t*)malloc(sizeof(int64_t) * n);
    t->lo_i = (int64_t*)malloc(sizeof(int64_t) * cap);
    t->hi_i = (int64_t*)malloc(sizeof(int64_t) * cap);
    t->child = (int64_t*)malloc(sizeof(int64_t) * cap);
    t->box = (float*)malloc(sizeof(float) * 6 * cap);
    t->nlab = (int64_t*)malloc(sizeof(int64_t) * cap);
    if (!t->idx || !t->lo_i || !t->hi_i || !t->child || !t->box || !t->nlab) return -1;
    for (int64_t i = 0; i < n; ++i) t->idx[i] = i;
    /* breadth-first: children of node k are appended in order, so a parent
     * always precedes its children (labels are computed children first by
     * walking the nodes backwards) */
    t->lo_i[0] = 0;
    t->hi_i[0] = n;
    t->nnodes = 1;
    for (int64_t k = 0; k < t->nnodes; ++k) {
        kd_box(t, k);
        int64_t lo = t->lo_i[k], hi = t->hi_i[k];
        t->child[k] = -1;
        if (hi - lo <= KD_LEAF) continue;
        const float* b = t->box + 6 * k;
        int a = 0;
        float w = b[3] - b[0];
        for (int j = 1; j < dim; ++j)
            if (b[3 + j] - b[j] > w) {
                w = b[3 + j] - b[j];
                a = j;
            }
        int64_t mid = lo + (hi - lo) / 2;
        kd_select(t, lo, hi, mid, a);
        if (t->nnodes + 2 > cap) return -1;
        int64_t c = t->nnodes;
        t->child[k] = c;
        t->lo_i[c] = lo;
        t->hi_i[c] = mid;
        t->lo_i[c + 1] = mid;
        t->hi_i[c + 1] = hi;
        t->nnodes += 2;
    }
    return 0;
}

static void kd_free(kdtree_t* t)
{
    free(t->idx);
    free(t->lo_i);
    free(t->hi_i);
    free(t->child);
    free(t->box);
    free(t->nlab);
}

/* Per node: the component shared by all its points, or -2. */
static void kd_labels(kdtree_t* t, const int64_t* lab)
{
    for (int64_t k = t->nnodes - 1; k >= 0; --k) {
        if (t->child[k] < 0) {
            int64_t l = lab[t->idx[t->lo_i[k]]];
            for (int64_t j = t->lo_i[k] + 1; j < t->hi_i[k] && l != -2; ++j)
                if (lab[t->idx[j]] != l) l = -2;
            t->nlab[k] = l;
        } else {
            int64_t a = t->nlab[t->child[k]], b = t->nlab[t->child[k] + 1];
            t->nlab[k] = a == b ? a : -2;
        }
    }
}

static inline float kd_lb(const kdtree_t* t, int64_t node, const float* p)
{
    const float* b = t->box + 6 * node;
    float g[3] = {0.f, 0.f, 0.f};
    for (int a = 0; a < t->dim; ++a) {
        float u = b[a] - p[a], v = p[a] - b[3 + a];
        float m = u > v ? u : v;
        g[a] = m > 0.f ? m : 0.f;
    }
    float r = g[0] * g[0];
    r = fmaf(g[1], g[1], r);
    if (t->dim == 3) r = fmaf(g[2], g[2], r);
    return r;
}

/* Nearest point q with lab[q] != lab[p] under (d2, q), searching only within
 * d2 <= bound.  Returns q or KD_NONE; *d2_out = its d2. */
static int64_t kd_nearest_outside(const kdtree_t* t, int64_t p, const int64_t* lab, float bound, float* d2_out)
{
    const float* P = t->sp + p * t->dim;
    const int64_t lp = lab[p];
    int64_t best = KD_NONE;
    float bd = bound;
    int64_t stack[128];
    int top = 0;
    stack[top++] = 0;
    while (top > 0) {
        int64_t k = stack[--top];
        if (t->nlab[k] == lp) continue;
        if (kd_lb(t, k, P) > bd) continue;
        if (t->child[k] < 0) {
            for (int64_t j = t->lo_i[k]; j < t->hi_i[k]; ++j) {
                int64_t q = t->idx[j];
                if (lab[q] == lp) continue;
                float d = kd_d2(P, t->sp + q * t->dim, t->dim);
                if (d < bd || (d == bd && (best == KD_NONE || q < best))) {
                    bd = d;
                    best = q;
                }
            }
            continue;
        }
        int64_t c0 = t->child[k], c1 = c0 + 1;
        float l0 = kd_lb(t, c0, P), l1 = kd_lb(t, c1, P);
        /* nearer child popped first */
        if (l0 <= l1) {
            stack[top++] = c1;
            stack[top++] = c0;
        } else {
            stack[top++] = c0;
            stack[top++] = c1;
        }
    }
    *d2_out = bd;
    return best;
}

static int64_t kd_find_root(const int64_t* ds, int64_t x)
{
    while (ds[x] != x) x = ds[x];
    return x;
}

static inline int kd_is_inf(int64_t a1, int64_t b1, float d1, int64_t a2, int64_t b2, float d2)
{
    if (d1 != d2) return d1 < d2;
    if (a1 != a2) return a1 < a2;
    return b1 < b2;
}

static inline uint32_t kd_fbits(float f)
{
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}

static inline float kd_bitsf(uint32_t u)
{
    float f;
    memcpy(&f, &u, 4);
    return f;
}

/*
 * Exact EMST of rescaled points sp (n * dim floats) by kd-tree Boruvka.
 * Outputs as oracle_emst (emst_oracle.c).  Returns the number of rounds, or a
 * negative error.
 */
int64_t oracle_emst_kd(const float* sp, int64_t n, int dim, int64_t* edges_out, int32_t* edge_round_out,
                       int64_t* round_edges_out, int64_t* labels_out)
{
    if (n <= 0 || (dim != 2 && dim != 3)) return -1;
    kdtree_t t;
    if (kd_build(&t, sp, n, dim) != 0) {
        kd_free(&t);
        return -2;
    }
    int64_t* ds = (int64_t*)malloc(sizeof(int64_t) * n);
    int64_t* par = (int64_t*)malloc(sizeof(int64_t) * n);
    int64_t* corr = (int64_t*)malloc(sizeof(int64_t) * n);
    float* dist = (float*)malloc(sizeof(float) * n);
    float* lbp = (float*)malloc(sizeof(float) * n);       /* lower bound of d2 to the nearest outside point */
    uint32_t* cbest = (uint32_t*)malloc(sizeof(uint32_t) * n); /* per root: smallest d2 found (float bits) */
    int64_t* cbest_w = (int64_t*)malloc(sizeof(int64_t) * n);
    char* fix = (char*)malloc(n);
    if (!ds || !par || !corr || !dist || !lbp || !cbest || !cbest_w || !fix) {
        free(ds); free(par); free(corr); free(dist); free(lbp); free(cbest); free(cbest_w); free(fix);
        kd_free(&t);
        return -3;
    }
    for (int64_t i = 0; i < n; ++i) {
        ds[i] = i;
        corr[i] = KD_NONE;
        lbp[i] = 0.f;
    }
    int64_t nedges = 0, iteration = 0;
    for (;;) {
        for (int64_t i = 0; i < n; ++i) par[i] = kd_find_root(ds, i);
        memcpy(ds, par, sizeof(int64_t) * n);
        int64_t r0 = ds[0], ncomp = 0;
        for (int64_t i = 0; i < n; ++i)
            if (ds[i] != r0) ncomp++;
        if (ncomp == 0 || iteration == KD_MAX_ROUNDS) break;
        iteration++;
        kd_labels(&t, ds);
        /* 1. partners still outside keep them (outside sets only shrink, and
         * every point nearer than the partner was inside, so it still is) */
        for (int64_t i = 0; i < n; ++i) cbest[i] = 0x7f800000u;
#pragma omp parallel for schedule(static)
        for (int64_t i = 0; i < n; ++i) {
            int64_t q = corr[i];
            if (q != KD_NONE && ds[q] != ds[i]) {
                uint32_t b = kd_fbits(dist[i]);
                uint32_t* slot = &cbest[ds[i]];
                uint32_t cur = __atomic_load_n(slot, __ATOMIC_RELAXED);
                while (b < cur && !__atomic_compare_exchange_n(slot, &cur, b, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
                }
            } else {
                corr[i] = KD_NONE;
            }
        }
        /* 2. the others search, each bounded by its component's best so far:
         * a point whose nearest outside point is farther than that cannot give
         * the component's minimum (ties at the bound are searched) */
#pragma omp parallel for schedule(dynamic, 512)
        for (int64_t i = 0; i < n; ++i) {
            if (corr[i] != KD_NONE) continue;
            uint32_t* slot = &cbest[ds[i]];
            float bound = kd_bitsf(__atomic_load_n(slot, __ATOMIC_RELAXED));
            if (lbp[i] > bound) continue;
            float d = 0.f;
            int64_t q = kd_nearest_outside(&t, i, ds, bound, &d);
            if (q == KD_NONE) {
                if (bound > lbp[i]) lbp[i] = bound; /* nothing outside within the bound */
                continue;
            }
            corr[i] = q;
            dist[i] = d;
            lbp[i] = d;
            uint32_t b = kd_fbits(d);
            uint32_t cur = __atomic_load_n(slot, __ATOMIC_RELAXED);
            while (b < cur && !__atomic_compare_exchange_n(slot, &cur, b, 1, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
            }
        }
        /* 3. per component, the minimum under (d2, min id, max id) */
        for (int64_t i = 0; i < n; ++i) {
            fix[i] = 0;
            cbest_w[i] = KD_NONE;
        }
        for (int64_t i = 0; i < n; ++i) {
            int64_t q = corr[i];
            if (q == KD_NONE) continue;
            int64_t c = ds[i], w = cbest_w[c];
            int64_t a1 = i < q ? i : q, b1 = i < q ? q : i;
            if (w == KD_NONE) {
                cbest_w[c] = i;
                continue;
            }
            int64_t qw = corr[w];
            int64_t a2 = w < qw ? w : qw, b2 = w < qw ? qw : w;
            if (kd_is_inf(a1, b1, dist[i], a2, b2, dist[w])) cbest_w[c] = i;
        }
        for (int64_t c = 0; c < n; ++c)
            if (cbest_w[c] != KD_NONE) fix[cbest_w[c]] = 1;
        /* 4. hook (EMSTOperators.h:1267-1303), roots read from a snapshot */
        memcpy(par, ds, sizeof(int64_t) * n);
        for (int64_t ps = 0; ps < n; ++ps) {
            if (!fix[ps]) continue;
            int64_t pq = corr[ps];
            int64_t rps = par[ps], rpq = par[pq];
            int mutual = fix[pq] && corr[pq] == ps;
            if (!mutual) ds[rps] = rpq;
            else if (ps < pq) ds[rpq] = rps;
            if (!mutual || ps < pq) {
                edges_out[2 * nedges] = ps < pq ? ps : pq;
                edges_out[2 * nedges + 1] = ps < pq ? pq : ps;
                if (edge_round_out) edge_round_out[nedges] = (int32_t)iteration;
                nedges++;
            }
        }
        if (round_edges_out) round_edges_out[iteration - 1] = nedges;
    }
    if (labels_out)
        for (int64_t i = 0; i < n; ++i) labels_out[i] = ds[i];
    free(ds); free(par); free(corr); free(dist); free(lbp); free(cbest); free(cbest_w); free(fix);
    kd_free(&t);
    return iteration;
}

/* ------------------------------------------------------------------------ */
/* k nearest neighbours (the round-1 neighbour lists)                        */
/* ------------------------------------------------------------------------ */

/* The k nearest other points of p under (d2, id), ascending; -1 / +inf past
 * the end when fewer than k other points exist.  A node is skipped only when
 * its box bound exceeds the k-th entry's d2 (a point at that d2 with a lower
 * id still enters). */
static void kd_knn_one(const kdtree_t* t, int64_t p, int k, int64_t* ids, float* d2s)
{
    const float* P = t->sp + p * t->dim;
    for (int j = 0; j < k; ++j) {
        ids[j] = KD_NONE;
        d2s[j] = INFINITY;
    }
    int64_t stack[128];
    int top = 0;
    stack[top++] = 0;
    while (top > 0) {
        int64_t node = stack[--top];
        if (kd_lb(t, node, P) > d2s[k - 1]) continue;
        if (t->child[node] < 0) {
            for (int64_t j = t->lo_i[node]; j < t->hi_i[node]; ++j) {
                int64_t q = t->idx[j];
                if (q == p) continue;
                float d = kd_d2(P, t->sp + q * t->dim, t->dim);
                if (!(d < d2s[k - 1] || (d == d2s[k - 1] && (ids[k - 1] == KD_NONE || q < ids[k - 1])))) continue;
                int s = k - 1;
                while (s > 0 && (d < d2s[s - 1] || (d == d2s[s - 1] && q < ids[s - 1]))) {
                    d2s[s] = d2s[s - 1];
                    ids[s] = ids[s - 1];
                    --s;
                }
                d2s[s] = d;
                ids[s] = q;
            }
            continue;
        }
        int64_t c0 = t->child[node], c1 = c0 + 1;
        if (kd_lb(t, c0, P) <= kd_lb(t, c1, P)) {
            stack[top++] = c1;
            stack[top++] = c0;
        } else {
            stack[top++] = c0;
            stack[top++] = c1;
        }
    }
}

/* Every point's k nearest other points: ids_out / d2_out hold n rows of k. */
int oracle_knn_kd(const float* sp, int64_t n, int dim, int k, int64_t* ids_out, float* d2_out)
{
    if (n < 1 || k < 1 || (dim != 2 && dim != 3)) return -1;
    kdtree_t t;
    if (kd_build(&t, sp, n, dim) != 0) {
        kd_free(&t);
        return -2;
    }
#pragma omp parallel for schedule(dynamic, 1024)
    for (int64_t i = 0; i < n; ++i) kd_knn_one(&t, i, k, ids_out + i * k, d2_out + i * k);
    kd_free(&t);
    return 0;
}
