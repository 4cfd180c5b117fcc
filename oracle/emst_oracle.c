/*
 * emst_oracle.c -- CPU restatement of the reference's GPU Boruvka EMST path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity oracle: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it, and
 * only as the checker or the timed CPU baseline.  The product library never
 * links or calls it.
 *
 * Parity is pinned against the reference's own golden outputs (the 3000-point
 * edge set in test_2D_2/outypu.links and the per-round edge counts / tree
 * lengths recorded in test_2D_2/output and test_3D_2/output); see
 * tests/test_oracle_golden.py.
 *
 * Every function names the reference file:line it restates (paths relative to
 * the reference project root).  Arithmetic follows the reference exactly:
 *   - coordinates are float; rescale is float(float(p - pMin) * float(unitX))
 *     with unitX computed in double (emst_coalition/src/SolutionEMST.cu:305-364);
 *   - squared distance is the float dot product f = dx*dx; f += dy*dy; f += dz*dz
 *     (basic_components/include/Node.h:241-250) with the GPU's FMA contraction
 *     (fmaf for the accumulating steps) -- metric variant 0; variant 1 keeps
 *     separate multiply and add roundings;
 *   - tie-break is lexicographic on (d2, min id, max id)
 *     (basic_components/include/macros_cuda.h:37, EMST_isInf).
 * Build with -ffp-contract=off so that the compiler adds no contraction of
 * its own.
 */
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_MAX_K 24
#define ORACLE_MAX_ROUNDS 100 /* SolutionEMSTOperators.cu:210: iteration == 100 cap */

/* ------------------------------------------------------------------------ */
/* Metric and tie-break                                                      */
/* ------------------------------------------------------------------------ */

static int g_metric_variant = 0;

void oracle_set_metric_variant(int v) { g_metric_variant = v; }

#ifdef _OPENMP
#include <omp.h>
void oracle_set_threads(int t) { omp_set_num_threads(t > 0 ? t : 1); }
int oracle_max_threads(void) { return omp_get_max_threads(); }
#else
void oracle_set_threads(int t) { (void)t; }
int oracle_max_threads(void) { return 1; }
#endif

/* Node.h:241-250 scalar product of (p1 - p2) with itself, in float. */
static inline float d2f(const float* a, const float* b, int dim)
{
    float dx = a[0] - b[0];
    float dy = a[1] - b[1];
    float r = dx * dx;
    if (g_metric_variant == 0) {
        r = fmaf(dy, dy, r);
        if (dim == 3) {
            float dz = a[2] - b[2];
            r = fmaf(dz, dz, r);
        }
    } else {
        float t = dy * dy;
        r = r + t;
        if (dim == 3) {
            float dz = a[2] - b[2];
            float u = dz * dz;
            r = r + u;
        }
    }
    return r;
}

float oracle_d2(const float* a, const float* b, int dim) { return d2f(a, b, dim); }

/* macros_cuda.h:37 EMST_isInf: (d1,a1,b1) < (d2,a2,b2) lexicographically. */
static inline int is_inf(int64_t a1, int64_t b1, double d1, int64_t a2, int64_t b2, double d2)
{
    if (d1 == d2) {
        if (a1 == a2) return b1 < b2;
        return a1 < a2;
    }
    return d1 < d2;
}

static inline int64_t mn(int64_t a, int64_t b) { return a <= b ? a : b; }
static inline int64_t mx(int64_t a, int64_t b) { return a >= b ? a : b; }

/* ------------------------------------------------------------------------ */
/* Rescale: SolutionEMST::initialize(NetLink&, pMin, pMax)                   */
/* ------------------------------------------------------------------------ */

/*
 * Bounding box as the readers compute it (InputRW.h:545-559: max with >=,
 * min with <, in float), then unitX (SolutionEMST.cu:305-341) and the rescale
 * loop (SolutionEMST.cu:361-364).
 * out: n*dim floats.  Returns unitX (double) through *unitx.
 */
int oracle_rescale(const float* pts, int64_t n, int dim, float* out, double* unitx,
                   float* pmin_out, float* pmax_out)
{
    float pmin[3] = {INFINITY, INFINITY, INFINITY};
    float pmax[3] = {-INFINITY, -INFINITY, -INFINITY};
    if (n <= 0) return -1;
    for (int64_t i = 0; i < n; ++i) {
        for (int k = 0; k < dim; ++k) {
            float c = pts[i * dim + k];
            if (c >= pmax[k]) pmax[k] = c;
            if (c < pmin[k]) pmin[k] = c;
        }
    }
    double wg = (double)(float)(pmax[0] - pmin[0]);
    double hg = (double)(float)(pmax[1] - pmin[1]);
    double dg = 0.0;
    if (dim >= 3) dg = (double)(float)(pmax[2] - pmin[2]);
    if (wg == 0) wg = 1;
    if (hg == 0) hg = 1;
    double nn = (double)n;
    double wnd = sqrt(nn * wg / hg) * 2;
    if (dim >= 3) {
        if (dg != 0)
            wnd = pow((nn * wg * wg) / (hg * dg), 0.333);
        else
            dg = 1;
    }
    double wndd = ceil(wnd) + 1;
    double ux = wndd / wg;
    float uxf = (float)ux;
    for (int64_t i = 0; i < n; ++i)
        for (int k = 0; k < dim; ++k) {
            float t = pts[i * dim + k] - pmin[k];
            out[i * dim + k] = t * uxf;
        }
    if (unitx) *unitx = ux;
    for (int k = 0; k < dim; ++k) {
        if (pmin_out) pmin_out[k] = pmin[k];
        if (pmax_out) pmax_out[k] = pmax[k];
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Region classification (NodeEMST.h:1207-1232)                             */
/* ------------------------------------------------------------------------ */

/*
 * Region index = face * NSLAB + slab.  face = 2*dir + (delta[dir] >= 0 ? 0 : 1)
 * for every dominant axis (|delta[dir]| >= max |delta|); slab bit j (over the
 * other axes in increasing order) is 0 when delta >= 0 and 1 when delta <= 0,
 * so zero components belong to both slabs.  Returns a bit mask over regions.
 */
static uint32_t region_mask(const float* d, int dim)
{
    const int nslab = dim == 3 ? 4 : 2;
    float ad[3] = {fabsf(d[0]), fabsf(d[1]), dim == 3 ? fabsf(d[2]) : 0.f};
    double maxd = 0;
    for (int k = 0; k < dim; ++k)
        if (ad[k] > maxd) maxd = ad[k];
    uint32_t mask = 0;
    for (int dir = 0; dir < dim; ++dir) {
        if (!(ad[dir] >= maxd)) continue;
        int f = dir * 2 + (d[dir] >= 0 ? 0 : 1);
        for (int s = 0; s < nslab; ++s) {
            int ok = 1, bit = 1;
            for (int i = 0; i < dim; ++i) {
                if (i == dir) continue;
                double sign = (s & bit) ? -1.0 : 1.0;
                ok = ok && (sign * d[i] >= 0);
                if (!ok) break;
                bit <<= 1;
            }
            if (ok) mask |= 1u << (f * nslab + s);
        }
    }
    return mask;
}

uint32_t oracle_region_mask(const float* delta, int dim) { return region_mask(delta, dim); }

/* ------------------------------------------------------------------------ */
/* Reference cell geometry: ViewGridQuadMD (ViewGrid.h:241-359)             */
/* ------------------------------------------------------------------------ */

typedef struct {
    int dim;
    int R;
    int pc[3], PC[3];
    int ext_dual[3];
    float p1[3]; /* FEuclid(FDual(0)) */
} vgrid_t;

/* SolutionEMST.cu:344-430 (extents from the rescaled box) + ViewGrid.h:254-265. */
static void vgrid_init(vgrid_t* g, const float* sp, int64_t n, int dim, int R)
{
    double mxn[3] = {-INFINITY, -INFINITY, 0}, mnn[3] = {INFINITY, INFINITY, 0};
    if (dim >= 3) { mxn[2] = -INFINITY; mnn[2] = INFINITY; }
    for (int64_t i = 0; i < n; ++i)
        for (int k = 0; k < dim; ++k) {
            double c = sp[i * dim + k];
            if (c >= mxn[k]) mxn[k] = c;
            if (c < mnn[k]) mnn[k] = c;
        }
    int ext[3] = {1, 1, 1};
    for (int k = 0; k < dim; ++k) ext[k] = (int)ceil(mxn[k] - mnn[k]) + 1;
    g->dim = dim;
    g->R = R;
    for (int k = 0; k < 3; ++k) {
        int e = k < dim ? ext[k] : 1;
        int pc = e / 2;
        int PC = (pc + (R - 1)) / R;
        int eb = (PC + 1) + ((e - pc) + (R - 1)) / R;
        int PCD = PC / 2;
        int ed = (PCD + 1) + ((eb - PC) + 1) / 2;
        g->pc[k] = pc;
        g->PC[k] = PC;
        g->ext_dual[k] = k < dim ? ed : 1;
        /* FDual(0) = F(FDualToBase(0)) = (PC % 2) * R - PC * R + pc */
        int lo = (PC % 2) * R - PC * R + pc;
        g->p1[k] = (float)lo;
    }
}

/* FEuclid(FDual(PD))[k] as float. */
static inline float vgrid_center(const vgrid_t* g, int k, int PD)
{
    int v = (2 * PD + g->PC[k] % 2) * g->R - g->PC[k] * g->R + g->pc[k];
    return (float)v;
}

/* ViewGrid.h:339-359 findCell. */
static void vgrid_find_cell(const vgrid_t* g, const float* p, int* c)
{
    double size_slab = (double)(float)(2 * g->R);
    for (int k = 0; k < g->dim; ++k) {
        float t = p[k] - g->p1[k];
        double li = (double)t + size_slab / 2;
        c[k] = (int)floor(li / size_slab);
    }
    for (int k = g->dim; k < 3; ++k) c[k] = 0;
}

static inline int vgrid_valid(const vgrid_t* g, const int* c)
{
    for (int k = 0; k < g->dim; ++k)
        if (c[k] < 0 || c[k] >= g->ext_dual[k]) return 0;
    return 1;
}

static inline int64_t vgrid_lin(const vgrid_t* g, const int* c)
{
    return ((int64_t)c[2] * g->ext_dual[1] + c[1]) * g->ext_dual[0] + c[0];
}

/* Cells as counting-sorted index lists (the reference's CellBMD buckets,
 * Cell.h:433-453, without the 32-slot cap; overflow is reported). */
typedef struct {
    vgrid_t g;
    int64_t ncell;
    int64_t* start; /* ncell + 1 */
    int64_t* items;
    int* cell_of;   /* per point: 3 ints */
    int max_occ;
} vcells_t;

static int vcells_build(vcells_t* vc, const float* sp, int64_t n, int dim, int R)
{
    vgrid_init(&vc->g, sp, n, dim, R);
    vc->ncell = (int64_t)vc->g.ext_dual[0] * vc->g.ext_dual[1] * vc->g.ext_dual[2];
    vc->start = (int64_t*)calloc((size_t)vc->ncell + 1, sizeof(int64_t));
    vc->items = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n > 0 ? n : 1));
    vc->cell_of = (int*)malloc(sizeof(int) * 3 * (size_t)(n > 0 ? n : 1));
    if (!vc->start || !vc->items || !vc->cell_of) return -1;
    for (int64_t i = 0; i < n; ++i) {
        int* c = vc->cell_of + 3 * i;
        vgrid_find_cell(&vc->g, sp + i * dim, c);
        if (!vgrid_valid(&vc->g, c)) return -2; /* reference: "erreur search" */
        vc->start[vgrid_lin(&vc->g, c) + 1]++;
    }
    vc->max_occ = 0;
    for (int64_t c = 0; c < vc->ncell; ++c) {
        if (vc->start[c + 1] > vc->max_occ) vc->max_occ = (int)vc->start[c + 1];
        vc->start[c + 1] += vc->start[c];
    }
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)vc->ncell);
    memcpy(fill, vc->start, sizeof(int64_t) * (size_t)vc->ncell);
    for (int64_t i = 0; i < n; ++i) vc->items[fill[vgrid_lin(&vc->g, vc->cell_of + 3 * i)]++] = i;
    free(fill);
    return 0;
}

static void vcells_free(vcells_t* vc)
{
    free(vc->start);
    free(vc->items);
    free(vc->cell_of);
}

/* ------------------------------------------------------------------------ */
/* Region table state                                                        */
/* ------------------------------------------------------------------------ */

/* Classify candidate q for query p and fold it into the table (NodeEMST.h:1193-1262). */
static inline int fold_candidate(int64_t p, int64_t q, const float* sp, int dim, const int64_t* lab,
                                 int64_t* tid, float* td2)
{
    float v = d2f(sp + p * dim, sp + q * dim, dim);
    if (!(v != 0 || (v == 0 && lab[q] != lab[p]))) return 0;
    float dl[3];
    for (int k = 0; k < dim; ++k) dl[k] = sp[q * dim + k] - sp[p * dim + k];
    uint32_t m = region_mask(dl, dim);
    int changed = 0;
    while (m) {
        int r = __builtin_ctz(m);
        m &= m - 1;
        int64_t cur = tid[r];
        if (cur == -1) {
            tid[r] = q;
            td2[r] = v;
            changed = 1;
        } else if (is_inf(mn(p, q), mx(p, q), v, mn(p, cur), mx(p, cur), td2[r])) {
            tid[r] = q;
            td2[r] = v;
            changed = 1;
        }
    }
    return changed;
}

/*
 * NodeComputeOctantMD::computeOctants (NodeEMST.h:1018-1296), one point,
 * faithful to the reference's ring / face / slab order and its per-face
 * closure rule.  tid/td2 hold the point's table (K entries) in and out.
 * Returns 1 when the reference would return true.
 */
static int faithful_compute_octants(int64_t p, const float* sp, const vcells_t* vc, const int64_t* lab,
                                    int64_t* tid_io, float* td2_io)
{
    const vgrid_t* g = &vc->g;
    const int dim = g->dim;
    const int nface = 2 * dim, nslab = dim == 3 ? 4 : 2, K = nface * nslab;
    int64_t tid[ORACLE_MAX_K];
    float td2[ORACLE_MAX_K];
    int faceV[6] = {0};
    int slabC[ORACLE_MAX_K];
    int allinit = 1, atleastonezero = 0, nozero = 1, ret = 0, modified = 0;
    for (int r = 0; r < K; ++r) {
        slabC[r] = 0;
        tid[r] = tid_io[r];
        td2[r] = td2_io[r];
        if (td2[r] == 0) {
            nozero = 0;
            atleastonezero = 1;
        } else if (tid[r] != -1)
            allinit = 0;
    }
    if (atleastonezero)
        for (int r = 0; r < K; ++r) {
            tid[r] = -1;
            td2[r] = INFINITY;
        }
    if (nozero && !allinit) return 1;
    const int* pc = vc->cell_of + 3 * p;
    const float* pps = sp + p * dim;
    int dmax = g->ext_dual[0];
    if (g->ext_dual[1] > dmax) dmax = g->ext_dual[1];
    if (g->ext_dual[2] > dmax) dmax = g->ext_dual[2];
    for (int radius = 0; radius <= dmax; ++radius) {
        int all = 1;
        for (int f = 0; f < nface; ++f) all = all && faceV[f];
        if (all) break;
        for (int f = 0; f < nface; ++f) {
            if (faceV[f]) continue;
            int dir = f / 2;
            int sens = (f % 2) ? -1 : 1;
            int base[3] = {pc[0], pc[1], pc[2]};
            base[dir] += radius * sens;
            if (!vgrid_valid(g, base)) {
                faceV[f] = 1;
                for (int s = 0; s < nslab; ++s) slabC[f * nslab + s] = 1;
            }
            if (!faceV[f] && radius > 0) {
                double ppsj = pps[dir];
                double size_slab = (double)(float)(2 * g->R);
                double cen = (double)vgrid_center(g, dir, base[dir]);
                double dist = fabs(cen - ppsj) - size_slab / 2;
                dist *= dist;
                for (int s = 0; s < nslab; ++s)
                    if (tid[f * nslab + s] != -1 && dist > (double)td2[f * nslab + s]) slabC[f * nslab + s] = 1;
            }
            if (!faceV[f]) {
                int v = 1;
                for (int s = 0; s < nslab; ++s) v = v && slabC[f * nslab + s];
                if (v) faceV[f] = 1;
            }
            if (faceV[f]) continue;
            for (int s = 0; s < nslab; ++s) {
                if (slabC[f * nslab + s]) continue;
                int sign[3] = {0, 0, 0}, ext[3] = {1, 1, 1}, bit = 1;
                for (int i = 0; i < dim; ++i) {
                    if (i == dir) continue;
                    sign[i] = (s & bit) ? -1 : 1;
                    ext[i] = radius + 1;
                    bit <<= 1;
                }
                for (int i2 = 0; i2 < ext[2]; ++i2)
                    for (int i1 = 0; i1 < ext[1]; ++i1)
                        for (int i0 = 0; i0 < ext[0]; ++i0) {
                            int idx[3] = {i0, i1, i2};
                            int c[3];
                            for (int k = 0; k < 3; ++k) c[k] = base[k] + idx[k] * sign[k];
                            if (dim == 2) c[2] = 0;
                            if (!vgrid_valid(g, c)) continue;
                            int64_t cl = vgrid_lin(g, c);
                            for (int64_t j = vc->start[cl]; j < vc->start[cl + 1]; ++j) {
                                int64_t q = vc->items[j];
                                if (q == p) continue;
                                if (fold_candidate(p, q, sp, dim, lab, tid, td2)) {
                                    modified = 1;
                                    ret = 1;
                                }
                            }
                        }
            }
        }
    }
    if (modified)
        for (int r = 0; r < K; ++r) {
            tid_io[r] = tid[r];
            td2_io[r] = td2[r];
        }
    return ret;
}

/* ------------------------------------------------------------------------ */
/* Exact region nearest neighbours (certified ring search)                   */
/* ------------------------------------------------------------------------ */

/*
 * Same per-region minimum as computeOctants intends -- for every region the
 * smallest (d2, id) over all points of the region that pass the zero-distance
 * filter -- computed by a ring search whose stop rule is certified per region
 * (a point of region R outside the scanned box crossed a box face the region's
 * cone can reach; its d2 is at least gap^2 through the dominant-axis face and
 * 2*gap^2 through a side face).  Independent of the cell size.
 */
static void exact_region_nn(int64_t p, const float* sp, const vcells_t* vc, const int64_t* lab,
                            int64_t* tid, float* td2)
{
    const vgrid_t* g = &vc->g;
    const int dim = g->dim;
    const int nslab = dim == 3 ? 4 : 2, K = 2 * dim * nslab;
    for (int r = 0; r < K; ++r) {
        tid[r] = -1;
        td2[r] = INFINITY;
    }
    const int* pc = vc->cell_of + 3 * p;
    const float* pps = sp + p * dim;
    int dmax = g->ext_dual[0];
    if (g->ext_dual[1] > dmax) dmax = g->ext_dual[1];
    if (g->ext_dual[2] > dmax) dmax = g->ext_dual[2];
    for (int radius = 0; radius <= dmax; ++radius) {
        int lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
        for (int k = 0; k < dim; ++k) {
            lo[k] = pc[k] - radius;
            hi[k] = pc[k] + radius;
        }
        for (int c2 = lo[2]; c2 <= hi[2]; ++c2)
            for (int c1 = lo[1]; c1 <= hi[1]; ++c1)
                for (int c0 = lo[0]; c0 <= hi[0]; ++c0) {
                    int c[3] = {c0, c1, c2};
                    int on_shell = 0;
                    for (int k = 0; k < dim; ++k)
                        if (c[k] == lo[k] || c[k] == hi[k]) on_shell = 1;
                    if (!on_shell) continue;
                    if (!vgrid_valid(g, c)) continue;
                    int64_t cl = vgrid_lin(g, c);
                    for (int64_t j = vc->start[cl]; j < vc->start[cl + 1]; ++j) {
                        int64_t q = vc->items[j];
                        if (q != p) fold_candidate(p, q, sp, dim, lab, tid, td2);
                    }
                }
        /* gaps to the box faces; INFINITY when the face is at / past the grid edge */
        double gap[3][2];
        for (int k = 0; k < dim; ++k) {
            double R = g->R;
            double lo_edge = (double)vgrid_center(g, k, lo[k]) - R;
            double hi_edge = (double)vgrid_center(g, k, hi[k]) + R;
            gap[k][0] = hi[k] >= g->ext_dual[k] - 1 ? INFINITY : hi_edge - (double)pps[k];
            gap[k][1] = lo[k] <= 0 ? INFINITY : (double)pps[k] - lo_edge;
        }
        int done = 1;
        for (int f = 0; f < 2 * dim && done; ++f) {
            int dir = f / 2, side = f % 2;
            for (int s = 0; s < nslab; ++s) {
                double lb = gap[dir][side] * gap[dir][side];
                int bit = 1;
                for (int i = 0; i < dim; ++i) {
                    if (i == dir) continue;
                    int sside = (s & bit) ? 1 : 0;
                    double gg = gap[i][sside];
                    if (2 * gg * gg < lb) lb = 2 * gg * gg;
                    bit <<= 1;
                }
                /* conservative margin: float rounding of d2 and of the gaps */
                if (!(isinf(lb) || (tid[f * nslab + s] != -1 && (double)td2[f * nslab + s] * (1 + 1e-5) + 1e-30 < lb))) {
                    done = 0;
                    break;
                }
            }
        }
        if (done) break;
    }
}

/* ------------------------------------------------------------------------ */
/* Boruvka driver: SolutionEMST::activate (SolutionEMSTOperators.cu:156-422) */
/* ------------------------------------------------------------------------ */

static int64_t find_root(const int64_t* ds, int64_t x)
{
    while (ds[x] != x) x = ds[x];
    return x;
}

/*
 * Full EMST on rescaled points sp (n*dim).
 * mode 0: faithful static pruning (reference ring process, levelRadius R);
 * mode 1: exact region nearest neighbours.
 * Outputs:
 *   edges_out: 2*(n-1) int64 (u < v), in the order the rounds produce them
 *              (round by round, winners in increasing point index);
 *   edge_round_out: round of each edge (1-based);
 *   round_edges_out: cumulative edge count after each round (<= 100 entries);
 *   labels_out: final disjoint-set labels (root point index per point);
 *   table_id_out / table_d2_out: the round-1 region table (n*K), optional.
 * Returns the number of rounds, or a negative error.
 */
int64_t oracle_emst(const float* sp, int64_t n, int dim, int mode, int R, int64_t* edges_out,
                    int32_t* edge_round_out, int64_t* round_edges_out, int64_t* labels_out,
                    int64_t* table_id_out, float* table_d2_out, int* max_occ_out)
{
    if (n <= 0 || (dim != 2 && dim != 3)) return -1;
    const int nslab = dim == 3 ? 4 : 2, K = 2 * dim * nslab;
    vcells_t vc;
    memset(&vc, 0, sizeof(vc));
    if (vcells_build(&vc, sp, n, dim, R) != 0) {
        vcells_free(&vc);
        return -2;
    }
    if (max_occ_out) *max_occ_out = vc.max_occ;
    int64_t* ds = (int64_t*)malloc(sizeof(int64_t) * n);
    int64_t* parent = (int64_t*)malloc(sizeof(int64_t) * n);
    int64_t* corr = (int64_t*)malloc(sizeof(int64_t) * n);
    float* dist = (float*)malloc(sizeof(float) * n);
    char* fix = (char*)malloc(n);
    int64_t* tid = (int64_t*)malloc(sizeof(int64_t) * n * K);
    float* td2 = (float*)malloc(sizeof(float) * n * K);
    int64_t* cbest_w = (int64_t*)malloc(sizeof(int64_t) * n);
    for (int64_t i = 0; i < n; ++i) {
        ds[i] = i; /* K_EMST_initDisjointSet, EMSTOperators.h:330-343 */
        for (int r = 0; r < K; ++r) {
            tid[i * K + r] = -1; /* NodeComputeOctantMD::init, NodeEMST.h:996-1011 */
            td2[i * K + r] = INFINITY;
        }
    }
    int64_t nedges = 0;
    int64_t iteration = 0;
    for (;;) {
        /* flatten (EMSTOperators.h:412-433): every point gets its root */
        for (int64_t i = 0; i < n; ++i) parent[i] = find_root(ds, i);
        memcpy(ds, parent, sizeof(int64_t) * n);
        /* testTermination (EMSTOperators.h:1517-1536) */
        int64_t r0 = find_root(ds, 0), ncomp = 0;
        for (int64_t i = 0; i < n; ++i)
            if (ds[i] != r0) ncomp++;
        if (ncomp == 0 || iteration == ORACLE_MAX_ROUNDS) break;
        iteration++;
        /* FIND MIN 1: reset, computeOctants, search */
        for (int64_t i = 0; i < n; ++i) {
            corr[i] = -1;
            dist[i] = INFINITY;
        }
        /* per-point work is independent within a round: parallel over points */
#pragma omp parallel for schedule(dynamic, 256)
        for (int64_t i = 0; i < n; ++i) {
            if (mode == 0) {
                faithful_compute_octants(i, sp, &vc, ds, tid + i * K, td2 + i * K);
            } else {
                /* same recompute rule as computeOctants: only on the first
                 * call, when nothing was found, or when a zero is held */
                int allinit = 1, zero = 0;
                for (int r = 0; r < K; ++r) {
                    if (td2[i * K + r] == 0) zero = 1;
                    else if (tid[i * K + r] != -1) allinit = 0;
                }
                if (zero || allinit) exact_region_nn(i, sp, &vc, ds, tid + i * K, td2 + i * K);
            }
            if (iteration == 1 && table_id_out) {
                for (int r = 0; r < K; ++r) {
                    table_id_out[i * K + r] = tid[i * K + r];
                    table_d2_out[i * K + r] = td2[i * K + r];
                }
            }
            /* NodeComputeOctantMD::search (NodeEMST.h:1303-1384) */
            int64_t best = -1;
            double bd = INFINITY;
            for (int r = 0; r < K; ++r) {
                int64_t q = tid[i * K + r];
                if (q == -1 || ds[q] == ds[i]) continue;
                double v = td2[i * K + r];
                if (best == -1 || is_inf(mn(i, q), mx(i, q), v, mn(i, best), mx(i, best), bd)) {
                    best = q;
                    bd = v;
                }
            }
            corr[i] = best;
            dist[i] = (float)bd;
        }
        /* FIND MIN 2: K_NEMST_findMinPair (NodeEMST.h:871-955) per component */
        for (int64_t i = 0; i < n; ++i) {
            fix[i] = 0;
            cbest_w[i] = -1;
        }
        for (int64_t i = 0; i < n; ++i) {
            if (corr[i] == -1) continue;
            int64_t c = ds[i];
            int64_t w = cbest_w[c];
            if (w == -1 || is_inf(mn(i, corr[i]), mx(i, corr[i]), dist[i], mn(w, corr[w]), mx(w, corr[w]), dist[w]))
                cbest_w[c] = i;
        }
        for (int64_t c = 0; c < n; ++c)
            if (cbest_w[c] != -1) fix[cbest_w[c]] = 1;
        /* union: K_EMST_connectComponentAndUnion_2 (EMSTOperators.h:1267-1303),
         * reading roots from the snapshot parent[] (EMSTOperators.h:1802-1814) */
        memcpy(parent, ds, sizeof(int64_t) * n);
        for (int64_t ps = 0; ps < n; ++ps) {
            if (!fix[ps]) continue;
            int64_t pq = corr[ps];
            int64_t rps = parent[ps], rpq = parent[pq];
            int mutual = fix[pq] && corr[pq] == ps;
            if (!mutual) {
                ds[rps] = rpq;
            } else if (ps < pq) {
                ds[rpq] = rps;
            }
            if (!mutual || ps < pq) {
                edges_out[2 * nedges] = mn(ps, pq);
                edges_out[2 * nedges + 1] = mx(ps, pq);
                if (edge_round_out) edge_round_out[nedges] = (int32_t)iteration;
                nedges++;
            }
        }
        if (round_edges_out) round_edges_out[iteration - 1] = nedges;
    }
    if (labels_out)
        for (int64_t i = 0; i < n; ++i) labels_out[i] = ds[i];
    free(ds);
    free(parent);
    free(corr);
    free(dist);
    free(fix);
    free(tid);
    free(td2);
    free(cbest_w);
    vcells_free(&vc);
    return iteration;
}

/* ------------------------------------------------------------------------ */
/* Region table only (for candidate-table parity)                            */
/* ------------------------------------------------------------------------ */

/* Round-1 table (all labels distinct) by the faithful or the exact search. */
int oracle_region_table(const float* sp, int64_t n, int dim, int mode, int R, int64_t* tid, float* td2)
{
    const int nslab = dim == 3 ? 4 : 2, K = 2 * dim * nslab;
    vcells_t vc;
    memset(&vc, 0, sizeof(vc));
    if (vcells_build(&vc, sp, n, dim, R) != 0) {
        vcells_free(&vc);
        return -2;
    }
    int64_t* lab = (int64_t*)malloc(sizeof(int64_t) * n);
    for (int64_t i = 0; i < n; ++i) lab[i] = i;
    for (int64_t i = 0; i < n; ++i) {
        for (int r = 0; r < K; ++r) {
            tid[i * K + r] = -1;
            td2[i * K + r] = INFINITY;
        }
        if (mode == 0)
            faithful_compute_octants(i, sp, &vc, lab, tid + i * K, td2 + i * K);
        else
            exact_region_nn(i, sp, &vc, lab, tid + i * K, td2 + i * K);
    }
    free(lab);
    vcells_free(&vc);
    return 0;
}

/* Brute-force region table, O(n^2), all labels distinct. */
int oracle_region_table_brute(const float* sp, int64_t n, int dim, int64_t* tid, float* td2)
{
    const int nslab = dim == 3 ? 4 : 2, K = 2 * dim * nslab;
    int64_t* lab = (int64_t*)malloc(sizeof(int64_t) * n);
    for (int64_t i = 0; i < n; ++i) lab[i] = i;
    for (int64_t i = 0; i < n; ++i) {
        for (int r = 0; r < K; ++r) {
            tid[i * K + r] = -1;
            td2[i * K + r] = INFINITY;
        }
        for (int64_t q = 0; q < n; ++q)
            if (q != i) fold_candidate(i, q, sp, dim, lab, tid + i * K, td2 + i * K);
    }
    free(lab);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Independent exact EMST: O(n^2) Prim under the same metric and tie-break   */
/* ------------------------------------------------------------------------ */

int oracle_prim(const float* sp, int64_t n, int dim, int64_t* edges_out)
{
    if (n <= 0) return -1;
    float* kd = (float*)malloc(sizeof(float) * n);
    int64_t* kfrom = (int64_t*)malloc(sizeof(int64_t) * n);
    char* in = (char*)calloc(n, 1);
    for (int64_t i = 0; i < n; ++i) {
        kd[i] = INFINITY;
        kfrom[i] = -1;
    }
    int64_t cur = 0, ne = 0;
    in[0] = 1;
    for (int64_t it = 1; it < n; ++it) {
        for (int64_t v = 0; v < n; ++v) {
            if (in[v]) continue;
            float d = d2f(sp + cur * dim, sp + v * dim, dim);
            if (kfrom[v] == -1 || is_inf(mn(cur, v), mx(cur, v), d, mn(kfrom[v], v), mx(kfrom[v], v), kd[v])) {
                kd[v] = d;
                kfrom[v] = cur;
            }
        }
        int64_t best = -1;
        for (int64_t v = 0; v < n; ++v) {
            if (in[v]) continue;
            if (best == -1 ||
                is_inf(mn(kfrom[v], v), mx(kfrom[v], v), kd[v], mn(kfrom[best], best), mx(kfrom[best], best), kd[best]))
                best = v;
        }
        in[best] = 1;
        edges_out[2 * ne] = mn(kfrom[best], best);
        edges_out[2 * ne + 1] = mx(kfrom[best], best);
        ne++;
        cur = best;
    }
    free(kd);
    free(kfrom);
    free(in);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* Tree length: K_EMST_evaluate_ST + K_sumReduction                          */
/* ------------------------------------------------------------------------ */

/*
 * EMSTOperators.h:262-292 and SolutionEMST.cu:567-573: sum over edges of
 * sqrt(double(float dot)) in the ORIGINAL coordinates.  The reference sums
 * each edge twice (once per endpoint) and halves; this sums once.
 */
double oracle_length(const float* orig, int dim, const int64_t* edges, int64_t ne)
{
    double s = 0;
    for (int64_t e = 0; e < ne; ++e) s += sqrt((double)d2f(orig + edges[2 * e] * dim, orig + edges[2 * e + 1] * dim, dim));
    return s;
}

/* ------------------------------------------------------------------------ */
/* Full-size checks                                                          */
/* ------------------------------------------------------------------------ */

/* Exact region table rows for selected query points only (all labels
 * distinct, as in round 1), using the certified ring search above. */
int oracle_region_rows(const float* sp, int64_t n, int dim, int R, const int64_t* rows, int64_t nrows, int64_t* tid,
                       float* td2)
{
    const int nslab = dim == 3 ? 4 : 2, K = 2 * dim * nslab;
    vcells_t vc;
    memset(&vc, 0, sizeof(vc));
    if (vcells_build(&vc, sp, n, dim, R) != 0) {
        vcells_free(&vc);
        return -2;
    }
    int64_t* lab = (int64_t*)malloc(sizeof(int64_t) * n);
    for (int64_t i = 0; i < n; ++i) lab[i] = i;
    for (int64_t k = 0; k < nrows; ++k) exact_region_nn(rows[k], sp, &vc, lab, tid + k * K, td2 + k * K);
    free(lab);
    vcells_free(&vc);
    return 0;
}

typedef struct {
    float d2;
    int64_t a, b;
} kedge_t;

static int kedge_cmp(const void* x, const void* y)
{
    const kedge_t* p = (const kedge_t*)x;
    const kedge_t* q = (const kedge_t*)y;
    if (is_inf(p->a, p->b, p->d2, q->a, q->b, q->d2)) return -1;
    if (is_inf(q->a, q->b, q->d2, p->a, p->b, p->d2)) return 1;
    return 0;
}

static int64_t uf_find(int64_t* par, int64_t x)
{
    while (par[x] != x) {
        par[x] = par[par[x]];
        x = par[x];
    }
    return x;
}

/* Kruskal under the (d2, min id, max id) order over an explicit candidate
 * graph: table ids (n*K, -1 = none) and their squared distances.  Returns
 * the number of MST edges written to edges_out (2 per edge, u < v). */
int64_t oracle_kruskal_table(int64_t n, int K, const int32_t* ids, const float* d2, int64_t* edges_out)
{
    int64_t m = 0;
    kedge_t* e = (kedge_t*)malloc(sizeof(kedge_t) * (size_t)(n * K > 0 ? n * K : 1));
    for (int64_t p = 0; p < n; ++p)
        for (int r = 0; r < K; ++r) {
            int64_t q = ids[p * K + r];
            if (q < 0) continue;
            e[m].d2 = d2[p * K + r];
            e[m].a = mn(p, q);
            e[m].b = mx(p, q);
            m++;
        }
    qsort(e, (size_t)m, sizeof(kedge_t), kedge_cmp);
    int64_t* par = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
    for (int64_t i = 0; i < n; ++i) par[i] = i;
    int64_t ne = 0;
    for (int64_t k = 0; k < m; ++k) {
        int64_t ra = uf_find(par, e[k].a), rb = uf_find(par, e[k].b);
        if (ra == rb) continue;
        par[ra] = rb;
        edges_out[2 * ne] = e[k].a;
        edges_out[2 * ne + 1] = e[k].b;
        ne++;
    }
    free(par);
    free(e);
    return ne;
}
