/*
 * CPU restatement of VariantDBSCAN's from-scratch clustering path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the GB300 library:
 * only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it.  The product (variantdbscan_gb300/) never links or calls it.
 *
 * It restates, in plain C, what the reference computes for one variant when
 * libVDBSCAN is called with numVariants=1 (the algDBScanParallel path):
 *
 *   - visit order: binDataset (src/main.cpp:459-605): a 300x300 grid over the
 *     bounding box (widths x1.01, max initialised to DBL_MIN at
 *     src/main.cpp:467-468), xbin = floor(((x+xoffset)/x_width)*300), points
 *     ordered by (xbin, ybin) and, inside one bin, by input index;
 *   - multiple-point boxes: groups of MBBsize consecutive visit-ordered points
 *     (src/main.cpp:404-436, src/structs.h:79-120) inserted in the R-tree;
 *   - the epsilon neighbourhood (src/DBScan.cpp:627-702): candidates are the
 *     points of every box that overlaps [x-eps,x+eps]x[y-eps,y+eps]
 *     (inclusive overlap, src/RTree.h:1613-1625); a candidate is kept when
 *     sqrt((px-qx)^2+(py-qy)^2) <= eps in FP64 without FMA contraction
 *     (src/DBScan.cpp:687, 699-702);
 *   - the expansion (src/DBScan.cpp:523-609): points visited in visit order,
 *     noise = 0, clusters numbered 1..K in the order their seeds are met,
 *     expansion skips points visited earlier (so such border points stay 0).
 *
 * Candidate generation uses a uniform grid instead of the R-tree; the grid is
 * only a candidate superset (cell width > eps), the predicate above decides.
 * The expansion is a depth-first search that marks points when they are pushed
 * instead of when they are popped; inside one expansion every pushed point is
 * popped and labelled before the main loop moves on, so the labelled set and
 * the labels are the same as the reference's (which pushes whole neighbour
 * lists, src/DBScan.cpp:565, 589).
 *
 * Build: gcc -O2 -std=c11 -ffp-contract=off -fopenmp -shared -fPIC
 * (-ffp-contract=off keeps fl(fl(dx*dx)+fl(dy*dy)) unfused on aarch64).
 */
#include <float.h>
#include <limits.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_OK 0
#define ORC_ERR_ARG 1
#define ORC_ERR_DEGENERATE 2
#define ORC_ERR_NOMEM 3

#define NUM_BINS 300

/* ---------------------------------------------------------------- visit order */

/* Bin keys and the stable order of src/main.cpp:459-605.  Returns
 * ORC_ERR_DEGENERATE where the reference would print "bins out of range" and
 * return early (zero or non-finite bin width). */
int orc_visit_keys(const double *x, const double *y, uint32_t n, uint32_t *keys)
{
    double min_x = DBL_MAX, min_y = DBL_MAX;
    double max_x = DBL_MIN, max_y = DBL_MIN; /* src/main.cpp:467-468 */
    for (uint32_t i = 0; i < n; i++) {
        if (x[i] < min_x) min_x = x[i];
        if (x[i] > max_x) max_x = x[i];
        if (y[i] < min_y) min_y = y[i];
        if (y[i] > max_y) max_y = y[i];
    }
    double x_width = (max_x - min_x) * 1.01;
    double y_width = (max_y - min_y) * 1.01;
    double xoffset = (min_x > 0) ? -min_x : fabs(min_x);
    double yoffset = (min_y > 0) ? -min_y : fabs(min_y);
    for (uint32_t i = 0; i < n; i++) {
        double fx = floor(((x[i] + xoffset) / x_width) * NUM_BINS);
        double fy = floor(((y[i] + yoffset) / y_width) * NUM_BINS);
        if (!(fx >= 0.0 && fx <= NUM_BINS - 1) || !(fy >= 0.0 && fy <= NUM_BINS - 1))
            return ORC_ERR_DEGENERATE;
        keys[i] = (uint32_t)fx * NUM_BINS + (uint32_t)fy;
    }
    return ORC_OK;
}

/* mapping[k] = input index of the point visited k-th (src/main.cpp:581-595). */
int orc_visit_order(const double *x, const double *y, uint32_t n, uint32_t *mapping)
{
    uint32_t *keys = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    uint32_t *cnt = (uint32_t *)calloc(NUM_BINS * NUM_BINS + 1, sizeof(uint32_t));
    if (!keys || !cnt) { free(keys); free(cnt); return ORC_ERR_NOMEM; }
    int rc = orc_visit_keys(x, y, n, keys);
    if (rc == ORC_OK) {
        for (uint32_t i = 0; i < n; i++) cnt[keys[i] + 1]++;
        for (uint32_t b = 0; b < NUM_BINS * NUM_BINS; b++) cnt[b + 1] += cnt[b];
        for (uint32_t i = 0; i < n; i++) mapping[cnt[keys[i]]++] = i; /* stable */
    }
    free(keys);
    free(cnt);
    return rc;
}

/* Largest double t with sqrt(t) <= eps (sqrt correctly rounded, monotone), so
 * that sqrt(d2) <= eps  <=>  d2 <= t.  -1 when no d2 >= 0 qualifies. */
double orc_eps_sq_threshold(double eps)
{
    if (!(eps >= 0.0)) return -1.0;
    if (isinf(eps)) return INFINITY;
    double t = eps * eps;
    while (t > 0.0 && sqrt(t) > eps) t = nextafter(t, 0.0);
    for (;;) {
        double u = nextafter(t, INFINITY);
        if (isinf(u) || sqrt(u) > eps) break;
        t = u;
    }
    return t;
}

/* ------------------------------------------------------------------ dataset */

typedef struct {
    uint32_t n;
    int mbb;
    double eps, thr;
    double sq_lo, sq_hi;          /* d2 <= sq_lo: sqrt(d2) <= eps; d2 > sq_hi: > eps */
    const double *vx, *vy;        /* visit order */
    double *mpb;                  /* [nmpb][4]: minx, maxx, miny, maxy */
    /* grid over visit-ordered points, cells of width >= eps */
    double x0, y0, w;
    int64_t ncx, ncy;
    int64_t *gkey;                /* sorted cell keys */
    uint32_t *gidx;               /* visit positions sorted by cell key */
    double *gx, *gy;              /* coordinates in cell order */
    uint32_t *cstart;             /* ncells+1 first positions (NULL: binary search) */
} orc_ctx;

typedef struct { int64_t key; uint32_t idx; } keyidx;

static int cmp_keyidx(const void *a, const void *b)
{
    const keyidx *p = (const keyidx *)a, *q = (const keyidx *)b;
    if (p->key != q->key) return p->key < q->key ? -1 : 1;
    return p->idx < q->idx ? -1 : (p->idx > q->idx);
}

static int ctx_build(orc_ctx *c, const double *vx, const double *vy, uint32_t n, double eps, int mbb)
{
    memset(c, 0, sizeof(*c));
    c->n = n; c->mbb = mbb; c->eps = eps; c->vx = vx; c->vy = vy;
    c->thr = orc_eps_sq_threshold(eps);
    /* sqrt is correctly rounded: outside eps^2 (1 -+ 1e-9) its comparison
     * with eps is decided by d2 alone (the relative error of these bounds is
     * far below 1e-9) */
    c->sq_lo = eps * eps * (1.0 - 1e-9);
    c->sq_hi = eps * eps * (1.0 + 1e-9);
    uint32_t nmpb = (n + (uint32_t)mbb - 1) / (uint32_t)mbb;
    c->mpb = (double *)malloc(sizeof(double) * 4 * (nmpb ? nmpb : 1));
    c->gkey = (int64_t *)malloc(sizeof(int64_t) * (n ? n : 1));
    c->gidx = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    c->gx = (double *)malloc(sizeof(double) * (n ? n : 1));
    c->gy = (double *)malloc(sizeof(double) * (n ? n : 1));
    keyidx *ki = (keyidx *)malloc(sizeof(keyidx) * (n ? n : 1));
    if (!c->mpb || !c->gkey || !c->gidx || !c->gx || !c->gy || !ki) { free(ki); return ORC_ERR_NOMEM; }
    for (uint32_t b = 0; b < nmpb; b++) {
        uint32_t s = b * (uint32_t)mbb, e = s + (uint32_t)mbb < n ? s + (uint32_t)mbb : n;
        double *m = c->mpb + 4 * (size_t)b;
        m[0] = m[1] = vx[s]; m[2] = m[3] = vy[s];
        for (uint32_t k = s; k < e; k++) {
            if (vx[k] < m[0]) m[0] = vx[k];
            if (vx[k] > m[1]) m[1] = vx[k];
            if (vy[k] < m[2]) m[2] = vy[k];
            if (vy[k] > m[3]) m[3] = vy[k];
        }
    }
    double minx = INFINITY, maxx = -INFINITY, miny = INFINITY, maxy = -INFINITY;
    for (uint32_t k = 0; k < n; k++) {
        if (vx[k] < minx) minx = vx[k];
        if (vx[k] > maxx) maxx = vx[k];
        if (vy[k] < miny) miny = vy[k];
        if (vy[k] > maxy) maxy = vy[k];
    }
    double range = fmax(maxx - minx, maxy - miny);
    double w = fmax(eps, 0x1p-500) * (1.0 + 0x1p-20);
    if (range / w > 0x1p28) w = range * 0x1p-28 * (1.0 + 0x1p-20);
    c->x0 = minx; c->y0 = miny; c->w = w;
    c->ncx = (int64_t)floor((maxx - minx) / w) + 1;
    c->ncy = (int64_t)floor((maxy - miny) / w) + 1;
    for (uint32_t k = 0; k < n; k++) {
        int64_t cx = (int64_t)floor((vx[k] - minx) / w);
        int64_t cy = (int64_t)floor((vy[k] - miny) / w);
        ki[k].key = cy * c->ncx + cx;
        ki[k].idx = k;
    }
    qsort(ki, n, sizeof(keyidx), cmp_keyidx);
    for (uint32_t k = 0; k < n; k++) {
        c->gkey[k] = ki[k].key; c->gidx[k] = ki[k].idx;
        c->gx[k] = vx[ki[k].idx]; c->gy[k] = vy[ki[k].idx];
    }
    free(ki);
    /* dense first-position array when the grid is not much larger than 2^26 cells */
    int64_t ncells = c->ncx * c->ncy;
    if (n && ncells <= ((int64_t)1 << 26)) {
        c->cstart = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(ncells + 1));
        if (c->cstart) {
            uint32_t k = 0;
            for (int64_t cell = 0; cell <= ncells; cell++) {
                while (k < n && c->gkey[k] < cell) k++;
                c->cstart[cell] = k;
            }
        }
    }
    return ORC_OK;
}

static void ctx_free(orc_ctx *c)
{
    free(c->mpb); free(c->gkey); free(c->gidx); free(c->gx); free(c->gy); free(c->cstart);
}

static uint32_t lower_bound64(const int64_t *a, uint32_t n, int64_t v)
{
    uint32_t lo = 0, hi = n;
    while (lo < hi) {
        uint32_t mid = lo + (hi - lo) / 2;
        if (a[mid] < v) lo = mid + 1; else hi = mid;
    }
    return lo;
}

/* sqrt(d2) <= eps (src/DBScan.cpp:687, 699-702), d2 = fl(fl(dx*dx)+fl(dy*dy)) */
static int within_eps(const orc_ctx *c, double px, double py, double qx, double qy)
{
    double dx = px - qx, dy = py - qy;
    double d2 = dx * dx + dy * dy; /* compiled with -ffp-contract=off */
    if (d2 <= c->sq_lo) return 1;
    if (d2 > c->sq_hi || d2 != d2) return 0;
    return sqrt(d2) <= c->eps;
}

/* The R-tree candidate rule (src/RTree.h:1613-1625): the multiple-point box of
 * visit position q overlaps the query box [p-eps, p+eps]^2
 * (src/DBScan.cpp:722-731). */
static int box_ok(const orc_ctx *c, double px, double py, uint32_t q)
{
    double bminx = px - c->eps, bmaxx = px + c->eps;
    double bminy = py - c->eps, bmaxy = py + c->eps;
    const double *m = c->mpb + 4 * (size_t)(q / (uint32_t)c->mbb);
    if (bminx > m[1] || m[0] > bmaxx) return 0;
    if (bminy > m[3] || m[2] > bmaxy) return 0;
    return 1;
}

/* box_ok for a candidate at (qx, qy): a point inside the query box lies in
 * its own multiple-point box, which then overlaps the query box, so only
 * points outside it need their box. */
static int box_rule(const orc_ctx *c, double px, double py, double qx, double qy, uint32_t q)
{
    double bminx = px - c->eps, bmaxx = px + c->eps;
    double bminy = py - c->eps, bmaxy = py + c->eps;
    if (!(bminx > qx || qx > bmaxx || bminy > qy || qy > bmaxy)) return 1;
    return box_ok(c, px, py, q);
}

/* q (visit position) is in N(p): src/DBScan.cpp:665-702 with the R-tree
 * candidate rule applied to q's multiple-point box. */
static int in_neighbourhood(const orc_ctx *c, uint32_t p, uint32_t q)
{
    double px = c->vx[p], py = c->vy[p];
    return within_eps(c, px, py, c->vx[q], c->vy[q]) && box_ok(c, px, py, q);
}

/* Calls fn(q) for every q in N(p); returns |N(p)|. */
static uint64_t neighbours(const orc_ctx *c, uint32_t p, uint32_t *out)
{
    if (!(c->eps >= 0.0)) return 0;
    double px = c->vx[p], py = c->vy[p];
    int64_t cx = (int64_t)floor((px - c->x0) / c->w);
    int64_t cy = (int64_t)floor((py - c->y0) / c->w);
    uint64_t cnt = 0;
    for (int64_t ry = cy - 1; ry <= cy + 1; ry++) {
        if (ry < 0 || ry >= c->ncy) continue;
        int64_t lo = cx - 1 < 0 ? 0 : cx - 1;
        int64_t hi = cx + 1 >= c->ncx ? c->ncx - 1 : cx + 1;
        uint32_t s, e;
        if (c->cstart) {
            s = c->cstart[ry * c->ncx + lo];
            e = c->cstart[ry * c->ncx + hi + 1];
        } else {
            s = lower_bound64(c->gkey, c->n, ry * c->ncx + lo);
            e = lower_bound64(c->gkey, c->n, ry * c->ncx + hi + 1);
        }
        for (uint32_t k = s; k < e; k++) {
            if (!within_eps(c, px, py, c->gx[k], c->gy[k])) continue;
            uint32_t q = c->gidx[k];
            if (!box_rule(c, px, py, c->gx[k], c->gy[k], q)) continue;
            if (out) out[cnt] = q;
            cnt++;
        }
    }
    return cnt;
}

static int prepare(const double *x, const double *y, uint32_t n, int mbb,
                   uint32_t **mapping, double **vx, double **vy)
{
    *mapping = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    *vx = (double *)malloc(sizeof(double) * (n ? n : 1));
    *vy = (double *)malloc(sizeof(double) * (n ? n : 1));
    if (!*mapping || !*vx || !*vy) return ORC_ERR_NOMEM;
    if (mbb <= 0) return ORC_ERR_ARG;
    int rc = orc_visit_order(x, y, n, *mapping);
    if (rc) return rc;
    for (uint32_t k = 0; k < n; k++) { (*vx)[k] = x[(*mapping)[k]]; (*vy)[k] = y[(*mapping)[k]]; }
    return ORC_OK;
}

/* |N(p)| for every input point (input order).  Returns the total in *pairs. */
int orc_neighbor_counts(const double *x, const double *y, uint32_t n, double eps, int mbb,
                        uint32_t *counts, uint64_t *pairs)
{
    uint32_t *mapping = NULL; double *vx = NULL, *vy = NULL;
    int rc = prepare(x, y, n, mbb, &mapping, &vx, &vy);
    orc_ctx c; memset(&c, 0, sizeof(c));
    if (rc == ORC_OK) rc = ctx_build(&c, vx, vy, n, eps, mbb);
    uint64_t tot = 0;
    if (rc == ORC_OK) {
        #pragma omp parallel for schedule(dynamic, 256) reduction(+ : tot)
        for (int64_t k = 0; k < (int64_t)n; k++) {
            uint64_t m = neighbours(&c, (uint32_t)k, NULL);
            counts[mapping[k]] = (uint32_t)m;
            tot += m;
        }
        if (pairs) *pairs = tot;
    }
    ctx_free(&c); free(mapping); free(vx); free(vy);
    return rc;
}

/* Exact neighbour lists, input indices, rows in input order (CSR).  offsets has
 * n+1 entries; nbrs must hold the total returned by orc_neighbor_counts. */
int orc_neighbor_lists(const double *x, const double *y, uint32_t n, double eps, int mbb,
                       const uint64_t *offsets, uint32_t *nbrs)
{
    uint32_t *mapping = NULL; double *vx = NULL, *vy = NULL;
    int rc = prepare(x, y, n, mbb, &mapping, &vx, &vy);
    orc_ctx c; memset(&c, 0, sizeof(c));
    if (rc == ORC_OK) rc = ctx_build(&c, vx, vy, n, eps, mbb);
    if (rc == ORC_OK) {
        #pragma omp parallel for schedule(dynamic, 256)
        for (int64_t k = 0; k < (int64_t)n; k++) {
            uint32_t *row = nbrs + offsets[mapping[k]];
            uint64_t m = neighbours(&c, (uint32_t)k, row);
            for (uint64_t j = 0; j < m; j++) row[j] = mapping[row[j]];
        }
    }
    ctx_free(&c); free(mapping); free(vx); free(vy);
    return rc;
}

/* Brute-force |N(p)| over all pairs (tests only; O(n^2)). */
int orc_neighbor_counts_bruteforce(const double *x, const double *y, uint32_t n, double eps,
                                   int mbb, uint32_t *counts)
{
    uint32_t *mapping = NULL; double *vx = NULL, *vy = NULL;
    int rc = prepare(x, y, n, mbb, &mapping, &vx, &vy);
    orc_ctx c; memset(&c, 0, sizeof(c));
    if (rc == ORC_OK) rc = ctx_build(&c, vx, vy, n, eps, mbb);
    if (rc == ORC_OK) {
        #pragma omp parallel for schedule(dynamic, 64)
        for (int64_t p = 0; p < (int64_t)n; p++) {
            uint32_t m = 0;
            for (uint32_t q = 0; q < n; q++) m += (uint32_t)in_neighbourhood(&c, (uint32_t)p, q);
            counts[mapping[p]] = m;
        }
    }
    ctx_free(&c); free(mapping); free(vx); free(vy);
    return rc;
}

/* splitmix64 finaliser (a published 64-bit mixer). */
static uint64_t mix64(uint64_t x)
{
    x ^= x >> 30;
    x *= 0xbf58476d1ce4e5b9ULL;
    x ^= x >> 27;
    x *= 0x94d049bb133111ebULL;
    x ^= x >> 31;
    return x;
}

/* Hash of the neighbour relation of one epsilon, as the GB300 library reports
 * it in vdb_stats.table_hash: the sum modulo 2^64 over p and q in N(p) of
 * mix64(p << 32 | q) + (p not in N(q) ? 0x9e3779b97f4a7c15 : 0), p and q
 * input indices.  Not a reference function: a checksum of N(p) for all p.
 * p in N(q) is the same predicate with the roles swapped: the distance is
 * the same bit for bit (fl(a-b) = -fl(b-a)), so only the box rule is
 * evaluated again, with p's multiple-point box against q's query box. */
int orc_table_hash(const double *x, const double *y, uint32_t n, double eps, int mbb,
                   uint64_t *hash)
{
    uint32_t *mapping = NULL; double *vx = NULL, *vy = NULL;
    int rc = prepare(x, y, n, mbb, &mapping, &vx, &vy);
    orc_ctx c; memset(&c, 0, sizeof(c));
    if (rc == ORC_OK) rc = ctx_build(&c, vx, vy, n, eps, mbb);
    uint32_t *gorig = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    if (rc == ORC_OK && !gorig) rc = ORC_ERR_NOMEM;
    uint64_t h = 0;
    if (rc == ORC_OK && eps >= 0.0) {
        for (uint32_t k = 0; k < n; k++) gorig[k] = mapping[c.gidx[k]];
        #pragma omp parallel for schedule(dynamic, 256) reduction(+ : h)
        for (int64_t kk = 0; kk < (int64_t)n; kk++) {
            uint32_t k = (uint32_t)kk;
            double px = vx[k], py = vy[k];
            const double *pm = c.mpb + 4 * (size_t)(k / (uint32_t)mbb);
            uint64_t prow = (uint64_t)mapping[k] << 32;
            int64_t cx = (int64_t)floor((px - c.x0) / c.w);
            int64_t cy = (int64_t)floor((py - c.y0) / c.w);
            for (int64_t ry = cy - 1; ry <= cy + 1; ry++) {
                if (ry < 0 || ry >= c.ncy) continue;
                int64_t lo = cx - 1 < 0 ? 0 : cx - 1;
                int64_t hi = cx + 1 >= c.ncx ? c.ncx - 1 : cx + 1;
                uint32_t s0, e0;
                if (c.cstart) {
                    s0 = c.cstart[ry * c.ncx + lo];
                    e0 = c.cstart[ry * c.ncx + hi + 1];
                } else {
                    s0 = lower_bound64(c.gkey, n, ry * c.ncx + lo);
                    e0 = lower_bound64(c.gkey, n, ry * c.ncx + hi + 1);
                }
                for (uint32_t j = s0; j < e0; j++) {
                    double qx = c.gx[j], qy = c.gy[j];
                    if (!within_eps(&c, px, py, qx, qy)) continue;
                    if (!box_rule(&c, px, py, qx, qy, c.gidx[j])) continue;
                    h += mix64(prow | gorig[j]);
                    /* p's box against q's query box [q-eps, q+eps]^2 */
                    double bminx = qx - eps, bmaxx = qx + eps;
                    double bminy = qy - eps, bmaxy = qy + eps;
                    if (bminx > pm[1] || pm[0] > bmaxx || bminy > pm[3] || pm[2] > bmaxy)
                        h += 0x9e3779b97f4a7c15ULL;
                }
            }
        }
    }
    if (rc == ORC_OK && hash) *hash = h;
    ctx_free(&c); free(mapping); free(vx); free(vy); free(gorig);
    return rc;
}

/* DBSCAN labels of one variant from the neighbour counts of its epsilon
 * (src/DBScan.cpp:523-609): the main loop in visit order, a stack expansion
 * from each unvisited core, visited points never re-labelled, then the
 * un-permutation of src/main.cpp:255-262.  row holds maxdeg entries. */
static int dfs_labels(const orc_ctx *c, const uint32_t *counts, uint64_t maxdeg, uint64_t mp,
                      const uint32_t *mapping, uint32_t *labels, uint32_t *nclusters)
{
    uint32_t n = c->n;
    uint8_t *visited = (uint8_t *)calloc(n ? n : 1, 1);
    uint32_t *lab = (uint32_t *)calloc(n ? n : 1, sizeof(uint32_t));
    uint32_t *stack = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    uint32_t *row = (uint32_t *)malloc(sizeof(uint32_t) * (maxdeg ? maxdeg : 1));
    int rc = ORC_OK;
    if (!visited || !lab || !stack || !row) rc = ORC_ERR_NOMEM;
    uint32_t cluster = 0;
    if (rc == ORC_OK) {
        for (uint32_t i = 0; i < n; i++) {
            if (visited[i]) continue;
            visited[i] = 1;
            if ((uint64_t)counts[i] < mp) { lab[i] = 0; continue; }
            cluster++;
            lab[i] = cluster;
            uint64_t top = 0;
            uint64_t m = neighbours(c, i, row);
            for (uint64_t j = 0; j < m; j++)
                if (!visited[row[j]]) { visited[row[j]] = 1; stack[top++] = row[j]; }
            while (top) {
                uint32_t v = stack[--top];
                lab[v] = cluster;
                if ((uint64_t)counts[v] >= mp) {
                    m = neighbours(c, v, row);
                    for (uint64_t j = 0; j < m; j++)
                        if (!visited[row[j]]) { visited[row[j]] = 1; stack[top++] = row[j]; }
                }
            }
        }
        for (uint32_t k = 0; k < n; k++) labels[mapping[k]] = lab[k];
        if (nclusters) *nclusters = cluster;
    }
    free(visited); free(lab); free(stack); free(row);
    return rc;
}

/* Neighbour counts of every visit position (parallel); returns the largest. */
static uint64_t visit_counts(const orc_ctx *c, uint32_t *counts)
{
    uint64_t maxdeg = 0;
    #pragma omp parallel for schedule(dynamic, 256) reduction(max : maxdeg)
    for (int64_t k = 0; k < (int64_t)c->n; k++) {
        uint64_t m = neighbours(c, (uint32_t)k, NULL);
        counts[k] = (uint32_t)m;
        if (m > maxdeg) maxdeg = m;
    }
    return maxdeg;
}

/* src/DBScan.cpp:69 stores minpts in an int and compares it with a size_t:
 * values above INT_MAX become huge and no point is core. */
static uint64_t minpts_bound(uint32_t minpts)
{
    return minpts > (uint32_t)INT_MAX ? UINT64_MAX : (uint64_t)minpts;
}

/* One variant, labels in input order (src/DBScan.cpp:523-609, then the
 * un-permutation of src/main.cpp:255-262).  nclusters = K (noise excluded). */
int orc_dbscan(const double *x, const double *y, uint32_t n, double eps, uint32_t minpts,
               int mbb, uint32_t *labels, uint32_t *nclusters)
{
    uint32_t *mapping = NULL; double *vx = NULL, *vy = NULL;
    int rc = prepare(x, y, n, mbb, &mapping, &vx, &vy);
    orc_ctx c; memset(&c, 0, sizeof(c));
    if (rc == ORC_OK) rc = ctx_build(&c, vx, vy, n, eps, mbb);
    uint32_t *counts = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    if (rc == ORC_OK && !counts) rc = ORC_ERR_NOMEM;
    if (rc == ORC_OK) {
        uint64_t maxdeg = visit_counts(&c, counts);
        rc = dfs_labels(&c, counts, maxdeg, minpts_bound(minpts), mapping, labels, nclusters);
    }
    ctx_free(&c); free(mapping); free(vx); free(vy); free(counts);
    return rc;
}

/* nv variants of one dataset, each clustered on its own exactly as
 * orc_dbscan does (labels[v*n + i], input order).  The visit order is computed
 * once; per distinct epsilon the grid and the neighbour counts are computed
 * once, and the variants of that epsilon are labelled in parallel threads
 * (the labelling of one variant is sequential, as in the reference). */
int orc_dbscan_many(const double *x, const double *y, uint32_t n, const double *eps,
                    const uint32_t *minpts, uint32_t nv, int mbb, uint32_t *labels)
{
    uint32_t *mapping = NULL; double *vx = NULL, *vy = NULL;
    int rc = prepare(x, y, n, mbb, &mapping, &vx, &vy);
    uint32_t *counts = (uint32_t *)malloc(sizeof(uint32_t) * (n ? n : 1));
    uint32_t *group = (uint32_t *)malloc(sizeof(uint32_t) * (nv ? nv : 1));
    uint8_t *done = (uint8_t *)calloc(nv ? nv : 1, 1);
    if (rc == ORC_OK && (!counts || !group || !done)) rc = ORC_ERR_NOMEM;
    for (uint32_t v0 = 0; rc == ORC_OK && v0 < nv; v0++) {
        if (done[v0]) continue;
        uint32_t ng = 0;
        for (uint32_t v = v0; v < nv; v++)
            if (!done[v] && (eps[v] == eps[v0] || (eps[v] != eps[v] && eps[v0] != eps[v0]))) {
                group[ng++] = v;
                done[v] = 1;
            }
        orc_ctx c; memset(&c, 0, sizeof(c));
        rc = ctx_build(&c, vx, vy, n, eps[v0], mbb);
        if (rc == ORC_OK) {
            uint64_t maxdeg = visit_counts(&c, counts);
            int bad = ORC_OK;
            #pragma omp parallel for schedule(dynamic, 1)
            for (int64_t g = 0; g < (int64_t)ng; g++) {
                uint32_t v = group[g];
                int r = dfs_labels(&c, counts, maxdeg, minpts_bound(minpts[v]), mapping,
                                   labels + (size_t)v * n, NULL);
                if (r != ORC_OK) {
                    #pragma omp critical
                    bad = r;
                }
            }
            rc = bad;
        }
        ctx_free(&c);
    }
    free(mapping); free(vx); free(vy); free(counts); free(group); free(done);
    return rc;
}
