/*
 * dpg_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY) for the 2D granular
 * contact hot path of mmccraw98/dpCUDA-v2: cell list + Verlet neighbour
 * build, harmonic disk contacts, NVE velocity Verlet, FIRE, Adam, stress /
 * pressure and the box-scaling / last-state pieces used by jamming.
 *
 * Used only by tests/ (as the parity checker) and by bench.py's CPU
 * baseline leg.  The product library never links or calls this file.
 *
 * Each function restates the reference algorithm in its own code and cites
 * the reference file:line it follows.  Compile with -ffp-contract=off so the
 * per-particle arithmetic matches the reference operation for operation.
 * Per-particle loops are OpenMP-parallel (independent items, so results do
 * not depend on the thread count); reductions are sequential sums in index
 * order.
 */
#include "dpg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PAR_MIN 2048 /* below this many items loops run on one thread */

struct orc_sys {
    int64_t n;
    double box[2];
    double e_c, n_c;
    /* particle arrays, current (cell-sorted) order */
    double *x, *y, *vx, *vy, *fx, *fy, *r, *m, *pe, *ke;
    double *tx, *ty, *tvx, *tvy, *tfx, *tfy, *tr, *tm; /* reorder targets */
    double *lnx, *lny, *lcx, *lcy, *nd2, *cd2;
    int64_t *cell_index, *pidx, *sidx, *cell_start;
    int64_t *key_tmp, *pidx_tmp, *sidx_tmp;
    int64_t *nlist, *ncount, cap;
    /* neighbour configuration (src/particles/base/particle.cu:1223-1272) */
    int method;
    double cutoff, nthr2;
    int64_t ncd, ncells;
    double cs, cthr2;
    int64_t n_rebuilds, n_cell_rebuilds;
    /* Adam moments and their swap twins (src/particles/base/particle.cu:319-322) */
    double *m1x, *m1y, *m2x, *m2y, *m1x_t, *m1y_t, *m2x_t, *m2y_t;
    int adam_ready;
    /* FIRE state (include/integrator/fire.h:15-35) */
    double f_alpha, f_alpha0, f_dt, f_dtmax, f_dtmin;
    int64_t f_ngood, f_nbad;
    int f_stopped;
    /* last state (src/particles/base/particle.cu:956-991) */
    double *sx, *sy, *svx, *svy, *sfx, *sfy, *sr, *sm;
    int64_t *spidx, *ssidx;
    double sbox[2];
    int saved;
};

/* --------------------------------------------------------------------- */
static double *dalloc(int64_t n) { return (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double)); }
static int64_t *lalloc(int64_t n) { return (int64_t *)calloc((size_t)(n > 0 ? n : 1), sizeof(int64_t)); }
static void lfill(int64_t *a, int64_t n, int64_t v) { for (int64_t i = 0; i < n; i++) a[i] = v; }
static void swapp(double **a, double **b) { double *t = *a; *a = *b; *b = t; }

void orc_set_threads(int nthreads) {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
}

/* mod with non-negative result: include/particles/base/kernels.cuh:53-55 */
static inline int64_t pmod(int64_t a, int64_t b) { return (a % b + b) % b; }

/* minimum image: include/particles/base/kernels.cuh:65-72 */
static inline double pbc(double x1, double x2, double size) {
    double d = x1 - x2;
    return d - size * round(d / size);
}

/* harmonic (power-law) contact, include/particles/base/kernels.cuh:154-183.
 * For n_c == 2 the reference's pow(overlap, 1.0) is exactly overlap. */
static inline double pair_interaction(const orc_sys *s, double xi, double yi, double ri, double xj,
                                      double yj, double rj, double *fx, double *fy) {
    double dx = pbc(xi, xj, s->box[0]);
    double dy = pbc(yi, yj, s->box[1]);
    double rs = ri + rj;
    double d2 = dx * dx + dy * dy;
    if (d2 >= rs * rs) { *fx = 0.0; *fy = 0.0; return 0.0; }
    double d = sqrt(d2);
    double ov = 1.0 - (d / rs);
    double ovp = (s->n_c == 2.0) ? ov : pow(ov, s->n_c - 1);
    double energy = s->e_c * ov * ovp / (2.0 * s->n_c);
    double fm = s->e_c * ovp / (rs * d);
    *fx = fm * dx;
    *fy = fm * dy;
    return energy;
}

/* cell coordinate, include/particles/base/kernels.cuh:285-301 */
static inline int64_t cell_coord(double p, double cs, int64_t ncd) {
    int64_t idx = (int64_t)floor(p / cs);
    return idx >= 0 ? idx % ncd : (idx % ncd + ncd) % ncd;
}

/* --------------------------------------------------------------------- */
orc_sys *orc_create(int64_t n, double box_x, double box_y, double e_c, double n_c) {
    orc_sys *s = (orc_sys *)calloc(1, sizeof(orc_sys));
    s->n = n; s->box[0] = box_x; s->box[1] = box_y; s->e_c = e_c; s->n_c = n_c;
    s->x = dalloc(n); s->y = dalloc(n); s->vx = dalloc(n); s->vy = dalloc(n);
    s->fx = dalloc(n); s->fy = dalloc(n); s->r = dalloc(n); s->m = dalloc(n);
    s->pe = dalloc(n); s->ke = dalloc(n);
    s->tx = dalloc(n); s->ty = dalloc(n); s->tvx = dalloc(n); s->tvy = dalloc(n);
    s->tfx = dalloc(n); s->tfy = dalloc(n); s->tr = dalloc(n); s->tm = dalloc(n);
    s->lnx = dalloc(n); s->lny = dalloc(n); s->lcx = dalloc(n); s->lcy = dalloc(n);
    s->nd2 = dalloc(n); s->cd2 = dalloc(n);
    s->cell_index = lalloc(n); s->pidx = lalloc(n); s->sidx = lalloc(n);
    s->key_tmp = lalloc(n); s->pidx_tmp = lalloc(n); s->sidx_tmp = lalloc(n);
    s->ncount = lalloc(n);
    for (int64_t i = 0; i < n; i++) { s->pidx[i] = i; s->sidx[i] = i; }
    s->cap = 4;
    s->nlist = lalloc(n * s->cap);
    lfill(s->nlist, n * s->cap, -1);
    s->cell_start = lalloc(1);
    s->method = -1;
    /* the reference's member defaults (include/particles/base/particle.h:173-187) */
    s->cutoff = -1; s->nthr2 = -1; s->cs = -1; s->cthr2 = -1; s->ncd = -1; s->ncells = -1;
    return s;
}

#define FREE(p) do { free(p); (p) = NULL; } while (0)
void orc_destroy(orc_sys *s) {
    if (!s) return;
    FREE(s->x); FREE(s->y); FREE(s->vx); FREE(s->vy); FREE(s->fx); FREE(s->fy);
    FREE(s->r); FREE(s->m); FREE(s->pe); FREE(s->ke);
    FREE(s->tx); FREE(s->ty); FREE(s->tvx); FREE(s->tvy); FREE(s->tfx); FREE(s->tfy);
    FREE(s->tr); FREE(s->tm); FREE(s->lnx); FREE(s->lny); FREE(s->lcx); FREE(s->lcy);
    FREE(s->nd2); FREE(s->cd2); FREE(s->cell_index); FREE(s->pidx); FREE(s->sidx);
    FREE(s->key_tmp); FREE(s->pidx_tmp); FREE(s->sidx_tmp); FREE(s->ncount);
    FREE(s->nlist); FREE(s->cell_start);
    FREE(s->m1x); FREE(s->m1y); FREE(s->m2x); FREE(s->m2y);
    FREE(s->m1x_t); FREE(s->m1y_t); FREE(s->m2x_t); FREE(s->m2y_t);
    FREE(s->sx); FREE(s->sy); FREE(s->svx); FREE(s->svy); FREE(s->sfx); FREE(s->sfy);
    FREE(s->sr); FREE(s->sm); FREE(s->spidx); FREE(s->ssidx);
    free(s);
}

/* Input arrays are given in static order; the slot of static particle k is
 * found through sidx (identity until the first cell sort). */
void orc_set_arrays(orc_sys *s, const double *x, const double *y, const double *vx,
                    const double *vy, const double *r, const double *m) {
    for (int64_t i = 0; i < s->n; i++) {
        int64_t k = s->sidx[i];
        if (x) s->x[i] = x[k];
        if (y) s->y[i] = y[k];
        if (vx) s->vx[i] = vx[k];
        if (vy) s->vy[i] = vy[k];
        if (r) s->r[i] = r[k];
        if (m) s->m[i] = m[k];
    }
}

void orc_set_forces(orc_sys *s, const double *fx, const double *fy) {
    for (int64_t i = 0; i < s->n; i++) {
        int64_t k = s->sidx[i];
        if (fx) s->fx[i] = fx[k];
        if (fy) s->fy[i] = fy[k];
    }
}

void orc_get_arrays(const orc_sys *s, double *x, double *y, double *vx, double *vy, double *fx,
                    double *fy, double *pe, double *r, double *m) {
    for (int64_t i = 0; i < s->n; i++) {
        int64_t k = s->sidx[i];
        if (x) x[k] = s->x[i];
        if (y) y[k] = s->y[i];
        if (vx) vx[k] = s->vx[i];
        if (vy) vy[k] = s->vy[i];
        if (fx) fx[k] = s->fx[i];
        if (fy) fy[k] = s->fy[i];
        if (pe) pe[k] = s->pe[i];
        if (r) r[k] = s->r[i];
        if (m) m[k] = s->m[i];
    }
}

void orc_get_current(const orc_sys *s, double *x, double *y, double *vx, double *vy, double *fx,
                     double *fy, double *pe, int64_t *static_index) {
    size_t b = (size_t)s->n * sizeof(double);
    if (x) memcpy(x, s->x, b);
    if (y) memcpy(y, s->y, b);
    if (vx) memcpy(vx, s->vx, b);
    if (vy) memcpy(vy, s->vy, b);
    if (fx) memcpy(fx, s->fx, b);
    if (fy) memcpy(fy, s->fy, b);
    if (pe) memcpy(pe, s->pe, b);
    if (static_index) memcpy(static_index, s->sidx, (size_t)s->n * sizeof(int64_t));
}

void orc_set_box(orc_sys *s, double bx, double by) { s->box[0] = bx; s->box[1] = by; }
void orc_get_box(const orc_sys *s, double *bx, double *by) { *bx = s->box[0]; *by = s->box[1]; }

static double max_diameter(const orc_sys *s) {
    double mx = -INFINITY;
    for (int64_t i = 0; i < s->n; i++) if (s->r[i] > mx) mx = s->r[i];
    return 2.0 * mx;
}

/* getParticleArea for disks: src/particles/disk/disk.cu:205-207 */
double orc_particle_area(const orc_sys *s) {
    double a = 0.0;
    for (int64_t i = 0; i < s->n; i++) a += s->r[i] * s->r[i];
    return a * 3.141592653589793238462643383279502884197;
}

static double box_area(const orc_sys *s) { return 1.0 * s->box[0] * s->box[1]; }

double orc_packing_fraction(const orc_sys *s) { return orc_particle_area(s) / box_area(s); }

/* ======================================================================
 *  Neighbour lists
 * ====================================================================== */

static void resize_list(orc_sys *s, int64_t cap) {
    free(s->nlist);
    s->cap = cap;
    s->nlist = lalloc(s->n * cap);
}

/* setNeighborSize: src/particles/base/particle.cu:1223-1234 */
static int set_neighbor_size(orc_sys *s, double cutoff_mult, double disp_mult) {
    s->cap = 4;
    s->cutoff = cutoff_mult * max_diameter(s);
    s->nthr2 = pow(disp_mult * s->cutoff, 2);
    double diag = sqrt(s->box[0] * s->box[0] + s->box[1] * s->box[1]);
    return s->cutoff < diag;
}

/* setCellSize: src/particles/base/particle.cu:1242-1272 */
static int set_cell_size(orc_sys *s, double ppc, double cdm) {
    const int64_t min_dim = 4;
    double density = (double)s->n / box_area(s);
    double trial = sqrt(ppc / density);
    double min_cs = 2.0 * max_diameter(s);
    s->ncd = (int64_t)floor(s->box[0] / trial);
    s->ncells = s->ncd * s->ncd;
    if (s->ncd < min_dim) { s->ncd = min_dim; s->ncells = s->ncd * s->ncd; }
    s->cs = s->box[0] / s->ncd;
    if (s->cs < min_cs) {
        s->cs = min_cs;
        s->ncd = (int64_t)floor(s->box[0] / s->cs);
        s->ncells = s->ncd * s->ncd;
        if (s->ncd < min_dim) return 0;
    }
    s->cthr2 = pow(cdm * s->cs, 2);
    return 1;
}

/* setNeighborMethod ("all" branch), src/particles/base/particle.cu:252-261 */
static void set_method(orc_sys *s, int method) {
    s->method = method;
    for (int64_t i = 0; i < s->n; i++) { s->pidx[i] = i; s->sidx[i] = i; }
    if (method == ORC_NEIGH_ALL) {
        double diag = sqrt(s->box[0] * s->box[0] + s->box[1] * s->box[1]);
        set_neighbor_size(s, 2.0 * diag / max_diameter(s), 0.0);
    }
}

/* kernelUpdateNeighborList (O(N^2)): src/particles/base/kernels.cu:256-293 */
static void build_all_pairs(orc_sys *s) {
    const int64_t n = s->n, cap = s->cap;
    const double c2 = s->cutoff * s->cutoff;
#pragma omp parallel for schedule(static) if (n >= PAR_MIN)
    for (int64_t i = 0; i < n; i++) {
        int64_t cnt = 0;
        double xi = s->x[i], yi = s->y[i];
        for (int64_t j = 0; j < n; j++) {
            if (j == i) continue;
            double dx = pbc(xi, s->x[j], s->box[0]);
            double dy = pbc(yi, s->y[j], s->box[1]);
            if (dx * dx + dy * dy < c2) {
                if (cnt < cap) s->nlist[i * cap + cnt] = j;
                cnt++;
            }
        }
        s->lnx[i] = xi; s->lny[i] = yi; s->nd2[i] = 0.0;
        s->ncount[i] = cnt;
    }
}

/* kernelUpdateCellNeighborList: src/particles/base/kernels.cu:440-505.
 * 3x3 cells, dy outer / dx inner, ascending slot inside a cell; an empty
 * cell's end is found by walking forward to the next non-empty start. */
static void build_from_cells(orc_sys *s) {
    const int64_t n = s->n, cap = s->cap, ncd = s->ncd;
    const double c2 = s->cutoff * s->cutoff;
#pragma omp parallel for schedule(static) if (n >= PAR_MIN)
    for (int64_t i = 0; i < n; i++) {
        int64_t cnt = 0;
        double xi = s->x[i], yi = s->y[i];
        int64_t cid = s->cell_index[i];
        int64_t cx = cid % ncd, cy = cid / ncd;
        for (int64_t oy = -1; oy <= 1; oy++) {
            int64_t yy = pmod(cy + oy, ncd);
            for (int64_t ox = -1; ox <= 1; ox++) {
                int64_t xx = pmod(cx + ox, ncd);
                int64_t nc = xx + yy * ncd;
                int64_t start = s->cell_start[nc];
                if (start == -1) continue;
                int64_t end = s->cell_start[nc + 1];
                while (end == -1) { nc++; end = s->cell_start[nc + 1]; }
                for (int64_t j = start; j < end; j++) {
                    if (j == i) continue;
                    double dx = pbc(xi, s->x[j], s->box[0]);
                    double dy = pbc(yi, s->y[j], s->box[1]);
                    if (dx * dx + dy * dy < c2) {
                        if (cnt < cap) s->nlist[i * cap + cnt] = j;
                        cnt++;
                    }
                }
            }
        }
        s->ncount[i] = cnt;
        s->nd2[i] = 0.0;
        s->lnx[i] = xi; s->lny[i] = yi;
    }
}

static int64_t max_count(const orc_sys *s) {
    int64_t mx = -1;
    for (int64_t i = 0; i < s->n; i++) if (s->ncount[i] > mx) mx = s->ncount[i];
    return mx;
}

/* power-of-two growth, src/particles/base/particle.cu:1124,1325 */
static int64_t grow_cap(int64_t max_neighbors) {
    return (int64_t)pow(2, ceil(log2((double)max_neighbors)));
}

/* updateVerletList: src/particles/base/particle.cu:1119-1131 */
static void update_verlet_list(orc_sys *s) {
    lfill(s->nlist, s->n * s->cap, -1);
    build_all_pairs(s);
    int64_t mx = max_count(s);
    if (mx > s->cap) {
        resize_list(s, grow_cap(mx));
        lfill(s->nlist, s->n * s->cap, -1);
        build_all_pairs(s);
    }
    s->n_rebuilds++;
}

/* updateCellNeighborList: src/particles/base/particle.cu:1320-1331 */
static void update_cell_neighbor_list(orc_sys *s) {
    lfill(s->nlist, s->n * s->cap, -1);
    build_from_cells(s);
    int64_t mx = max_count(s);
    if (mx > s->cap) {
        resize_list(s, grow_cap(mx));
        lfill(s->nlist, s->n * s->cap, -1);
        build_from_cells(s);
    }
    s->n_rebuilds++;
}

/* updateCellList + reorderParticleData + kernelGetFirstParticleIndexForCell:
 * src/particles/base/particle.cu:1292-1317, src/particles/base/kernels.cu:309-438,508-543.
 * The reference stable-sorts (particle_index, static_particle_index) by
 * cell_index; a stable counting sort gives the same permutation.  Empty cells
 * get cell_start = -1 and cell_start[n_cells] = N. */
static void update_cell_list(orc_sys *s) {
    const int64_t n = s->n, ncd = s->ncd, nc = s->ncells;
    s->cell_start[nc] = n;
#pragma omp parallel for schedule(static) if (n >= PAR_MIN)
    for (int64_t i = 0; i < n; i++) {
        int64_t xi = cell_coord(s->x[i], s->cs, ncd);
        int64_t yi = cell_coord(s->y[i], s->cs, ncd);
        s->cell_index[i] = xi + yi * ncd;
        s->pidx[i] = i;
    }
    /* stable counting sort by cell */
    int64_t *cnt = lalloc(nc + 1);
    for (int64_t i = 0; i < n; i++) cnt[s->cell_index[i] + 1]++;
    for (int64_t c = 0; c < nc; c++) cnt[c + 1] += cnt[c];
    for (int64_t c = 0; c < nc; c++) s->cell_start[c] = (cnt[c + 1] > cnt[c]) ? cnt[c] : -1;
    int64_t *cur = lalloc(nc);
    memcpy(cur, cnt, (size_t)nc * sizeof(int64_t));
    for (int64_t i = 0; i < n; i++) {
        int64_t c = s->cell_index[i];
        int64_t slot = cur[c]++;
        s->key_tmp[slot] = c;
        s->pidx_tmp[slot] = s->pidx[i];
        s->sidx_tmp[slot] = s->sidx[i];
    }
    free(cnt); free(cur);
    memcpy(s->cell_index, s->key_tmp, (size_t)n * sizeof(int64_t));
    memcpy(s->pidx, s->pidx_tmp, (size_t)n * sizeof(int64_t));
    memcpy(s->sidx, s->sidx_tmp, (size_t)n * sizeof(int64_t));
    /* gather (kernelReorderParticleData) */
#pragma omp parallel for schedule(static) if (n >= PAR_MIN)
    for (int64_t i = 0; i < n; i++) {
        int64_t o = s->pidx[i];
        s->tx[i] = s->x[o]; s->ty[i] = s->y[o];
        s->tfx[i] = s->fx[o]; s->tfy[i] = s->fy[o];
        s->tvx[i] = s->vx[o]; s->tvy[i] = s->vy[o];
        s->tm[i] = s->m[o]; s->tr[i] = s->r[o];
        s->lcx[i] = s->x[o]; s->lcy[i] = s->y[o];
        s->cd2[i] = 0.0;
    }
    swapp(&s->x, &s->tx); swapp(&s->y, &s->ty);
    swapp(&s->fx, &s->tfx); swapp(&s->fy, &s->tfy);
    swapp(&s->vx, &s->tvx); swapp(&s->vy, &s->tvy);
    swapp(&s->m, &s->tm); swapp(&s->r, &s->tr);
    /* The reference swaps the Adam moments with their (un-gathered) twins
     * (src/particles/base/particle.cu:1302-1303); restated as is. */
    if (s->adam_ready) {
        swapp(&s->m1x, &s->m1x_t); swapp(&s->m1y, &s->m1y_t);
        swapp(&s->m2x, &s->m2x_t); swapp(&s->m2y, &s->m2y_t);
    }
    s->n_cell_rebuilds++;
}

/* initVerletListVariables: src/particles/base/particle.cu:1171-1178 */
static void init_verlet_vars(orc_sys *s) {
    resize_list(s, s->cap);
    lfill(s->nlist, s->n * s->cap, -1);
    for (int64_t i = 0; i < s->n; i++) {
        s->ncount[i] = 0; s->lnx[i] = 0; s->lny[i] = 0; s->nd2[i] = 0;
        s->lcx[i] = 0; s->lcy[i] = 0; s->cd2[i] = 0;
    }
}

static void init_neighbor_list(orc_sys *s) {
    if (s->method == ORC_NEIGH_CELL) {
        /* initCellList: src/particles/base/particle.cu:1209-1221 */
        init_verlet_vars(s);
        for (int64_t i = 0; i < s->n; i++) s->cell_index[i] = -1;
        free(s->cell_start);
        s->cell_start = lalloc(s->ncells + 1);
        for (int64_t i = 0; i < s->n; i++) { s->pidx[i] = i; s->sidx[i] = i; }
        update_cell_list(s);
        update_cell_neighbor_list(s);
    } else if (s->method == ORC_NEIGH_VERLET) {
        /* initVerletList: src/particles/base/particle.cu:1180-1184 */
        init_verlet_vars(s);
        update_verlet_list(s);
    } else {
        /* initAllToAllList: src/particles/base/particle.cu:1186-1200 */
        s->cap = s->n - 1;
        init_verlet_vars(s);
        s->cutoff = 10.0 * sqrt(s->box[0] * s->box[0] + s->box[1] * s->box[1]);
        s->nthr2 = s->cutoff * s->cutoff;
        update_verlet_list(s);
    }
}

/* setupNeighbors: src/particles/base/particle.cu:71-100 (including the
 * calculateForces at the end, which accumulates onto the existing F, PE). */
int orc_setup_neighbors(orc_sys *s, int method, double cutoff_mult, double disp_mult,
                        double ppc, double cdm) {
    set_method(s, method);
    set_neighbor_size(s, cutoff_mult, disp_mult);
    if (s->method == ORC_NEIGH_CELL) {
        if (!set_cell_size(s, ppc, cdm)) set_method(s, ORC_NEIGH_VERLET);
        if (!set_neighbor_size(s, cutoff_mult, disp_mult)) set_method(s, ORC_NEIGH_ALL);
    }
    if (s->method == ORC_NEIGH_VERLET) {
        if (!set_neighbor_size(s, cutoff_mult, disp_mult)) set_method(s, ORC_NEIGH_ALL);
    }
    init_neighbor_list(s);
    orc_calculate_forces(s);
    return s->method;
}

/* updateNeighborList through the method pointer */
void orc_update_neighbor_list(orc_sys *s) {
    if (s->method == ORC_NEIGH_CELL) update_cell_neighbor_list(s);
    else update_verlet_list(s);
}

static double max_of(const double *a, int64_t n) {
    double mx = 0.0; /* thrust::reduce(..., 0.0, maximum) */
    for (int64_t i = 0; i < n; i++) if (a[i] > mx) mx = a[i];
    return mx;
}

/* checkForCellListUpdate / checkForVerletListUpdate / checkForAllToAllUpdate:
 * src/particles/base/particle.cu:1133-1161 (tolerance 3) */
int orc_check_for_neighbor_update(orc_sys *s) {
    const double tol = 3.0;
    if (s->method == ORC_NEIGH_ALL) return 0;
    if (s->method == ORC_NEIGH_VERLET) {
        if (tol * max_of(s->nd2, s->n) > s->nthr2) { update_verlet_list(s); return 1; }
        return 0;
    }
    if (tol * max_of(s->cd2, s->n) > s->cthr2) {
        update_cell_list(s);
        update_cell_neighbor_list(s);
        return 2;
    }
    if (tol * max_of(s->nd2, s->n) > s->nthr2) { update_cell_neighbor_list(s); return 1; }
    return 0;
}

void orc_neighbor_info(const orc_sys *s, int *method, double *cutoff, double *thr2,
                       int64_t *ncd, double *cs, double *cthr2, int64_t *cap) {
    if (method) *method = s->method;
    if (cutoff) *cutoff = s->cutoff;
    if (thr2) *thr2 = s->nthr2;
    if (ncd) *ncd = s->ncd;
    if (cs) *cs = s->cs;
    if (cthr2) *cthr2 = s->cthr2;
    if (cap) *cap = s->cap;
}

void orc_get_neighbors(const orc_sys *s, int64_t *list, int64_t *counts) {
    if (list) memcpy(list, s->nlist, (size_t)(s->n * s->cap) * sizeof(int64_t));
    if (counts) memcpy(counts, s->ncount, (size_t)s->n * sizeof(int64_t));
}

void orc_get_cells(const orc_sys *s, int64_t *cell_index, int64_t *cell_start) {
    if (cell_index) memcpy(cell_index, s->cell_index, (size_t)s->n * sizeof(int64_t));
    if (cell_start && s->method == ORC_NEIGH_CELL)
        memcpy(cell_start, s->cell_start, (size_t)(s->ncells + 1) * sizeof(int64_t));
}

int64_t orc_num_rebuilds(const orc_sys *s, int64_t *n_cell) {
    if (n_cell) *n_cell = s->n_cell_rebuilds;
    return s->n_rebuilds;
}

/* ======================================================================
 *  Forces and dynamics
 * ====================================================================== */

/* kernelZeroForceAndPotentialEnergy: src/particles/base/kernels.cu:150-161 */
void orc_zero_force_and_pe(orc_sys *s) {
    for (int64_t i = 0; i < s->n; i++) { s->fx[i] = 0.0; s->fy[i] = 0.0; s->pe[i] = 0.0; }
}

/* kernelCalcDiskForces: src/particles/disk/kernels.cu:11-57 */
void orc_calculate_forces(orc_sys *s) {
    const int64_t n = s->n, cap = s->cap;
#pragma omp parallel for schedule(static) if (n >= PAR_MIN)
    for (int64_t i = 0; i < n; i++) {
        int64_t nn = s->ncount[i];
        if (nn == 0) continue;
        double xi = s->x[i], yi = s->y[i], ri = s->r[i];
        double ax = 0.0, ay = 0.0, en = 0.0;
        for (int64_t k = 0; k < nn; k++) {
            int64_t j = s->nlist[i * cap + k];
            if (j == -1 || j == i) continue;
            double fx, fy;
            double e = pair_interaction(s, xi, yi, ri, s->x[j], s->y[j], s->r[j], &fx, &fy);
            ax += fx; ay += fy; en += e;
        }
        s->fx[i] += ax; s->fy[i] += ay; s->pe[i] += en;
    }
}

/* kernelUpdateVelocities: src/particles/base/kernels.cu:117-139 */
void orc_update_velocities(orc_sys *s, double dt) {
    const int64_t n = s->n;
#pragma omp parallel for schedule(static) if (n >= PAR_MIN)
    for (int64_t i = 0; i < n; i++) {
        double dtm = dt / s->m[i];
        s->vx[i] = s->vx[i] + s->fx[i] * dtm;
        s->vy[i] = s->vy[i] + s->fy[i] * dtm;
    }
}

/* kernelUpdatePositions: src/particles/base/kernels.cu:48-81 */
void orc_update_positions(orc_sys *s, double dt) {
    const int64_t n = s->n;
#pragma omp parallel for schedule(static) if (n >= PAR_MIN)
    for (int64_t i = 0; i < n; i++) {
        double px = s->x[i] + s->vx[i] * dt;
        double py = s->y[i] + s->vy[i] * dt;
        s->x[i] = px; s->y[i] = py;
        double dxn = px - s->lnx[i], dyn = py - s->lny[i];
        s->nd2[i] = dxn * dxn + dyn * dyn;
        double dxc = px - s->lcx[i], dyc = py - s->lcy[i];
        s->cd2[i] = dxc * dxc + dyc * dyc;
    }
}

/* kernelMixVelocitiesAndForces (per-particle FIRE mix):
 * src/particles/base/kernels.cu:91-112 */
void orc_mix_velocities_and_forces(orc_sys *s, double alpha) {
    const int64_t n = s->n;
#pragma omp parallel for schedule(static) if (n >= PAR_MIN)
    for (int64_t i = 0; i < n; i++) {
        double fx = s->fx[i], fy = s->fy[i], vx = s->vx[i], vy = s->vy[i];
        double fn = sqrt(fx * fx + fy * fy);
        double vn = sqrt(vx * vx + vy * vy);
        double mix = 0.0;
        if (fn > 1e-16) mix = vn / fn * alpha;
        else { vx = 0.0; vy = 0.0; mix = 0.0; }
        s->vx[i] = vx * (1 - alpha) + fx * mix;
        s->vy[i] = vy * (1 - alpha) + fy * mix;
    }
}

void orc_set_velocities_zero(orc_sys *s) {
    memset(s->vx, 0, (size_t)s->n * sizeof(double));
    memset(s->vy, 0, (size_t)s->n * sizeof(double));
}

/* getPowerFire: src/particles/base/particle.cu:993-1009 (x sum + y sum) */
double orc_power_fire(orc_sys *s) {
    double px = 0.0, py = 0.0;
    for (int64_t i = 0; i < s->n; i++) px += s->fx[i] * s->vx[i];
    for (int64_t i = 0; i < s->n; i++) py += s->fy[i] * s->vy[i];
    return px + py;
}

/* totalPotentialEnergy: src/particles/base/particle.cu:1078-1080 */
double orc_total_pe(orc_sys *s) {
    double e = 0.0;
    for (int64_t i = 0; i < s->n; i++) e += s->pe[i];
    return e;
}

/* kernelCalculateTranslationalKineticEnergy + totalKineticEnergy:
 * src/particles/base/kernels.cu:163-180, src/particles/base/particle.cu:1074-1076 */
double orc_total_ke(orc_sys *s) {
    double e = 0.0;
    for (int64_t i = 0; i < s->n; i++) {
        double v2 = s->vx[i] * s->vx[i] + s->vy[i] * s->vy[i];
        s->ke[i] = 0.5 * s->m[i] * v2;
        e += s->ke[i];
    }
    return e;
}

double orc_max_force(orc_sys *s) {
    double mx = 0.0;
    for (int64_t i = 0; i < s->n; i++) {
        double f = sqrt(s->fx[i] * s->fx[i] + s->fy[i] * s->fy[i]);
        if (f > mx) mx = f;
    }
    return mx;
}

/* getForceBalance: src/particles/base/particle.cu:231-235 */
double orc_force_balance(orc_sys *s) {
    double fx = 0.0, fy = 0.0;
    for (int64_t i = 0; i < s->n; i++) { fx += s->fx[i]; fy += s->fy[i]; }
    return sqrt(fx * fx + fy * fy);
}

/* NVE::step: src/integrator/nve.cu:15-25 */
void orc_nve_steps(orc_sys *s, double dt, int64_t n_steps) {
    for (int64_t t = 0; t < n_steps; t++) {
        orc_update_velocities(s, 0.5 * dt);
        orc_update_positions(s, dt);
        orc_check_for_neighbor_update(s);
        orc_zero_force_and_pe(s);
        orc_calculate_forces(s);
        orc_update_velocities(s, 0.5 * dt);
    }
}

/* kernelCalculateDampedForces: src/particles/base/kernels.cu:83-89 */
void orc_damped_forces(orc_sys *s, double gamma) {
    const int64_t n = s->n;
#pragma omp parallel for schedule(static) if (n >= PAR_MIN)
    for (int64_t i = 0; i < n; i++) {
        s->fx[i] -= gamma * s->vx[i];
        s->fy[i] -= gamma * s->vy[i];
    }
}

/* DampedNVE::step: src/integrator/damped_nve.cu:15-27 */
void orc_damped_nve_steps(orc_sys *s, double dt, double gamma, int64_t n_steps) {
    for (int64_t t = 0; t < n_steps; t++) {
        orc_update_velocities(s, 0.5 * dt);
        orc_update_positions(s, dt);
        orc_check_for_neighbor_update(s);
        orc_zero_force_and_pe(s);
        orc_damped_forces(s, gamma);
        orc_calculate_forces(s);
        orc_update_velocities(s, 0.5 * dt);
    }
}

/* kernelCalcDiskForceDistancePairs (src/particles/disk/kernels.cu:73-175) after
 * the fills of Disk::calculateForceDistancePairs (src/particles/disk/disk.cu:228-255).
 * d[16]: potential, force x/y, distance x/y, overlap, radius sum, separation angle,
 * pair Hessian xx/xy/yx/yy, self Hessian xx/xy/yx/yy; n * cap each, row-major
 * [slot * cap + k] in the current order; ids are static indices. */
void orc_pair_dump(orc_sys *s, double *const *d, int64_t *this_id, int64_t *other_id) {
    const int64_t n = s->n, cap = s->cap, m = n * cap;
    const double fill[16] = {-1, 0, 0, -1, -1, -1, -1, -1, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 16; k++)
        if (d[k]) for (int64_t q = 0; q < m; q++) d[k][q] = fill[k];
    for (int64_t q = 0; q < m; q++) { this_id[q] = -1; other_id[q] = -1; }
    for (int64_t i = 0; i < n; i++) {
        if (s->ncount[i] == 0) continue;
        const double xi = s->x[i], yi = s->y[i], ri = s->r[i];
        for (int64_t k = 0; k < cap; k++) {
            const int64_t j = s->nlist[i * cap + k];
            if (j == -1 || j == i) continue;
            double fx, fy;
            const double e = pair_interaction(s, xi, yi, ri, s->x[j], s->y[j], s->r[j], &fx, &fy);
            const int64_t q = i * cap + k;
            const double dx = pbc(xi, s->x[j], s->box[0]), dy = pbc(yi, s->y[j], s->box[1]);
            const double rj = s->r[j];
            if (d[0]) d[0][q] = e;
            if (d[1]) d[1][q] = fx;
            if (d[2]) d[2][q] = fy;
            if (d[3]) d[3][q] = dx;
            if (d[4]) d[4][q] = dy;
            this_id[q] = s->sidx[i];
            other_id[q] = s->sidx[j];
            const double dist = sqrt(dx * dx + dy * dy);
            if (d[5]) d[5][q] = dist - (ri + rj);
            if (d[6]) d[6][q] = ri + rj;
            if (d[7]) d[7][q] = atan2(dy, dx);
            if (dist < ri + rj) {
                const double radsum = ri + rj;
                const double t_ij = -s->e_c / radsum * (1 - dist / radsum);
                const double c_ij = s->e_c / (radsum * radsum);
                double hij[4] = {0.0, 0.0, 0.0, 0.0}, hii[4] = {0.0, 0.0, 0.0, 0.0};
                for (int a = 0; a < 2; a++) {
                    for (int b = 0; b < 2; b++) {
                        const double dia_x = 1 * (a == 0), dia_y = 1 * (a == 1);
                        const double djb_x = -1 * (b == 0), djb_y = -1 * (b == 1);
                        const double q_ia = dx * dia_x + dy * dia_y;
                        const double q_jb = dx * djb_x + dy * djb_y;
                        const double dia_q_jb = dia_x * djb_x + dx * 0.0 + dia_y * djb_y + dy * 0.0;
                        hij[a * 2 + b] += c_ij * (q_ia * q_jb) / (dist * dist) +
                                          t_ij * (dia_q_jb / dist - (q_ia * q_jb) / (dist * dist * dist));
                        const double dib_x = 1 * (b == 0), dib_y = 1 * (b == 1);
                        const double q_ib = dx * dib_x + dy * dib_y;
                        const double dia_q_ib = dia_x * dib_x + dx * 0.0 + dia_y * dib_y + dy * 0.0;
                        hii[a * 2 + b] += c_ij * (q_ia * q_ib) / (dist * dist) +
                                          t_ij * (dia_q_ib / dist - (q_ia * q_ib) / (dist * dist * dist));
                    }
                }
                for (int c = 0; c < 4; c++) {
                    if (d[8 + c]) d[8 + c][q] += hij[c];
                    if (d[12 + c]) d[12 + c][q] += hii[c];
                }
            }
        }
    }
}

/* calcWallInteraction + kernelCalcDiskWallForces (+= into F, PE):
 * include/particles/base/kernels.cuh:185-235, src/particles/disk/kernels.cu:59-71 */
void orc_wall_forces(orc_sys *s) {
    const int64_t n = s->n;
    const double L0 = s->box[0], L1 = s->box[1], e_c = s->e_c, n_c = s->n_c;
#pragma omp parallel for schedule(static) if (n >= PAR_MIN)
    for (int64_t i = 0; i < n; i++) {
        const double px = s->x[i], py = s->y[i], rad = s->r[i];
        double fx = 0.0, fy = 0.0, en = 0.0;
        const double dist[4] = {px, L0 - px, py, L1 - py};
        const int near[4] = {px < rad, px > L0 - rad, py < rad, py > L1 - rad};
        for (int w = 0; w < 4; w++) {
            if (!near[w]) continue;
            double ov = rad - dist[w];
            if (!(ov > 0)) continue;
            double ovp = pow(ov / rad, n_c - 1);
            double f = e_c * ovp / rad;
            if (w == 0) fx += f;
            else if (w == 1) fx -= f;
            else if (w == 2) fy += f;
            else fy -= f;
            en += e_c * ov * ovp / (n_c * rad);
        }
        s->fx[i] += fx; s->fy[i] += fy; s->pe[i] += en;
    }
}

/* NVE::wall_step: src/integrator/nve.cu:27-38 */
void orc_nve_wall_steps(orc_sys *s, double dt, int64_t n_steps) {
    for (int64_t t = 0; t < n_steps; t++) {
        orc_update_velocities(s, 0.5 * dt);
        orc_update_positions(s, dt);
        orc_check_for_neighbor_update(s);
        orc_zero_force_and_pe(s);
        orc_wall_forces(s);
        orc_calculate_forces(s);
        orc_update_velocities(s, 0.5 * dt);
    }
}

/* kernelGradDescStep: src/particles/base/kernels.cu:613-637 */
void orc_update_positions_grad_desc(orc_sys *s, double alpha) {
    const int64_t n = s->n;
#pragma omp parallel for schedule(static) if (n >= PAR_MIN)
    for (int64_t i = 0; i < n; i++) {
        double px = s->x[i] + alpha * s->fx[i];
        double py = s->y[i] + alpha * s->fy[i];
        s->x[i] = px; s->y[i] = py;
        double dxn = px - s->lnx[i], dyn = py - s->lny[i];
        s->nd2[i] = dxn * dxn + dyn * dyn;
        double dxc = px - s->lcx[i], dyc = py - s->lcy[i];
        s->cd2[i] = dxc * dxc + dyc * dyc;
    }
}

/* GradDesc::step: src/integrator/grad_desc.cu:11-17 */
void orc_grad_desc_steps(orc_sys *s, double alpha, int64_t n_steps) {
    for (int64_t t = 0; t < n_steps; t++) {
        orc_zero_force_and_pe(s);
        orc_check_for_neighbor_update(s);
        orc_calculate_forces(s);
        orc_update_positions_grad_desc(s, alpha);
    }
}

/* ======================================================================
 *  FIRE: src/integrator/fire.cu:3-46, include/integrator/fire.h:15-35
 * ====================================================================== */
void orc_fire_init(orc_sys *s, double alpha_init, double dt) {
    s->f_alpha = alpha_init; s->f_alpha0 = alpha_init; s->f_dt = dt;
    s->f_dtmax = 10.0 * dt; s->f_dtmin = 0.001 * dt;
    s->f_ngood = 0; s->f_nbad = 0; s->f_stopped = 0;
}

int orc_fire_step(orc_sys *s) {
    const double f_inc = 1.1, f_dec = 0.5, f_a = 0.99;
    const int64_t n_min = 5, n_bad_max = 10;
    double power = orc_power_fire(s);
    if (power > 0) {
        s->f_ngood++;
        s->f_nbad = 0;
        if (s->f_ngood > n_min) {
            double d = s->f_dt * f_inc;
            s->f_dt = d < s->f_dtmax ? d : s->f_dtmax;
            s->f_alpha *= f_a;
        }
    } else {
        s->f_ngood = 0;
        s->f_nbad++;
        if (s->f_nbad > n_bad_max) { s->f_stopped = 1; return 1; }
        double d = s->f_dt * f_dec;
        s->f_dt = d > s->f_dtmin ? d : s->f_dtmin;
        s->f_alpha = s->f_alpha0;
        orc_update_positions(s, -s->f_dt / 2.0);
        orc_set_velocities_zero(s);
    }
    orc_update_velocities(s, s->f_dt / 2.0);
    orc_mix_velocities_and_forces(s, s->f_alpha);
    orc_update_positions(s, s->f_dt);
    orc_zero_force_and_pe(s);
    orc_check_for_neighbor_update(s);
    orc_calculate_forces(s);
    orc_update_velocities(s, s->f_dt / 2.0);
    return 0;
}

void orc_fire_state(const orc_sys *s, double *alpha, double *dt, int64_t *ng, int64_t *nb,
                    int *stopped) {
    if (alpha) *alpha = s->f_alpha;
    if (dt) *dt = s->f_dt;
    if (ng) *ng = s->f_ngood;
    if (nb) *nb = s->f_nbad;
    if (stopped) *stopped = s->f_stopped;
}

/* minimizeFire: src/routines/minimization.cu:75-112 (dof = N).
 * fmax_target > 0 adds a max|F_i| stop, checked after the PE tests. */
int64_t orc_minimize_fire(orc_sys *s, double alpha_init, double dt, double pe_target,
                          double pe_diff_target, int64_t num_steps, double fmax_target,
                          int *stopped_out) {
    orc_fire_init(s, alpha_init, dt);
    int64_t step = 0;
    double dof = (double)s->n;
    orc_set_velocities_zero(s);
    orc_zero_force_and_pe(s);
    orc_check_for_neighbor_update(s);
    orc_calculate_forces(s);
    double last = orc_total_pe(s) / dof;
    while (step < num_steps) {
        orc_fire_step(s);
        double avg = orc_total_pe(s) / dof;
        double diff = fabs(avg / last - 1);
        last = avg;
        if (diff < pe_diff_target || avg < pe_target || s->f_stopped) break;
        if (fmax_target > 0 && orc_max_force(s) <= fmax_target) break;
        step++;
    }
    orc_set_velocities_zero(s);
    if (stopped_out) *stopped_out = s->f_stopped;
    return step;
}

/* ======================================================================
 *  Adam: src/particles/base/kernels.cu:550-611, src/particles/base/particle.cu:319-333,
 *        src/integrator/adam.cu:11-17, src/routines/minimization.cu:3-33
 * ====================================================================== */
void orc_init_adam(orc_sys *s) {
    double **bufs[8] = {&s->m1x, &s->m1y, &s->m2x, &s->m2y, &s->m1x_t, &s->m1y_t, &s->m2x_t, &s->m2y_t};
    for (int k = 0; k < 8; k++) { free(*bufs[k]); *bufs[k] = dalloc(s->n); }
    s->adam_ready = 1;
}

void orc_adam_step(orc_sys *s, int64_t step, double alpha, double b1, double b2, double eps) {
    double c1 = 1 - pow(b1, step + 1);
    double c2 = 1 - pow(b2, step + 1);
    const int64_t n = s->n;
#pragma omp parallel for schedule(static) if (n >= PAR_MIN)
    for (int64_t i = 0; i < n; i++) {
        double fx = s->fx[i], fy = s->fy[i];
        double m1x = fma(b1, s->m1x[i], (b1 - 1) * fx);
        double m1y = fma(b1, s->m1y[i], (b1 - 1) * fy);
        double m2x = fma(b2, s->m2x[i], (1 - b2) * fx * fx);
        double m2y = fma(b2, s->m2y[i], (1 - b2) * fy * fy);
        double mhx = m1x / c1, mhy = m1y / c1;
        double vhx = m2x / c2, vhy = m2y / c2;
        double ux = -alpha * mhx / (sqrt(vhx) + eps);
        double uy = -alpha * mhy / (sqrt(vhy) + eps);
        double px = s->x[i] + ux, py = s->y[i] + uy;
        s->x[i] = px; s->y[i] = py;
        double dxn = px - s->lnx[i], dyn = py - s->lny[i];
        s->nd2[i] = dxn * dxn + dyn * dyn;
        double dxc = px - s->lcx[i], dyc = py - s->lcy[i];
        s->cd2[i] = dxc * dxc + dyc * dyc;
        s->m1x[i] = m1x; s->m1y[i] = m1y; s->m2x[i] = m2x; s->m2y[i] = m2y;
    }
}

int64_t orc_minimize_adam(orc_sys *s, double alpha, double b1, double b2, double eps,
                          double pe_target, double pe_diff_target, int64_t num_steps) {
    orc_init_adam(s);
    int64_t step = 0;
    double dof = (double)(s->n * 2);
    double last = 0.0;
    while (step < num_steps) {
        orc_zero_force_and_pe(s);
        orc_check_for_neighbor_update(s);
        orc_calculate_forces(s);
        orc_adam_step(s, step, alpha, b1, b2, eps);
        double avg = orc_total_pe(s) / dof;
        double diff = fabs(avg / last - 1);
        last = avg;
        if (diff < pe_diff_target || avg < pe_target) break;
        step++;
    }
    return step;
}

/* ======================================================================
 *  Stress, pressure, contacts, scaling, last state
 * ====================================================================== */

/* kernelCalcDiskStressTensor + getStressTensor: src/particles/disk/kernels.cu:203-252,
 * src/particles/base/particle.cu:1378-1384; components summed over particles */
void orc_stress_tensor(orc_sys *s, double out[4]) {
    const int64_t n = s->n, cap = s->cap;
    double area = s->box[0] * s->box[1];
    double *sxx = dalloc(n), *sxy = dalloc(n), *syx = dalloc(n), *syy = dalloc(n);
#pragma omp parallel for schedule(static) if (n >= PAR_MIN)
    for (int64_t i = 0; i < n; i++) {
        double xi = s->x[i], yi = s->y[i], mi = s->m[i], ri = s->r[i];
        double vx = s->vx[i], vy = s->vy[i];
        double axx = mi * vx * vx, axy = mi * vx * vy, ayx = axy, ayy = mi * vy * vy;
        for (int64_t k = 0; k < cap; k++) {
            int64_t j = s->nlist[i * cap + k];
            if (j == -1 || j == i) continue;
            double dx = pbc(xi, s->x[j], s->box[0]);
            double dy = pbc(yi, s->y[j], s->box[1]);
            double fx, fy;
            pair_interaction(s, xi, yi, ri, s->x[j], s->y[j], s->r[j], &fx, &fy);
            axx += dx * fx / 2; axy += dx * fy / 2;
            ayx += dy * fx / 2; ayy += dy * fy / 2;
        }
        sxx[i] = axx / area; sxy[i] = axy / area; syx[i] = ayx / area; syy[i] = ayy / area;
    }
    double a = 0, b = 0, c = 0, d = 0;
    for (int64_t i = 0; i < n; i++) { a += sxx[i]; b += sxy[i]; c += syx[i]; d += syy[i]; }
    out[0] = a; out[1] = b; out[2] = c; out[3] = d;
    free(sxx); free(sxy); free(syx); free(syy);
}

/* getPressure: src/particles/base/particle.cu:1371-1376 */
double orc_pressure(orc_sys *s) {
    double st[4];
    orc_stress_tensor(s, st);
    return (st[0] + st[3]) / 2;
}

/* kernelCountDiskContacts + getContactCount: src/particles/disk/kernels.cu:177-201,
 * src/particles/base/particle.cu:1367-1369 */
double orc_contact_count(orc_sys *s) {
    const int64_t cap = s->cap;
    int64_t total = 0;
    for (int64_t i = 0; i < s->n; i++) {
        int64_t nn = s->ncount[i], c = 0;
        for (int64_t k = 0; k < nn; k++) {
            int64_t j = s->nlist[i * cap + k];
            if (j == -1 || j == i) continue;
            double dx = pbc(s->x[i], s->x[j], s->box[0]);
            double dy = pbc(s->y[i], s->y[j], s->box[1]);
            if (sqrt(dx * dx + dy * dy) < s->r[i] + s->r[j]) c++;
        }
        total += c;
    }
    return (double)total;
}

/* updateCellSize: src/particles/base/particle.cu:1236-1240 (n_cells_dim frozen) */
static void update_cell_size(orc_sys *s) {
    if (s->ncd > 0) s->cs = s->box[0] / s->ncd;
}

/* scaleToPackingFractionFull: src/particles/base/particle.cu:1047-1055 */
void orc_scale_to_packing_fraction(orc_sys *s, double phi) {
    double new_l = pow(orc_particle_area(s) / phi, 1.0 / 2);
    double l = pow(box_area(s), 1.0 / 2);
    double f = new_l / l;
    for (int64_t i = 0; i < s->n; i++) { s->x[i] *= f; s->y[i] *= f; }
    s->box[0] = new_l; s->box[1] = new_l;
    update_cell_size(s);
}

/* scaleBox: src/particles/base/particle.cu:1057-1064 */
void orc_scale_box(orc_sys *s, double factor) {
    for (int64_t i = 0; i < s->n; i++) { s->x[i] *= factor; s->y[i] *= factor; }
    double l = pow(box_area(s), 1.0 / 2);
    double nl = l * factor;
    s->box[0] = nl; s->box[1] = nl;
    update_cell_size(s);
}

/* setLastState / revertToLastState: src/particles/base/particle.cu:956-991.
 * Revert restores the saved arrays and box and rebuilds only the neighbour
 * list (through updateNeighborList), leaving the cell arrays as they are. */
void orc_set_last_state(orc_sys *s) {
    int64_t n = s->n;
    if (!s->sx) {
        s->sx = dalloc(n); s->sy = dalloc(n); s->svx = dalloc(n); s->svy = dalloc(n);
        s->sfx = dalloc(n); s->sfy = dalloc(n); s->sr = dalloc(n); s->sm = dalloc(n);
        s->spidx = lalloc(n); s->ssidx = lalloc(n);
    }
    size_t b = (size_t)n * sizeof(double), bl = (size_t)n * sizeof(int64_t);
    memcpy(s->sx, s->x, b); memcpy(s->sy, s->y, b); memcpy(s->svx, s->vx, b);
    memcpy(s->svy, s->vy, b); memcpy(s->sfx, s->fx, b); memcpy(s->sfy, s->fy, b);
    memcpy(s->sr, s->r, b); memcpy(s->sm, s->m, b);
    memcpy(s->spidx, s->pidx, bl); memcpy(s->ssidx, s->sidx, bl);
    s->sbox[0] = s->box[0]; s->sbox[1] = s->box[1];
    s->saved = 1;
}

void orc_revert_to_last_state(orc_sys *s) {
    if (!s->saved) return;
    int64_t n = s->n;
    size_t b = (size_t)n * sizeof(double), bl = (size_t)n * sizeof(int64_t);
    memcpy(s->x, s->sx, b); memcpy(s->y, s->sy, b); memcpy(s->vx, s->svx, b);
    memcpy(s->vy, s->svy, b); memcpy(s->fx, s->sfx, b); memcpy(s->fy, s->sfy, b);
    memcpy(s->r, s->sr, b); memcpy(s->m, s->sm, b);
    memcpy(s->pidx, s->spidx, bl); memcpy(s->sidx, s->ssidx, bl);
    s->box[0] = s->sbox[0]; s->box[1] = s->sbox[1];
    orc_update_neighbor_list(s);
}

/* ======================================================================
 *  Seeded initialisation: include/functors.h:17-50, src/data/data_1d.cu:85-93.
 *  thrust::default_random_engine is minstd (a = 48271, m = 2^31 - 1);
 *  uniform_real maps (u - 1) / (m - 1) onto [lo, hi); the normal sampler the
 *  reference runs on the GPU is the inverse-erfc transform of one draw.
 * ====================================================================== */
static const uint64_t MINSTD_A = 48271u, MINSTD_M = 2147483647u;

static uint32_t minstd_seed(uint32_t s) {
    uint32_t x = (uint32_t)(s % MINSTD_M);
    return x == 0 ? 1u : x;
}

static uint32_t minstd_jump(uint32_t x, uint64_t z) {
    uint64_t mul = MINSTD_A, acc = 1;
    while (z) {
        if (z & 1) acc = (acc * mul) % MINSTD_M;
        mul = (mul * mul) % MINSTD_M;
        z >>= 1;
    }
    return (uint32_t)((acc * x) % MINSTD_M);
}

static uint32_t minstd_next(uint32_t x) { return (uint32_t)(((uint64_t)x * MINSTD_A) % MINSTD_M); }

void orc_fill_uniform(double *out, int64_t n, double lo, double hi, int64_t seed_offset,
                      int64_t seed) {
    uint32_t useed = (uint32_t)seed;
    for (int64_t i = 0; i < n; i++) {
        uint32_t k = (uint32_t)(seed + seed_offset + i);
        uint32_t st = minstd_jump(minstd_seed(useed + k), k);
        st = minstd_next(st);
        double u = (double)(st - 1u);
        u /= (1.0 + (double)(MINSTD_M - 2u));
        out[i] = u * (hi - lo) + lo;
    }
}

/* inverse complementary error function by Halley iteration on libm erfc,
 * started from Winitzki's closed-form erfinv estimate */
double orc_erfcinv(double z) {
    if (z <= 0.0) return INFINITY;
    if (z >= 2.0) return -INFINITY;
    if (z > 1.0) return -orc_erfcinv(2.0 - z);
    const double a = 0.147, pi = 3.141592653589793238462643383279502884197;
    double l = log(z * (2.0 - z));
    double t = 2.0 / (pi * a) + 0.5 * l;
    double y = sqrt(sqrt(t * t - l / a) - t);
    const double k = 1.1283791670955125738961589031215452; /* 2/sqrt(pi) */
    for (int it = 0; it < 50; it++) {
        double f = erfc(y) - z;
        double fp = -k * exp(-y * y);
        double rr = f / fp;
        double dy = rr / (1.0 + y * rr);
        y -= dy;
        if (fabs(dy) <= 1e-17 * fabs(y)) break;
    }
    return y;
}

void orc_fill_normal(double *out, int64_t n, double mean, double stddev, int64_t seed_offset,
                     int64_t seed) {
    const uint32_t range = (uint32_t)(MINSTD_M - 2u); /* max - min */
    const double s1 = 1. / (double)range, s2 = s1 / 2;
    for (int64_t i = 0; i < n; i++) {
        uint32_t k = (uint32_t)(seed + seed_offset + i);
        uint32_t st = minstd_jump(minstd_seed((uint32_t)seed), k);
        st = minstd_next(st);
        uint32_t u = st - 1u;
        double s3 = -1.4142135623730950488016887242097;
        if (u > range / 2) { u = range - u; s3 = -s3; }
        double p = fma((double)u, s1, s2);
        out[i] = fma(stddev * s3, orc_erfcinv(2 * p), mean);
    }
}

/* ======================================================================
 *  Jamming drivers: the run scripts' control flow restated
 * ====================================================================== */

/* Disk::load (src/particles/disk/disk.cu:35-96): arrays in static order, the
 * slot order becomes the static order, velocities / forces / PE zero. */
void orc_load_state(orc_sys *s, const double *x, const double *y, const double *r,
                    const double *m) {
    for (int64_t i = 0; i < s->n; i++) {
        s->pidx[i] = i; s->sidx[i] = i;
        s->x[i] = x[i]; s->y[i] = y[i]; s->r[i] = r[i]; s->m[i] = m[i];
        s->vx[i] = 0; s->vy[i] = 0; s->fx[i] = 0; s->fy[i] = 0; s->pe[i] = 0;
    }
}

static double jam_box_length(const orc_sys *s) { return pow(box_area(s), 1.0 / 2); }

/* scripts/runArthurJamWithFire.cpp:36-106 */
void orc_jam_pressure(orc_sys *s, double p_low, double p_high, double rate, double length_tol,
                      double decompress, int64_t max_steps, double fa, double fdt, double pet,
                      double pedt, int64_t fsteps, int method, double cm, double dm, double ppc,
                      double cdm, orc_jam_result *r) {
    int64_t total = 0, n = s->n;
    double P;
    for (int guard = 0; guard < 10000; guard++) {
        total += orc_minimize_fire(s, fa, fdt, 1e-16, 0.0, fsteps, 0.0, NULL) + 1;
        P = orc_pressure(s);
        if (P < p_low) break;
        orc_scale_box(s, decompress);
    }
    double *sx = dalloc(n), *sy = dalloc(n), *sr = dalloc(n), *sm = dalloc(n);
    double sbx = 0, sby = 0;
    double L_low = -1, L_high = -1, L_last = -1, contacts = 0;
    int64_t step = 0;
    int status = 2;
    while (step < max_steps) {
        total += orc_minimize_fire(s, fa, fdt, pet, pedt, fsteps, 0.0, NULL) + 1;
        P = orc_pressure(s);
        contacts = orc_contact_count(s);
        double L = jam_box_length(s), L_prior = L;
        if (P < p_low) {
            L_low = L;
            orc_get_arrays(s, sx, sy, NULL, NULL, NULL, NULL, NULL, sr, sm);
            sbx = s->box[0]; sby = s->box[1];
            L_last = L;
            if (L_high != -1) { L = (L_high + L_low) / 2; L_high = -1; }
            else L = L * rate;
        } else {
            if (P > p_high) {
                L_high = L;
                s->box[0] = sbx; s->box[1] = sby;
                orc_load_state(s, sx, sy, sr, sm);
                orc_setup_neighbors(s, method, cm, dm, ppc, cdm);
                L_prior = L_last;
                L = (L_high + L_low) / 2;
            } else if (contacts > 2 * n) {
                status = 0;
                break;
            }
        }
        if (L_low > 0 && L_high > 0 && fabs(L_low / L_high - 1) < length_tol) { status = 1; break; }
        orc_scale_box(s, L / L_prior);
        step++;
    }
    free(sx); free(sy); free(sr); free(sm);
    r->pressure = orc_pressure(s);
    r->contacts = orc_contact_count(s);
    r->packing_fraction = orc_packing_fraction(s);
    r->box_length = jam_box_length(s);
    r->compression_steps = step;
    r->fire_steps_total = total;
    r->status = status;
}

/* scripts/runJam.cpp:15-106 */
void orc_jam_phi(orc_sys *s, double tol, double dtol, double phi_tol, double inc, double dstab,
                 int64_t max_steps, orc_jam_result *r) {
    int64_t total = 0;
    double dof = (double)s->n;
    for (int guard = 0; guard < 10000; guard++) {
        total += orc_minimize_fire(s, 0.1, 1e-2, tol, dtol, 100000, 0.0, NULL) + 1;
        if (orc_total_pe(s) / dof < tol) break;
        orc_scale_box(s, 1.1);
    }
    orc_set_last_state(s);
    double phi_low = orc_packing_fraction(s), phi, phi_high = -1.0;
    int64_t step = 0;
    int status = 2;
    while (step < max_steps) {
        phi = orc_packing_fraction(s);
        total += orc_minimize_fire(s, 0.1, 1e-2, tol, dtol, 1000000, 0.0, NULL) + 1;
        double pe = orc_total_pe(s) / dof;
        if (pe > tol) {
            phi_high = phi;
            phi = (phi_high + phi_low) / 2.0;
            orc_revert_to_last_state(s);
        } else {
            orc_set_last_state(s);
            phi_low = phi;
            if (phi_high > 0) phi = (phi_high + phi_low) / 2.0;
            else phi += inc;
        }
        if (fabs(phi_high / phi_low - 1) < phi_tol) {
            orc_set_last_state(s);
            orc_scale_to_packing_fraction(s, orc_packing_fraction(s) + dstab);
            total += orc_minimize_fire(s, 0.1, 1e-2, tol, dtol, 100000, 0.0, NULL) + 1;
            double fin = orc_total_pe(s) / dof;
            orc_revert_to_last_state(s);
            if (fin > 1e-1 * pow(dstab, s->n_c)) { status = 0; break; }
            phi_low = phi;
            phi_high = -1.0;
            phi = orc_packing_fraction(s);
            orc_set_last_state(s);
        }
        orc_scale_to_packing_fraction(s, phi);
        step++;
    }
    r->pressure = orc_pressure(s);
    r->contacts = orc_contact_count(s);
    r->packing_fraction = orc_packing_fraction(s);
    r->box_length = jam_box_length(s);
    r->compression_steps = step;
    r->fire_steps_total = total;
    r->status = status;
}
