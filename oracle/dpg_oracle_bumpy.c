/*
 * dpg_oracle_bumpy.c -- CPU oracle (TEST INFRASTRUCTURE ONLY) for the rigid
 * bumpy bodies of mmccraw98/dpCUDA-v2: rigid bodies made of vertex disks on a
 * circle, vertex-vertex harmonic contacts reduced to body force and torque.
 *
 * Restates src/particles/rigid_bumpy/{rigid_bumpy.cu,kernels.cu} and the
 * base-class sequences they plug into (src/particles/base/particle.cu), with
 * per-function citations.  Used only by tests/ and bench.py's CPU leg.
 * Compile with -ffp-contract=off.  Arrays are SoA in the reference's layout:
 * vertices of a body are contiguous, body b owns vertices
 * [start[b], start[b] + nvb[b]).
 */
#include "dpg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define PAR_MIN 2048
#define PI_REF 3.141592653589793238462643383279502884197

typedef struct orcb_sys {
    int64_t nb, nv;
    double box[2], e_c, n_c, rv, seg;
    int rotation;
    /* bodies (current, cell-sorted order) */
    double *x, *y, *th, *vx, *vy, *w, *fx, *fy, *tq, *pe, *m, *r, *I, *ke;
    double *lpx, *lpy, *dx, *dy, *dth; /* last positions and deltas for the vertex move */
    int64_t *nvb, *start;
    /* reorder targets */
    double *tx, *ty, *tth, *tvx, *tvy, *tw, *tfx, *tfy, *ttq, *tm, *tr, *tI;
    int64_t *tnvb, *tstart, *o2n;
    /* vertices */
    double *px, *py, *vfx, *vfy, *vtq, *vpe, *vm;
    int64_t *vbody, *svidx;
    double *tpx, *tpy, *tvm;
    int64_t *tvbody, *tsvidx;
    /* body neighbours (same scheme as disks) */
    double *lnx, *lny, *lcx, *lcy, *nd2, *cd2;
    int64_t *cell_index, *pidx, *sidx, *cell_start, *key_tmp, *pidx_tmp, *sidx_tmp;
    int64_t *nlist, *ncount, cap;
    int method;
    double cutoff, nthr2, cs, cthr2;
    int64_t ncd, ncells;
    /* vertex neighbours */
    int64_t *vnlist, *vncount, vcap;
    double vcutoff, vpcutoff;
    int64_t n_rebuilds, n_cell_rebuilds;
    /* FIRE */
    double f_alpha, f_alpha0, f_dt, f_dtmax, f_dtmin;
    int64_t f_ngood, f_nbad;
    int f_stopped;
    /* Adam moments: the translational ones are swapped with never-gathered
     * twins on a re-sort, the angular ones stay with their slot */
    double *m1x, *m1y, *m2x, *m2y, *tm1x, *tm1y, *tm2x, *tm2y, *m1a, *m2a;
    /* per-body stress tensor and contact counts */
    double *sxx, *sxy, *syx, *syy;
    int64_t *cc, *vcc;
    /* setLastState snapshot */
    double *s_x, *s_y, *s_vx, *s_vy, *s_fx, *s_fy, *s_r, *s_m, *s_th, *s_w, *s_tq, *s_px, *s_py;
    int64_t *s_pidx, *s_sidx, *s_nvb, *s_start, *s_vbody, *s_svidx;
    double s_box[2];
} orcb_sys;

static double *dz(int64_t n) { return (double *)calloc((size_t)(n > 0 ? n : 1), sizeof(double)); }
static int64_t *lz(int64_t n) { return (int64_t *)calloc((size_t)(n > 0 ? n : 1), sizeof(int64_t)); }
static void lset(int64_t *a, int64_t n, int64_t v) { for (int64_t i = 0; i < n; i++) a[i] = v; }
#define SWAPP(a, b) do { void *t_ = (void *)(a); (a) = (b); (b) = t_; } while (0)

static inline int64_t bmod(int64_t a, int64_t b) { return (a % b + b) % b; }
static inline double bpbc(double a, double b, double L) { double d = a - b; return d - L * round(d / L); }
static inline int64_t bcell(double p, double cs, int64_t ncd) {
    int64_t idx = (int64_t)floor(p / cs);
    return idx >= 0 ? idx % ncd : (idx % ncd + ncd) % ncd;
}

/* calcPointPointInteraction with both radii = vertex radius:
 * include/particles/base/kernels.cuh:154-183 */
static inline double vpair(const orcb_sys *s, double xi, double yi, double xj, double yj, double *fx,
                           double *fy) {
    double ddx = bpbc(xi, xj, s->box[0]);
    double ddy = bpbc(yi, yj, s->box[1]);
    double rs = s->rv + s->rv;
    double d2 = ddx * ddx + ddy * ddy;
    if (d2 >= rs * rs) { *fx = 0.0; *fy = 0.0; return 0.0; }
    double d = sqrt(d2);
    double ov = 1.0 - (d / rs);
    double ovp = (s->n_c == 2.0) ? ov : pow(ov, s->n_c - 1);
    double en = s->e_c * ov * ovp / (2.0 * s->n_c);
    double fm = s->e_c * ovp / (rs * d);
    *fx = fm * ddx;
    *fy = fm * ddy;
    return en;
}

orcb_sys *orcb_create(int64_t nb, int64_t nv, double bx, double by, double e_c, double n_c,
                      double vertex_radius, double seg, int rotation) {
    orcb_sys *s = (orcb_sys *)calloc(1, sizeof(orcb_sys));
    s->nb = nb; s->nv = nv; s->box[0] = bx; s->box[1] = by; s->e_c = e_c; s->n_c = n_c;
    s->rv = vertex_radius; s->seg = seg; s->rotation = rotation;
    double **bd[] = {&s->x, &s->y, &s->th, &s->vx, &s->vy, &s->w, &s->fx, &s->fy, &s->tq, &s->pe,
                     &s->m, &s->r, &s->I, &s->ke, &s->lpx, &s->lpy, &s->dx, &s->dy, &s->dth,
                     &s->tx, &s->ty, &s->tth, &s->tvx, &s->tvy, &s->tw, &s->tfx, &s->tfy, &s->ttq,
                     &s->tm, &s->tr, &s->tI, &s->lnx, &s->lny, &s->lcx, &s->lcy, &s->nd2, &s->cd2,
                     &s->m1x, &s->m1y, &s->m2x, &s->m2y, &s->tm1x, &s->tm1y, &s->tm2x, &s->tm2y,
                     &s->m1a, &s->m2a, &s->sxx, &s->sxy, &s->syx, &s->syy, &s->s_x, &s->s_y,
                     &s->s_vx, &s->s_vy, &s->s_fx, &s->s_fy, &s->s_r, &s->s_m, &s->s_th, &s->s_w,
                     &s->s_tq};
    for (size_t k = 0; k < sizeof(bd) / sizeof(bd[0]); k++) *bd[k] = dz(nb);
    int64_t **bl[] = {&s->nvb, &s->start, &s->tnvb, &s->tstart, &s->o2n, &s->cell_index, &s->pidx,
                      &s->sidx, &s->key_tmp, &s->pidx_tmp, &s->sidx_tmp, &s->ncount, &s->cc,
                      &s->vcc, &s->s_pidx, &s->s_sidx, &s->s_nvb, &s->s_start};
    for (size_t k = 0; k < sizeof(bl) / sizeof(bl[0]); k++) *bl[k] = lz(nb);
    double **vd[] = {&s->px, &s->py, &s->vfx, &s->vfy, &s->vtq, &s->vpe, &s->vm, &s->tpx, &s->tpy,
                     &s->tvm, &s->s_px, &s->s_py};
    for (size_t k = 0; k < sizeof(vd) / sizeof(vd[0]); k++) *vd[k] = dz(nv);
    int64_t **vl[] = {&s->vbody, &s->svidx, &s->tvbody, &s->tsvidx, &s->vncount, &s->s_vbody,
                      &s->s_svidx};
    for (size_t k = 0; k < sizeof(vl) / sizeof(vl[0]); k++) *vl[k] = lz(nv);
    for (int64_t i = 0; i < nb; i++) { s->pidx[i] = i; s->sidx[i] = i; }
    for (int64_t v = 0; v < nv; v++) s->svidx[v] = v;
    s->cap = 4; s->vcap = 4;
    s->nlist = lz(nb * 4); s->vnlist = lz(nv * 4);
    lset(s->nlist, nb * 4, -1); lset(s->vnlist, nv * 4, -1);
    s->cell_start = lz(1);
    s->method = -1;
    return s;
}

void orcb_destroy(orcb_sys *s) {
    if (!s) return;
    void *ptrs[] = {s->x, s->y, s->th, s->vx, s->vy, s->w, s->fx, s->fy, s->tq, s->pe, s->m, s->r,
                    s->I, s->ke, s->lpx, s->lpy, s->dx, s->dy, s->dth, s->tx, s->ty, s->tth, s->tvx,
                    s->tvy, s->tw, s->tfx, s->tfy, s->ttq, s->tm, s->tr, s->tI, s->lnx, s->lny,
                    s->lcx, s->lcy, s->nd2, s->cd2, s->nvb, s->start, s->tnvb, s->tstart, s->o2n,
                    s->cell_index, s->pidx, s->sidx, s->key_tmp, s->pidx_tmp, s->sidx_tmp,
                    s->ncount, s->px, s->py, s->vfx, s->vfy, s->vtq, s->vpe, s->vm, s->tpx, s->tpy,
                    s->tvm, s->vbody, s->svidx, s->tvbody, s->tsvidx, s->vncount, s->nlist,
                    s->vnlist, s->cell_start, s->m1x, s->m1y, s->m2x, s->m2y, s->tm1x, s->tm1y,
                    s->tm2x, s->tm2y, s->m1a, s->m2a, s->sxx, s->sxy, s->syx, s->syy, s->cc, s->vcc,
                    s->s_x, s->s_y, s->s_vx, s->s_vy, s->s_fx, s->s_fy, s->s_r, s->s_m, s->s_th,
                    s->s_w, s->s_tq, s->s_px, s->s_py, s->s_pidx, s->s_sidx, s->s_nvb, s->s_start,
                    s->s_vbody, s->s_svidx};
    for (size_t k = 0; k < sizeof(ptrs) / sizeof(ptrs[0]); k++) free(ptrs[k]);
    free(s);
}

/* setParticleStartIndex + setVertexParticleIndex:
 * src/particles/rigid_bumpy/rigid_bumpy.cu:476-478,562-568, kernels.cu:1099-1113 */
static void index_vertices(orcb_sys *s) {
    int64_t acc = 0;
    for (int64_t b = 0; b < s->nb; b++) { s->start[b] = acc; acc += s->nvb[b]; }
    for (int64_t b = 0; b < s->nb; b++)
        for (int64_t k = 0; k < s->nvb[b]; k++) s->vbody[s->start[b] + k] = b;
}

/* Bodies in static order (before the first cell sort the order is the input order). */
int orcb_set_bodies(orcb_sys *s, const double *x, const double *y, const double *th,
                    const double *vx, const double *vy, const double *w, const double *r,
                    const int64_t *nvb) {
    int64_t tot = 0;
    for (int64_t b = 0; b < s->nb; b++) tot += nvb[b];
    if (tot != s->nv) return -1;
    for (int64_t b = 0; b < s->nb; b++) {
        s->x[b] = x[b]; s->y[b] = y[b]; s->th[b] = th ? th[b] : 0.0;
        s->vx[b] = vx ? vx[b] : 0.0; s->vy[b] = vy ? vy[b] : 0.0; s->w[b] = w ? w[b] : 0.0;
        s->r[b] = r[b]; s->nvb[b] = nvb[b];
    }
    index_vertices(s);
    return 0;
}

/* kernelInitializeVerticesOnParticles: src/particles/rigid_bumpy/kernels.cu:1137-1162 */
void orcb_init_vertices(orcb_sys *s) {
    for (int64_t b = 0; b < s->nb; b++) {
        double inc = 2 * PI_REF / s->nvb[b];
        double ir = s->r[b] - s->rv;
        for (int64_t i = 0; i < s->nvb[b]; i++) {
            double a = i * inc + s->th[b];
            s->px[s->start[b] + i] = s->x[b] + ir * cos(a);
            s->py[s->start[b] + i] = s->y[b] + ir * sin(a);
        }
    }
}

void orcb_set_vertices(orcb_sys *s, const double *px, const double *py) {
    for (int64_t v = 0; v < s->nv; v++) { s->px[v] = px[s->svidx[v]]; s->py[v] = py[s->svidx[v]]; }
}

/* RigidBumpy::setMass: masses, kernelGetVertexMasses, kernelGetMomentsOfInertia
 * (src/particles/rigid_bumpy/rigid_bumpy.cu:1068-1080, kernels.cu:1164-1189) */
void orcb_set_mass(orcb_sys *s, double mass) {
    for (int64_t b = 0; b < s->nb; b++) s->m[b] = mass;
    for (int64_t v = 0; v < s->nv; v++) {
        int64_t b = s->vbody[v];
        s->vm[v] = s->m[b] / (double)s->nvb[b];
    }
    for (int64_t b = 0; b < s->nb; b++) {
        int64_t f = s->start[b];
        double mv = s->vm[f], acc = 0.0;
        for (int64_t i = 0; i < s->nvb[b]; i++) {
            double rx = s->px[f + i] - s->x[b], ry = s->py[f + i] - s->y[b];
            acc += mv * (rx * rx + ry * ry);
        }
        s->I[b] = acc;
    }
}

/* ---------------- neighbours ---------------------------------------------- */
static double bmaxd(const orcb_sys *s) {
    double mx = -INFINITY;
    for (int64_t i = 0; i < s->nb; i++) if (s->r[i] > mx) mx = s->r[i];
    return 2.0 * mx;
}
static double barea(const orcb_sys *s) { return 1.0 * s->box[0] * s->box[1]; }

/* RigidBumpy::setNeighborSize: src/particles/rigid_bumpy/rigid_bumpy.cu:1229-1250 */
static int bset_neighbor_size(orcb_sys *s, double cm, double dm) {
    s->cap = 4; s->vcap = 4;
    s->cutoff = cm * bmaxd(s);
    s->vcutoff = cm * 2.0 * s->rv;
    s->vpcutoff = bmaxd(s);
    s->nthr2 = pow(dm * s->seg * s->rv, 2);
    double diag = sqrt(s->box[0] * s->box[0] + s->box[1] * s->box[1]);
    return s->cutoff < diag;
}

static int bset_cell_size(orcb_sys *s, double ppc, double cdm) {
    const int64_t min_dim = 4;
    double density = (double)s->nb / barea(s);
    double trial = sqrt(ppc / density);
    double min_cs = 2.0 * bmaxd(s);
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

static void bset_method(orcb_sys *s, int method) {
    s->method = method;
    for (int64_t i = 0; i < s->nb; i++) { s->pidx[i] = i; s->sidx[i] = i; }
    if (method == ORC_NEIGH_ALL) {
        double diag = sqrt(s->box[0] * s->box[0] + s->box[1] * s->box[1]);
        bset_neighbor_size(s, 2.0 * diag / bmaxd(s), 0.0);
    }
}

static int64_t bmaxcnt(const int64_t *c, int64_t n) {
    int64_t mx = -1;
    for (int64_t i = 0; i < n; i++) if (c[i] > mx) mx = c[i];
    return mx;
}
static int64_t bgrow(int64_t m) { return (int64_t)pow(2, ceil(log2((double)m))); }

static void body_list_all(orcb_sys *s) {
    const double c2 = s->cutoff * s->cutoff;
    for (int64_t i = 0; i < s->nb; i++) {
        int64_t cnt = 0;
        for (int64_t j = 0; j < s->nb; j++) {
            if (j == i) continue;
            double ddx = bpbc(s->x[i], s->x[j], s->box[0]), ddy = bpbc(s->y[i], s->y[j], s->box[1]);
            if (ddx * ddx + ddy * ddy < c2) {
                if (cnt < s->cap) s->nlist[i * s->cap + cnt] = j;
                cnt++;
            }
        }
        s->lnx[i] = s->x[i]; s->lny[i] = s->y[i]; s->nd2[i] = 0.0; s->ncount[i] = cnt;
    }
}

static void body_list_cells(orcb_sys *s) {
    const double c2 = s->cutoff * s->cutoff;
    const int64_t ncd = s->ncd;
    for (int64_t i = 0; i < s->nb; i++) {
        int64_t cnt = 0, cid = s->cell_index[i], cx = cid % ncd, cy = cid / ncd;
        for (int64_t oy = -1; oy <= 1; oy++) {
            int64_t yy = bmod(cy + oy, ncd);
            for (int64_t ox = -1; ox <= 1; ox++) {
                int64_t nc = bmod(cx + ox, ncd) + yy * ncd;
                int64_t st = s->cell_start[nc];
                if (st == -1) continue;
                int64_t en = s->cell_start[nc + 1];
                while (en == -1) { nc++; en = s->cell_start[nc + 1]; }
                for (int64_t j = st; j < en; j++) {
                    if (j == i) continue;
                    double ddx = bpbc(s->x[i], s->x[j], s->box[0]);
                    double ddy = bpbc(s->y[i], s->y[j], s->box[1]);
                    if (ddx * ddx + ddy * ddy < c2) {
                        if (cnt < s->cap) s->nlist[i * s->cap + cnt] = j;
                        cnt++;
                    }
                }
            }
        }
        s->ncount[i] = cnt; s->nd2[i] = 0.0; s->lnx[i] = s->x[i]; s->lny[i] = s->y[i];
    }
}

/* kernelUpdateVertexNeighborList: src/particles/rigid_bumpy/kernels.cu:870-922 */
static void vertex_list_kernel(orcb_sys *s) {
    const double c2 = s->vcutoff * s->vcutoff, pc2 = s->vpcutoff * s->vpcutoff;
#pragma omp parallel for schedule(static) if (s->nv >= PAR_MIN)
    for (int64_t v = 0; v < s->nv; v++) {
        int64_t cnt = 0, b = s->vbody[v];
        double xv = s->px[v], yv = s->py[v];
        for (int64_t k = 0; k < s->ncount[b]; k++) {
            int64_t ob = s->nlist[b * s->cap + k];
            if (ob == -1 || ob == b) continue;
            double ddx = bpbc(xv, s->x[ob], s->box[0]), ddy = bpbc(yv, s->y[ob], s->box[1]);
            if (!(ddx * ddx + ddy * ddy < pc2)) continue;
            int64_t f = s->start[ob];
            for (int64_t u = f; u < f + s->nvb[ob]; u++) {
                double ex = bpbc(xv, s->px[u], s->box[0]), ey = bpbc(yv, s->py[u], s->box[1]);
                if (ex * ex + ey * ey < c2) {
                    if (cnt < s->vcap) s->vnlist[v * s->vcap + cnt] = u;
                    cnt++;
                }
            }
        }
        s->vncount[v] = cnt;
    }
}

/* RigidBumpy::updateVertexVerletList: src/particles/rigid_bumpy/rigid_bumpy.cu:1198-1212 */
static void update_vertex_list(orcb_sys *s) {
    lset(s->vnlist, s->nv * s->vcap, -1);
    vertex_list_kernel(s);
    int64_t mx = bmaxcnt(s->vncount, s->nv);
    if (mx > s->vcap) {
        s->vcap = bgrow(mx);
        free(s->vnlist);
        s->vnlist = lz(s->nv * s->vcap);
        lset(s->vnlist, s->nv * s->vcap, -1);
        vertex_list_kernel(s);
    }
}

static void update_body_list(orcb_sys *s, int cells) {
    lset(s->nlist, s->nb * s->cap, -1);
    if (cells) body_list_cells(s); else body_list_all(s);
    int64_t mx = bmaxcnt(s->ncount, s->nb);
    if (mx > s->cap) {
        s->cap = bgrow(mx);
        free(s->nlist);
        s->nlist = lz(s->nb * s->cap);
        lset(s->nlist, s->nb * s->cap, -1);
        if (cells) body_list_cells(s); else body_list_all(s);
    }
    s->n_rebuilds++;
    update_vertex_list(s);
}

/* updateCellList + RigidBumpy::reorderParticleData:
 * src/particles/base/particle.cu:1307-1317, src/particles/rigid_bumpy/rigid_bumpy.cu:1303-1376,
 * kernels.cu:796-868 */
static void update_cell_list(orcb_sys *s) {
    const int64_t nb = s->nb, ncd = s->ncd, nc = s->ncells;
    s->cell_start[nc] = nb;
    for (int64_t i = 0; i < nb; i++) {
        s->cell_index[i] = bcell(s->x[i], s->cs, ncd) + bcell(s->y[i], s->cs, ncd) * ncd;
        s->pidx[i] = i;
    }
    int64_t *cnt = lz(nc + 1), *cur = lz(nc);
    for (int64_t i = 0; i < nb; i++) cnt[s->cell_index[i] + 1]++;
    for (int64_t c = 0; c < nc; c++) cnt[c + 1] += cnt[c];
    for (int64_t c = 0; c < nc; c++) s->cell_start[c] = (cnt[c + 1] > cnt[c]) ? cnt[c] : -1;
    memcpy(cur, cnt, (size_t)nc * sizeof(int64_t));
    for (int64_t i = 0; i < nb; i++) {
        int64_t c = s->cell_index[i], slot = cur[c]++;
        s->key_tmp[slot] = c; s->pidx_tmp[slot] = s->pidx[i]; s->sidx_tmp[slot] = s->sidx[i];
    }
    free(cnt); free(cur);
    memcpy(s->cell_index, s->key_tmp, (size_t)nb * sizeof(int64_t));
    memcpy(s->pidx, s->pidx_tmp, (size_t)nb * sizeof(int64_t));
    memcpy(s->sidx, s->sidx_tmp, (size_t)nb * sizeof(int64_t));
    for (int64_t n = 0; n < nb; n++) {
        int64_t o = s->pidx[n];
        s->o2n[o] = n;
        s->tx[n] = s->x[o]; s->ty[n] = s->y[o]; s->tfx[n] = s->fx[o]; s->tfy[n] = s->fy[o];
        s->tvx[n] = s->vx[o]; s->tvy[n] = s->vy[o]; s->tw[n] = s->w[o]; s->ttq[n] = s->tq[o];
        s->tth[n] = s->th[o]; s->tm[n] = s->m[o]; s->tr[n] = s->r[o]; s->tI[n] = s->I[o];
        s->tnvb[n] = s->nvb[o];
        s->lcx[n] = s->x[o]; s->lcy[n] = s->y[o]; s->cd2[n] = 0.0;
    }
    int64_t acc = 0;
    for (int64_t n = 0; n < nb; n++) { s->tstart[n] = acc; acc += s->tnvb[n]; }
    for (int64_t ov = 0; ov < s->nv; ov++) {
        int64_t ob = s->vbody[ov], nbn = s->o2n[ob];
        int64_t nvid = s->tstart[nbn] + (ov - s->start[ob]);
        s->tvbody[nvid] = nbn;
        s->tpx[nvid] = s->px[ov]; s->tpy[nvid] = s->py[ov];
        s->tvm[nvid] = s->vm[ov]; s->tsvidx[nvid] = s->svidx[ov];
    }
    SWAPP(s->x, s->tx); SWAPP(s->y, s->ty); SWAPP(s->fx, s->tfx); SWAPP(s->fy, s->tfy);
    SWAPP(s->vx, s->tvx); SWAPP(s->vy, s->tvy); SWAPP(s->w, s->tw); SWAPP(s->tq, s->ttq);
    SWAPP(s->th, s->tth); SWAPP(s->m, s->tm); SWAPP(s->r, s->tr); SWAPP(s->I, s->tI);
    SWAPP(s->nvb, s->tnvb); SWAPP(s->start, s->tstart);
    SWAPP(s->px, s->tpx); SWAPP(s->py, s->tpy); SWAPP(s->vm, s->tvm);
    SWAPP(s->vbody, s->tvbody); SWAPP(s->svidx, s->tsvidx);
    /* first_moment.swap(), second_moment.swap() without a gather (rigid_bumpy.cu:1370-1371);
     * the angular moments are neither gathered nor swapped */
    SWAPP(s->m1x, s->tm1x); SWAPP(s->m1y, s->tm1y); SWAPP(s->m2x, s->tm2x); SWAPP(s->m2y, s->tm2y);
    s->n_cell_rebuilds++;
}

void orcb_calculate_forces(orcb_sys *s);

/* Particle::setupNeighbors with the RigidBumpy overrides
 * (src/particles/base/particle.cu:71-100, rigid_bumpy.cu:1214-1255) */
int orcb_setup_neighbors(orcb_sys *s, int method, double cm, double dm, double ppc, double cdm) {
    bset_method(s, method);
    bset_neighbor_size(s, cm, dm);
    if (s->method == ORC_NEIGH_CELL) {
        if (!bset_cell_size(s, ppc, cdm)) bset_method(s, ORC_NEIGH_VERLET);
        if (!bset_neighbor_size(s, cm, dm)) bset_method(s, ORC_NEIGH_ALL);
    }
    if (s->method == ORC_NEIGH_VERLET) {
        if (!bset_neighbor_size(s, cm, dm)) bset_method(s, ORC_NEIGH_ALL);
    }
    /* initVerletListVariables (+ vertex list) */
    if (s->method == ORC_NEIGH_ALL) s->cap = s->nb - 1;
    free(s->nlist); s->nlist = lz(s->nb * s->cap); lset(s->nlist, s->nb * s->cap, -1);
    free(s->vnlist); s->vnlist = lz(s->nv * s->vcap); lset(s->vnlist, s->nv * s->vcap, -1);
    for (int64_t i = 0; i < s->nb; i++) {
        s->ncount[i] = 0; s->lnx[i] = 0; s->lny[i] = 0; s->nd2[i] = 0; s->lcx[i] = 0; s->lcy[i] = 0;
        s->cd2[i] = 0;
    }
    for (int64_t v = 0; v < s->nv; v++) s->vncount[v] = 0;
    if (s->method == ORC_NEIGH_CELL) {
        for (int64_t i = 0; i < s->nb; i++) { s->cell_index[i] = -1; s->pidx[i] = i; s->sidx[i] = i; }
        for (int64_t v = 0; v < s->nv; v++) s->svidx[v] = v;
        free(s->cell_start);
        s->cell_start = lz(s->ncells + 1);
        update_cell_list(s);
        update_body_list(s, 1);
    } else {
        if (s->method == ORC_NEIGH_ALL) {
            s->cutoff = 10.0 * sqrt(s->box[0] * s->box[0] + s->box[1] * s->box[1]);
            s->nthr2 = s->cutoff * s->cutoff;
        }
        update_body_list(s, 0);
    }
    orcb_calculate_forces(s);
    return s->method;
}

int orcb_check_for_neighbor_update(orcb_sys *s) {
    const double tol = 3.0;
    double mn = 0.0, mc = 0.0;
    for (int64_t i = 0; i < s->nb; i++) { if (s->nd2[i] > mn) mn = s->nd2[i]; if (s->cd2[i] > mc) mc = s->cd2[i]; }
    if (s->method == ORC_NEIGH_ALL) return 0;
    if (s->method == ORC_NEIGH_VERLET) {
        if (tol * mn > s->nthr2) { update_body_list(s, 0); return 1; }
        return 0;
    }
    if (tol * mc > s->cthr2) { update_cell_list(s); update_body_list(s, 1); return 2; }
    if (tol * mn > s->nthr2) { update_body_list(s, 1); return 1; }
    return 0;
}

/* ---------------- forces and dynamics ------------------------------------ */
/* kernelZeroRigidBumpy{Particle,Vertex}ForceAndPotentialEnergy: kernels.cu:234-252 */
void orcb_zero(orcb_sys *s) {
    for (int64_t b = 0; b < s->nb; b++) { s->fx[b] = 0; s->fy[b] = 0; s->tq[b] = 0; s->pe[b] = 0; }
    for (int64_t v = 0; v < s->nv; v++) { s->vfx[v] = 0; s->vfy[v] = 0; s->vtq[v] = 0; s->vpe[v] = 0; }
}

/* kernelCalcRigidBumpyForces1 + kernelCalcRigidBumpyParticleForces1:
 * src/particles/rigid_bumpy/kernels.cu:366-442 (+= into zeroed arrays) */
void orcb_calculate_forces(orcb_sys *s) {
#pragma omp parallel for schedule(static) if (s->nv >= PAR_MIN)
    for (int64_t v = 0; v < s->nv; v++) {
        int64_t nn = s->vncount[v];
        if (nn == 0) continue;
        double xv = s->px[v], yv = s->py[v];
        int64_t b = s->vbody[v];
        double ax = 0.0, ay = 0.0, en = 0.0;
        for (int64_t k = 0; k < nn; k++) {
            int64_t u = s->vnlist[v * s->vcap + k];
            if (u == -1 || u == v) continue;
            double fx, fy;
            double e = vpair(s, xv, yv, s->px[u], s->py[u], &fx, &fy);
            ax += fx; ay += fy; en += e;
        }
        double rx = xv - s->x[b], ry = yv - s->y[b];
        double t = ay * rx - ax * ry;
        s->vfx[v] += ax; s->vfy[v] += ay; s->vtq[v] += t; s->vpe[v] += en;
    }
    for (int64_t b = 0; b < s->nb; b++) {
        double ax = 0.0, ay = 0.0, at = 0.0, en = 0.0;
        for (int64_t k = 0; k < s->nvb[b]; k++) {
            int64_t v = s->start[b] + k;
            ax += s->vfx[v]; ay += s->vfy[v]; at += s->vtq[v]; en += s->vpe[v];
        }
        s->fx[b] += ax; s->fy[b] += ay; s->tq[b] += at; s->pe[b] += en;
    }
}

/* kernelUpdateRigidVelocities: kernels.cu:123-150 */
void orcb_update_velocities(orcb_sys *s, double dt) {
    for (int64_t b = 0; b < s->nb; b++) {
        double w = s->w[b];
        if (s->rotation) w += s->tq[b] * dt / s->I[b];
        else w = 0.0;
        s->vx[b] += s->fx[b] * dt / s->m[b];
        s->vy[b] += s->fy[b] * dt / s->m[b];
        s->w[b] = w;
    }
}

/* kernelUpdateRigidPositions + kernelTranslateAndRotateVertices1: kernels.cu:21-78,152-201 */
void orcb_update_positions(orcb_sys *s, double dt) {
    for (int64_t b = 0; b < s->nb; b++) {
        double ox = s->x[b], oy = s->y[b], a = s->th[b];
        s->lpx[b] = ox; s->lpy[b] = oy;
        double ddx = s->vx[b] * dt, ddy = s->vy[b] * dt, dth = s->w[b] * dt;
        s->dx[b] = ddx; s->dy[b] = ddy; s->dth[b] = dth;
        double nx = ox + ddx, ny = oy + ddy;
        s->x[b] = nx; s->y[b] = ny; s->th[b] = a + dth;
        double a1 = nx - s->lnx[b], a2 = ny - s->lny[b];
        s->nd2[b] = a1 * a1 + a2 * a2;
        double c1 = nx - s->lcx[b], c2 = ny - s->lcy[b];
        s->cd2[b] = c1 * c1 + c2 * c2;
    }
    for (int64_t v = 0; v < s->nv; v++) {
        int64_t b = s->vbody[v];
        double rx = s->px[v] - s->lpx[b], ry = s->py[v] - s->lpy[b];
        double ca = cos(s->dth[b]), sa = sin(s->dth[b]);
        double rxr = rx * ca - ry * sa, ryr = rx * sa + ry * ca;
        s->px[v] = s->x[b] + rxr;
        s->py[v] = s->y[b] + ryr;
    }
}

/* kernelMixRigidVelocitiesAndForces: kernels.cu:89-121 */
void orcb_mix(orcb_sys *s, double alpha) {
    for (int64_t b = 0; b < s->nb; b++) {
        double fx = s->fx[b], fy = s->fy[b], vx = s->vx[b], vy = s->vy[b];
        double fn = sqrt(fx * fx + fy * fy), vn = sqrt(vx * vx + vy * vy), mix = 0.0;
        if (fn > 1e-16) mix = vn / fn * alpha;
        else { vx = 0.0; vy = 0.0; }
        double w = s->w[b], t = s->tq[b];
        double tn = fabs(t), wn = fabs(w), tmix = 0.0;
        if (tn > 1e-16) tmix = wn / tn * alpha;
        else { w = 0.0; tmix = 0.0; }
        s->vx[b] = vx * (1 - alpha) + fx * mix;
        s->vy[b] = vy * (1 - alpha) + fy * mix;
        s->w[b] = w * (1 - alpha) + t * tmix;
    }
}

void orcb_set_velocities_zero(orcb_sys *s) {
    for (int64_t b = 0; b < s->nb; b++) { s->vx[b] = 0; s->vy[b] = 0; s->w[b] = 0; }
}

/* RigidBumpy::getPowerFire: rigid_bumpy.cu:1181-1190 */
double orcb_power_fire(orcb_sys *s) {
    double px = 0, py = 0, pr = 0;
    for (int64_t b = 0; b < s->nb; b++) px += s->fx[b] * s->vx[b];
    for (int64_t b = 0; b < s->nb; b++) py += s->fy[b] * s->vy[b];
    for (int64_t b = 0; b < s->nb; b++) pr += s->tq[b] * s->w[b];
    return (px + py) + pr;
}

double orcb_total_pe(orcb_sys *s) {
    double e = 0;
    for (int64_t b = 0; b < s->nb; b++) e += s->pe[b];
    return e;
}

/* kernelCalculateTranslationalAndRotationalKineticEnergy: kernels.cu:254-269 */
double orcb_total_ke(orcb_sys *s) {
    double e = 0;
    for (int64_t b = 0; b < s->nb; b++) {
        double k;
        if (s->rotation)
            k = 0.5 * s->m[b] * (s->vx[b] * s->vx[b] + s->vy[b] * s->vy[b]) + 0.5 * s->I[b] * s->w[b] * s->w[b];
        else
            k = 0.5 * s->m[b] * (s->vx[b] * s->vx[b] + s->vy[b] * s->vy[b]);
        s->ke[b] = k;
        e += k;
    }
    return e;
}

void orcb_max_force_torque(orcb_sys *s, double *fmax, double *tmax) {
    double a = 0, t = 0;
    for (int64_t b = 0; b < s->nb; b++) {
        double f = sqrt(s->fx[b] * s->fx[b] + s->fy[b] * s->fy[b]);
        if (f > a) a = f;
        if (fabs(s->tq[b]) > t) t = fabs(s->tq[b]);
    }
    *fmax = a; *tmax = t;
}

void orcb_nve_steps(orcb_sys *s, double dt, int64_t n) {
    for (int64_t t = 0; t < n; t++) {
        orcb_update_velocities(s, 0.5 * dt);
        orcb_update_positions(s, dt);
        orcb_check_for_neighbor_update(s);
        orcb_zero(s);
        orcb_calculate_forces(s);
        orcb_update_velocities(s, 0.5 * dt);
    }
}

void orcb_fire_init(orcb_sys *s, double alpha_init, double dt) {
    s->f_alpha = alpha_init; s->f_alpha0 = alpha_init; s->f_dt = dt;
    s->f_dtmax = 10.0 * dt; s->f_dtmin = 0.001 * dt;
    s->f_ngood = 0; s->f_nbad = 0; s->f_stopped = 0;
}

/* Fire::step with the RigidBumpy overrides: src/integrator/fire.cu:13-46 */
int orcb_fire_step(orcb_sys *s) {
    double power = orcb_power_fire(s);
    if (power > 0) {
        s->f_ngood++;
        s->f_nbad = 0;
        if (s->f_ngood > 5) {
            double d = s->f_dt * 1.1;
            s->f_dt = d < s->f_dtmax ? d : s->f_dtmax;
            s->f_alpha *= 0.99;
        }
    } else {
        s->f_ngood = 0;
        s->f_nbad++;
        if (s->f_nbad > 10) { s->f_stopped = 1; return 1; }
        double d = s->f_dt * 0.5;
        s->f_dt = d > s->f_dtmin ? d : s->f_dtmin;
        s->f_alpha = s->f_alpha0;
        orcb_update_positions(s, -s->f_dt / 2.0);
        orcb_set_velocities_zero(s);
    }
    orcb_update_velocities(s, s->f_dt / 2.0);
    orcb_mix(s, s->f_alpha);
    orcb_update_positions(s, s->f_dt);
    orcb_zero(s);
    orcb_check_for_neighbor_update(s);
    orcb_calculate_forces(s);
    orcb_update_velocities(s, s->f_dt / 2.0);
    return 0;
}

/* minimizeFire (src/routines/minimization.cu:75-112); fmax/tmax > 0 add
 * max|F_b| <= fmax and max|tau_b| <= tmax stops. */
int64_t orcb_minimize_fire(orcb_sys *s, double alpha_init, double dt, double pe_target,
                           double pe_diff_target, int64_t num_steps, double fmax, double tmax,
                           int *stopped_out) {
    orcb_fire_init(s, alpha_init, dt);
    int64_t step = 0;
    double dof = (double)s->nb;
    orcb_set_velocities_zero(s);
    orcb_zero(s);
    orcb_check_for_neighbor_update(s);
    orcb_calculate_forces(s);
    double last = orcb_total_pe(s) / dof;
    while (step < num_steps) {
        orcb_fire_step(s);
        double avg = orcb_total_pe(s) / dof;
        double diff = fabs(avg / last - 1);
        last = avg;
        if (diff < pe_diff_target || avg < pe_target || s->f_stopped) break;
        if (fmax > 0) {
            double a, t;
            orcb_max_force_torque(s, &a, &t);
            if (a <= fmax && t <= tmax) break;
        }
        step++;
    }
    orcb_set_velocities_zero(s);
    if (stopped_out) *stopped_out = s->f_stopped;
    return step;
}

/* ---------------- Adam --------------------------------------------------- */
/* RigidBumpy::initAdamVariables (rigid_bumpy.cu:1461-1465): every moment, and
 * the twins the translational ones swap with, starts at zero */
void orcb_adam_init(orcb_sys *s) {
    double *arr[] = {s->m1x, s->m1y, s->m2x, s->m2y, s->tm1x, s->tm1y, s->tm2x, s->tm2y, s->m1a, s->m2a};
    for (size_t k = 0; k < sizeof(arr) / sizeof(arr[0]); k++)
        for (int64_t b = 0; b < s->nb; b++) arr[k][b] = 0.0;
}

/* RigidBumpy::updatePositionsAdam: kernelRigidBumpyAdamStep then
 * kernelTranslateAndRotateVertices1 (rigid_bumpy.cu:1473-1486,
 * kernels.cu:1004-1093,152-201).  With rotation off the angle and its delta
 * are left alone, so the vertices turn by the slot's last angle delta. */
void orcb_adam_step(orcb_sys *s, int64_t step, double alpha, double b1, double b2, double eps) {
    const double c1 = 1 - pow(b1, step + 1), c2 = 1 - pow(b2, step + 1);
    for (int64_t b = 0; b < s->nb; b++) {
        double fx = s->fx[b], fy = s->fy[b], t = s->tq[b];
        double m1x = fma(b1, s->m1x[b], (b1 - 1) * fx);
        double m1y = fma(b1, s->m1y[b], (b1 - 1) * fy);
        double m1a = fma(b1, s->m1a[b], (b1 - 1) * t);
        double m2x = fma(b2, s->m2x[b], (1 - b2) * fx * fx);
        double m2y = fma(b2, s->m2y[b], (1 - b2) * fy * fy);
        double m2a = fma(b2, s->m2a[b], (1 - b2) * t * t);
        double ux = -alpha * (m1x / c1) / (sqrt(m2x / c2) + eps);
        double uy = -alpha * (m1y / c1) / (sqrt(m2y / c2) + eps);
        double ua = -alpha * (m1a / c1) / (sqrt(m2a / c2) + eps);
        double px = s->x[b], py = s->y[b];
        s->lpx[b] = px; s->lpy[b] = py;
        px += ux; py += uy;
        s->dx[b] = ux; s->dy[b] = uy;
        if (s->rotation) { s->th[b] += ua; s->dth[b] = ua; }
        s->x[b] = px; s->y[b] = py;
        double a1 = px - s->lnx[b], a2 = py - s->lny[b];
        s->nd2[b] = a1 * a1 + a2 * a2;
        double e1 = px - s->lcx[b], e2 = py - s->lcy[b];
        s->cd2[b] = e1 * e1 + e2 * e2;
        s->m1x[b] = m1x; s->m1y[b] = m1y; s->m1a[b] = m1a;
        s->m2x[b] = m2x; s->m2y[b] = m2y; s->m2a[b] = m2a;
    }
    for (int64_t v = 0; v < s->nv; v++) {
        int64_t b = s->vbody[v];
        double rx = s->px[v] - s->lpx[b], ry = s->py[v] - s->lpy[b];
        double ca = cos(s->dth[b]), sa = sin(s->dth[b]);
        s->px[v] = s->x[b] + (rx * ca - ry * sa);
        s->py[v] = s->y[b] + (rx * sa + ry * ca);
    }
}

/* minimizeAdam (src/routines/minimization.cu:3-33) with Adam::minimize
 * (src/integrator/adam.cu:11-17); dof = n_dof = 3 N with rotation, else 2 N
 * (rigid_bumpy.cu:618-624).  Returns the final step index. */
int64_t orcb_minimize_adam(orcb_sys *s, double alpha, double b1, double b2, double eps,
                           double pe_target, double pe_diff_target, int64_t num_steps) {
    orcb_adam_init(s);
    int64_t step = 0;
    double dof = (double)(s->nb * (s->rotation ? 3 : 2)), last = 0.0;
    while (step < num_steps) {
        orcb_zero(s);
        orcb_check_for_neighbor_update(s);
        orcb_calculate_forces(s);
        orcb_adam_step(s, step, alpha, b1, b2, eps);
        double avg = orcb_total_pe(s) / dof;
        double diff = fabs(avg / last - 1);
        last = avg;
        if (diff < pe_diff_target || avg < pe_target) break;
        step++;
    }
    return step;
}

/* n steps of Adam::minimize (src/integrator/adam.cu:11-17) without the stop test */
void orcb_adam_steps(orcb_sys *s, double alpha, double b1, double b2, double eps, int64_t n) {
    orcb_adam_init(s);
    for (int64_t t = 0; t < n; t++) {
        orcb_zero(s);
        orcb_check_for_neighbor_update(s);
        orcb_calculate_forces(s);
        orcb_adam_step(s, t, alpha, b1, b2, eps);
    }
}

/* Rigid gradient descent (no reference counterpart: GradDesc::step on a
 * RigidBumpy runs the disk kernelGradDescStep, src/particles/base/kernels.cu:
 * 613-637, which moves the body centres but neither the angles nor the
 * vertices).  Here x += alpha F as that kernel, theta += alpha tau with
 * rotation, and the vertices follow as in kernelTranslateAndRotateVertices1. */
void orcb_grad_desc_step(orcb_sys *s, double alpha) {
    for (int64_t b = 0; b < s->nb; b++) {
        double px = s->x[b], py = s->y[b];
        s->lpx[b] = px; s->lpy[b] = py;
        px += alpha * s->fx[b];
        py += alpha * s->fy[b];
        double dth = 0.0;
        if (s->rotation) {
            dth = alpha * s->tq[b];
            s->th[b] += dth;
        }
        s->dx[b] = px - s->lpx[b]; s->dy[b] = py - s->lpy[b];
        s->x[b] = px; s->y[b] = py;
        double a1 = px - s->lnx[b], a2 = py - s->lny[b];
        s->nd2[b] = a1 * a1 + a2 * a2;
        double e1 = px - s->lcx[b], e2 = py - s->lcy[b];
        s->cd2[b] = e1 * e1 + e2 * e2;
        s->ke[b] = dth; /* scratch: this step's angle increment */
    }
    for (int64_t v = 0; v < s->nv; v++) {
        int64_t b = s->vbody[v];
        double rx = s->px[v] - s->lpx[b], ry = s->py[v] - s->lpy[b];
        double ca = cos(s->ke[b]), sa = sin(s->ke[b]);
        s->px[v] = s->x[b] + (rx * ca - ry * sa);
        s->py[v] = s->y[b] + (rx * sa + ry * ca);
    }
}

/* GradDesc::step (src/integrator/grad_desc.cu:11-17) n times with the rigid step */
void orcb_grad_desc_steps(orcb_sys *s, double alpha, int64_t n) {
    for (int64_t t = 0; t < n; t++) {
        orcb_zero(s);
        orcb_check_for_neighbor_update(s);
        orcb_calculate_forces(s);
        orcb_grad_desc_step(s, alpha);
    }
}

/* ---------------- damping and walls --------------------------------------- */
/* kernelCalculateRigidDampedForces: kernels.cu:80-87 */
void orcb_damped_forces(orcb_sys *s, double g) {
    for (int64_t b = 0; b < s->nb; b++) {
        s->fx[b] -= g * s->vx[b];
        s->fy[b] -= g * s->vy[b];
        s->tq[b] -= g * s->w[b];
    }
}

/* DampedNVE::step with the rigid overrides: src/integrator/damped_nve.cu:15-25 */
void orcb_damped_nve_steps(orcb_sys *s, double dt, double g, int64_t n) {
    for (int64_t t = 0; t < n; t++) {
        orcb_update_velocities(s, 0.5 * dt);
        orcb_update_positions(s, dt);
        orcb_check_for_neighbor_update(s);
        orcb_zero(s);
        orcb_damped_forces(s, g);
        orcb_calculate_forces(s);
        orcb_update_velocities(s, 0.5 * dt);
    }
}

/* calcWallInteraction: include/particles/base/kernels.cuh:185-235 (box walls
 * at 0 and L on both axes) */
static double bwall(const orcb_sys *s, double x, double y, double rad, double *fx, double *fy) {
    double en = 0.0;
    const double pos[4] = {x, x, y, y};
    const double dist[4] = {x, s->box[0] - x, y, s->box[1] - y};
    *fx = 0.0; *fy = 0.0;
    for (int k = 0; k < 4; k++) {
        int near = (k % 2 == 0) ? (pos[k] < rad) : (pos[k] > s->box[k / 2] - rad);
        if (!near) continue;
        double ov = rad - dist[k];
        if (!(ov > 0)) continue;
        double ovp = pow(ov / rad, s->n_c - 1);
        double f = s->e_c * ovp / rad;
        if (k == 0) *fx += f;
        else if (k == 1) *fx -= f;
        else if (k == 2) *fy += f;
        else *fy -= f;
        en += s->e_c * ov * ovp / (s->n_c * rad);
    }
    return en;
}

/* kernelCalcRigidBumpyWallForces (kernels.cu:348-362): += into the vertex
 * arrays, torque about the body centre without the minimum image */
void orcb_wall_forces(orcb_sys *s) {
    for (int64_t v = 0; v < s->nv; v++) {
        int64_t b = s->vbody[v];
        double fx, fy;
        double e = bwall(s, s->px[v], s->py[v], s->rv, &fx, &fy);
        double rx = s->px[v] - s->x[b], ry = s->py[v] - s->y[b];
        s->vfx[v] += fx; s->vfy[v] += fy; s->vtq[v] += fy * rx - fx * ry; s->vpe[v] += e;
    }
}

/* calculateWallForces_onlyWallContacts (rigid_bumpy.cu:1495-1499): the wall
 * terms, then kernelCalcRigidBumpyParticleForces1's per-body sums */
void orcb_wall_only(orcb_sys *s) {
    orcb_wall_forces(s);
    for (int64_t b = 0; b < s->nb; b++) {
        double ax = 0.0, ay = 0.0, at = 0.0, en = 0.0;
        for (int64_t k = 0; k < s->nvb[b]; k++) {
            int64_t v = s->start[b] + k;
            ax += s->vfx[v]; ay += s->vfy[v]; at += s->vtq[v]; en += s->vpe[v];
        }
        s->fx[b] += ax; s->fy[b] += ay; s->tq[b] += at; s->pe[b] += en;
    }
}

/* calculateWallForces then calculateForces, the pair NVE::wall_step calls */
void orcb_wall_and_pair_forces(orcb_sys *s) {
    orcb_wall_forces(s);
    orcb_calculate_forces(s);
}

/* NVE::wall_step with the rigid overrides: src/integrator/nve.cu:27-38 */
void orcb_nve_wall_steps(orcb_sys *s, double dt, int64_t n) {
    for (int64_t t = 0; t < n; t++) {
        orcb_update_velocities(s, 0.5 * dt);
        orcb_update_positions(s, dt);
        orcb_check_for_neighbor_update(s);
        orcb_zero(s);
        orcb_wall_forces(s);
        orcb_calculate_forces(s);
        orcb_update_velocities(s, 0.5 * dt);
    }
}

/* ---------------- stress, pressure, contacts ------------------------------ */
/* kernelCalcRigidBumpyStressTensor (kernels.cu:705-789): per body, the kinetic
 * term of every vertex (body velocity plus omega x r through atan2 / sin /
 * cos when omega != 0) and half the virial of its vertex contacts with other
 * bodies, in vertex then list order, divided by the box area.  out = the four
 * component sums over bodies (xx, xy, yx, yy). */
void orcb_stress(orcb_sys *s, double *out) {
    const double area = s->box[0] * s->box[1];
#pragma omp parallel for schedule(static) if (s->nb >= PAR_MIN)
    for (int64_t b = 0; b < s->nb; b++) {
        double axx = 0.0, axy = 0.0, ayx = 0.0, ayy = 0.0;
        double cx = s->x[b], cy = s->y[b], ux = s->vx[b], uy = s->vy[b], w = s->w[b];
        for (int64_t k = 0; k < s->nvb[b]; k++) {
            int64_t v = s->start[b] + k;
            double qx = s->px[v], qy = s->py[v], mv = s->vm[v];
            double rx = qx - cx, ry = qy - cy;
            double prad = sqrt(rx * rx + ry * ry);
            double wx = ux, wy = uy;
            if (w != 0.0) {
                double a = atan2(ry, rx);
                wx -= sin(a) * w * prad;
                wy += cos(a) * w * prad;
            }
            axx += mv * wx * wx;
            axy += mv * wx * wy;
            ayx += mv * wy * wx;
            ayy += mv * wy * wy;
            for (int64_t t = 0; t < s->vncount[v]; t++) {
                int64_t u = s->vnlist[v * s->vcap + t];
                if (u == -1 || u == v || s->vbody[u] == b) continue;
                double dx = bpbc(qx, s->px[u], s->box[0]);
                double dy = bpbc(qy, s->py[u], s->box[1]);
                double fx, fy;
                vpair(s, qx, qy, s->px[u], s->py[u], &fx, &fy);
                axx += dx * fx / 2;
                axy += dx * fy / 2;
                ayx += dy * fx / 2;
                ayy += dy * fy / 2;
            }
        }
        s->sxx[b] = axx / area; s->sxy[b] = axy / area; s->syx[b] = ayx / area; s->syy[b] = ayy / area;
    }
    double t[4] = {0, 0, 0, 0};
    for (int64_t b = 0; b < s->nb; b++) { t[0] += s->sxx[b]; t[1] += s->sxy[b]; t[2] += s->syx[b]; t[3] += s->syy[b]; }
    if (out) for (int k = 0; k < 4; k++) out[k] = t[k];
}

/* getPressure after calculateStressTensor (src/particles/base/particle.cu:1371-1376) */
double orcb_pressure(orcb_sys *s) {
    double t[4];
    orcb_stress(s, t);
    return (t[0] + t[3]) / 2;
}

/* kernelCountRigidBumpyContacts (kernels.cu:924-997): a neighbour body counts
 * once if any vertex pair of the two bodies overlaps; the vertex count adds,
 * per neighbour body, the overlapping partners of the FIRST vertex (in body
 * vertex order) that has one.  Returns getContactCount (the sum of the body
 * counts). */
double orcb_count_contacts(orcb_sys *s) {
    const double rs = 2 * s->rv;
#pragma omp parallel for schedule(static) if (s->nb >= PAR_MIN)
    for (int64_t b = 0; b < s->nb; b++) {
        int64_t nc = 0, nvc = 0;
        for (int64_t k = 0; k < s->ncount[b]; k++) {
            int64_t ob = s->nlist[b * s->cap + k];
            if (ob == -1 || ob == b) continue;
            int contact = 0;
            for (int64_t i = 0; i < s->nvb[b]; i++) {
                int64_t v = s->start[b] + i;
                for (int64_t t = 0; t < s->vncount[v]; t++) {
                    int64_t u = s->vnlist[v * s->vcap + t];
                    if (u == -1 || u == v || s->vbody[u] != ob) continue;
                    double dx = bpbc(s->px[v], s->px[u], s->box[0]);
                    double dy = bpbc(s->py[v], s->py[u], s->box[1]);
                    if (sqrt(dx * dx + dy * dy) < rs) {
                        if (!contact) nc++;
                        nvc++;
                        contact = 1;
                    }
                }
                if (contact) break;
            }
        }
        s->cc[b] = nc;
        s->vcc[b] = nvc;
    }
    int64_t tot = 0;
    for (int64_t b = 0; b < s->nb; b++) tot += s->cc[b];
    return (double)tot;
}

/* per-body stress components and contact counts in static order */
void orcb_get_stress(const orcb_sys *s, double *sxx, double *sxy, double *syx, double *syy) {
    for (int64_t b = 0; b < s->nb; b++) {
        int64_t k = s->sidx[b];
        if (sxx) sxx[k] = s->sxx[b];
        if (sxy) sxy[k] = s->sxy[b];
        if (syx) syx[k] = s->syx[b];
        if (syy) syy[k] = s->syy[b];
    }
}

void orcb_get_contacts(const orcb_sys *s, int64_t *cc, int64_t *vcc) {
    for (int64_t b = 0; b < s->nb; b++) {
        int64_t k = s->sidx[b];
        if (cc) cc[k] = s->cc[b];
        if (vcc) vcc[k] = s->vcc[b];
    }
}

/* ---------------- pair and Hessian dump ------------------------------------ */
/* RigidBumpy::calculateForceDistancePairs (rigid_bumpy.cu:1383-1459) with
 * kernelCalcRigidBumpyForceDistancePairs (kernels.cu:482-703).  Entry
 * [slot * cap + k] describes the k-th listed neighbour body of the body in
 * slot `slot`.  out[30] (NULL skipped): pair energy, force x, y, separation x,
 * y, overlap (distance - radius sum), radius sum, separation angle, angle i,
 * angle j, friction coefficient, summed vertex overlap, pair Hessian xx, xy,
 * xt, yx, yy, yt, tx, ty, tt, self Hessian in the same order; ids: static
 * body indices and the count of this body's vertices touching the other body.
 * Returns cap (entries = n_bodies * cap). */
static const double k_pair_fill_b[30] = {-1, 0, 0, -1, -1, -1, -1, -1, -1, -1, -1, 0,
                                         0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};

int64_t orcb_pair_dump(orcb_sys *s, double **out, int64_t *this_id, int64_t *other_id,
                       int64_t *vcount) {
    const int64_t cap = s->cap, m = s->nb * cap;
    if (!out) return cap;
    for (int k = 0; k < 30; k++)
        if (out[k]) for (int64_t q = 0; q < m; q++) out[k][q] = k_pair_fill_b[k];
    for (int64_t q = 0; q < m; q++) { this_id[q] = -1; other_id[q] = -1; vcount[q] = -1; }
    const double rs = s->rv * 2.0;
#pragma omp parallel for schedule(static) if (s->nb >= PAR_MIN)
    for (int64_t b = 0; b < s->nb; b++) {
        if (s->ncount[b] == 0) continue;
        const double cx = s->x[b], cy = s->y[b], thi = s->th[b], rad = s->r[b];
        for (int64_t k = 0; k < s->ncount[b]; k++) {
            int64_t ob = s->nlist[b * cap + k];
            if (ob == -1 || ob == b) continue;
            const double ox = s->x[ob], oy = s->y[ob], thj = s->th[ob], orad = s->r[ob];
            double fx = 0.0, fy = 0.0, en = 0.0, vov = 0.0;
            int64_t vci = 0;
            double hij[9] = {0}, hii[9] = {0};
            for (int64_t u = 0; u < s->nvb[b]; u++) {
                const int64_t v = s->start[b] + u;
                const double qx = s->px[v], qy = s->py[v];
                const double phu = (double)(u * 2) * PI_REF / (double)s->nvb[b];
                const double rdx = qx - cx, rdy = qy - cy;
                const double Ri = sqrt(rdx * rdx + rdy * rdy);
                int contact = 0;
                for (int64_t t = 0; t < s->vncount[v]; t++) {
                    const int64_t w = s->vnlist[v * s->vcap + t];
                    if (w == -1 || w == v || s->vbody[w] != ob) continue;
                    const double wx = s->px[w], wy = s->py[w];
                    const int64_t iv = w - s->start[ob];
                    const double phv = (double)(iv * 2) * PI_REF / (double)s->nvb[ob];
                    const double odx = wx - ox, ody = wy - oy;
                    const double Rj = sqrt(odx * odx + ody * ody);
                    double tfx, tfy;
                    const double te = vpair(s, qx, qy, wx, wy, &tfx, &tfy);
                    en += te;
                    fx += tfx;
                    fy += tfy;
                    if (te > 0.0) {
                        contact = 1;
                        const double dx = bpbc(qx, wx, s->box[0]), dy = bpbc(qy, wy, s->box[1]);
                        vov += rs - sqrt(dx * dx + dy * dy);
                        const double dist = sqrt(dx * dx + dy * dy);
                        const double tij = -s->e_c / rs * (1 - dist / rs);
                        const double cij = s->e_c / (rs * rs);
                        const double si = sin(thi + phu), ci = cos(thi + phu);
                        const double sj = sin(thj + phv), cj = cos(thj + phv);
                        for (int a = 0; a < 3; a++) {
                            for (int c = 0; c < 3; c++) {
                                const double dia_x = (double)(a == 0) - Ri * si * (double)(a == 2);
                                const double dia_y = (double)(a == 1) + Ri * ci * (double)(a == 2);
                                const double djb_x = -1.0 * ((double)(c == 0) - Rj * sj * (double)(c == 2));
                                const double djb_y = -1.0 * ((double)(c == 1) + Rj * cj * (double)(c == 2));
                                const double qia = dx * dia_x + dy * dia_y;
                                const double qjb = dx * djb_x + dy * djb_y;
                                const double dqjb = (dia_x * djb_x + dia_y * djb_y) / dist;
                                hij[a * 3 + c] += cij * qia * qjb / (dist * dist) +
                                                  tij * (dqjb - qia * qjb / (dist * dist * dist));
                                const double dib_x = (double)(c == 0) - Ri * si * (double)(c == 2);
                                const double dib_y = (double)(c == 1) + Ri * ci * (double)(c == 2);
                                const double d2x = -Ri * ci * (double)(a == 2) * (double)(c == 2);
                                const double d2y = -Ri * si * (double)(a == 2) * (double)(c == 2);
                                const double qib = dx * dib_x + dy * dib_y;
                                const double dqib = (dia_x * dib_x + dx * d2x + dia_y * dib_y + dy * d2y) / dist;
                                hii[a * 3 + c] += cij * qia * qib / (dist * dist) +
                                                  tij * (dqib - qia * qib / (dist * dist * dist));
                            }
                        }
                    }
                }
                if (contact) vci++;
            }
            const int64_t q = b * cap + k;
            const double xd = bpbc(cx, ox, s->box[0]), yd = bpbc(cy, oy, s->box[1]);
            const double dist = sqrt(xd * xd + yd * yd);
            double fric = 0.0;
            if (fx != 0.0 || fy != 0.0) {
                const double nfx = fx * xd / dist, nfy = fy * yd / dist;
                const double nf = sqrt(nfx * nfx + nfy * nfy);
                const double tfx = fx - nfx, tfy = fy - nfy;
                fric = sqrt(tfx * tfx + tfy * tfy) / nf;
            }
            const double vals[12] = {en, fx, fy, xd, yd, dist - (rad + orad), rad + orad,
                                     atan2(yd, xd), thi, thj, fric, vov};
            for (int e = 0; e < 12; e++) if (out[e]) out[e][q] = vals[e];
            for (int e = 0; e < 9; e++) {
                if (out[12 + e]) out[12 + e][q] += hij[e];
                if (out[21 + e]) out[21 + e][q] += hii[e];
            }
            this_id[q] = s->sidx[b];
            other_id[q] = s->sidx[ob];
            vcount[q] = vci;
        }
    }
    return cap;
}

/* ---------------- setLastState / revertToLastState ------------------------- */
/* RigidBumpy::setLastState (rigid_bumpy.cu:1144-1166 over particle.cu:956-973) */
void orcb_save_state(orcb_sys *s) {
    const size_t B = (size_t)s->nb * sizeof(double), L = (size_t)s->nb * sizeof(int64_t);
    const size_t VB = (size_t)s->nv * sizeof(double), VL = (size_t)s->nv * sizeof(int64_t);
    memcpy(s->s_x, s->x, B); memcpy(s->s_y, s->y, B); memcpy(s->s_vx, s->vx, B);
    memcpy(s->s_vy, s->vy, B); memcpy(s->s_fx, s->fx, B); memcpy(s->s_fy, s->fy, B);
    memcpy(s->s_r, s->r, B); memcpy(s->s_m, s->m, B); memcpy(s->s_th, s->th, B);
    memcpy(s->s_w, s->w, B); memcpy(s->s_tq, s->tq, B);
    memcpy(s->s_pidx, s->pidx, L); memcpy(s->s_sidx, s->sidx, L);
    memcpy(s->s_nvb, s->nvb, L); memcpy(s->s_start, s->start, L);
    memcpy(s->s_px, s->px, VB); memcpy(s->s_py, s->py, VB);
    memcpy(s->s_vbody, s->vbody, VL); memcpy(s->s_svidx, s->svidx, VL);
    s->s_box[0] = s->box[0]; s->s_box[1] = s->box[1];
}

/* RigidBumpy::revertToLastStateVariables + Particle::revertToLastState
 * (rigid_bumpy.cu:1168-1179, particle.cu:975-991): the saved arrays go back
 * slot by slot; moments of inertia, vertex masses, Adam moments and the cell
 * arrays stay as they are; then the box and updateNeighborList (body list
 * from the current cell arrays, then the vertex list) */
void orcb_restore_state(orcb_sys *s) {
    const size_t B = (size_t)s->nb * sizeof(double), L = (size_t)s->nb * sizeof(int64_t);
    const size_t VB = (size_t)s->nv * sizeof(double), VL = (size_t)s->nv * sizeof(int64_t);
    memcpy(s->x, s->s_x, B); memcpy(s->y, s->s_y, B); memcpy(s->vx, s->s_vx, B);
    memcpy(s->vy, s->s_vy, B); memcpy(s->fx, s->s_fx, B); memcpy(s->fy, s->s_fy, B);
    memcpy(s->r, s->s_r, B); memcpy(s->m, s->s_m, B); memcpy(s->th, s->s_th, B);
    memcpy(s->w, s->s_w, B); memcpy(s->tq, s->s_tq, B);
    memcpy(s->pidx, s->s_pidx, L); memcpy(s->sidx, s->s_sidx, L);
    memcpy(s->nvb, s->s_nvb, L); memcpy(s->start, s->s_start, L);
    memcpy(s->px, s->s_px, VB); memcpy(s->py, s->s_py, VB);
    memcpy(s->vbody, s->s_vbody, VL); memcpy(s->svidx, s->s_svidx, VL);
    s->box[0] = s->s_box[0]; s->box[1] = s->s_box[1];
    update_body_list(s, s->method == ORC_NEIGH_CELL);
}

void orcb_get_box(const orcb_sys *s, double *bx, double *by) {
    if (bx) *bx = s->box[0];
    if (by) *by = s->box[1];
}

/* ---------------- state access -------------------------------------------- */
void orcb_get_bodies(const orcb_sys *s, double *x, double *y, double *th, double *vx, double *vy,
                     double *w, double *fx, double *fy, double *tq, double *pe, double *I) {
    for (int64_t b = 0; b < s->nb; b++) {
        int64_t k = s->sidx[b];
        if (x) x[k] = s->x[b];
        if (y) y[k] = s->y[b];
        if (th) th[k] = s->th[b];
        if (vx) vx[k] = s->vx[b];
        if (vy) vy[k] = s->vy[b];
        if (w) w[k] = s->w[b];
        if (fx) fx[k] = s->fx[b];
        if (fy) fy[k] = s->fy[b];
        if (tq) tq[k] = s->tq[b];
        if (pe) pe[k] = s->pe[b];
        if (I) I[k] = s->I[b];
    }
}

void orcb_get_vertices(const orcb_sys *s, double *px, double *py) {
    for (int64_t v = 0; v < s->nv; v++) {
        int64_t k = s->svidx[v];
        if (px) px[k] = s->px[v];
        if (py) py[k] = s->py[v];
    }
}

/* vertex neighbour lists keyed by static vertex index: list[nv * cap] (static
 * vertex indices, -1 padded), counts[nv]; returns cap */
int64_t orcb_get_vertex_neighbors(const orcb_sys *s, int64_t *list, int64_t *counts) {
    if (list && counts) {
        for (int64_t v = 0; v < s->nv; v++) {
            int64_t k = s->svidx[v];
            counts[k] = s->vncount[v];
            for (int64_t t = 0; t < s->vcap; t++) {
                int64_t u = (t < s->vncount[v]) ? s->vnlist[v * s->vcap + t] : -1;
                list[k * s->vcap + t] = u >= 0 ? s->svidx[u] : -1;
            }
        }
    }
    return s->vcap;
}

void orcb_neighbor_info(const orcb_sys *s, int *method, double *cutoff, double *vcutoff,
                        double *thr2, int64_t *cap, int64_t *vcap, int64_t *n_rebuilds,
                        int64_t *n_cell_rebuilds) {
    if (method) *method = s->method;
    if (cutoff) *cutoff = s->cutoff;
    if (vcutoff) *vcutoff = s->vcutoff;
    if (thr2) *thr2 = s->nthr2;
    if (cap) *cap = s->cap;
    if (vcap) *vcap = s->vcap;
    if (n_rebuilds) *n_rebuilds = s->n_rebuilds;
    if (n_cell_rebuilds) *n_cell_rebuilds = s->n_cell_rebuilds;
}

/* vertex radius rule (calculateVertexRadius, rigid_bumpy.cu:570-580) */
double orcb_vertex_radius(double min_diameter, int64_t n_vertices_small, double seg) {
    double ang = 2 * PI_REF / n_vertices_small;
    return min_diameter / (1 + seg / sin(ang / 2)) / 2.0;
}
