/*
 * ref_bumpy_driver.cpp -- drives the reference's OWN rigid-bumpy kernel
 * sources (src/particles/rigid_bumpy/kernels.cu + base kernels, compiled as
 * host C++ through shim/) to pin the bumpy oracle (oracle/dpg_oracle_bumpy.c).
 * TEST INFRASTRUCTURE ONLY.
 *
 * Host sequences restated from src/particles/rigid_bumpy/rigid_bumpy.cu:
 * initializeFromConfig pieces (setParticleStartIndex, setVertexParticleIndex,
 * setVertexPositions, setMass), setNeighborSize / initCellList /
 * updateCellNeighborList / updateVertexVerletList / reorderParticleData,
 * calculateForces, updatePositions, updateVelocities, getPowerFire,
 * mixVelocitiesAndForces, and the base Fire / NVE / minimizeFire sequences.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

#include "cuda_host_shim.h"
#include "particles/base/kernels.cuh"
#include "particles/rigid_bumpy/kernels.cuh"

typedef std::vector<double> dvec;
typedef std::vector<long> lvec;

template <class F>
static void launchb(long n, F &&f) {
#pragma omp parallel for schedule(static) if (n >= 2048)
    for (long i = 0; i < n; i++) {
        blockIdx = {(unsigned)i, 0, 0};
        threadIdx = {0, 0, 0};
        blockDim = {1, 1, 1};
        f();
    }
}

struct refb_sys {
    long nb, nv;
    double box[2], e_c, n_c, rv, seg;
    bool rotation;
    dvec x, y, th, vx, vy, w, fx, fy, tq, pe, m, r, I, ke, lpx, lpy, dx, dy, dth;
    dvec tx, ty, tth, tvx, tvy, tw, tfx, tfy, ttq, tm, tr, tI;
    lvec nvb, start, tnvb, tstart, o2n;
    dvec px, py, vfx, vfy, vtq, vpe, vm, tpx, tpy, tvm;
    lvec vbody, svidx, tvbody, tsvidx;
    dvec lnx, lny, lcx, lcy, nd2, cd2;
    lvec cell_index, pidx, sidx, cell_start, nlist, ncount, vnlist, vncount;
    long cap = 4, vcap = 4, ncd = -1, ncells = -1;
    int method = -1;
    double cutoff = -1, vcutoff = -1, vpcutoff = -1, nthr2 = -1, cs = -1, cthr2 = -1;
    long n_rebuilds = 0, n_cell_rebuilds = 0;
    double f_alpha, f_alpha0, f_dt, f_dtmax, f_dtmin;
    long f_ngood = 0, f_nbad = 0;
    int f_stopped = 0;
    // Adam moments (first_moment / second_moment and their swap twins, the angular ones)
    dvec m1x, m1y, m2x, m2y, tm1x, tm1y, tm2x, tm2y, m1a, m2a;
    dvec sxx, sxy, syx, syy;
    lvec cc, vcc;
    // setLastState copies
    dvec s_x, s_y, s_vx, s_vy, s_fx, s_fy, s_r, s_m, s_th, s_w, s_tq, s_px, s_py;
    lvec s_pidx, s_sidx, s_nvb, s_start, s_vbody, s_svidx;
    double s_box[2] = {0, 0};
};

static void bsync(refb_sys *s) {
    d_n_particles = s->nb;
    d_n_vertices = s->nv;
    d_box_size[0] = s->box[0];
    d_box_size[1] = s->box[1];
    d_e_c = s->e_c;
    d_n_c = s->n_c;
    d_num_neighbors_ptr = s->ncount.data();
    d_neighbor_list_ptr = s->nlist.data();
    d_max_neighbors_allocated = s->cap;
    d_n_cells = s->ncells;
    d_n_cells_dim = s->ncd;
    d_cell_size = s->cs;
    d_vertex_radius = s->rv;
    d_num_vertex_neighbors_ptr = s->vncount.data();
    d_vertex_neighbor_list_ptr = s->vnlist.data();
    d_max_vertex_neighbors_allocated = s->vcap;
    d_particle_start_index_ptr = s->start.data();
    d_num_vertices_in_particle_ptr = s->nvb.data();
    d_vertex_particle_index_ptr = s->vbody.data();
}

static double bmaxd(refb_sys *s) { return 2.0 * *std::max_element(s->r.begin(), s->r.end()); }

extern "C" {

refb_sys *refb_create(int64_t nb, int64_t nv, double bx, double by, double e_c, double n_c,
                      double rv, double seg, int rotation) {
    refb_sys *s = new refb_sys();
    s->nb = nb; s->nv = nv; s->box[0] = bx; s->box[1] = by; s->e_c = e_c; s->n_c = n_c;
    s->rv = rv; s->seg = seg; s->rotation = rotation != 0;
    dvec *bd[] = {&s->x, &s->y, &s->th, &s->vx, &s->vy, &s->w, &s->fx, &s->fy, &s->tq, &s->pe,
                  &s->m, &s->r, &s->I, &s->ke, &s->lpx, &s->lpy, &s->dx, &s->dy, &s->dth, &s->tx,
                  &s->ty, &s->tth, &s->tvx, &s->tvy, &s->tw, &s->tfx, &s->tfy, &s->ttq, &s->tm,
                  &s->tr, &s->tI, &s->lnx, &s->lny, &s->lcx, &s->lcy, &s->nd2, &s->cd2,
                  &s->m1x, &s->m1y, &s->m2x, &s->m2y, &s->tm1x, &s->tm1y, &s->tm2x, &s->tm2y,
                  &s->m1a, &s->m2a, &s->sxx, &s->sxy, &s->syx, &s->syy};
    for (dvec *d : bd) d->assign(nb, 0.0);
    lvec *bl[] = {&s->nvb, &s->start, &s->tnvb, &s->tstart, &s->o2n, &s->cell_index, &s->pidx,
                  &s->sidx, &s->ncount, &s->cc, &s->vcc};
    for (lvec *l : bl) l->assign(nb, 0);
    dvec *vd[] = {&s->px, &s->py, &s->vfx, &s->vfy, &s->vtq, &s->vpe, &s->vm, &s->tpx, &s->tpy, &s->tvm};
    for (dvec *d : vd) d->assign(nv, 0.0);
    lvec *vl[] = {&s->vbody, &s->svidx, &s->tvbody, &s->tsvidx, &s->vncount};
    for (lvec *l : vl) l->assign(nv, 0);
    std::iota(s->pidx.begin(), s->pidx.end(), 0L);
    std::iota(s->sidx.begin(), s->sidx.end(), 0L);
    std::iota(s->svidx.begin(), s->svidx.end(), 0L);
    s->nlist.assign(nb * 4, -1);
    s->vnlist.assign(nv * 4, -1);
    s->cell_start.assign(1, 0);
    return s;
}

void refb_destroy(refb_sys *s) { delete s; }

int refb_set_bodies(refb_sys *s, const double *x, const double *y, const double *th,
                    const double *vx, const double *vy, const double *w, const double *r,
                    const int64_t *nvb) {
    long tot = 0;
    for (long b = 0; b < s->nb; b++) tot += nvb[b];
    if (tot != s->nv) return -1;
    for (long b = 0; b < s->nb; b++) {
        s->x[b] = x[b]; s->y[b] = y[b]; s->th[b] = th ? th[b] : 0.0;
        s->vx[b] = vx ? vx[b] : 0.0; s->vy[b] = vy ? vy[b] : 0.0; s->w[b] = w ? w[b] : 0.0;
        s->r[b] = r[b]; s->nvb[b] = nvb[b];
    }
    /* setParticleStartIndex (exclusive scan) + kernelSetVertexParticleIndex */
    std::exclusive_scan(s->nvb.begin(), s->nvb.end(), s->start.begin(), 0L);
    bsync(s);
    launchb(s->nb, [&] { kernelSetVertexParticleIndex(s->nvb.data(), s->start.data(), s->vbody.data()); });
    return 0;
}

void refb_init_vertices(refb_sys *s) {
    bsync(s);
    launchb(s->nb, [&] {
        kernelInitializeVerticesOnParticles(s->x.data(), s->y.data(), s->r.data(), s->th.data(),
                                            s->start.data(), s->nvb.data(), s->px.data(), s->py.data());
    });
}

void refb_set_vertices(refb_sys *s, const double *px, const double *py) {
    for (long v = 0; v < s->nv; v++) { s->px[v] = px[s->svidx[v]]; s->py[v] = py[s->svidx[v]]; }
}

void refb_set_mass(refb_sys *s, double mass) {
    std::fill(s->m.begin(), s->m.end(), mass);
    bsync(s);
    launchb(s->nv, [&] { kernelGetVertexMasses(s->r.data(), s->vm.data(), s->m.data()); });
    launchb(s->nb, [&] {
        kernelGetMomentsOfInertia(s->x.data(), s->y.data(), s->px.data(), s->py.data(), s->vm.data(),
                                  s->I.data());
    });
}

static bool set_neighbor_size(refb_sys *s, double cm, double dm) {
    s->cap = 4; s->vcap = 4;
    s->cutoff = cm * bmaxd(s);
    s->vcutoff = cm * 2.0 * s->rv;
    s->vpcutoff = bmaxd(s);
    s->nthr2 = std::pow(dm * s->seg * s->rv, 2);
    double diag = std::sqrt(s->box[0] * s->box[0] + s->box[1] * s->box[1]);
    return s->cutoff < diag;
}

static bool set_cell_size(refb_sys *s, double ppc, double cdm) {
    long min_dim = 4;
    double density = s->nb / (1.0 * s->box[0] * s->box[1]);
    double trial = std::sqrt(ppc / density);
    double min_cs = 2.0 * bmaxd(s);
    s->ncd = (long)std::floor(s->box[0] / trial);
    s->ncells = s->ncd * s->ncd;
    if (s->ncd < min_dim) { s->ncd = min_dim; s->ncells = s->ncd * s->ncd; }
    s->cs = s->box[0] / s->ncd;
    if (s->cs < min_cs) {
        s->cs = min_cs;
        s->ncd = (long)std::floor(s->box[0] / s->cs);
        s->ncells = s->ncd * s->ncd;
        if (s->ncd < min_dim) return false;
    }
    s->cthr2 = std::pow(cdm * s->cs, 2);
    return true;
}

static void set_method(refb_sys *s, int m) {
    s->method = m;
    std::iota(s->pidx.begin(), s->pidx.end(), 0L);
    std::iota(s->sidx.begin(), s->sidx.end(), 0L);
    if (m == 2) {
        double diag = std::sqrt(s->box[0] * s->box[0] + s->box[1] * s->box[1]);
        set_neighbor_size(s, 2.0 * diag / bmaxd(s), 0.0);
    }
}

static long maxl(const lvec &a) {
    long m = -1;
    for (long v : a) m = std::max(m, v);
    return m;
}

static void vertex_kernel(refb_sys *s) {
    bsync(s);
    launchb(s->nv, [&] {
        kernelUpdateVertexNeighborList(s->px.data(), s->py.data(), s->x.data(), s->y.data(),
                                       s->vcutoff, s->vpcutoff);
    });
}

static void update_vertex_list(refb_sys *s) {
    std::fill(s->vnlist.begin(), s->vnlist.end(), -1L);
    vertex_kernel(s);
    long mx = maxl(s->vncount);
    if (mx > s->vcap) {
        s->vcap = (long)std::pow(2, std::ceil(std::log2(mx)));
        s->vnlist.assign(s->nv * s->vcap, -1);
        vertex_kernel(s);
    }
}

static void body_kernel(refb_sys *s, bool cells) {
    bsync(s);
    if (cells)
        launchb(s->nb, [&] {
            kernelUpdateCellNeighborList(s->x.data(), s->y.data(), s->lnx.data(), s->lny.data(),
                                         s->cutoff, s->cell_index.data(), s->cell_start.data(),
                                         s->nd2.data());
        });
    else
        launchb(s->nb, [&] {
            kernelUpdateNeighborList(s->x.data(), s->y.data(), s->lnx.data(), s->lny.data(),
                                     s->nd2.data(), s->cutoff);
        });
}

static void update_body_list(refb_sys *s, bool cells) {
    std::fill(s->nlist.begin(), s->nlist.end(), -1L);
    body_kernel(s, cells);
    long mx = maxl(s->ncount);
    if (mx > s->cap) {
        s->cap = (long)std::pow(2, std::ceil(std::log2(mx)));
        s->nlist.assign(s->nb * s->cap, -1);
        body_kernel(s, cells);
    }
    s->n_rebuilds++;
    update_vertex_list(s);
}

static void update_cell_list(refb_sys *s) {
    s->cell_start[s->ncells] = s->nb;
    bsync(s);
    launchb(s->nb, [&] { kernelGetCellIndexForParticle(s->x.data(), s->y.data(), s->cell_index.data(), s->pidx.data()); });
    std::vector<long> order(s->nb);
    std::iota(order.begin(), order.end(), 0L);
    std::stable_sort(order.begin(), order.end(),
                     [&](long a, long b) { return s->cell_index[a] < s->cell_index[b]; });
    lvec ci(s->nb), pi(s->nb), si(s->nb);
    for (long k = 0; k < s->nb; k++) {
        ci[k] = s->cell_index[order[k]]; pi[k] = s->pidx[order[k]]; si[k] = s->sidx[order[k]];
    }
    s->cell_index = ci; s->pidx = pi; s->sidx = si;
    launchb(s->nb, [&] {
        kernelReorderRigidBumpyParticleData(
            s->pidx.data(), s->o2n.data(), s->nvb.data(), s->tnvb.data(), s->x.data(), s->y.data(),
            s->tx.data(), s->ty.data(), s->fx.data(), s->fy.data(), s->tfx.data(), s->tfy.data(),
            s->vx.data(), s->vy.data(), s->tvx.data(), s->tvy.data(), s->w.data(), s->tq.data(),
            s->tw.data(), s->ttq.data(), s->th.data(), s->tth.data(), s->m.data(), s->r.data(),
            s->tm.data(), s->tr.data(), s->I.data(), s->tI.data(), s->lcx.data(), s->lcy.data(),
            s->cd2.data());
    });
    std::exclusive_scan(s->tnvb.begin(), s->tnvb.end(), s->tstart.begin(), 0L);
    launchb(s->nv, [&] {
        kernelReorderRigidBumpyVertexData(s->vbody.data(), s->tvbody.data(), s->o2n.data(),
                                          s->start.data(), s->tstart.data(), s->px.data(),
                                          s->py.data(), s->tpx.data(), s->tpy.data(), s->vm.data(),
                                          s->tvm.data(), s->svidx.data(), s->tsvidx.data());
    });
    std::swap(s->x, s->tx); std::swap(s->y, s->ty); std::swap(s->fx, s->tfx); std::swap(s->fy, s->tfy);
    std::swap(s->vx, s->tvx); std::swap(s->vy, s->tvy); std::swap(s->w, s->tw); std::swap(s->th, s->tth);
    std::swap(s->tq, s->ttq); std::swap(s->m, s->tm); std::swap(s->r, s->tr); std::swap(s->I, s->tI);
    std::swap(s->nvb, s->tnvb); std::swap(s->start, s->tstart);
    std::swap(s->px, s->tpx); std::swap(s->py, s->tpy); std::swap(s->vm, s->tvm);
    std::swap(s->vbody, s->tvbody); std::swap(s->svidx, s->tsvidx);
    // first_moment.swap(); second_moment.swap() (rigid_bumpy.cu:1370-1371), no gather
    std::swap(s->m1x, s->tm1x); std::swap(s->m1y, s->tm1y);
    std::swap(s->m2x, s->tm2x); std::swap(s->m2y, s->tm2y);
    bsync(s);
    long width = s->ncells > 0 ? s->nb / s->ncells : 0;
    launchb(s->ncells, [&] { kernelGetFirstParticleIndexForCell(s->cell_index.data(), s->cell_start.data(), 2, width); });
    s->n_cell_rebuilds++;
}

void refb_calculate_forces(refb_sys *s);

int refb_setup_neighbors(refb_sys *s, int method, double cm, double dm, double ppc, double cdm) {
    set_method(s, method);
    set_neighbor_size(s, cm, dm);
    if (s->method == 0) {
        if (!set_cell_size(s, ppc, cdm)) set_method(s, 1);
        if (!set_neighbor_size(s, cm, dm)) set_method(s, 2);
    }
    if (s->method == 1) {
        if (!set_neighbor_size(s, cm, dm)) set_method(s, 2);
    }
    if (s->method == 2) s->cap = s->nb - 1;
    s->nlist.assign(s->nb * s->cap, -1);
    std::fill(s->ncount.begin(), s->ncount.end(), 0L);
    dvec *ds[] = {&s->lnx, &s->lny, &s->nd2, &s->lcx, &s->lcy, &s->cd2};
    for (dvec *d : ds) std::fill(d->begin(), d->end(), 0.0);
    s->vnlist.assign(s->nv * s->vcap, -1);
    std::fill(s->vncount.begin(), s->vncount.end(), 0L);
    if (s->method == 0) {
        std::fill(s->cell_index.begin(), s->cell_index.end(), -1L);
        s->cell_start.assign(s->ncells + 1, 0);
        std::iota(s->pidx.begin(), s->pidx.end(), 0L);
        std::iota(s->sidx.begin(), s->sidx.end(), 0L);
        std::iota(s->svidx.begin(), s->svidx.end(), 0L);
        update_cell_list(s);
        update_body_list(s, true);
    } else {
        if (s->method == 2) {
            s->cutoff = 10.0 * std::sqrt(s->box[0] * s->box[0] + s->box[1] * s->box[1]);
            s->nthr2 = s->cutoff * s->cutoff;
        }
        update_body_list(s, false);
    }
    refb_calculate_forces(s);
    return s->method;
}

int refb_check_for_neighbor_update(refb_sys *s) {
    const double tol = 3.0;
    double mn = 0, mc = 0;
    for (long b = 0; b < s->nb; b++) { mn = std::max(mn, s->nd2[b]); mc = std::max(mc, s->cd2[b]); }
    if (s->method == 2) return 0;
    if (s->method == 1) {
        if (tol * mn > s->nthr2) { update_body_list(s, false); return 1; }
        return 0;
    }
    if (tol * mc > s->cthr2) { update_cell_list(s); update_body_list(s, true); return 2; }
    if (tol * mn > s->nthr2) { update_body_list(s, true); return 1; }
    return 0;
}

void refb_zero(refb_sys *s) {
    bsync(s);
    launchb(s->nb, [&] { kernelZeroRigidBumpyParticleForceAndPotentialEnergy(s->fx.data(), s->fy.data(), s->tq.data(), s->pe.data()); });
    launchb(s->nv, [&] { kernelZeroRigidBumpyVertexForceAndPotentialEnergy(s->vfx.data(), s->vfy.data(), s->vtq.data(), s->vpe.data()); });
}

void refb_calculate_forces(refb_sys *s) {
    bsync(s);
    launchb(s->nv, [&] {
        kernelCalcRigidBumpyForces1(s->x.data(), s->y.data(), s->px.data(), s->py.data(),
                                    s->vfx.data(), s->vfy.data(), s->vtq.data(), s->vpe.data());
    });
    launchb(s->nb, [&] {
        kernelCalcRigidBumpyParticleForces1(s->vfx.data(), s->vfy.data(), s->vtq.data(), s->vpe.data(),
                                            s->fx.data(), s->fy.data(), s->tq.data(), s->pe.data());
    });
}

void refb_update_velocities(refb_sys *s, double dt) {
    bsync(s);
    launchb(s->nb, [&] {
        kernelUpdateRigidVelocities(s->vx.data(), s->vy.data(), s->w.data(), s->fx.data(), s->fy.data(),
                                    s->tq.data(), s->m.data(), s->I.data(), dt, s->rotation);
    });
}

void refb_update_positions(refb_sys *s, double dt) {
    bsync(s);
    launchb(s->nb, [&] {
        kernelUpdateRigidPositions(s->lpx.data(), s->lpy.data(), s->x.data(), s->y.data(), s->th.data(),
                                   s->dx.data(), s->dy.data(), s->dth.data(), s->lnx.data(), s->lny.data(),
                                   s->lcx.data(), s->lcy.data(), s->nd2.data(), s->cd2.data(),
                                   s->vx.data(), s->vy.data(), s->w.data(), dt);
    });
    launchb(s->nv, [&] {
        kernelTranslateAndRotateVertices1(s->lpx.data(), s->lpy.data(), s->x.data(), s->y.data(),
                                          s->px.data(), s->py.data(), s->dx.data(), s->dy.data(),
                                          s->dth.data());
    });
}

void refb_mix(refb_sys *s, double alpha) {
    bsync(s);
    launchb(s->nb, [&] {
        kernelMixRigidVelocitiesAndForces(s->vx.data(), s->vy.data(), s->w.data(), s->fx.data(),
                                          s->fy.data(), s->tq.data(), alpha);
    });
}

void refb_set_velocities_zero(refb_sys *s) {
    std::fill(s->vx.begin(), s->vx.end(), 0.0);
    std::fill(s->vy.begin(), s->vy.end(), 0.0);
    std::fill(s->w.begin(), s->w.end(), 0.0);
}

double refb_power_fire(refb_sys *s) {
    double px = 0, py = 0, pr = 0;
    for (long b = 0; b < s->nb; b++) px += s->fx[b] * s->vx[b];
    for (long b = 0; b < s->nb; b++) py += s->fy[b] * s->vy[b];
    for (long b = 0; b < s->nb; b++) pr += s->tq[b] * s->w[b];
    return (px + py) + pr;
}

double refb_total_pe(refb_sys *s) {
    double e = 0;
    for (double v : s->pe) e += v;
    return e;
}

double refb_total_ke(refb_sys *s) {
    bsync(s);
    if (s->rotation)
        launchb(s->nb, [&] {
            kernelCalculateTranslationalAndRotationalKineticEnergy(s->vx.data(), s->vy.data(), s->m.data(),
                                                                   s->w.data(), s->I.data(), s->ke.data());
        });
    else
        launchb(s->nb, [&] { kernelCalculateTranslationalKineticEnergy(s->vx.data(), s->vy.data(), s->m.data(), s->ke.data()); });
    double e = 0;
    for (double v : s->ke) e += v;
    return e;
}

void refb_nve_steps(refb_sys *s, double dt, int64_t n) {
    for (int64_t t = 0; t < n; t++) {
        refb_update_velocities(s, 0.5 * dt);
        refb_update_positions(s, dt);
        refb_check_for_neighbor_update(s);
        refb_zero(s);
        refb_calculate_forces(s);
        refb_update_velocities(s, 0.5 * dt);
    }
}

void refb_fire_init(refb_sys *s, double alpha_init, double dt) {
    s->f_alpha = alpha_init; s->f_alpha0 = alpha_init; s->f_dt = dt;
    s->f_dtmax = 10.0 * dt; s->f_dtmin = 0.001 * dt;
    s->f_ngood = 0; s->f_nbad = 0; s->f_stopped = 0;
}

int refb_fire_step(refb_sys *s) {
    double power = refb_power_fire(s);
    if (power > 0) {
        s->f_ngood++;
        s->f_nbad = 0;
        if (s->f_ngood > 5) { s->f_dt = std::min(s->f_dt * 1.1, s->f_dtmax); s->f_alpha *= 0.99; }
    } else {
        s->f_ngood = 0;
        s->f_nbad++;
        if (s->f_nbad > 10) { s->f_stopped = 1; return 1; }
        s->f_dt = std::max(s->f_dt * 0.5, s->f_dtmin);
        s->f_alpha = s->f_alpha0;
        refb_update_positions(s, -s->f_dt / 2.0);
        refb_set_velocities_zero(s);
    }
    refb_update_velocities(s, s->f_dt / 2.0);
    refb_mix(s, s->f_alpha);
    refb_update_positions(s, s->f_dt);
    refb_zero(s);
    refb_check_for_neighbor_update(s);
    refb_calculate_forces(s);
    refb_update_velocities(s, s->f_dt / 2.0);
    return 0;
}

void refb_get_bodies(refb_sys *s, double *x, double *y, double *th, double *vx, double *vy, double *w,
                     double *fx, double *fy, double *tq, double *pe, double *I) {
    for (long b = 0; b < s->nb; b++) {
        long k = s->sidx[b];
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

void refb_get_vertices(refb_sys *s, double *px, double *py) {
    for (long v = 0; v < s->nv; v++) {
        long k = s->svidx[v];
        if (px) px[k] = s->px[v];
        if (py) py[k] = s->py[v];
    }
}

int64_t refb_get_vertex_neighbors(refb_sys *s, int64_t *list, int64_t *counts) {
    if (list && counts) {
        for (long v = 0; v < s->nv; v++) {
            long k = s->svidx[v];
            counts[k] = s->vncount[v];
            for (long t = 0; t < s->vcap; t++) {
                long u = (t < s->vncount[v]) ? s->vnlist[v * s->vcap + t] : -1;
                list[k * s->vcap + t] = u >= 0 ? s->svidx[u] : -1;
            }
        }
    }
    return s->vcap;
}

// ---- Adam: RigidBumpy::initAdamVariables / updatePositionsAdam (rigid_bumpy.cu:1461-1486)
void refb_adam_init(refb_sys *s) {
    dvec *m[] = {&s->m1x, &s->m1y, &s->m2x, &s->m2y, &s->tm1x, &s->tm1y, &s->tm2x, &s->tm2y, &s->m1a, &s->m2a};
    for (dvec *d : m) std::fill(d->begin(), d->end(), 0.0);
}

void refb_adam_step(refb_sys *s, int64_t step, double alpha, double b1, double b2, double eps) {
    double c1 = 1 - std::pow(b1, step + 1), c2 = 1 - std::pow(b2, step + 1);
    bsync(s);
    launchb(s->nb, [&] {
        kernelRigidBumpyAdamStep(s->lpx.data(), s->lpy.data(), s->m1x.data(), s->m1y.data(), s->m1a.data(),
                                 s->m2x.data(), s->m2y.data(), s->m2a.data(), s->x.data(), s->y.data(),
                                 s->th.data(), s->dx.data(), s->dy.data(), s->dth.data(), s->fx.data(),
                                 s->fy.data(), s->tq.data(), alpha, b1, b2, c1, c2, eps, s->lnx.data(),
                                 s->lny.data(), s->nd2.data(), s->lcx.data(), s->lcy.data(), s->cd2.data(),
                                 s->rotation);
    });
    launchb(s->nv, [&] {
        kernelTranslateAndRotateVertices1(s->lpx.data(), s->lpy.data(), s->x.data(), s->y.data(),
                                          s->px.data(), s->py.data(), s->dx.data(), s->dy.data(),
                                          s->dth.data());
    });
}

// Adam::minimize steps (src/integrator/adam.cu:11-17) without the stop test
void refb_adam_steps(refb_sys *s, double alpha, double b1, double b2, double eps, int64_t n) {
    refb_adam_init(s);
    for (int64_t t = 0; t < n; t++) {
        refb_zero(s);
        refb_check_for_neighbor_update(s);
        refb_calculate_forces(s);
        refb_adam_step(s, t, alpha, b1, b2, eps);
    }
}

// ---- DampedNVE::step (src/integrator/damped_nve.cu:15-25) with RigidBumpy::calculateDampedForces
void refb_damped_nve_steps(refb_sys *s, double dt, double g, int64_t n) {
    for (int64_t t = 0; t < n; t++) {
        refb_update_velocities(s, 0.5 * dt);
        refb_update_positions(s, dt);
        refb_check_for_neighbor_update(s);
        refb_zero(s);
        bsync(s);
        launchb(s->nb, [&] {
            kernelCalculateRigidDampedForces(s->fx.data(), s->fy.data(), s->tq.data(), s->vx.data(),
                                             s->vy.data(), s->w.data(), g);
        });
        refb_calculate_forces(s);
        refb_update_velocities(s, 0.5 * dt);
    }
}

// ---- walls: RigidBumpy::calculateWallForces (rigid_bumpy.cu:1488-1493)
static void wall_kernel(refb_sys *s) {
    bsync(s);
    launchb(s->nv, [&] {
        kernelCalcRigidBumpyWallForces(s->x.data(), s->y.data(), s->px.data(), s->py.data(),
                                       s->vfx.data(), s->vfy.data(), s->vtq.data(), s->vpe.data());
    });
}

// calculateWallForces_onlyWallContacts (rigid_bumpy.cu:1495-1499)
void refb_wall_only(refb_sys *s) {
    wall_kernel(s);
    launchb(s->nb, [&] {
        kernelCalcRigidBumpyParticleForces1(s->vfx.data(), s->vfy.data(), s->vtq.data(), s->vpe.data(),
                                            s->fx.data(), s->fy.data(), s->tq.data(), s->pe.data());
    });
}

// calculateWallForces then calculateForces, as NVE::wall_step calls them
void refb_wall_and_pair_forces(refb_sys *s) {
    wall_kernel(s);
    refb_calculate_forces(s);
}

// NVE::wall_step (src/integrator/nve.cu:27-38)
void refb_nve_wall_steps(refb_sys *s, double dt, int64_t n) {
    for (int64_t t = 0; t < n; t++) {
        refb_update_velocities(s, 0.5 * dt);
        refb_update_positions(s, dt);
        refb_check_for_neighbor_update(s);
        refb_zero(s);
        wall_kernel(s);
        refb_calculate_forces(s);
        refb_update_velocities(s, 0.5 * dt);
    }
}

// ---- calculateStressTensor + getPressure (rigid_bumpy.cu:1513-1519, particle.cu:1371-1376);
// the component sums run in body order here (thrust::reduce in the reference)
void refb_stress(refb_sys *s, double *out) {
    bsync(s);
    launchb(s->nb, [&] {
        kernelCalcRigidBumpyStressTensor(s->x.data(), s->y.data(), s->vx.data(), s->vy.data(), s->w.data(),
                                         s->px.data(), s->py.data(), s->vm.data(), s->sxx.data(),
                                         s->sxy.data(), s->syx.data(), s->syy.data());
    });
    double t[4] = {0, 0, 0, 0};
    for (long b = 0; b < s->nb; b++) { t[0] += s->sxx[b]; t[1] += s->sxy[b]; t[2] += s->syx[b]; t[3] += s->syy[b]; }
    for (int k = 0; k < 4; k++) out[k] = t[k];
}

// ---- countContacts (rigid_bumpy.cu:1505-1511) + getContactCount
double refb_count_contacts(refb_sys *s) {
    std::fill(s->cc.begin(), s->cc.end(), 0L);
    std::fill(s->vcc.begin(), s->vcc.end(), 0L);
    bsync(s);
    launchb(s->nb, [&] {
        kernelCountRigidBumpyContacts(s->x.data(), s->y.data(), s->px.data(), s->py.data(), s->r.data(),
                                      s->cc.data(), s->vcc.data());
    });
    long tot = 0;
    for (long v : s->cc) tot += v;
    return (double)tot;
}

void refb_get_stress(refb_sys *s, double *sxx, double *sxy, double *syx, double *syy) {
    for (long b = 0; b < s->nb; b++) {
        long k = s->sidx[b];
        if (sxx) sxx[k] = s->sxx[b];
        if (sxy) sxy[k] = s->sxy[b];
        if (syx) syx[k] = s->syx[b];
        if (syy) syy[k] = s->syy[b];
    }
}

void refb_get_contacts(refb_sys *s, int64_t *cc, int64_t *vcc) {
    for (long b = 0; b < s->nb; b++) {
        long k = s->sidx[b];
        if (cc) cc[k] = s->cc[b];
        if (vcc) vcc[k] = s->vcc[b];
    }
}

// ---- RigidBumpy::setLastState / revertToLastStateVariables + Particle::revertToLastState
// (rigid_bumpy.cu:1144-1179, particle.cu:956-991)
void refb_save_state(refb_sys *s) {
    s->s_x = s->x; s->s_y = s->y; s->s_vx = s->vx; s->s_vy = s->vy; s->s_fx = s->fx; s->s_fy = s->fy;
    s->s_r = s->r; s->s_m = s->m; s->s_th = s->th; s->s_w = s->w; s->s_tq = s->tq;
    s->s_px = s->px; s->s_py = s->py;
    s->s_pidx = s->pidx; s->s_sidx = s->sidx; s->s_nvb = s->nvb; s->s_start = s->start;
    s->s_vbody = s->vbody; s->s_svidx = s->svidx;
    s->s_box[0] = s->box[0]; s->s_box[1] = s->box[1];
}

void refb_restore_state(refb_sys *s) {
    s->x = s->s_x; s->y = s->s_y; s->vx = s->s_vx; s->vy = s->s_vy; s->fx = s->s_fx; s->fy = s->s_fy;
    s->r = s->s_r; s->m = s->s_m; s->th = s->s_th; s->w = s->s_w; s->tq = s->s_tq;
    s->px = s->s_px; s->py = s->s_py;
    s->pidx = s->s_pidx; s->sidx = s->s_sidx; s->nvb = s->s_nvb; s->start = s->s_start;
    s->vbody = s->s_vbody; s->svidx = s->s_svidx;
    s->box[0] = s->s_box[0]; s->box[1] = s->s_box[1];
    update_body_list(s, s->method == 0);
}

// ---- RigidBumpy::calculateForceDistancePairs (rigid_bumpy.cu:1383-1459): the
// reference's fills, then its kernel; out[30] in the order of orcb_pair_dump
int64_t refb_pair_dump(refb_sys *s, double **out, int64_t *this_id, int64_t *other_id,
                       int64_t *vcount) {
    const long m = s->nb * s->cap;
    if (!out) return s->cap;
    static const double fill[30] = {-1, 0, 0, -1, -1, -1, -1, -1, -1, -1, -1, 0,
                                    0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    std::vector<dvec> a(30);
    for (int k = 0; k < 30; k++) a[k].assign(m, fill[k]);
    lvec ti(m, -1), oi(m, -1), vc(m, -1);
    bsync(s);
    // kernel argument order: potential, force x/y, distance x/y, ids, overlap, radsum,
    // radii, static index, separation angle, angle i/j, vertex contacts, angles,
    // friction, vertex overlaps, pair Hessian xx xy yx yy xt yt tt tx ty, self Hessian same
    launchb(s->nb, [&] {
        kernelCalcRigidBumpyForceDistancePairs(
            s->x.data(), s->y.data(), s->px.data(), s->py.data(), a[0].data(), a[1].data(),
            a[2].data(), a[3].data(), a[4].data(), ti.data(), oi.data(), a[5].data(), a[6].data(),
            s->r.data(), s->sidx.data(), a[7].data(), a[8].data(), a[9].data(), vc.data(),
            s->th.data(), a[10].data(), a[11].data(),
            a[12].data(), a[13].data(), a[15].data(), a[16].data(), a[14].data(), a[17].data(),
            a[20].data(), a[18].data(), a[19].data(),
            a[21].data(), a[22].data(), a[24].data(), a[25].data(), a[23].data(), a[26].data(),
            a[29].data(), a[27].data(), a[28].data());
    });
    for (int k = 0; k < 30; k++)
        if (out[k]) std::copy(a[k].begin(), a[k].end(), out[k]);
    for (long q = 0; q < m; q++) { this_id[q] = ti[q]; other_id[q] = oi[q]; vcount[q] = vc[q]; }
    return s->cap;
}

void refb_neighbor_info(refb_sys *s, int *method, double *cutoff, double *vcutoff, double *thr2,
                        int64_t *cap, int64_t *vcap, int64_t *nr, int64_t *ncr) {
    if (method) *method = s->method;
    if (cutoff) *cutoff = s->cutoff;
    if (vcutoff) *vcutoff = s->vcutoff;
    if (thr2) *thr2 = s->nthr2;
    if (cap) *cap = s->cap;
    if (vcap) *vcap = s->vcap;
    if (nr) *nr = s->n_rebuilds;
    if (ncr) *ncr = s->n_cell_rebuilds;
}

}  // extern "C"
