/*
 * ref_driver.cpp -- drives the reference's OWN kernel sources
 * (src/particles/{base,disk}/kernels.cu of mmccraw98/dpCUDA-v2, compiled as
 * host C++ through shim/cuda_host_shim.h) to pin the oracle.
 * TEST INFRASTRUCTURE ONLY; built by oracle/ref/build_ref.sh into
 * oracle/_ref/ and used by tests/golden/make_golden.py and the CPU tests.
 *
 * The reference's host classes need nlohmann_json, which is not available, so
 * the host sequences are restated here (second, independent restatement,
 * beside oracle/dpg_oracle.c):
 *   setupNeighbors / setNeighborSize / setCellSize    src/particles/base/particle.cu:71-100,1223-1272
 *   updateCellList / reorderParticleData              src/particles/base/particle.cu:1292-1317
 *   updateCellNeighborList / updateVerletList         src/particles/base/particle.cu:1119-1131,1320-1331
 *   checkForCellListUpdate / checkForVerletListUpdate src/particles/base/particle.cu:1141-1161
 *   NVE::step, Fire::step, Adam::minimize             src/integrator/{nve,fire,adam}.cu
 *   minimizeFire / minimizeAdam                       src/routines/minimization.cu:3-112
 * thrust::sort_by_key is restated with std::stable_sort, thrust reductions
 * with sequential sums.  Every per-item computation is the reference kernel.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

#include "cuda_host_shim.h"
#include "particles/base/kernels.cuh"
#include "particles/disk/kernels.cuh"

#define THRUST_DEVICE_SYSTEM THRUST_DEVICE_SYSTEM_CPP
#include "functors.h"

thread_local shim_dim3 blockIdx, threadIdx, blockDim, gridDim;

typedef std::vector<double> dvec;
typedef std::vector<long> lvec;

template <class F>
static void launch(long n, F &&f) {
#pragma omp parallel for schedule(static) if (n >= 2048)
    for (long i = 0; i < n; i++) {
        blockIdx = {(unsigned)i, 0, 0};
        threadIdx = {0, 0, 0};
        blockDim = {1, 1, 1};
        gridDim = {(unsigned)n, 1, 1};
        f();
    }
}

enum { M_CELL = 0, M_VERLET = 1, M_ALL = 2 };

struct ref_sys {
    long n;
    double box[2], e_c, n_c;
    dvec x, y, vx, vy, fx, fy, r, m, pe, ke;
    dvec tx, ty, tvx, tvy, tfx, tfy, tr, tm;
    dvec lnx, lny, lcx, lcy, nd2, cd2;
    lvec cell_index, pidx, sidx, cell_start, nlist, ncount;
    long cap = 4;
    int method = -1;
    double cutoff = -1, nthr2 = -1, cs = -1, cthr2 = -1;
    long ncd = -1, ncells = -1;
    long n_rebuilds = 0, n_cell_rebuilds = 0;
    dvec m1x, m1y, m2x, m2y, m1x_t, m1y_t, m2x_t, m2y_t;
    bool adam_ready = false;
    double f_alpha, f_alpha0, f_dt, f_dtmax, f_dtmin;
    long f_ngood = 0, f_nbad = 0;
    int f_stopped = 0;
    dvec sx, sy, svx, svy, sfx, sfy, sr, sm;
    lvec spidx, ssidx;
    double sbox[2];
    bool saved = false;
};

/* publish the system into the reference's global constants */
static void sync(ref_sys *s) {
    d_n_particles = s->n;
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
}

static double max_diam(ref_sys *s) { return 2.0 * *std::max_element(s->r.begin(), s->r.end()); }
static double area(ref_sys *s) {
    double a = 0.0;
    for (double v : s->r) a += v * v;
    return a * PI;
}
static double box_area(ref_sys *s) { return 1.0 * s->box[0] * s->box[1]; }

extern "C" {

ref_sys *ref_create(int64_t n, double bx, double by, double e_c, double n_c) {
    ref_sys *s = new ref_sys();
    s->n = n; s->box[0] = bx; s->box[1] = by; s->e_c = e_c; s->n_c = n_c;
    dvec *ds[] = {&s->x, &s->y, &s->vx, &s->vy, &s->fx, &s->fy, &s->r, &s->m, &s->pe, &s->ke,
                  &s->tx, &s->ty, &s->tvx, &s->tvy, &s->tfx, &s->tfy, &s->tr, &s->tm,
                  &s->lnx, &s->lny, &s->lcx, &s->lcy, &s->nd2, &s->cd2};
    for (dvec *d : ds) d->assign(n, 0.0);
    s->cell_index.assign(n, -1);
    s->pidx.resize(n); s->sidx.resize(n);
    std::iota(s->pidx.begin(), s->pidx.end(), 0L);
    std::iota(s->sidx.begin(), s->sidx.end(), 0L);
    s->ncount.assign(n, 0);
    s->nlist.assign(n * s->cap, -1);
    s->cell_start.assign(1, 0);
    return s;
}

void ref_destroy(ref_sys *s) { delete s; }

void ref_set_arrays(ref_sys *s, const double *x, const double *y, const double *vx,
                    const double *vy, const double *r, const double *m) {
    for (long i = 0; i < s->n; i++) {
        long k = s->sidx[i];
        if (x) s->x[i] = x[k];
        if (y) s->y[i] = y[k];
        if (vx) s->vx[i] = vx[k];
        if (vy) s->vy[i] = vy[k];
        if (r) s->r[i] = r[k];
        if (m) s->m[i] = m[k];
    }
}

void ref_get_arrays(ref_sys *s, double *x, double *y, double *vx, double *vy, double *fx,
                    double *fy, double *pe, double *r, double *m) {
    for (long i = 0; i < s->n; i++) {
        long k = s->sidx[i];
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

void ref_get_current(ref_sys *s, double *x, double *y, double *vx, double *vy, double *fx,
                     double *fy, double *pe, int64_t *sidx) {
    size_t b = s->n * sizeof(double);
    if (x) memcpy(x, s->x.data(), b);
    if (y) memcpy(y, s->y.data(), b);
    if (vx) memcpy(vx, s->vx.data(), b);
    if (vy) memcpy(vy, s->vy.data(), b);
    if (fx) memcpy(fx, s->fx.data(), b);
    if (fy) memcpy(fy, s->fy.data(), b);
    if (pe) memcpy(pe, s->pe.data(), b);
    if (sidx) for (long i = 0; i < s->n; i++) sidx[i] = s->sidx[i];
}

void ref_get_box(ref_sys *s, double *bx, double *by) { *bx = s->box[0]; *by = s->box[1]; }

/* ------------------------------------------------------------------ */
static bool set_neighbor_size(ref_sys *s, double cm, double dm) {
    s->cap = 4;
    s->cutoff = cm * max_diam(s);
    s->nthr2 = std::pow(dm * s->cutoff, 2);
    double diag = std::sqrt(s->box[0] * s->box[0] + s->box[1] * s->box[1]);
    return s->cutoff < diag;
}

static bool set_cell_size(ref_sys *s, double ppc, double cdm) {
    long min_dim = 4;
    double density = s->n / box_area(s);
    double trial = std::sqrt(ppc / density);
    double min_cs = 2.0 * max_diam(s);
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

static void set_method(ref_sys *s, int method) {
    s->method = method;
    std::iota(s->pidx.begin(), s->pidx.end(), 0L);
    std::iota(s->sidx.begin(), s->sidx.end(), 0L);
    if (method == M_ALL) {
        double diag = std::sqrt(s->box[0] * s->box[0] + s->box[1] * s->box[1]);
        set_neighbor_size(s, 2.0 * diag / max_diam(s), 0.0);
    }
}

static long max_count(ref_sys *s) {
    long mx = -1;
    for (long c : s->ncount) mx = std::max(mx, c);
    return mx;
}

static void verlet_kernel(ref_sys *s) {
    sync(s);
    launch(s->n, [&] {
        kernelUpdateNeighborList(s->x.data(), s->y.data(), s->lnx.data(), s->lny.data(),
                                 s->nd2.data(), s->cutoff);
    });
}

static void update_verlet_list(ref_sys *s) {
    std::fill(s->nlist.begin(), s->nlist.end(), -1L);
    verlet_kernel(s);
    long mx = max_count(s);
    if (mx > s->cap) {
        s->cap = (long)std::pow(2, std::ceil(std::log2(mx)));
        s->nlist.assign(s->n * s->cap, -1);
        verlet_kernel(s);
    }
    s->n_rebuilds++;
}

static void cell_nl_kernel(ref_sys *s) {
    sync(s);
    launch(s->n, [&] {
        kernelUpdateCellNeighborList(s->x.data(), s->y.data(), s->lnx.data(), s->lny.data(),
                                     s->cutoff, s->cell_index.data(), s->cell_start.data(),
                                     s->nd2.data());
    });
}

static void update_cell_neighbor_list(ref_sys *s) {
    std::fill(s->nlist.begin(), s->nlist.end(), -1L);
    cell_nl_kernel(s);
    long mx = max_count(s);
    if (mx > s->cap) {
        s->cap = (long)std::pow(2, std::ceil(std::log2(mx)));
        s->nlist.assign(s->n * s->cap, -1);
        cell_nl_kernel(s);
    }
    s->n_rebuilds++;
}

static void update_cell_list(ref_sys *s) {
    s->cell_start[s->ncells] = s->n;
    sync(s);
    launch(s->n, [&] {
        kernelGetCellIndexForParticle(s->x.data(), s->y.data(), s->cell_index.data(),
                                      s->pidx.data());
    });
    /* thrust::sort_by_key(cell_index, zip(particle_index, static_particle_index)) */
    std::vector<long> order(s->n);
    std::iota(order.begin(), order.end(), 0L);
    std::stable_sort(order.begin(), order.end(),
                     [&](long a, long b) { return s->cell_index[a] < s->cell_index[b]; });
    lvec ci(s->n), pi(s->n), si(s->n);
    for (long k = 0; k < s->n; k++) {
        ci[k] = s->cell_index[order[k]];
        pi[k] = s->pidx[order[k]];
        si[k] = s->sidx[order[k]];
    }
    s->cell_index = ci; s->pidx = pi; s->sidx = si;
    launch(s->n, [&] {
        kernelReorderParticleData(s->pidx.data(), s->x.data(), s->y.data(), s->fx.data(),
                                  s->fy.data(), s->vx.data(), s->vy.data(), s->m.data(),
                                  s->r.data(), s->tx.data(), s->ty.data(), s->tfx.data(),
                                  s->tfy.data(), s->tvx.data(), s->tvy.data(), s->tm.data(),
                                  s->tr.data(), s->lcx.data(), s->lcy.data(), s->cd2.data());
    });
    std::swap(s->x, s->tx); std::swap(s->y, s->ty);
    std::swap(s->fx, s->tfx); std::swap(s->fy, s->tfy);
    std::swap(s->vx, s->tvx); std::swap(s->vy, s->tvy);
    std::swap(s->m, s->tm); std::swap(s->r, s->tr);
    if (s->adam_ready) {
        std::swap(s->m1x, s->m1x_t); std::swap(s->m1y, s->m1y_t);
        std::swap(s->m2x, s->m2x_t); std::swap(s->m2y, s->m2y_t);
    }
    /* kernelGetFirstParticleIndexForCell, one item per cell */
    long width = s->ncells > 0 ? s->n / s->ncells : 0;
    launch(s->ncells, [&] {
        kernelGetFirstParticleIndexForCell(s->cell_index.data(), s->cell_start.data(), 2, width);
    });
    s->n_cell_rebuilds++;
}

static void init_verlet_vars(ref_sys *s) {
    s->nlist.assign(s->n * s->cap, -1);
    std::fill(s->ncount.begin(), s->ncount.end(), 0L);
    dvec *ds[] = {&s->lnx, &s->lny, &s->nd2, &s->lcx, &s->lcy, &s->cd2};
    for (dvec *d : ds) std::fill(d->begin(), d->end(), 0.0);
}

void ref_calculate_forces(ref_sys *s);

int ref_setup_neighbors(ref_sys *s, int method, double cm, double dm, double ppc, double cdm) {
    set_method(s, method);
    set_neighbor_size(s, cm, dm);
    if (s->method == M_CELL) {
        if (!set_cell_size(s, ppc, cdm)) set_method(s, M_VERLET);
        if (!set_neighbor_size(s, cm, dm)) set_method(s, M_ALL);
    }
    if (s->method == M_VERLET) {
        if (!set_neighbor_size(s, cm, dm)) set_method(s, M_ALL);
    }
    if (s->method == M_CELL) {
        init_verlet_vars(s);
        std::fill(s->cell_index.begin(), s->cell_index.end(), -1L);
        s->cell_start.assign(s->ncells + 1, 0);
        std::iota(s->pidx.begin(), s->pidx.end(), 0L);
        std::iota(s->sidx.begin(), s->sidx.end(), 0L);
        update_cell_list(s);
        update_cell_neighbor_list(s);
    } else if (s->method == M_VERLET) {
        init_verlet_vars(s);
        update_verlet_list(s);
    } else {
        s->cap = s->n - 1;
        init_verlet_vars(s);
        s->cutoff = 10.0 * std::sqrt(s->box[0] * s->box[0] + s->box[1] * s->box[1]);
        s->nthr2 = s->cutoff * s->cutoff;
        update_verlet_list(s);
    }
    ref_calculate_forces(s);
    return s->method;
}

void ref_update_neighbor_list(ref_sys *s) {
    if (s->method == M_CELL) update_cell_neighbor_list(s);
    else update_verlet_list(s);
}

static double max_of(const dvec &a) {
    double mx = 0.0;
    for (double v : a) mx = std::max(mx, v);
    return mx;
}

int ref_check_for_neighbor_update(ref_sys *s) {
    const double tol = 3.0;
    if (s->method == M_ALL) return 0;
    if (s->method == M_VERLET) {
        if (tol * max_of(s->nd2) > s->nthr2) { update_verlet_list(s); return 1; }
        return 0;
    }
    if (tol * max_of(s->cd2) > s->cthr2) {
        update_cell_list(s);
        update_cell_neighbor_list(s);
        return 2;
    }
    if (tol * max_of(s->nd2) > s->nthr2) { update_cell_neighbor_list(s); return 1; }
    return 0;
}

void ref_neighbor_info(ref_sys *s, int *method, double *cutoff, double *thr2, int64_t *ncd,
                       double *cs, double *cthr2, int64_t *cap) {
    if (method) *method = s->method;
    if (cutoff) *cutoff = s->cutoff;
    if (thr2) *thr2 = s->nthr2;
    if (ncd) *ncd = s->ncd;
    if (cs) *cs = s->cs;
    if (cthr2) *cthr2 = s->cthr2;
    if (cap) *cap = s->cap;
}

void ref_get_neighbors(ref_sys *s, int64_t *list, int64_t *counts) {
    if (list) for (size_t i = 0; i < s->nlist.size(); i++) list[i] = s->nlist[i];
    if (counts) for (long i = 0; i < s->n; i++) counts[i] = s->ncount[i];
}

void ref_get_cells(ref_sys *s, int64_t *cell_index, int64_t *cell_start) {
    if (cell_index) for (long i = 0; i < s->n; i++) cell_index[i] = s->cell_index[i];
    if (cell_start && s->method == M_CELL)
        for (long c = 0; c <= s->ncells; c++) cell_start[c] = s->cell_start[c];
}

int64_t ref_num_rebuilds(ref_sys *s, int64_t *n_cell) {
    if (n_cell) *n_cell = s->n_cell_rebuilds;
    return s->n_rebuilds;
}

/* ------------------------------------------------------------------ */
void ref_zero_force_and_pe(ref_sys *s) {
    sync(s);
    launch(s->n, [&] { kernelZeroForceAndPotentialEnergy(s->fx.data(), s->fy.data(), s->pe.data()); });
}

void ref_calculate_forces(ref_sys *s) {
    sync(s);
    launch(s->n, [&] {
        kernelCalcDiskForces(s->x.data(), s->y.data(), s->r.data(), s->fx.data(), s->fy.data(),
                             s->pe.data());
    });
}

void ref_update_velocities(ref_sys *s, double dt) {
    sync(s);
    launch(s->n, [&] {
        kernelUpdateVelocities(s->vx.data(), s->vy.data(), s->fx.data(), s->fy.data(),
                               s->m.data(), dt);
    });
}

void ref_update_positions(ref_sys *s, double dt) {
    sync(s);
    launch(s->n, [&] {
        kernelUpdatePositions(s->x.data(), s->y.data(), s->lnx.data(), s->lny.data(),
                              s->lcx.data(), s->lcy.data(), s->nd2.data(), s->cd2.data(),
                              s->vx.data(), s->vy.data(), dt);
    });
}

void ref_mix_velocities_and_forces(ref_sys *s, double alpha) {
    sync(s);
    launch(s->n, [&] {
        kernelMixVelocitiesAndForces(s->vx.data(), s->vy.data(), s->fx.data(), s->fy.data(), alpha);
    });
}

void ref_set_velocities_zero(ref_sys *s) {
    std::fill(s->vx.begin(), s->vx.end(), 0.0);
    std::fill(s->vy.begin(), s->vy.end(), 0.0);
}

double ref_power_fire(ref_sys *s) {
    double px = 0, py = 0;
    for (long i = 0; i < s->n; i++) px += s->fx[i] * s->vx[i];
    for (long i = 0; i < s->n; i++) py += s->fy[i] * s->vy[i];
    return px + py;
}

double ref_total_pe(ref_sys *s) {
    double e = 0;
    for (double v : s->pe) e += v;
    return e;
}

double ref_total_ke(ref_sys *s) {
    sync(s);
    launch(s->n, [&] {
        kernelCalculateTranslationalKineticEnergy(s->vx.data(), s->vy.data(), s->m.data(),
                                                  s->ke.data());
    });
    double e = 0;
    for (double v : s->ke) e += v;
    return e;
}

double ref_max_force(ref_sys *s) {
    double mx = 0;
    for (long i = 0; i < s->n; i++) mx = std::max(mx, std::sqrt(s->fx[i] * s->fx[i] + s->fy[i] * s->fy[i]));
    return mx;
}

void ref_nve_steps(ref_sys *s, double dt, int64_t n_steps) {
    for (int64_t t = 0; t < n_steps; t++) {
        ref_update_velocities(s, 0.5 * dt);
        ref_update_positions(s, dt);
        ref_check_for_neighbor_update(s);
        ref_zero_force_and_pe(s);
        ref_calculate_forces(s);
        ref_update_velocities(s, 0.5 * dt);
    }
}

/* DampedNVE::step (src/integrator/damped_nve.cu:15-27) over the reference kernels */
void ref_damped_nve_steps(ref_sys *s, double dt, double gamma, int64_t n_steps) {
    for (int64_t t = 0; t < n_steps; t++) {
        ref_update_velocities(s, 0.5 * dt);
        ref_update_positions(s, dt);
        ref_check_for_neighbor_update(s);
        ref_zero_force_and_pe(s);
        sync(s);
        launch(s->n, [&] {
            kernelCalculateDampedForces(s->fx.data(), s->fy.data(), s->vx.data(), s->vy.data(), gamma);
        });
        ref_calculate_forces(s);
        ref_update_velocities(s, 0.5 * dt);
    }
}

/* Disk::calculateForceDistancePairs (src/particles/disk/disk.cu:228-255): the
 * reference's fills, then its kernel; 18 arrays of n * cap, row-major
 * [slot * cap + k] in the current order (ids are static indices) */
void ref_pair_dump(ref_sys *s, double *const *d, int64_t *this_id, int64_t *other_id) {
    const long m = s->n * s->cap;
    std::vector<double> v[16];
    const double fill[16] = {-1, 0, 0, -1, -1, -1, -1, -1, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int k = 0; k < 16; k++) v[k].assign(m, fill[k]);
    std::vector<long> ti(m, -1), oi(m, -1);
    sync(s);
    launch(s->n, [&] {
        kernelCalcDiskForceDistancePairs(s->x.data(), s->y.data(), v[0].data(), v[1].data(), v[2].data(),
                                         v[3].data(), v[4].data(), ti.data(), oi.data(), v[5].data(),
                                         v[6].data(), s->r.data(), s->sidx.data(), v[7].data(),
                                         v[8].data(), v[9].data(), v[10].data(), v[11].data(),
                                         v[12].data(), v[13].data(), v[14].data(), v[15].data());
    });
    for (int k = 0; k < 16; k++)
        if (d[k]) std::copy(v[k].begin(), v[k].end(), d[k]);
    for (long q = 0; q < m; q++) { this_id[q] = ti[q]; other_id[q] = oi[q]; }
}

/* Disk::calculateWallForces (src/particles/disk/disk.cu:257-259) */
void ref_wall_forces(ref_sys *s) {
    sync(s);
    launch(s->n, [&] {
        kernelCalcDiskWallForces(s->x.data(), s->y.data(), s->r.data(), s->fx.data(), s->fy.data(),
                                 s->pe.data());
    });
}

/* NVE::wall_step (src/integrator/nve.cu:27-38) over the reference kernels */
void ref_nve_wall_steps(ref_sys *s, double dt, int64_t n_steps) {
    for (int64_t t = 0; t < n_steps; t++) {
        ref_update_velocities(s, 0.5 * dt);
        ref_update_positions(s, dt);
        ref_check_for_neighbor_update(s);
        ref_zero_force_and_pe(s);
        ref_wall_forces(s);
        ref_calculate_forces(s);
        ref_update_velocities(s, 0.5 * dt);
    }
}

/* GradDesc::step (src/integrator/grad_desc.cu:11-17) over the reference kernels */
void ref_grad_desc_steps(ref_sys *s, double alpha, int64_t n_steps) {
    for (int64_t t = 0; t < n_steps; t++) {
        ref_zero_force_and_pe(s);
        ref_check_for_neighbor_update(s);
        ref_calculate_forces(s);
        sync(s);
        launch(s->n, [&] {
            kernelGradDescStep(s->x.data(), s->y.data(), s->fx.data(), s->fy.data(), s->lnx.data(),
                               s->lny.data(), s->nd2.data(), s->lcx.data(), s->lcy.data(),
                               s->cd2.data(), alpha);
        });
    }
}

void ref_fire_init(ref_sys *s, double alpha_init, double dt) {
    s->f_alpha = alpha_init; s->f_alpha0 = alpha_init; s->f_dt = dt;
    s->f_dtmax = 10.0 * dt; s->f_dtmin = 0.001 * dt;
    s->f_ngood = 0; s->f_nbad = 0; s->f_stopped = 0;
}

int ref_fire_step(ref_sys *s) {
    double power = ref_power_fire(s);
    if (power > 0) {
        s->f_ngood++;
        s->f_nbad = 0;
        if (s->f_ngood > 5) {
            s->f_dt = std::min(s->f_dt * 1.1, s->f_dtmax);
            s->f_alpha *= 0.99;
        }
    } else {
        s->f_ngood = 0;
        s->f_nbad++;
        if (s->f_nbad > 10) { s->f_stopped = 1; return 1; }
        s->f_dt = std::max(s->f_dt * 0.5, s->f_dtmin);
        s->f_alpha = s->f_alpha0;
        ref_update_positions(s, -s->f_dt / 2.0);
        ref_set_velocities_zero(s);
    }
    ref_update_velocities(s, s->f_dt / 2.0);
    ref_mix_velocities_and_forces(s, s->f_alpha);
    ref_update_positions(s, s->f_dt);
    ref_zero_force_and_pe(s);
    ref_check_for_neighbor_update(s);
    ref_calculate_forces(s);
    ref_update_velocities(s, s->f_dt / 2.0);
    return 0;
}

void ref_fire_state(ref_sys *s, double *alpha, double *dt, int64_t *ng, int64_t *nb, int *stopped) {
    if (alpha) *alpha = s->f_alpha;
    if (dt) *dt = s->f_dt;
    if (ng) *ng = s->f_ngood;
    if (nb) *nb = s->f_nbad;
    if (stopped) *stopped = s->f_stopped;
}

int64_t ref_minimize_fire(ref_sys *s, double alpha_init, double dt, double pe_target,
                          double pe_diff_target, int64_t num_steps, double fmax_target,
                          int *stopped_out) {
    ref_fire_init(s, alpha_init, dt);
    int64_t step = 0;
    double dof = (double)s->n;
    ref_set_velocities_zero(s);
    ref_zero_force_and_pe(s);
    ref_check_for_neighbor_update(s);
    ref_calculate_forces(s);
    double last = ref_total_pe(s) / dof;
    while (step < num_steps) {
        ref_fire_step(s);
        double avg = ref_total_pe(s) / dof;
        double diff = std::abs(avg / last - 1);
        last = avg;
        if (diff < pe_diff_target || avg < pe_target || s->f_stopped) break;
        if (fmax_target > 0 && ref_max_force(s) <= fmax_target) break;
        step++;
    }
    ref_set_velocities_zero(s);
    if (stopped_out) *stopped_out = s->f_stopped;
    return step;
}

void ref_init_adam(ref_sys *s) {
    dvec *ds[] = {&s->m1x, &s->m1y, &s->m2x, &s->m2y, &s->m1x_t, &s->m1y_t, &s->m2x_t, &s->m2y_t};
    for (dvec *d : ds) d->assign(s->n, 0.0);
    s->adam_ready = true;
}

void ref_adam_step(ref_sys *s, int64_t step, double alpha, double b1, double b2, double eps) {
    double c1 = 1 - std::pow(b1, step + 1);
    double c2 = 1 - std::pow(b2, step + 1);
    sync(s);
    launch(s->n, [&] {
        kernelAdamStep(s->m1x.data(), s->m1y.data(), s->m2x.data(), s->m2y.data(), s->x.data(),
                       s->y.data(), s->fx.data(), s->fy.data(), alpha, b1, b2, c1, c2, eps,
                       s->lnx.data(), s->lny.data(), s->nd2.data(), s->lcx.data(), s->lcy.data(),
                       s->cd2.data());
    });
}

int64_t ref_minimize_adam(ref_sys *s, double alpha, double b1, double b2, double eps,
                          double pe_target, double pe_diff_target, int64_t num_steps) {
    ref_init_adam(s);
    int64_t step = 0;
    double dof = (double)(s->n * 2), last = 0.0;
    while (step < num_steps) {
        ref_zero_force_and_pe(s);
        ref_check_for_neighbor_update(s);
        ref_calculate_forces(s);
        ref_adam_step(s, step, alpha, b1, b2, eps);
        double avg = ref_total_pe(s) / dof;
        double diff = std::abs(avg / last - 1);
        last = avg;
        if (diff < pe_diff_target || avg < pe_target) break;
        step++;
    }
    return step;
}

void ref_stress_tensor(ref_sys *s, double out[4]) {
    dvec sxx(s->n, 0), sxy(s->n, 0), syx(s->n, 0), syy(s->n, 0);
    sync(s);
    launch(s->n, [&] {
        kernelCalcDiskStressTensor(s->x.data(), s->y.data(), s->vx.data(), s->vy.data(),
                                   s->m.data(), s->r.data(), sxx.data(), sxy.data(), syx.data(),
                                   syy.data());
    });
    double a = 0, b = 0, c = 0, d = 0;
    for (long i = 0; i < s->n; i++) { a += sxx[i]; b += sxy[i]; c += syx[i]; d += syy[i]; }
    out[0] = a; out[1] = b; out[2] = c; out[3] = d;
}

double ref_pressure(ref_sys *s) {
    double st[4];
    ref_stress_tensor(s, st);
    return (st[0] + st[3]) / N_DIM;
}

double ref_contact_count(ref_sys *s) {
    lvec counts(s->n, 0);
    sync(s);
    launch(s->n, [&] { kernelCountDiskContacts(s->x.data(), s->y.data(), s->r.data(), counts.data()); });
    long t = 0;
    for (long c : counts) t += c;
    return (double)t;
}

double ref_particle_area(ref_sys *s) { return area(s); }
double ref_packing_fraction(ref_sys *s) { return area(s) / box_area(s); }

static void update_cell_size(ref_sys *s) {
    if (s->ncd > 0) s->cs = s->box[0] / s->ncd;
}

void ref_scale_to_packing_fraction(ref_sys *s, double phi) {
    double new_l = std::pow(area(s) / phi, 1.0 / N_DIM);
    double l = std::pow(box_area(s), 1.0 / N_DIM);
    double f = new_l / l;
    for (long i = 0; i < s->n; i++) { s->x[i] *= f; s->y[i] *= f; }
    s->box[0] = new_l; s->box[1] = new_l;
    update_cell_size(s);
}

void ref_scale_box(ref_sys *s, double factor) {
    for (long i = 0; i < s->n; i++) { s->x[i] *= factor; s->y[i] *= factor; }
    double l = std::pow(box_area(s), 1.0 / N_DIM);
    double nl = l * factor;
    s->box[0] = nl; s->box[1] = nl;
    update_cell_size(s);
}

void ref_set_last_state(ref_sys *s) {
    s->sx = s->x; s->sy = s->y; s->svx = s->vx; s->svy = s->vy; s->sfx = s->fx; s->sfy = s->fy;
    s->sr = s->r; s->sm = s->m; s->spidx = s->pidx; s->ssidx = s->sidx;
    s->sbox[0] = s->box[0]; s->sbox[1] = s->box[1];
    s->saved = true;
}

void ref_revert_to_last_state(ref_sys *s) {
    if (!s->saved) return;
    s->x = s->sx; s->y = s->sy; s->vx = s->svx; s->vy = s->svy; s->fx = s->sfx; s->fy = s->sfy;
    s->r = s->sr; s->m = s->sm; s->pidx = s->spidx; s->sidx = s->ssidx;
    s->box[0] = s->sbox[0]; s->box[1] = s->sbox[1];
    ref_update_neighbor_list(s);
}

/* the reference's own generator functors (include/functors.h:17-50), host build */
void ref_fill_uniform(double *out, int64_t n, double lo, double hi, int64_t seed_offset,
                      int64_t seed) {
    RandomUniform f(lo, hi, (unsigned int)seed);
    for (int64_t i = 0; i < n; i++) out[i] = f((unsigned int)(seed + seed_offset + i));
}

} /* extern "C" */
