// disk_system.cu -- host side of the plain FP64 disk system and the C ABI
// (include/dpg.h).  Compiled with --fmad=false together with disk_kernels.cuh.
//
// A dpg_system owns the device buffers, a DevSys block in device memory and a
// stream.  Single operations (dpg_kick, dpg_drift, ...) map one-to-one onto
// the reference's Particle methods.  The loops (dpg_nve_steps,
// dpg_fire_minimize, dpg_adam_minimize) run device-resident: the rebuild
// decision, the FIRE dt/alpha logic and the convergence tests are made on
// the GPU, and the loop body is a CUDA graph whose neighbour rebuild sits
// under a conditional (IF) node inside a WHILE node, so a whole minimisation is
// one graph launch with no host round trips.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/dpg.h"
#include "disk_kernels.cuh"
#include "host_common.h"

using namespace dpg;

// ---------------------------------------------------------------------------
// errors
// ---------------------------------------------------------------------------
static thread_local char g_err[512] = "";

int dpg::set_error(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}
#define set_err dpg::set_error

#define CK(x)                                                                        \
    do {                                                                             \
        cudaError_t e_ = (x);                                                        \
        if (e_ != cudaSuccess)                                                       \
            return set_err(DPG_ERR_CUDA, "%s:%d %s: %s", __FILE__, __LINE__, #x,      \
                           cudaGetErrorString(e_));                                  \
    } while (0)

#define TRY(x)                    \
    do {                          \
        int r_ = (x);             \
        if (r_ != DPG_OK) return r_; \
    } while (0)

extern "C" const char *dpg_last_error(void) { return g_err; }
extern "C" int dpg_version(void) { return 1; }

// ---------------------------------------------------------------------------
// the system object
// ---------------------------------------------------------------------------
enum LoopKind { kLoopFire = 0, kLoopNve = 1, kLoopCount = 2 };
enum LoopMode { kModeStream = 0, kModeGraph = 1, kModeCond = 2 };

struct dpg_system {
    int n = 0;
    dpg_params prm{};
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    DevSys *d = nullptr;  // device block
    DevSys h{};           // host mirror of params and the initial buffer pointers
    DevState *hs = nullptr;  // pinned readback of the device state
    std::vector<double> h_rad;  // radii in static order
    bool have_state = false, have_neighbors = false, adam_ready = false;
    // neighbour configuration (Particle members)
    int method = -1, ncd = 0, ncells = 0, cap = 4;
    double cutoff = -1, nthr2 = -1, cs = -1, cthr2 = -1;
    // buffers owned here
    std::vector<void *> allocs;
    int *nbr = nullptr;
    int *cell_buf = nullptr;
    double *xfer = nullptr;  // staging for static-order transfers (2 n doubles)
    // loops
    int mode = kModeCond;
    cudaGraphExec_t loop_exec[kLoopCount] = {nullptr, nullptr};
    cudaGraphConditionalHandle h_loop[kLoopCount] = {0, 0}, h_rb[kLoopCount] = {0, 0};
    cudaGraphExec_t chunk_exec[kLoopCount] = {nullptr, nullptr};
    double chunk_dt = 0.0;
    int kernel_launches = 0;  // launches issued by the last loop call (bench bookkeeping)

    // threads per block of the per-particle kernels: small systems use small
    // blocks so the grid still spreads over every SM
    int tpb = kTPB;
    int grid(int count) const { return std::max(1, (count + tpb - 1) / tpb); }
    int grid_full(int count) const { return std::max(1, (count + kTPB - 1) / kTPB); }
    // force kernels: fg threads per particle (bit-identical sums, more warps
    // in flight for small systems), ftpb threads per block
    int fg = 1;
    int ftpb = kTPB;
    int fgrid() const { return std::max(1, (int)(((long long)n * fg + ftpb - 1) / ftpb)); }
    // mixed form (precision DPG_MIXED): FP32 pair kernels, one thread per particle
    bool mixed = false;
    double switch_fmax = 1e-6;
    void *fire_force_fn() const {
        if (mixed) return (void *)k_fire_force<1, true>;
        switch (fg) {
            case 2: return (void *)k_fire_force<2, false>;
            case 4: return (void *)k_fire_force<4, false>;
            case 8: return (void *)k_fire_force<8, false>;
            default: return (void *)k_fire_force<1, false>;
        }
    }
    void *nve_second_fn() const {
        if (mixed) return (void *)k_nve_second<1, true>;
        switch (fg) {
            case 2: return (void *)k_nve_second<2, false>;
            case 4: return (void *)k_nve_second<4, false>;
            case 8: return (void *)k_nve_second<8, false>;
            default: return (void *)k_nve_second<1, false>;
        }
    }
    void *force_acc_fn() const {
        if (mixed) return (void *)k_force_acc<1, true>;
        switch (fg) {
            case 2: return (void *)k_force_acc<2, false>;
            case 4: return (void *)k_force_acc<4, false>;
            case 8: return (void *)k_force_acc<8, false>;
            default: return (void *)k_force_acc<1, false>;
        }
    }
};

static int dalloc(dpg_system *s, void **p, size_t bytes) {
    CK(cudaMalloc(p, bytes > 0 ? bytes : 16));
    CK(cudaMemsetAsync(*p, 0, bytes > 0 ? bytes : 16, s->stream));
    s->allocs.push_back(*p);
    return DPG_OK;
}

static void free_graphs(dpg_system *s) {
    for (int k = 0; k < kLoopCount; k++) {
        if (s->loop_exec[k]) cudaGraphExecDestroy(s->loop_exec[k]);
        if (s->chunk_exec[k]) cudaGraphExecDestroy(s->chunk_exec[k]);
        s->loop_exec[k] = nullptr;
        s->chunk_exec[k] = nullptr;
    }
}

static int push_params(dpg_system *s) {
    mixed_grid_update(s->h.p);
    CK(cudaMemcpyAsync(&s->d->p, &s->h.p, sizeof(DevParams), cudaMemcpyHostToDevice, s->stream));
    return DPG_OK;
}

static int pull_state(dpg_system *s) {
    CK(cudaMemcpyAsync(s->hs, &s->d->s, sizeof(DevState), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return DPG_OK;
}

template <class T>
static int put_field(dpg_system *s, T *dev_field, const T &val) {
    CK(cudaMemcpyAsync(dev_field, &val, sizeof(T), cudaMemcpyHostToDevice, s->stream));
    return DPG_OK;
}

static int check_launch(dpg_system *s) {
    (void)s;
    CK(cudaGetLastError());
    return DPG_OK;
}

#define LAUNCH(kern, blocks, threads, ...)                              \
    do {                                                                \
        kern<<<(blocks), (threads), 0, s->stream>>>(__VA_ARGS__);       \
        TRY(check_launch(s));                                           \
    } while (0)

// launch of a kernel chosen at run time (the force kernels' group size)
template <class... A>
static int launch_fn(dpg_system *s, void *fn, int blocks, int threads, A... a) {
    void *args[] = {(void *)&a...};
    CK(cudaLaunchKernel(fn, dim3(blocks), dim3(threads), args, 0, s->stream));
    return DPG_OK;
}

// mixed form: offsets from the current positions (after any host-side or
// single-operation change of positions or box; the loop kernels keep them
// current themselves)
static int mixed_refresh(dpg_system *s) {
    if (!s->mixed) return DPG_OK;
    k_mixed_refresh<<<s->grid(s->n), s->tpb, 0, s->stream>>>(s->d);
    CK(cudaGetLastError());
    return DPG_OK;
}

static int launch_force_acc(dpg_system *s) {
    TRY(mixed_refresh(s));
    return launch_fn(s, s->force_acc_fn(), s->fgrid(), s->ftpb, s->d);
}
static int launch_fire_force(dpg_system *s, int mode) {
    if (mode != 0) TRY(mixed_refresh(s));
    return launch_fn(s, s->fire_force_fn(), s->fgrid(), s->ftpb, s->d, mode);
}
static int launch_nve_second(dpg_system *s, double dt_half) {
    return launch_fn(s, s->nve_second_fn(), s->fgrid(), s->ftpb, s->d, dt_half);
}

// ---------------------------------------------------------------------------
// creation / destruction
// ---------------------------------------------------------------------------
extern "C" int dpg_create(const dpg_params *p, void *cuda_stream, dpg_handle *out) {
    if (!p || !out) return set_err(DPG_ERR_ARG, "dpg_create: null argument");
    if (p->n_particles <= 0 || p->n_particles > (1LL << 30))
        return set_err(DPG_ERR_ARG, "dpg_create: n_particles must be in [1, 2^30]");
    if (!(p->box_x > 0) || !(p->box_y > 0)) return set_err(DPG_ERR_ARG, "dpg_create: box must be > 0");
    if (p->precision != DPG_FP64 && p->precision != DPG_MIXED)
        return set_err(DPG_ERR_ARG, "dpg_create: precision must be DPG_FP64 or DPG_MIXED");
    dpg_system *s = new dpg_system();
    s->n = (int)p->n_particles;
    s->prm = *p;
    if (cuda_stream) {
        s->stream = (cudaStream_t)cuda_stream;
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { delete s; return set_err(DPG_ERR_CUDA, "stream: %s", cudaGetErrorString(e)); }
        s->own_stream = true;
    }
    const char *m = getenv("DPG_LOOP_MODE");
    if (m && !strcmp(m, "stream")) s->mode = kModeStream;
    else if (m && !strcmp(m, "graph")) s->mode = kModeGraph;
    const size_t n = s->n;
    int dev = 0, nsm = 148;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    s->tpb = kTPB;
    while (s->tpb > 32 && (long long)s->n < (long long)s->tpb * 2 * nsm) s->tpb >>= 1;
    const char *tp = getenv("DPG_TPB");
    if (tp && atoi(tp) >= 32 && atoi(tp) <= kTPB) s->tpb = atoi(tp) & ~31;
    // group size for the force kernels: enough threads to give every SM about
    // 6 warps, at most 8 lanes per particle (measured at N = 16384 on GB300:
    // 52.7, 37.8, 42.2, 55.1 us per FIRE force pass for 1, 2, 4, 8 lanes)
    s->fg = 1;
    while (s->fg < 8 && (long long)s->n * s->fg < (long long)nsm * 192) s->fg <<= 1;
    const char *fgs = getenv("DPG_FORCE_GROUP");
    if (fgs) {
        int g = atoi(fgs);
        if (g == 1 || g == 2 || g == 4 || g == 8) s->fg = g;
    }
    s->ftpb = kTPB;
    s->mixed = p->precision == DPG_MIXED;
    if (s->mixed) s->fg = 1;
    int rc = DPG_OK;
    auto A = [&](void **pp, size_t b) { if (rc == DPG_OK) rc = dalloc(s, pp, b); };
    DevView &v = s->h.v;
    DevScratch &w = s->h.w;
    A((void **)&v.pos, n * 16); A((void **)&v.vel, n * 16); A((void **)&v.frc, n * 16);
    A((void **)&v.rad, n * 8); A((void **)&v.mass, n * 8); A((void **)&v.sidx, n * 4);
    A((void **)&v.pos_t, n * 16); A((void **)&v.vel_t, n * 16); A((void **)&v.frc_t, n * 16);
    A((void **)&v.rad_t, n * 8); A((void **)&v.mass_t, n * 8); A((void **)&v.sidx_t, n * 4);
    A((void **)&v.m1, n * 16); A((void **)&v.m2, n * 16); A((void **)&v.m1_t, n * 16); A((void **)&v.m2_t, n * 16);
    if (s->mixed) A((void **)&v.pk, n * 16);
    A((void **)&w.pos_n, n * 16); A((void **)&w.pos_c, n * 16); A((void **)&w.pe, n * 8);
    A((void **)&w.count, n * 4); A((void **)&w.cell_raw, n * 4); A((void **)&w.cell_of, n * 4);
    A((void **)&w.perm, n * 4);
    // partials for the widest force group (8 lanes), so the group can change later
    const int fg8 = std::max(1, (int)(((long long)s->n * 8 + s->ftpb - 1) / s->ftpb));
    w.max_blocks = std::max(std::max(s->grid(s->n), s->grid_full(s->n)), std::max(s->fgrid(), fg8));
    A((void **)&w.partials, (size_t)w.max_blocks * 8 * 8);
    A((void **)&w.s_pos, n * 16); A((void **)&w.s_vel, n * 16); A((void **)&w.s_frc, n * 16);
    A((void **)&w.s_rad, n * 8); A((void **)&w.s_mass, n * 8); A((void **)&w.s_sidx, n * 4);
    A((void **)&s->xfer, n * 16);
    A((void **)&s->d, sizeof(DevSys));
    if (rc == DPG_OK) {
        cudaError_t e = cudaMallocHost((void **)&s->hs, sizeof(DevState));
        if (e != cudaSuccess) rc = set_err(DPG_ERR_CUDA, "pinned: %s", cudaGetErrorString(e));
    }
    if (rc != DPG_OK) { dpg_destroy(s); return rc; }
    DevParams &pp = s->h.p;
    pp.n = s->n; pp.method = -1; pp.cap = 4; pp.precision = p->precision;
    pp.box[0] = p->box_x; pp.box[1] = p->box_y; pp.e_c = p->e_c; pp.n_c = p->n_c;
    if (s->mixed) {
        mixed_grid_init(pp);
        mixed_grid_update(pp);
    }
    memset(&s->h.s, 0, sizeof(DevState));
    rc = [&]() -> int {
        CK(cudaMemcpyAsync(s->d, &s->h, sizeof(DevSys), cudaMemcpyHostToDevice, s->stream));
        LAUNCH(k_iota_sidx, s->grid(s->n), s->tpb, s->d);
        CK(cudaStreamSynchronize(s->stream));
        return DPG_OK;
    }();
    if (rc != DPG_OK) { dpg_destroy(s); return rc; }
    s->h_rad.assign(n, 0.0);
    *out = s;
    return DPG_OK;
}

extern "C" int dpg_destroy(dpg_handle s) {
    if (!s) return DPG_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    free_graphs(s);
    for (void *p : s->allocs) cudaFree(p);
    if (s->nbr) cudaFree(s->nbr);
    if (s->cell_buf) cudaFree(s->cell_buf);
    if (s->hs) cudaFreeHost(s->hs);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return DPG_OK;
}

extern "C" int dpg_get_params(dpg_handle s, dpg_params *p) {
    if (!s || !p) return set_err(DPG_ERR_ARG, "null argument");
    *p = s->prm;
    p->box_x = s->h.p.box[0];
    p->box_y = s->h.p.box[1];
    return DPG_OK;
}

extern "C" int dpg_synchronize(dpg_handle s) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    CK(cudaStreamSynchronize(s->stream));
    return DPG_OK;
}

// ---------------------------------------------------------------------------
// state transfer
// ---------------------------------------------------------------------------
// Copy a static-order array to device staging (or use it in place).
static int stage_in(dpg_system *s, const double *src, int where, int slot, const double **dev) {
    if (!src) { *dev = nullptr; return DPG_OK; }
    if (where == DPG_DEVICE) { *dev = src; return DPG_OK; }
    double *dst = s->xfer + (size_t)slot * s->n;
    CK(cudaMemcpyAsync(dst, src, sizeof(double) * s->n, cudaMemcpyHostToDevice, s->stream));
    *dev = dst;
    return DPG_OK;
}

static int put_xy(dpg_system *s, int which, const double *x, const double *y, int where) {
    if (!x && !y) return DPG_OK;
    const double *dx, *dy;
    TRY(stage_in(s, x, where, 0, &dx));
    TRY(stage_in(s, y, where, 1, &dy));
    LAUNCH(k_put_xy, s->grid(s->n), s->tpb, s->d, which, dx, dy);
    if (where == DPG_HOST) CK(cudaStreamSynchronize(s->stream));
    return DPG_OK;
}

extern "C" int dpg_set_state(dpg_handle s, const double *x, const double *y, const double *vx,
                             const double *vy, const double *radii, const double *masses,
                             int where) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (where != DPG_HOST && where != DPG_DEVICE) return set_err(DPG_ERR_ARG, "bad `where`");
    TRY(put_xy(s, 0, x, y, where));
    TRY(put_xy(s, 1, vx, vy, where));
    const double *scal[2] = {radii, masses};
    for (int k = 0; k < 2; k++) {
        if (!scal[k]) continue;
        const double *dp;
        TRY(stage_in(s, scal[k], where, 0, &dp));
        LAUNCH(k_put_scalar, s->grid(s->n), s->tpb, s->d, k, dp);
        if (where == DPG_HOST) CK(cudaStreamSynchronize(s->stream));
    }
    if (radii) {
        if (where == DPG_HOST) {
            memcpy(s->h_rad.data(), radii, sizeof(double) * s->n);
        } else {
            CK(cudaMemcpyAsync(s->h_rad.data(), radii, sizeof(double) * s->n, cudaMemcpyDeviceToHost, s->stream));
            CK(cudaStreamSynchronize(s->stream));
        }
    }
    if (x && y && radii) s->have_state = true;
    return DPG_OK;
}

extern "C" int dpg_load_state(dpg_handle s, const double *x, const double *y, const double *vx,
                              const double *vy, const double *radii, const double *masses,
                              int where) {
    if (!s || !x || !y || !radii || !masses) return set_err(DPG_ERR_ARG, "dpg_load_state: null argument");
    LAUNCH(k_iota_sidx, s->grid(s->n), s->tpb, s->d);
    LAUNCH(k_zero_force, s->grid(s->n), s->tpb, s->d);
    LAUNCH(k_zero_vel, s->grid(s->n), s->tpb, s->d);
    return dpg_set_state(s, x, y, vx, vy, radii, masses, where);
}

extern "C" int dpg_get_static_params(dpg_handle s, double *radii, double *masses) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    double *outs[2] = {radii, masses};
    for (int k = 0; k < 2; k++) {
        if (!outs[k]) continue;
        LAUNCH(k_get_scalar, s->grid(s->n), s->tpb, s->d, k, s->xfer);
        CK(cudaMemcpyAsync(outs[k], s->xfer, sizeof(double) * s->n, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    return DPG_OK;
}

extern "C" int dpg_set_forces(dpg_handle s, const double *fx, const double *fy, int where) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    return put_xy(s, 2, fx, fy, where);
}

extern "C" int dpg_get_state(dpg_handle s, double *x, double *y, double *vx, double *vy,
                             double *fx, double *fy, double *pe, int where) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (where != DPG_HOST && where != DPG_DEVICE) return set_err(DPG_ERR_ARG, "bad `where`");
    double *outs[3][2] = {{x, y}, {vx, vy}, {fx, fy}};
    const size_t nb = sizeof(double) * s->n;
    for (int k = 0; k < 3; k++) {
        double *ox = outs[k][0], *oy = outs[k][1];
        if (!ox && !oy) continue;
        if (where == DPG_DEVICE) {
            LAUNCH(k_get_xy, s->grid(s->n), s->tpb, s->d, k, ox, oy);
        } else {
            double *sx = s->xfer, *sy = s->xfer + s->n;
            LAUNCH(k_get_xy, s->grid(s->n), s->tpb, s->d, k, ox ? sx : nullptr, oy ? sy : nullptr);
            if (ox) CK(cudaMemcpyAsync(ox, sx, nb, cudaMemcpyDeviceToHost, s->stream));
            if (oy) CK(cudaMemcpyAsync(oy, sy, nb, cudaMemcpyDeviceToHost, s->stream));
            CK(cudaStreamSynchronize(s->stream));
        }
    }
    if (pe) {
        double *dst = where == DPG_DEVICE ? pe : s->xfer;
        LAUNCH(k_get_pe, s->grid(s->n), s->tpb, s->d, dst);
        if (where == DPG_HOST) {
            CK(cudaMemcpyAsync(pe, dst, nb, cudaMemcpyDeviceToHost, s->stream));
            CK(cudaStreamSynchronize(s->stream));
        }
    }
    return DPG_OK;
}

extern "C" int dpg_set_box(dpg_handle s, double bx, double by) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (!(bx > 0) || !(by > 0)) return set_err(DPG_ERR_ARG, "box must be > 0");
    s->h.p.box[0] = bx;
    s->h.p.box[1] = by;
    return push_params(s);
}

extern "C" int dpg_get_box(dpg_handle s, double *bx, double *by) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (bx) *bx = s->h.p.box[0];
    if (by) *by = s->h.p.box[1];
    return DPG_OK;
}

// ---------------------------------------------------------------------------
// neighbours: host restatement of setupNeighbors and friends
// (src/particles/base/particle.cu:71-100, 237-265, 1119-1331)
// ---------------------------------------------------------------------------
static double max_diameter(const dpg_system *s) {
    return 2.0 * *std::max_element(s->h_rad.begin(), s->h_rad.end());
}

static double particle_area(const dpg_system *s) {
    double a = 0.0;
    for (double r : s->h_rad) a += r * r;
    return a * 3.141592653589793238462643383279502884197;
}

// Disk::getParticleArea (src/particles/disk/disk.cu:205-207) sums r^2 over the
// CURRENT (cell-sorted) order, so the box scalings that use it round like the
// reference only when the sum runs in that order.
static int current_area(dpg_system *s, double *area) {
    DevView v;
    CK(cudaMemcpyAsync(&v, &s->d->v, sizeof(DevView), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    std::vector<double> r(s->n);
    CK(cudaMemcpyAsync(r.data(), v.rad, sizeof(double) * s->n, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    double a = 0.0;
    for (double x : r) a += x * x;
    *area = a * 3.141592653589793238462643383279502884197;
    return DPG_OK;
}

static double box_area(const dpg_system *s) { return 1.0 * s->h.p.box[0] * s->h.p.box[1]; }

static bool set_neighbor_size(dpg_system *s, double cm, double dm) {
    s->cap = 4;
    s->cutoff = cm * max_diameter(s);
    s->nthr2 = std::pow(dm * s->cutoff, 2);
    double diag = std::sqrt(s->h.p.box[0] * s->h.p.box[0] + s->h.p.box[1] * s->h.p.box[1]);
    return s->cutoff < diag;
}

static bool set_cell_size(dpg_system *s, double ppc, double cdm) {
    const int min_dim = 4;
    double density = s->n / box_area(s);
    double trial = std::sqrt(ppc / density);
    double min_cs = 2.0 * max_diameter(s);
    s->ncd = (int)std::floor(s->h.p.box[0] / trial);
    s->ncells = s->ncd * s->ncd;
    if (s->ncd < min_dim) { s->ncd = min_dim; s->ncells = s->ncd * s->ncd; }
    s->cs = s->h.p.box[0] / s->ncd;
    if (s->cs < min_cs) {
        s->cs = min_cs;
        s->ncd = (int)std::floor(s->h.p.box[0] / s->cs);
        s->ncells = s->ncd * s->ncd;
        if (s->ncd < min_dim) return false;
    }
    s->cthr2 = std::pow(cdm * s->cs, 2);
    return true;
}

static int set_method(dpg_system *s, int m) {
    s->method = m;
    LAUNCH(k_iota_sidx, s->grid(s->n), s->tpb, s->d);
    if (m == DPG_NEIGH_ALL) {
        double diag = std::sqrt(s->h.p.box[0] * s->h.p.box[0] + s->h.p.box[1] * s->h.p.box[1]);
        set_neighbor_size(s, 2.0 * diag / max_diameter(s), 0.0);
    }
    return DPG_OK;
}

static int sync_neighbor_params(dpg_system *s) {
    DevParams &p = s->h.p;
    p.method = s->method;
    p.ncd = s->ncd;
    p.ncells = s->ncells;
    p.cap = s->cap;
    p.cutoff2 = s->cutoff * s->cutoff;
    p.cell_size = s->cs;
    p.nthr2 = s->nthr2;
    p.cthr2 = s->cthr2;
    return push_params(s);
}

static int alloc_nbr(dpg_system *s, int cap) {
    if (s->nbr) { CK(cudaStreamSynchronize(s->stream)); CK(cudaFree(s->nbr)); s->nbr = nullptr; }
    CK(cudaMalloc((void **)&s->nbr, (size_t)s->n * cap * sizeof(int)));
    CK(cudaMemsetAsync(s->nbr, 0xff, (size_t)s->n * cap * sizeof(int), s->stream));
    s->cap = cap;
    s->h.p.cap = cap;
    s->h.v.nbr = s->nbr;
    TRY(put_field(s, &s->d->v.nbr, s->nbr));
    TRY(put_field(s, &s->d->p.cap, cap));
    return DPG_OK;
}

static int enqueue_nlist(dpg_system *s) {
    if (s->method == DPG_NEIGH_CELL) LAUNCH(k_nlist_cell, s->grid(s->n), s->tpb, s->d);
    else LAUNCH(k_nlist_all, s->grid_full(s->n), kTPB, s->d);
    return DPG_OK;
}

// the rebuild kernels; each one checks DevState.rebuild itself
static int enqueue_rebuild(dpg_system *s) {
    if (s->method == DPG_NEIGH_CELL) {
        LAUNCH(k_cell_index, s->grid(s->n), s->tpb, s->d);
        LAUNCH(k_cell_scan, 1, kScanTPB, s->d);
        LAUNCH(k_cell_scatter, s->grid(s->n), s->tpb, s->d);
        LAUNCH(k_cell_sort, s->grid(s->ncells), s->tpb, s->d);
        LAUNCH(k_reorder, s->grid(s->n), s->tpb, s->d);
    }
    return enqueue_nlist(s);
}

static int pow2_ceil(int x) {
    return (int)std::pow(2, std::ceil(std::log2((double)x)));
}

// After a build: grow the capacity to the next power of two and rebuild the
// neighbour list when it overflowed (updateCellNeighborList /
// updateVerletList resize path, src/particles/base/particle.cu:1122-1130,1323-1330).
static int resolve_overflow(dpg_system *s) {
    for (int tries = 0; tries < 8; tries++) {
        TRY(pull_state(s));
        if (s->hs->flags & kError) return set_err(DPG_ERR_STATE, "device error flag set");
        if (!(s->hs->flags & kOverflow)) return DPG_OK;
        int mx = s->hs->max_count;
        int newcap = pow2_ceil(mx);
        if ((size_t)newcap * s->n > (size_t)1 << 31)
            return set_err(DPG_ERR_OVERFLOW, "neighbour list would exceed 2^31 entries (max count %d)", mx);
        TRY(alloc_nbr(s, newcap));
        TRY(put_field(s, &s->d->s.flags, s->hs->flags & ~kOverflow));
        TRY(put_field(s, &s->d->s.rebuild, 1));
        TRY(put_field(s, &s->d->s.n_rebuilds, s->hs->n_rebuilds - 1));
        TRY(enqueue_nlist(s));
    }
    return set_err(DPG_ERR_OVERFLOW, "neighbour capacity did not settle");
}

static int rebuild_now(dpg_system *s, int kind) {
    LAUNCH(k_set_rebuild, 1, 1, s->d, kind);
    TRY(enqueue_rebuild(s));
    return resolve_overflow(s);
}

extern "C" int dpg_setup_neighbors(dpg_handle s, const dpg_neighbor_config *cfg, dpg_neighbor_info *info) {
    if (!s || !cfg) return set_err(DPG_ERR_ARG, "null argument");
    if (!s->have_state) return set_err(DPG_ERR_STATE, "dpg_setup_neighbors: set positions and radii first");
    if (cfg->method < 0 || cfg->method > 2) return set_err(DPG_ERR_ARG, "bad neighbour method");
    free_graphs(s);
    const double cm = cfg->cutoff_multiplier, dm = cfg->displacement_multiplier;
    TRY(set_method(s, cfg->method));
    set_neighbor_size(s, cm, dm);
    if (s->method == DPG_NEIGH_CELL) {
        if (!set_cell_size(s, cfg->particles_per_cell, cfg->cell_displacement_multiplier))
            TRY(set_method(s, DPG_NEIGH_VERLET));
        if (!set_neighbor_size(s, cm, dm)) TRY(set_method(s, DPG_NEIGH_ALL));
    }
    if (s->method == DPG_NEIGH_VERLET) {
        if (!set_neighbor_size(s, cm, dm)) TRY(set_method(s, DPG_NEIGH_ALL));
    }
    if (s->method != DPG_NEIGH_CELL) { s->ncd = 0; s->ncells = 0; s->cs = -1; s->cthr2 = -1; }
    if (s->method == DPG_NEIGH_ALL) {
        s->cap = s->n - 1 > 0 ? s->n - 1 : 1;
        s->cutoff = 10.0 * std::sqrt(s->h.p.box[0] * s->h.p.box[0] + s->h.p.box[1] * s->h.p.box[1]);
        s->nthr2 = s->cutoff * s->cutoff;
    }
    // initVerletListVariables / initCellListVariables
    TRY(alloc_nbr(s, s->cap));
    CK(cudaMemsetAsync(s->h.w.count, 0, sizeof(int) * s->n, s->stream));
    CK(cudaMemsetAsync(s->h.w.pos_n, 0, 16 * (size_t)s->n, s->stream));
    CK(cudaMemsetAsync(s->h.w.pos_c, 0, 16 * (size_t)s->n, s->stream));
    if (s->method == DPG_NEIGH_CELL) {
        if (s->cell_buf) { CK(cudaStreamSynchronize(s->stream)); CK(cudaFree(s->cell_buf)); s->cell_buf = nullptr; }
        size_t nc = (size_t)s->ncells + 1;
        CK(cudaMalloc((void **)&s->cell_buf, 3 * nc * sizeof(int)));
        CK(cudaMemsetAsync(s->cell_buf, 0, 3 * nc * sizeof(int), s->stream));
        s->h.w.cell_cnt = s->cell_buf;
        s->h.w.cell_cur = s->cell_buf + nc;
        s->h.w.cell_start = s->cell_buf + 2 * nc;
        TRY(put_field(s, &s->d->w.cell_cnt, s->h.w.cell_cnt));
        TRY(put_field(s, &s->d->w.cell_cur, s->h.w.cell_cur));
        TRY(put_field(s, &s->d->w.cell_start, s->h.w.cell_start));
    }
    TRY(sync_neighbor_params(s));
    TRY(rebuild_now(s, s->method == DPG_NEIGH_CELL ? 2 : 1));
    s->have_neighbors = true;
    // setupNeighbors ends with calculateForces (accumulating)
    TRY(launch_force_acc(s));
    CK(cudaStreamSynchronize(s->stream));
    if (info) return dpg_neighbor_info_get(s, info);
    return DPG_OK;
}

extern "C" int dpg_neighbor_info_get(dpg_handle s, dpg_neighbor_info *info) {
    if (!s || !info) return set_err(DPG_ERR_ARG, "null argument");
    TRY(pull_state(s));
    info->method = s->method;
    info->capacity = s->cap;
    info->n_cells_dim = s->ncd;
    info->cutoff = s->cutoff;
    info->neighbor_threshold_sq = s->nthr2;
    info->cell_size = s->cs;
    info->cell_threshold_sq = s->cthr2;
    info->n_rebuilds = s->hs->n_rebuilds;
    info->n_cell_rebuilds = s->hs->n_cell_rebuilds;
    return DPG_OK;
}

static int need_neighbors(dpg_system *s) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (!s->have_neighbors) return set_err(DPG_ERR_STATE, "call dpg_setup_neighbors first");
    return DPG_OK;
}

extern "C" int dpg_build_neighbors(dpg_handle s) {
    TRY(need_neighbors(s));
    return rebuild_now(s, 1);
}

extern "C" int dpg_check_neighbors(dpg_handle s, int *rebuilt) {
    TRY(need_neighbors(s));
    LAUNCH(k_decide_rebuild, 1, 1, s->d);
    TRY(pull_state(s));
    int kind = s->hs->rebuild;
    if (rebuilt) *rebuilt = kind;
    if (kind == 0) return DPG_OK;
    TRY(enqueue_rebuild(s));
    return resolve_overflow(s);
}

extern "C" int dpg_get_neighbors(dpg_handle s, int32_t *list, int32_t *counts, int *cap) {
    TRY(need_neighbors(s));
    if (!cap) return set_err(DPG_ERR_ARG, "cap is required");
    int cap_out = *cap;
    *cap = s->cap;
    if (!list || !counts || cap_out <= 0) return DPG_OK;
    int *dl = nullptr, *dc = nullptr;
    CK(cudaMalloc((void **)&dl, (size_t)s->n * cap_out * sizeof(int)));
    CK(cudaMalloc((void **)&dc, (size_t)s->n * sizeof(int)));
    k_get_nbrs<<<s->grid(s->n), s->tpb, 0, s->stream>>>(s->d, dl, dc, cap_out);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(list, dl, (size_t)s->n * cap_out * 4, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(counts, dc, (size_t)s->n * 4, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(dl);
    cudaFree(dc);
    if (e != cudaSuccess) return set_err(DPG_ERR_CUDA, "get_neighbors: %s", cudaGetErrorString(e));
    return DPG_OK;
}

extern "C" int dpg_get_cells(dpg_handle s, int64_t *cell_index, int64_t *cell_start, int64_t *static_index) {
    TRY(need_neighbors(s));
    size_t nci = (size_t)s->n * 8, ncs = ((size_t)s->ncells + 1) * 8;
    long long *d = nullptr;
    CK(cudaMalloc((void **)&d, 2 * nci + ncs));
    long long *dci = d, *dsi = d + s->n, *dcs = d + 2 * (size_t)s->n;
    int g = s->grid(std::max(s->n, s->ncells + 1));
    k_get_cells<<<g, s->tpb, 0, s->stream>>>(s->d, dci, s->method == DPG_NEIGH_CELL ? dcs : nullptr, dsi);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && cell_index) e = cudaMemcpyAsync(cell_index, dci, nci, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess && static_index) e = cudaMemcpyAsync(static_index, dsi, nci, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess && cell_start && s->method == DPG_NEIGH_CELL)
        e = cudaMemcpyAsync(cell_start, dcs, ncs, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(d);
    if (e != cudaSuccess) return set_err(DPG_ERR_CUDA, "get_cells: %s", cudaGetErrorString(e));
    return DPG_OK;
}

// ---------------------------------------------------------------------------
// single operations
// ---------------------------------------------------------------------------
extern "C" int dpg_zero_forces(dpg_handle s) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    LAUNCH(k_zero_force, s->grid(s->n), s->tpb, s->d);
    return DPG_OK;
}

extern "C" int dpg_compute_forces(dpg_handle s) {
    TRY(need_neighbors(s));
    TRY(launch_force_acc(s));
    return DPG_OK;
}

extern "C" int dpg_kick(dpg_handle s, double dt) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    LAUNCH(k_kick, s->grid(s->n), s->tpb, s->d, dt);
    return DPG_OK;
}

extern "C" int dpg_drift(dpg_handle s, double dt) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    LAUNCH(k_drift, s->grid(s->n), s->tpb, s->d, dt);
    return DPG_OK;
}

extern "C" int dpg_mix(dpg_handle s, double alpha) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    LAUNCH(k_mix, s->grid(s->n), s->tpb, s->d, alpha);
    return DPG_OK;
}

extern "C" int dpg_zero_velocities(dpg_handle s) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    LAUNCH(k_zero_vel, s->grid(s->n), s->tpb, s->d);
    return DPG_OK;
}

static int observe(dpg_system *s) {
    LAUNCH(k_observables, s->grid(s->n), s->tpb, s->d);
    return pull_state(s);
}

extern "C" int dpg_power_fire(dpg_handle s, double *power) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    TRY(observe(s));
    if (power) *power = s->hs->power;
    return DPG_OK;
}

extern "C" int dpg_reduce_energies(dpg_handle s, double *pe, double *ke) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    TRY(observe(s));
    if (pe) *pe = s->hs->pe;
    if (ke) *ke = s->hs->ke;
    return DPG_OK;
}

extern "C" int dpg_force_stats(dpg_handle s, double *max_force, double *balance) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    TRY(observe(s));
    if (max_force) *max_force = std::sqrt(s->hs->fmax2);
    if (balance) *balance = std::sqrt(s->hs->fsum_x * s->hs->fsum_x + s->hs->fsum_y * s->hs->fsum_y);
    return DPG_OK;
}

extern "C" int dpg_pressure(dpg_handle s, double *pressure, double stress[4]) {
    TRY(need_neighbors(s));
    LAUNCH(k_stress, s->grid(s->n), s->tpb, s->d);
    TRY(pull_state(s));
    if (stress) for (int k = 0; k < 4; k++) stress[k] = s->hs->stress[k];
    if (pressure) *pressure = (s->hs->stress[0] + s->hs->stress[3]) / 2;
    return DPG_OK;
}

extern "C" int dpg_contact_count(dpg_handle s, double *contacts) {
    TRY(need_neighbors(s));
    LAUNCH(k_contacts, s->grid(s->n), s->tpb, s->d);
    TRY(pull_state(s));
    if (contacts) *contacts = s->hs->contacts;
    return DPG_OK;
}

extern "C" int dpg_packing_fraction(dpg_handle s, double *phi) {
    if (!s || !phi) return set_err(DPG_ERR_ARG, "null argument");
    double a;
    TRY(current_area(s, &a));
    *phi = a / box_area(s);
    return DPG_OK;
}

// updateCellSize: src/particles/base/particle.cu:1236-1240 (n_cells_dim frozen)
static int update_cell_size(dpg_system *s) {
    if (s->ncd > 0) {
        s->cs = s->h.p.box[0] / s->ncd;
        s->h.p.cell_size = s->cs;
    }
    return push_params(s);
}

extern "C" int dpg_scale_box(dpg_handle s, double factor) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (!(factor > 0)) return set_err(DPG_ERR_ARG, "factor must be > 0");
    LAUNCH(k_scale_pos, s->grid(s->n), s->tpb, s->d, factor);
    double l = std::pow(box_area(s), 1.0 / 2);
    double nl = l * factor;
    s->h.p.box[0] = nl;
    s->h.p.box[1] = nl;
    return update_cell_size(s);
}

extern "C" int dpg_scale_to_packing_fraction(dpg_handle s, double phi) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (!(phi > 0)) return set_err(DPG_ERR_ARG, "phi must be > 0");
    double a;
    TRY(current_area(s, &a));
    double new_l = std::pow(a / phi, 1.0 / 2);
    double l = std::pow(box_area(s), 1.0 / 2);
    double f = new_l / l;
    LAUNCH(k_scale_pos, s->grid(s->n), s->tpb, s->d, f);
    s->h.p.box[0] = new_l;
    s->h.p.box[1] = new_l;
    return update_cell_size(s);
}

extern "C" int dpg_save_state(dpg_handle s) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    LAUNCH(k_snapshot, s->grid(s->n), s->tpb, s->d, 0);
    s->h.w.s_box[0] = s->h.p.box[0];
    s->h.w.s_box[1] = s->h.p.box[1];
    return DPG_OK;
}

// revertToLastState: restore the arrays and the box, then updateNeighborList
// (neighbour list only; the cell arrays are left as they are, like the reference).
extern "C" int dpg_restore_state(dpg_handle s) {
    TRY(need_neighbors(s));
    LAUNCH(k_snapshot, s->grid(s->n), s->tpb, s->d, 1);
    s->h.p.box[0] = s->h.w.s_box[0];
    s->h.p.box[1] = s->h.w.s_box[1];
    TRY(push_params(s));
    return rebuild_now(s, 1);
}

// ---------------------------------------------------------------------------
// Adam
// ---------------------------------------------------------------------------
extern "C" int dpg_adam_init(dpg_handle s) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    DevView &v = s->h.v;
    // both the moments and their twins (whichever is current) start at zero
    double2 *bufs[4] = {v.m1, v.m2, v.m1_t, v.m2_t};
    for (double2 *b : bufs) CK(cudaMemsetAsync(b, 0, 16 * (size_t)s->n, s->stream));
    s->adam_ready = true;
    return DPG_OK;
}

extern "C" int dpg_adam_step(dpg_handle s, int64_t step, double alpha, double b1, double b2, double eps) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (!s->adam_ready) return set_err(DPG_ERR_STATE, "call dpg_adam_init first");
    double c1 = 1 - std::pow(b1, step + 1);
    double c2 = 1 - std::pow(b2, step + 1);
    LAUNCH(k_adam, s->grid(s->n), s->tpb, s->d, alpha, b1, b2, c1, c2, eps);
    return DPG_OK;
}

// minimizeAdam: src/routines/minimization.cu:3-33 (dof = 2N); the loop runs on
// the host like the reference's because each step's bias corrections are host
// scalars; the per-step PE reduction is one small readback.
extern "C" int dpg_adam_minimize(dpg_handle s, double alpha, double b1, double b2, double eps,
                                 double pe_target, double pe_diff_target, int64_t max_steps,
                                 int64_t *steps) {
    TRY(need_neighbors(s));
    TRY(dpg_adam_init(s));
    int64_t step = 0;
    double dof = (double)(2 * (int64_t)s->n), last = 0.0;
    while (step < max_steps) {
        LAUNCH(k_zero_force, s->grid(s->n), s->tpb, s->d);
        int rb = 0;
        TRY(dpg_check_neighbors(s, &rb));
        TRY(launch_force_acc(s));
        TRY(dpg_adam_step(s, step, alpha, b1, b2, eps));
        TRY(observe(s));
        double avg = s->hs->pe / dof;
        double diff = std::fabs(avg / last - 1);
        last = avg;
        if (diff < pe_diff_target || avg < pe_target) break;
        step++;
    }
    if (steps) *steps = step;
    return DPG_OK;
}

// ---------------------------------------------------------------------------
// device-resident loops
// ---------------------------------------------------------------------------
// rebuild kernels of one loop iteration, in order (they sit under the IF node)
struct KNode {
    void *fn;
    int blocks, threads;
};

static std::vector<KNode> rebuild_nodes(const dpg_system *s) {
    std::vector<KNode> rb;
    int G = s->grid(s->n);
    if (s->method == DPG_NEIGH_CELL) {
        rb.push_back({(void *)k_cell_index, G, s->tpb});
        rb.push_back({(void *)k_cell_scan, 1, kScanTPB});
        rb.push_back({(void *)k_cell_scatter, G, s->tpb});
        rb.push_back({(void *)k_cell_sort, s->grid(s->ncells), s->tpb});
        rb.push_back({(void *)k_reorder, G, s->tpb});
        rb.push_back({(void *)k_nlist_cell, G, s->tpb});
    } else {
        rb.push_back({(void *)k_nlist_all, s->grid_full(s->n), kTPB});
    }
    return rb;
}

// Launch one iteration directly on the stream (modes stream / chunked graph).
static int enqueue_iteration(dpg_system *s, int kind) {
    int G = s->grid(s->n);
    if (kind == kLoopFire) LAUNCH(k_fire_move, G, s->tpb, s->d);
    else LAUNCH(k_nve_first, G, s->tpb, s->d, 0.5 * s->chunk_dt, s->chunk_dt);
    TRY(enqueue_rebuild(s));
    if (kind == kLoopFire) TRY(launch_fire_force(s, 0));
    else TRY(launch_nve_second(s, 0.5 * s->chunk_dt));
    return DPG_OK;
}

static const int kChunk = 32;

static int build_chunk_graph(dpg_system *s, int kind) {
    if (s->chunk_exec[kind]) return DPG_OK;
    cudaGraph_t g;
    CK(cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal));
    int rc = DPG_OK;
    for (int i = 0; i < kChunk && rc == DPG_OK; i++) rc = enqueue_iteration(s, kind);
    cudaError_t e = cudaStreamEndCapture(s->stream, &g);
    if (rc != DPG_OK) return rc;
    CK(e);
    e = cudaGraphInstantiate(&s->chunk_exec[kind], g, 0);
    cudaGraphDestroy(g);
    CK(e);
    return DPG_OK;
}

static cudaGraphNode_t add_kernel(cudaGraph_t g, cudaGraphNode_t dep, void *fn, int blocks,
                                  int threads, void **args, cudaError_t *err) {
    cudaKernelNodeParams kp = {};
    kp.func = fn;
    kp.gridDim = dim3(blocks);
    kp.blockDim = dim3(threads);
    kp.sharedMemBytes = 0;
    kp.kernelParams = args;
    cudaGraphNode_t node = nullptr;
    cudaError_t e = cudaGraphAddKernelNode(&node, g, dep ? &dep : nullptr, dep ? 1 : 0, &kp);
    if (e != cudaSuccess && *err == cudaSuccess) *err = e;
    return node;
}

// WHILE(loop) { pre ; IF(rebuild) { rebuild kernels } ; post ; guard }
static int build_cond_graph(dpg_system *s, int kind) {
    if (s->loop_exec[kind]) return DPG_OK;
    cudaGraph_t g;
    CK(cudaGraphCreate(&g, 0));
    cudaError_t err = cudaSuccess;
    cudaGraphConditionalHandle hloop = 0, hrb = 0;
    err = cudaGraphConditionalHandleCreate(&hloop, g, 1, cudaGraphCondAssignDefault);
    cudaGraphNodeParams wp = {};
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = hloop;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wnode = nullptr;
    if (err == cudaSuccess) err = cudaGraphAddNode(&wnode, g, nullptr, nullptr, 0, &wp);
    cudaGraph_t body = (err == cudaSuccess) ? wp.conditional.phGraph_out[0] : nullptr;
    if (err == cudaSuccess) err = cudaGraphConditionalHandleCreate(&hrb, body, 0, 0);
    double dt_half_arg = 0.5 * s->chunk_dt, dt_arg = s->chunk_dt;  // copied at node creation
    int mode0 = 0;
    void *a_d[] = {&s->d};
    void *a_nve1[] = {&s->d, &dt_half_arg, &dt_arg};
    void *a_nve2[] = {&s->d, &dt_half_arg};
    void *a_ff[] = {&s->d, &mode0};
    int G = s->grid(s->n);
    cudaGraphNode_t last = nullptr;
    if (err == cudaSuccess) {
        if (kind == kLoopFire) last = add_kernel(body, nullptr, (void *)k_fire_move, G, s->tpb, a_d, &err);
        else last = add_kernel(body, nullptr, (void *)k_nve_first, G, s->tpb, a_nve1, &err);
    }
    cudaGraphNodeParams ip = {};
    ip.type = cudaGraphNodeTypeConditional;
    ip.conditional.handle = hrb;
    ip.conditional.type = cudaGraphCondTypeIf;
    ip.conditional.size = 1;
    cudaGraphNode_t inode = nullptr;
    if (err == cudaSuccess) err = cudaGraphAddNode(&inode, body, &last, nullptr, 1, &ip);
    if (err == cudaSuccess) {
        cudaGraph_t ib = ip.conditional.phGraph_out[0];
        cudaGraphNode_t prev = nullptr;
        for (auto &k : rebuild_nodes(s)) prev = add_kernel(ib, prev, k.fn, k.blocks, k.threads, a_d, &err);
        last = inode;
        if (kind == kLoopFire) last = add_kernel(body, last, s->fire_force_fn(), s->fgrid(), s->ftpb, a_ff, &err);
        else last = add_kernel(body, last, s->nve_second_fn(), s->fgrid(), s->ftpb, a_nve2, &err);
        last = add_kernel(body, last, (void *)k_loop_guard, 1, 1, a_d, &err);
    }
    if (err == cudaSuccess) err = cudaGraphInstantiate(&s->loop_exec[kind], g, 0);
    cudaGraphDestroy(g);
    if (err != cudaSuccess) {
        s->loop_exec[kind] = nullptr;
        return set_err(DPG_ERR_CUDA, "conditional graph: %s", cudaGetErrorString(err));
    }
    s->h_loop[kind] = hloop;
    s->h_rb[kind] = hrb;
    return DPG_OK;
}

// Run iterations until the device says done (or halts on overflow).
// Returns after a host-visible stop; *halted_overflow tells the caller to
// finish the interrupted iteration.
static int run_loop(dpg_system *s, int kind, int *halted_overflow) {
    *halted_overflow = 0;
    TRY(mixed_refresh(s));
    if (s->mode == kModeCond) {
        int rc = build_cond_graph(s, kind);
        if (rc != DPG_OK) {
            fprintf(stderr, "dpg: %s; falling back to chunked graphs\n", g_err);
            s->mode = kModeGraph;
        } else {
            TRY(put_field(s, &s->d->s.h_loop, (unsigned long long)s->h_loop[kind]));
            TRY(put_field(s, &s->d->s.h_rb, (unsigned long long)s->h_rb[kind]));
            CK(cudaGraphLaunch(s->loop_exec[kind], s->stream));
            TRY(put_field(s, &s->d->s.h_loop, 0ULL));
            TRY(put_field(s, &s->d->s.h_rb, 0ULL));
            TRY(pull_state(s));
            if (s->hs->flags & kOverflow) *halted_overflow = 1;
            return DPG_OK;
        }
    }
    for (;;) {
        if (s->mode == kModeGraph) {
            TRY(build_chunk_graph(s, kind));
            CK(cudaGraphLaunch(s->chunk_exec[kind], s->stream));
        } else {
            for (int i = 0; i < kChunk; i++) TRY(enqueue_iteration(s, kind));
        }
        TRY(pull_state(s));
        if (s->hs->flags & kOverflow) { *halted_overflow = 1; return DPG_OK; }
        if (s->hs->flags) return DPG_OK;
    }
}

// Overflow mid-loop: grow, rebuild the list for the current positions, then
// run the interrupted iteration's second half.
static int finish_after_overflow(dpg_system *s, int kind) {
    TRY(resolve_overflow(s));
    if (kind == kLoopFire) TRY(launch_fire_force(s, 0));
    else TRY(launch_nve_second(s, 0.5 * s->chunk_dt));
    return pull_state(s);
}

extern "C" int dpg_nve_steps(dpg_handle s, double dt, int64_t n_steps) {
    TRY(need_neighbors(s));
    if (n_steps <= 0) return DPG_OK;
    if (s->chunk_dt != dt) {  // dt is baked into the graphs
        free_graphs(s);
        s->chunk_dt = dt;
    }
    TRY(put_field(s, &s->d->s.flags, 0));
    TRY(put_field(s, &s->d->s.nve_steps_done, 0LL));
    TRY(put_field(s, &s->d->s.max_steps, (long long)n_steps));
    for (int attempt = 0; attempt < 64; attempt++) {
        TRY(put_field(s, &s->d->s.guard, 0LL));
        TRY(put_field(s, &s->d->s.guard_limit, (long long)n_steps + 4));
        int ovf = 0;
        TRY(run_loop(s, kLoopNve, &ovf));
        if (ovf) TRY(finish_after_overflow(s, kLoopNve));
        if (s->hs->nve_steps_done >= n_steps) break;
        if (s->hs->flags & kError) return set_err(DPG_ERR_STATE, "NVE loop guard tripped");
        TRY(put_field(s, &s->d->s.flags, 0));
    }
    TRY(pull_state(s));
    if (s->hs->nve_steps_done != n_steps)
        return set_err(DPG_ERR_STATE, "NVE loop ended after %lld of %lld steps",
                       s->hs->nve_steps_done, (long long)n_steps);
    TRY(put_field(s, &s->d->s.flags, 0));
    return DPG_OK;
}

extern "C" int dpg_set_mixed_switch(dpg_handle s, double switch_fmax) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (!s->mixed) return set_err(DPG_ERR_STATE, "not a DPG_MIXED system");
    if (!(switch_fmax >= 0)) return set_err(DPG_ERR_ARG, "switch_fmax must be >= 0");
    s->switch_fmax = switch_fmax;
    return DPG_OK;
}

// ---- damped NVE and gradient descent -------------------------------------
extern "C" int dpg_damped_forces(dpg_handle s, double damping) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    LAUNCH(k_damp, s->grid(s->n), s->tpb, s->d, damping);
    return DPG_OK;
}

extern "C" int dpg_damped_nve_steps(dpg_handle s, double dt, double damping, int64_t n_steps) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    TRY(put_field(s, &s->d->s.damping, damping));
    int rc = dpg_nve_steps(s, dt, n_steps);
    int rc2 = put_field(s, &s->d->s.damping, 0.0);
    return rc != DPG_OK ? rc : rc2;
}

extern "C" int dpg_pair_dump(dpg_handle s, double *const *out, int64_t *this_id,
                             int64_t *other_id, int where) {
    TRY(need_neighbors(s));
    if (!out || !this_id || !other_id) return set_err(DPG_ERR_ARG, "dpg_pair_dump: null argument");
    if (where != DPG_HOST && where != DPG_DEVICE) return set_err(DPG_ERR_ARG, "bad where");
    const long long m = (long long)s->n * s->cap;
    PairOut o{};
    std::vector<void *> tmp;
    auto release = [&]() { for (void *p : tmp) cudaFree(p); };
    for (int k = 0; k < 16; k++) {
        if (!out[k]) continue;
        if (where == DPG_DEVICE) { o.d[k] = out[k]; continue; }
        void *p = nullptr;
        cudaError_t e = cudaMalloc(&p, 8 * (size_t)m);
        if (e != cudaSuccess) { release(); return set_err(DPG_ERR_CUDA, "pair dump: %s", cudaGetErrorString(e)); }
        tmp.push_back(p);
        o.d[k] = (double *)p;
    }
    if (where == DPG_DEVICE) {
        o.this_id = (long long *)this_id;
        o.other_id = (long long *)other_id;
    } else {
        void *a = nullptr, *b = nullptr;
        cudaError_t e = cudaMalloc(&a, 8 * (size_t)m);
        if (e == cudaSuccess) { tmp.push_back(a); e = cudaMalloc(&b, 8 * (size_t)m); }
        if (e != cudaSuccess) { release(); return set_err(DPG_ERR_CUDA, "pair dump: %s", cudaGetErrorString(e)); }
        tmp.push_back(b);
        o.this_id = (long long *)a;
        o.other_id = (long long *)b;
    }
    const int fb = (int)((m + 255) / 256);
    k_pair_fill<<<fb, 256, 0, s->stream>>>(o, m);
    k_pair_dump<<<s->grid(s->n), s->tpb, 0, s->stream>>>(s->d, o);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && where == DPG_HOST) {
        for (int k = 0; k < 16 && e == cudaSuccess; k++)
            if (out[k]) e = cudaMemcpyAsync(out[k], o.d[k], 8 * (size_t)m, cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(this_id, o.this_id, 8 * (size_t)m, cudaMemcpyDeviceToHost, s->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(other_id, o.other_id, 8 * (size_t)m, cudaMemcpyDeviceToHost, s->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    release();
    if (e != cudaSuccess) return set_err(DPG_ERR_CUDA, "pair dump: %s", cudaGetErrorString(e));
    return DPG_OK;
}

extern "C" int dpg_wall_forces(dpg_handle s) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    LAUNCH(k_wall_force, s->grid(s->n), s->tpb, s->d);
    return DPG_OK;
}

extern "C" int dpg_nve_wall_steps(dpg_handle s, double dt, int64_t n_steps) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    TRY(put_field(s, &s->d->s.walls, 1));
    int rc = dpg_nve_steps(s, dt, n_steps);
    int rc2 = put_field(s, &s->d->s.walls, 0);
    return rc != DPG_OK ? rc : rc2;
}

extern "C" int dpg_grad_desc_step(dpg_handle s, double alpha) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    LAUNCH(k_grad_desc, s->grid(s->n), s->tpb, s->d, alpha);
    return DPG_OK;
}

extern "C" int dpg_grad_desc_steps(dpg_handle s, double alpha, int64_t n_steps) {
    TRY(need_neighbors(s));
    for (int64_t t = 0; t < n_steps; t++) {
        TRY(dpg_zero_forces(s));
        TRY(dpg_check_neighbors(s, nullptr));
        TRY(launch_force_acc(s));
        TRY(dpg_grad_desc_step(s, alpha));
    }
    return DPG_OK;
}

// ---- FIRE ---------------------------------------------------------------
extern "C" int dpg_fire_init(dpg_handle s, double alpha_init, double dt) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    DevState st;
    TRY(pull_state(s));
    st = *s->hs;
    st.f_alpha = alpha_init; st.f_alpha0 = alpha_init; st.f_dt = dt;
    st.f_dtmax = 10.0 * dt; st.f_dtmin = 0.001 * dt;
    st.f_ngood = 0; st.f_nbad = 0; st.f_stopped = 0; st.f_converged = 0;
    st.fire_uphill = 0;
    CK(cudaMemcpyAsync(&s->d->s, &st, sizeof(DevState), cudaMemcpyHostToDevice, s->stream));
    return DPG_OK;
}

extern "C" int dpg_fire_get(dpg_handle s, double *alpha, double *dt, int64_t *n_good, int64_t *n_bad, int *stopped) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    TRY(pull_state(s));
    if (alpha) *alpha = s->hs->f_alpha;
    if (dt) *dt = s->hs->f_dt;
    if (n_good) *n_good = s->hs->f_ngood;
    if (n_bad) *n_bad = s->hs->f_nbad;
    if (stopped) *stopped = s->hs->f_stopped;
    return DPG_OK;
}

// Fire::step: power and decision, move, neighbour check, forces, kick.
extern "C" int dpg_fire_step(dpg_handle s, int *stopped) {
    TRY(need_neighbors(s));
    TRY(put_field(s, &s->d->s.flags, 0));
    LAUNCH(k_fire_power_decide, s->grid(s->n), s->tpb, s->d);
    LAUNCH(k_fire_move, s->grid(s->n), s->tpb, s->d);
    TRY(enqueue_rebuild(s));
    TRY(resolve_overflow(s));
    TRY(launch_fire_force(s, 2));
    TRY(pull_state(s));
    if (stopped) *stopped = s->hs->f_stopped;
    TRY(put_field(s, &s->d->s.flags, 0));
    return DPG_OK;
}

extern "C" int dpg_fire_minimize(dpg_handle s, const dpg_fire_params *p, dpg_fire_result *r) {
    TRY(need_neighbors(s));
    if (!p) return set_err(DPG_ERR_ARG, "null params");
    if (p->max_steps <= 0) return set_err(DPG_ERR_ARG, "max_steps must be > 0");
    TRY(dpg_fire_init(s, p->alpha_init, p->dt));
    TRY(pull_state(s));
    DevState st = *s->hs;
    st.flags = 0;
    st.iter = 0;
    st.max_steps = p->max_steps;
    st.result_step = 0;
    st.pe_target = p->avg_pe_target;
    st.pe_diff_target = p->avg_pe_diff_target;
    st.fmax_target = p->fmax_target;
    st.dof = (double)s->n;
    st.guard = 0;
    st.guard_limit = p->max_steps + 4;
    st.h_loop = 0;
    st.h_rb = 0;
    st.fp64_now = 0;  // mixed form: FP32 pairs first, FP64 refinement after the switch
    st.switch_fmax = s->switch_fmax;
    st.best_f2 = INFINITY;
    st.best_it = 0;
    CK(cudaMemcpyAsync(&s->d->s, &st, sizeof(DevState), cudaMemcpyHostToDevice, s->stream));
    // minimizeFire setup: v = 0, zero, neighbour check, forces, last PE
    LAUNCH(k_zero_vel, s->grid(s->n), s->tpb, s->d);
    LAUNCH(k_decide_rebuild, 1, 1, s->d);
    TRY(enqueue_rebuild(s));
    TRY(resolve_overflow(s));
    TRY(launch_fire_force(s, 1));
    for (int guard = 0; guard < 64; guard++) {
        TRY(pull_state(s));
        if (s->hs->flags & kDone) break;
        int ovf = 0;
        TRY(run_loop(s, kLoopFire, &ovf));
        if (ovf) TRY(finish_after_overflow(s, kLoopFire));
        if (s->hs->flags & kDone) break;
        TRY(put_field(s, &s->d->s.guard, 0LL));
        TRY(put_field(s, &s->d->s.flags, s->hs->flags & kDone));
    }
    TRY(pull_state(s));
    if (!(s->hs->flags & kDone)) return set_err(DPG_ERR_STATE, "FIRE loop did not finish");
    // minimizeFire ends with setVelocitiesToZero
    LAUNCH(k_zero_vel, s->grid(s->n), s->tpb, s->d);
    TRY(observe(s));
    TRY(put_field(s, &s->d->s.fp64_now, 0));  // later calls start in FP32 again
    if (r) {
        r->steps = s->hs->result_step;
        r->stopped = s->hs->f_stopped;
        r->converged = s->hs->f_converged;
        r->avg_pe = s->hs->pe / (double)s->n;
        r->max_force = std::sqrt(s->hs->fmax2);
        r->alpha = s->hs->f_alpha;
        r->dt = s->hs->f_dt;
    }
    TRY(put_field(s, &s->d->s.flags, 0));
    return DPG_OK;
}

// ---------------------------------------------------------------------------
// measurement hook
// ---------------------------------------------------------------------------
extern "C" int dpg_profile_loop(dpg_handle s, int kind, int iters, double dt, double *avg_us,
                                int64_t *counts) {
    TRY(need_neighbors(s));
    if (iters <= 0 || (kind != 0 && kind != 1)) return set_err(DPG_ERR_ARG, "bad profile arguments");
    TRY(pull_state(s));
    long long nb0 = s->hs->n_rebuilds, nc0 = s->hs->n_cell_rebuilds;
    if (kind == 0) {
        dpg_fire_params p = {0.1, dt > 0 ? dt : 1e-2, 0.0, 0.0, (int64_t)iters + 1, 0.0};
        TRY(dpg_fire_init(s, p.alpha_init, p.dt));
        TRY(pull_state(s));
        DevState st = *s->hs;
        st.flags = 0; st.iter = 0; st.max_steps = p.max_steps; st.pe_target = 0; st.pe_diff_target = 0;
        st.fmax_target = 0; st.dof = (double)s->n; st.h_loop = 0; st.h_rb = 0;
        CK(cudaMemcpyAsync(&s->d->s, &st, sizeof(DevState), cudaMemcpyHostToDevice, s->stream));
        LAUNCH(k_zero_vel, s->grid(s->n), s->tpb, s->d);
        LAUNCH(k_decide_rebuild, 1, 1, s->d);
        TRY(enqueue_rebuild(s));
        TRY(resolve_overflow(s));
        TRY(launch_fire_force(s, 1));
    } else {
        TRY(put_field(s, &s->d->s.flags, 0));
        TRY(put_field(s, &s->d->s.nve_steps_done, 0LL));
        TRY(put_field(s, &s->d->s.max_steps, (long long)iters + 1));
    }
    TRY(mixed_refresh(s));
    std::vector<cudaEvent_t> ev(4 * (size_t)iters);
    for (auto &e : ev) CK(cudaEventCreate(&e));
    int rc = DPG_OK;
    int G = s->grid(s->n);
    for (int i = 0; i < iters && rc == DPG_OK; i++) {
        cudaEventRecord(ev[4 * i + 0], s->stream);
        if (kind == 0) k_fire_move<<<G, s->tpb, 0, s->stream>>>(s->d);
        else k_nve_first<<<G, s->tpb, 0, s->stream>>>(s->d, 0.5 * dt, dt);
        cudaEventRecord(ev[4 * i + 1], s->stream);
        rc = enqueue_rebuild(s);
        cudaEventRecord(ev[4 * i + 2], s->stream);
        if (rc == DPG_OK) rc = (kind == 0) ? launch_fire_force(s, 0) : launch_nve_second(s, 0.5 * dt);
        cudaEventRecord(ev[4 * i + 3], s->stream);
    }
    cudaError_t e = cudaStreamSynchronize(s->stream);
    double acc[3] = {0, 0, 0};
    if (rc == DPG_OK && e == cudaSuccess) {
        for (int i = 0; i < iters; i++)
            for (int k = 0; k < 3; k++) {
                float ms = 0;
                cudaEventElapsedTime(&ms, ev[4 * i + k], ev[4 * i + k + 1]);
                acc[k] += ms * 1e3;
            }
    }
    for (auto &x : ev) cudaEventDestroy(x);
    if (rc != DPG_OK) return rc;
    if (e != cudaSuccess) return set_err(DPG_ERR_CUDA, "profile: %s", cudaGetErrorString(e));
    TRY(pull_state(s));
    if (s->hs->flags & kOverflow) return set_err(DPG_ERR_OVERFLOW, "profile run overflowed the neighbour list");
    for (int k = 0; k < 3; k++) avg_us[k] = acc[k] / iters;
    if (counts) {
        counts[0] = iters;
        counts[1] = s->hs->n_rebuilds - nb0;
        counts[2] = s->hs->n_cell_rebuilds - nc0;
    }
    TRY(put_field(s, &s->d->s.flags, 0));
    return DPG_OK;
}

// ---------------------------------------------------------------------------
// threads per particle of the FP64 force kernels
// ---------------------------------------------------------------------------
extern "C" int dpg_set_force_group(dpg_handle s, int lanes) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8)
        return set_err(DPG_ERR_ARG, "lanes per particle must be 1, 2, 4 or 8");
    if (s->mixed && lanes != 1) return set_err(DPG_ERR_ARG, "DPG_MIXED systems use one lane per particle");
    if (s->fg != lanes) {
        s->fg = lanes;
        free_graphs(s);  // the graphs hold the kernels and grids of the old group
    }
    return DPG_OK;
}

// Autotuner for the threads per particle of the FP64 force kernels (every
// group gives bit-identical sums): times `iters` force passes with 1, 2, 4 and
// 8 lanes per particle on the current positions and lists (CUDA events on the
// system's stream), keeps the fastest, and restores the forces and energies.
extern "C" int dpg_autotune_force_group(dpg_handle s, int iters, int *chosen, double *us_per_pass) {
    TRY(need_neighbors(s));
    if (iters <= 0) return set_err(DPG_ERR_ARG, "iters must be > 0");
    if (s->mixed) {
        if (chosen) *chosen = 1;
        return DPG_OK;
    }
    DevView v;
    CK(cudaMemcpyAsync(&v, &s->d->v, sizeof(DevView), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    double2 *f_save = nullptr;
    double *pe_save = nullptr;
    CK(cudaMalloc((void **)&f_save, 16 * (size_t)s->n));
    cudaError_t e = cudaMalloc((void **)&pe_save, 8 * (size_t)s->n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(f_save, v.frc, 16 * (size_t)s->n, cudaMemcpyDeviceToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(pe_save, s->h.w.pe, 8 * (size_t)s->n, cudaMemcpyDeviceToDevice, s->stream);
    cudaEvent_t a = nullptr, b = nullptr;
    if (e == cudaSuccess) e = cudaEventCreate(&a);
    if (e == cudaSuccess) e = cudaEventCreate(&b);
    const int groups[4] = {1, 2, 4, 8};
    double best_us = INFINITY;
    int best = s->fg, rc = DPG_OK;
    for (int k = 0; k < 4 && e == cudaSuccess && rc == DPG_OK; k++) {
        s->fg = groups[k];
        rc = launch_force_acc(s);  // untimed first pass
        e = cudaEventRecord(a, s->stream);
        for (int t = 0; t < iters && rc == DPG_OK; t++) rc = launch_force_acc(s);
        if (e == cudaSuccess) e = cudaEventRecord(b, s->stream);
        if (e == cudaSuccess) e = cudaEventSynchronize(b);
        float ms = 0.f;
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, b);
        const double us = 1e3 * ms / iters;
        if (us_per_pass) us_per_pass[k] = us;
        if (us < best_us) { best_us = us; best = groups[k]; }
    }
    s->fg = best;
    free_graphs(s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(v.frc, f_save, 16 * (size_t)s->n, cudaMemcpyDeviceToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->h.w.pe, pe_save, 8 * (size_t)s->n, cudaMemcpyDeviceToDevice, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    cudaFree(f_save);
    cudaFree(pe_save);
    if (rc != DPG_OK) return rc;
    if (e != cudaSuccess) return set_err(DPG_ERR_CUDA, "autotune: %s", cudaGetErrorString(e));
    if (chosen) *chosen = best;
    return DPG_OK;
}
