// bumpy_system.cu -- host side of the plain FP64 rigid-bumpy system and its C
// ABI (dpg_bumpy_* in include/dpg.h).  Compiled with --fmad=false.
//
// The body-level cell list and body neighbour list reuse the disk kernels (the
// bodies sit in the embedded DevSys); the vertex list, vertex forces and the
// rigid-body integration are the kernels in bumpy_kernels.cuh.  Loops are
// device-resident CUDA graphs (WHILE node, rebuild under an IF node), as for
// disks.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "bumpy_kernels.cuh"
#include "host_common.h"

using namespace dpg;

#define CK DPG_CK
#define TRY DPG_TRY
#define set_err dpg::set_error

struct dpg_bumpy_system {
    int nb = 0, nv = 0;
    dpg_bumpy_params prm{};
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    BumpySys *d = nullptr;
    BumpySys h{};
    DevState *hs = nullptr;
    BumpyExt *hx = nullptr;  // pinned readback of the extension block
    std::vector<double> h_rad;
    bool have_state = false, have_neighbors = false;
    int method = -1, ncd = 0, ncells = 0, cap = 4, capv = 4;
    double cutoff = -1, nthr2 = -1, cs = -1, cthr2 = -1, vcutoff = -1, vpcutoff = -1;
    std::vector<void *> allocs;
    int *nbr = nullptr, *vnbr = nullptr, *cell_buf = nullptr;
    double *xfer = nullptr;
    int mode = 2;
    cudaGraphExec_t loop_exec[2] = {nullptr, nullptr};
    cudaGraphConditionalHandle h_loop[2] = {0, 0}, h_rb[2] = {0, 0};
    double loop_dt = 0.0, loop_tmax = 0.0;
    bool adam_ready = false, have_snapshot = false;
    double snap_box[2] = {0.0, 0.0};
    double switch_fmax = 1e-6;  // mixed form: FP32 vertex pairs until max(|F|, |tau|) <= this
    int gb(int count) const { return std::max(1, (count + kTPB - 1) / kTPB); }
    int gw(int bodies) const { return std::max(1, (bodies + kWarpsPerBlock - 1) / kWarpsPerBlock); }
    DevSys *ds() const { return &d->b; }
};

typedef dpg_bumpy_system BS;

#define LAUNCH(kern, blocks, threads, ...)                        \
    do {                                                          \
        kern<<<(blocks), (threads), 0, s->stream>>>(__VA_ARGS__); \
        CK(cudaGetLastError());                                   \
    } while (0)

// mixed form: vertex offsets from the current vertex positions, before a force
// evaluation that follows host-side or single-operation changes (the loop
// kernels keep them current themselves)
static int vrefresh(BS *s) {
    if (s->prm.precision != DPG_MIXED) return DPG_OK;
    kb_mixed_refresh<<<(s->nv + kTPB - 1) / kTPB, kTPB, 0, s->stream>>>(s->d);
    CK(cudaGetLastError());
    return DPG_OK;
}

static int balloc(BS *s, void **p, size_t bytes) {
    CK(cudaMalloc(p, bytes > 0 ? bytes : 16));
    CK(cudaMemsetAsync(*p, 0, bytes > 0 ? bytes : 16, s->stream));
    s->allocs.push_back(*p);
    return DPG_OK;
}

template <class T>
static int put(BS *s, T *dev, const T &v) {
    CK(cudaMemcpyAsync(dev, &v, sizeof(T), cudaMemcpyHostToDevice, s->stream));
    return DPG_OK;
}

static int pull(BS *s) {
    CK(cudaMemcpyAsync(s->hs, &s->d->b.s, sizeof(DevState), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaMemcpyAsync(s->hx, &s->d->x, sizeof(BumpyExt), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return DPG_OK;
}

static void free_graphs(BS *s) {
    for (int k = 0; k < 2; k++) {
        if (s->loop_exec[k]) cudaGraphExecDestroy(s->loop_exec[k]);
        s->loop_exec[k] = nullptr;
    }
}

extern "C" int dpg_bumpy_destroy(dpg_bumpy_handle s) {
    if (!s) return DPG_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    free_graphs(s);
    for (void *p : s->allocs) cudaFree(p);
    if (s->nbr) cudaFree(s->nbr);
    if (s->vnbr) cudaFree(s->vnbr);
    if (s->cell_buf) cudaFree(s->cell_buf);
    if (s->hs) cudaFreeHost(s->hs);
    if (s->hx) cudaFreeHost(s->hx);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return DPG_OK;
}

extern "C" int dpg_bumpy_create(const dpg_bumpy_params *p, void *cuda_stream, dpg_bumpy_handle *out) {
    if (!p || !out) return set_err(DPG_ERR_ARG, "dpg_bumpy_create: null argument");
    if (p->n_bodies <= 0 || p->n_vertices < p->n_bodies || p->n_vertices > (1LL << 30))
        return set_err(DPG_ERR_ARG, "dpg_bumpy_create: need 1 <= n_bodies <= n_vertices <= 2^30");
    if (!(p->box_x > 0) || !(p->box_y > 0) || !(p->vertex_radius > 0))
        return set_err(DPG_ERR_ARG, "dpg_bumpy_create: box and vertex radius must be > 0");
    if (p->precision != DPG_FP64 && p->precision != DPG_MIXED)
        return set_err(DPG_ERR_ARG, "dpg_bumpy_create: precision must be DPG_FP64 or DPG_MIXED");
    BS *s = new BS();
    s->nb = (int)p->n_bodies;
    s->nv = (int)p->n_vertices;
    s->prm = *p;
    if (cuda_stream) {
        s->stream = (cudaStream_t)cuda_stream;
    } else {
        cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { delete s; return set_err(DPG_ERR_CUDA, "stream: %s", cudaGetErrorString(e)); }
        s->own_stream = true;
    }
    const char *m = getenv("DPG_LOOP_MODE");
    if (m && (!strcmp(m, "stream") || !strcmp(m, "graph"))) s->mode = 0;
    const size_t nb = s->nb, nv = s->nv;
    int rc = DPG_OK;
    auto A = [&](void **pp, size_t b) { if (rc == DPG_OK) rc = balloc(s, pp, b); };
    DevView &v = s->h.b.v;
    DevScratch &w = s->h.b.w;
    BumpyExt &x = s->h.x;
    A((void **)&v.pos, nb * 16); A((void **)&v.vel, nb * 16); A((void **)&v.frc, nb * 16);
    A((void **)&v.rad, nb * 8); A((void **)&v.mass, nb * 8); A((void **)&v.sidx, nb * 4);
    A((void **)&v.pos_t, nb * 16); A((void **)&v.vel_t, nb * 16); A((void **)&v.frc_t, nb * 16);
    A((void **)&v.rad_t, nb * 8); A((void **)&v.mass_t, nb * 8); A((void **)&v.sidx_t, nb * 4);
    A((void **)&v.m1, nb * 16); A((void **)&v.m2, nb * 16); A((void **)&v.m1_t, nb * 16); A((void **)&v.m2_t, nb * 16);
    A((void **)&w.pos_n, nb * 16); A((void **)&w.pos_c, nb * 16); A((void **)&w.pe, nb * 8);
    A((void **)&w.count, nb * 4); A((void **)&w.cell_raw, nb * 4); A((void **)&w.cell_of, nb * 4);
    A((void **)&w.perm, nb * 4);
    w.max_blocks = std::max(s->gb(s->nb), s->gw(s->nb));
    A((void **)&w.partials, (size_t)w.max_blocks * 8 * 8);
    A((void **)&x.w, nb * 8); A((void **)&x.th, nb * 8); A((void **)&x.tq, nb * 8); A((void **)&x.I, nb * 8);
    A((void **)&x.nvb, nb * 4); A((void **)&x.start, nb * 4);
    A((void **)&x.w_t, nb * 8); A((void **)&x.th_t, nb * 8); A((void **)&x.tq_t, nb * 8); A((void **)&x.I_t, nb * 8);
    A((void **)&x.nvb_t, nb * 4); A((void **)&x.start_t, nb * 4); A((void **)&x.o2n, nb * 4);
    A((void **)&x.vpos, nv * 16); A((void **)&x.vpos_t, nv * 16); A((void **)&x.vmass, nv * 8);
    A((void **)&x.vmass_t, nv * 8); A((void **)&x.vbody, nv * 4); A((void **)&x.vbody_t, nv * 4);
    A((void **)&x.svidx, nv * 4); A((void **)&x.svidx_t, nv * 4); A((void **)&x.vcount, nv * 4);
    if (p->precision == DPG_MIXED) A((void **)&x.vpk, nv * 16);
    A((void **)&x.adelta, nb * 8); A((void **)&x.m1a, nb * 8); A((void **)&x.m2a, nb * 8);
    A((void **)&x.stress_b, nb * 32); A((void **)&x.ccount, nb * 4); A((void **)&x.vccount, nb * 4);
    A((void **)&w.s_pos, nb * 16); A((void **)&w.s_vel, nb * 16); A((void **)&w.s_frc, nb * 16);
    A((void **)&w.s_rad, nb * 8); A((void **)&w.s_mass, nb * 8); A((void **)&w.s_sidx, nb * 4);
    A((void **)&x.s_w, nb * 8); A((void **)&x.s_th, nb * 8); A((void **)&x.s_tq, nb * 8);
    A((void **)&x.s_nvb, nb * 4); A((void **)&x.s_start, nb * 4); A((void **)&x.s_vpos, nv * 16);
    A((void **)&x.s_vbody, nv * 4); A((void **)&x.s_svidx, nv * 4);
    A((void **)&s->xfer, std::max(nb * 32, nv * 16));  // also 4 doubles per body (stress)
    A((void **)&s->d, sizeof(BumpySys));
    if (rc == DPG_OK) {
        cudaError_t e = cudaMallocHost((void **)&s->hs, sizeof(DevState));
        if (e == cudaSuccess) e = cudaMallocHost((void **)&s->hx, sizeof(BumpyExt));
        if (e != cudaSuccess) rc = set_err(DPG_ERR_CUDA, "pinned: %s", cudaGetErrorString(e));
    }
    if (rc != DPG_OK) { dpg_bumpy_destroy(s); return rc; }
    DevParams &pp = s->h.b.p;
    // the body kernels shared with disks run in FP64; the mixed form lives in
    // the vertex kernels (BumpyExt.mixed, vpk) on the same mixed grid
    pp.n = s->nb; pp.method = -1; pp.cap = 4; pp.precision = DPG_FP64;
    pp.box[0] = p->box_x; pp.box[1] = p->box_y; pp.e_c = p->e_c; pp.n_c = p->n_c;
    if (p->precision == DPG_MIXED) {
        mixed_grid_init(pp);
        mixed_grid_update(pp);
    }
    memset(&s->h.b.s, 0, sizeof(DevState));
    x.nv = s->nv; x.capv = 4; x.rotation = p->rotation ? 1 : 0; x.rv = p->vertex_radius;
    x.mixed = p->precision == DPG_MIXED ? 1 : 0;
    x.vlist_built = 0;
    s->h_rad.assign(nb, 0.0);
    cudaError_t e = cudaMemcpyAsync(s->d, &s->h, sizeof(BumpySys), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) {
        k_iota_sidx<<<s->gb(s->nb), kTPB, 0, s->stream>>>(&s->d->b);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) { dpg_bumpy_destroy(s); return set_err(DPG_ERR_CUDA, "create: %s", cudaGetErrorString(e)); }
    *out = s;
    return DPG_OK;
}

// ---------------------------------------------------------------------------
// state
// ---------------------------------------------------------------------------
static int to_dev(BS *s, const double *src, size_t count, int slot, const double **dev) {
    if (!src) { *dev = nullptr; return DPG_OK; }
    size_t n = std::max(s->nb, s->nv);
    double *dst = s->xfer + (size_t)slot * n;
    CK(cudaMemcpyAsync(dst, src, sizeof(double) * count, cudaMemcpyHostToDevice, s->stream));
    *dev = dst;
    return DPG_OK;
}

// Re-sorts swap buffers on the device; a fresh set of bodies restarts from the
// host's buffer assignment.
static int reset_views(BS *s) {
    CK(cudaMemcpyAsync(&s->d->b.v, &s->h.b.v, sizeof(DevView), cudaMemcpyHostToDevice, s->stream));
    BumpyExt cur;
    CK(cudaMemcpyAsync(&cur, &s->d->x, sizeof(BumpyExt), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    const BumpyExt &h = s->h.x;
    cur.w = h.w; cur.th = h.th; cur.tq = h.tq; cur.I = h.I; cur.nvb = h.nvb; cur.start = h.start;
    cur.w_t = h.w_t; cur.th_t = h.th_t; cur.tq_t = h.tq_t; cur.I_t = h.I_t; cur.nvb_t = h.nvb_t;
    cur.start_t = h.start_t; cur.vpos = h.vpos; cur.vpos_t = h.vpos_t; cur.vmass = h.vmass;
    cur.vmass_t = h.vmass_t; cur.vbody = h.vbody; cur.vbody_t = h.vbody_t; cur.svidx = h.svidx;
    cur.svidx_t = h.svidx_t;
    CK(cudaMemcpyAsync(&s->d->x, &cur, sizeof(BumpyExt), cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return DPG_OK;
}

extern "C" int dpg_bumpy_set_bodies(dpg_bumpy_handle s, const double *x, const double *y,
                                    const double *angle, const double *vx, const double *vy,
                                    const double *omega, const double *radii, const int32_t *nvb) {
    if (!s || !x || !y || !radii || !nvb) return set_err(DPG_ERR_ARG, "dpg_bumpy_set_bodies: null argument");
    long long tot = 0;
    for (int b = 0; b < s->nb; b++) {
        if (nvb[b] < 1) return set_err(DPG_ERR_ARG, "every body needs at least one vertex");
        tot += nvb[b];
    }
    if (tot != s->nv) return set_err(DPG_ERR_ARG, "vertex counts sum to %lld, expected %d", tot, s->nv);
    TRY(reset_views(s));
    // bodies are still in input order here (no cell sort yet): plain copies
    std::vector<double> zeros(s->nb, 0.0);
    std::vector<double2> buf(s->nb);
    for (int b = 0; b < s->nb; b++) buf[b] = make_double2(x[b], y[b]);
    CK(cudaMemcpyAsync(s->h.b.v.pos, buf.data(), 16 * (size_t)s->nb, cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    for (int b = 0; b < s->nb; b++) buf[b] = make_double2(vx ? vx[b] : 0.0, vy ? vy[b] : 0.0);
    CK(cudaMemcpyAsync(s->h.b.v.vel, buf.data(), 16 * (size_t)s->nb, cudaMemcpyHostToDevice, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    CK(cudaMemcpyAsync(s->h.b.v.rad, radii, 8 * (size_t)s->nb, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(s->h.x.th, angle ? angle : zeros.data(), 8 * (size_t)s->nb, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(s->h.x.w, omega ? omega : zeros.data(), 8 * (size_t)s->nb, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(s->h.x.nvb, nvb, 4 * (size_t)s->nb, cudaMemcpyHostToDevice, s->stream));
    std::vector<int> start(s->nb);
    int acc = 0;
    for (int b = 0; b < s->nb; b++) { start[b] = acc; acc += nvb[b]; }
    CK(cudaMemcpyAsync(s->h.x.start, start.data(), 4 * (size_t)s->nb, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemsetAsync(s->h.x.adelta, 0, 8 * (size_t)s->nb, s->stream));
    LAUNCH(k_iota_sidx, s->gb(s->nb), kTPB, &s->d->b);
    LAUNCH(kb_index_vertices, s->gw(s->nb), kTPB, s->d);
    LAUNCH(kb_init_vertices, s->gw(s->nb), kTPB, s->d);
    CK(cudaStreamSynchronize(s->stream));
    memcpy(s->h_rad.data(), radii, 8 * (size_t)s->nb);
    s->have_state = true;
    return DPG_OK;
}

extern "C" int dpg_bumpy_set_vertices(dpg_bumpy_handle s, const double *px, const double *py) {
    if (!s || !px || !py) return set_err(DPG_ERR_ARG, "null argument");
    const double *dx, *dy;
    TRY(to_dev(s, px, s->nv, 0, &dx));
    TRY(to_dev(s, py, s->nv, 1, &dy));
    LAUNCH(kb_put_vertices, s->gb(s->nv), kTPB, s->d, dx, dy);
    CK(cudaStreamSynchronize(s->stream));
    return DPG_OK;
}

extern "C" int dpg_bumpy_set_mass(dpg_bumpy_handle s, double mass) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (!(mass > 0)) return set_err(DPG_ERR_ARG, "mass must be > 0");
    LAUNCH(kb_set_mass, s->gw(s->nb), kTPB, s->d, mass);
    return DPG_OK;
}

extern "C" int dpg_bumpy_get_bodies(dpg_bumpy_handle s, double *x, double *y, double *angle,
                                    double *vx, double *vy, double *omega, double *fx,
                                    double *fy, double *torque, double *pe, double *inertia) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    const size_t n = s->nb, nb8 = 8 * n;
    double *d0 = s->xfer, *d1 = s->xfer + n;
    double *xy[3][2] = {{x, y}, {vx, vy}, {fx, fy}};
    for (int k = 0; k < 3; k++) {
        if (!xy[k][0] && !xy[k][1]) continue;
        LAUNCH(k_get_xy, s->gb(s->nb), kTPB, &s->d->b, k, d0, d1);
        if (xy[k][0]) CK(cudaMemcpyAsync(xy[k][0], d0, nb8, cudaMemcpyDeviceToHost, s->stream));
        if (xy[k][1]) CK(cudaMemcpyAsync(xy[k][1], d1, nb8, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    double *sc[4] = {angle, omega, torque, inertia};
    for (int k = 0; k < 4; k++) {
        if (!sc[k]) continue;
        LAUNCH(kb_get_body_scalar, s->gb(s->nb), kTPB, s->d, k, d0);
        CK(cudaMemcpyAsync(sc[k], d0, nb8, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    if (pe) {
        LAUNCH(k_get_pe, s->gb(s->nb), kTPB, &s->d->b, d0);
        CK(cudaMemcpyAsync(pe, d0, nb8, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    return DPG_OK;
}

extern "C" int dpg_bumpy_get_vertices(dpg_bumpy_handle s, double *px, double *py) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    size_t n = std::max(s->nb, s->nv);
    double *d0 = s->xfer, *d1 = s->xfer + n;
    LAUNCH(kb_get_vertices, s->gb(s->nv), kTPB, s->d, d0, d1);
    if (px) CK(cudaMemcpyAsync(px, d0, 8 * (size_t)s->nv, cudaMemcpyDeviceToHost, s->stream));
    if (py) CK(cudaMemcpyAsync(py, d1, 8 * (size_t)s->nv, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return DPG_OK;
}

// ---------------------------------------------------------------------------
// neighbours (Particle::setupNeighbors with the RigidBumpy overrides)
// ---------------------------------------------------------------------------
static double bmaxd(const BS *s) { return 2.0 * *std::max_element(s->h_rad.begin(), s->h_rad.end()); }
static double barea(const BS *s) { return 1.0 * s->h.b.p.box[0] * s->h.b.p.box[1]; }

static bool set_neighbor_size(BS *s, double cm, double dm) {
    s->cap = 4; s->capv = 4;
    s->cutoff = cm * bmaxd(s);
    s->vcutoff = cm * 2.0 * s->prm.vertex_radius;
    s->vpcutoff = bmaxd(s);
    s->nthr2 = std::pow(dm * s->prm.segment_length_per_vertex_diameter * s->prm.vertex_radius, 2);
    double diag = std::sqrt(s->h.b.p.box[0] * s->h.b.p.box[0] + s->h.b.p.box[1] * s->h.b.p.box[1]);
    return s->cutoff < diag;
}

static bool set_cell_size(BS *s, double ppc, double cdm) {
    const int min_dim = 4;
    double density = s->nb / barea(s);
    double trial = std::sqrt(ppc / density);
    double min_cs = 2.0 * bmaxd(s);
    s->ncd = (int)std::floor(s->h.b.p.box[0] / trial);
    s->ncells = s->ncd * s->ncd;
    if (s->ncd < min_dim) { s->ncd = min_dim; s->ncells = s->ncd * s->ncd; }
    s->cs = s->h.b.p.box[0] / s->ncd;
    if (s->cs < min_cs) {
        s->cs = min_cs;
        s->ncd = (int)std::floor(s->h.b.p.box[0] / s->cs);
        s->ncells = s->ncd * s->ncd;
        if (s->ncd < min_dim) return false;
    }
    s->cthr2 = std::pow(cdm * s->cs, 2);
    return true;
}

static int set_method(BS *s, int m) {
    s->method = m;
    LAUNCH(k_iota_sidx, s->gb(s->nb), kTPB, &s->d->b);
    if (m == DPG_NEIGH_ALL) {
        double diag = std::sqrt(s->h.b.p.box[0] * s->h.b.p.box[0] + s->h.b.p.box[1] * s->h.b.p.box[1]);
        set_neighbor_size(s, 2.0 * diag / bmaxd(s), 0.0);
    }
    return DPG_OK;
}

static int alloc_lists(BS *s, int cap, int capv) {
    CK(cudaStreamSynchronize(s->stream));
    if (cap != s->h.b.p.cap || !s->nbr) {
        if (s->nbr) CK(cudaFree(s->nbr));
        CK(cudaMalloc((void **)&s->nbr, (size_t)s->nb * cap * 4));
        CK(cudaMemsetAsync(s->nbr, 0xff, (size_t)s->nb * cap * 4, s->stream));
        s->cap = cap;
        s->h.b.p.cap = cap;
        s->h.b.v.nbr = s->nbr;
        TRY(put(s, &s->d->b.v.nbr, s->nbr));
        TRY(put(s, &s->d->b.p.cap, cap));
    }
    if (capv != s->h.x.capv || !s->vnbr) {
        if (s->vnbr) CK(cudaFree(s->vnbr));
        CK(cudaMalloc((void **)&s->vnbr, (size_t)s->nv * capv * 4));
        CK(cudaMemsetAsync(s->vnbr, 0xff, (size_t)s->nv * capv * 4, s->stream));
        s->capv = capv;
        s->h.x.capv = capv;
        s->h.x.vnbr = s->vnbr;
        TRY(put(s, &s->d->x.vnbr, s->vnbr));
        TRY(put(s, &s->d->x.capv, capv));
    }
    return DPG_OK;
}

static int enqueue_rebuild(BS *s) {
    DevSys *ds = &s->d->b;
    if (s->method == DPG_NEIGH_CELL) {
        LAUNCH(k_cell_index, s->gb(s->nb), kTPB, ds);
        LAUNCH(k_cell_scan, 1, kScanTPB, ds);
        LAUNCH(k_cell_scatter, s->gb(s->nb), kTPB, ds);
        LAUNCH(k_cell_sort, s->gb(s->ncells), kTPB, ds);
        LAUNCH(kb_reorder_bodies, s->gb(s->nb), kTPB, s->d);
        LAUNCH(kb_scan_starts, 1, kScanTPB, s->d);
        LAUNCH(kb_reorder_vertices, s->gw(s->nb), kTPB, s->d);
        LAUNCH(k_nlist_cell, s->gb(s->nb), kTPB, ds);
    } else {
        LAUNCH(k_nlist_all, s->gb(s->nb), kTPB, ds);
    }
    LAUNCH(kb_vlist, s->gw(s->nb), kTPB, s->d);
    return DPG_OK;
}

static int pow2ceil(int x) { return (int)std::pow(2, std::ceil(std::log2((double)x))); }

// grow whichever list overflowed (power of two) and rebuild it, as the
// reference's updateCellNeighborList / updateVertexVerletList resize paths
static int resolve_overflow(BS *s) {
    for (int tries = 0; tries < 8; tries++) {
        TRY(pull(s));
        if (!(s->hs->flags & kOverflow)) return DPG_OK;
        int mb = s->hs->max_count, mv = s->hx->max_vcount;
        bool body = mb > s->cap;
        int ncap = body ? pow2ceil(mb) : s->cap;
        int ncapv = (!body && mv > s->capv) ? pow2ceil(mv) : s->capv;
        if ((size_t)ncapv * s->nv > ((size_t)1 << 31) || (size_t)ncap * s->nb > ((size_t)1 << 31))
            return set_err(DPG_ERR_OVERFLOW, "neighbour list would exceed 2^31 entries");
        TRY(alloc_lists(s, ncap, ncapv));
        TRY(put(s, &s->d->b.s.flags, s->hs->flags & ~kOverflow));
        if (body) {
            TRY(put(s, &s->d->b.s.rebuild, 1));
            TRY(put(s, &s->d->b.s.n_rebuilds, s->hs->n_rebuilds - 1));
            // the vertex list was built from the truncated body list: rebuild it too
            TRY(put(s, &s->d->x.vlist_built, -1LL));
            if (s->method == DPG_NEIGH_CELL) LAUNCH(k_nlist_cell, s->gb(s->nb), kTPB, &s->d->b);
            else LAUNCH(k_nlist_all, s->gb(s->nb), kTPB, &s->d->b);
        } else {
            TRY(put(s, &s->d->x.vlist_built, s->hs->n_rebuilds - 1));
        }
        LAUNCH(kb_vlist, s->gw(s->nb), kTPB, s->d);
    }
    return set_err(DPG_ERR_OVERFLOW, "neighbour capacity did not settle");
}

static int rebuild_now(BS *s, int kind) {
    LAUNCH(k_set_rebuild, 1, 1, &s->d->b, kind);
    TRY(enqueue_rebuild(s));
    return resolve_overflow(s);
}

extern "C" int dpg_bumpy_neighbor_info_get(dpg_bumpy_handle s, dpg_neighbor_info *info, int *vcap) {
    if (!s || !info) return set_err(DPG_ERR_ARG, "null argument");
    TRY(pull(s));
    info->method = s->method;
    info->capacity = s->cap;
    info->n_cells_dim = s->ncd;
    info->cutoff = s->cutoff;
    info->neighbor_threshold_sq = s->nthr2;
    info->cell_size = s->cs;
    info->cell_threshold_sq = s->cthr2;
    info->n_rebuilds = s->hs->n_rebuilds;
    info->n_cell_rebuilds = s->hs->n_cell_rebuilds;
    if (vcap) *vcap = s->capv;
    return DPG_OK;
}

extern "C" int dpg_bumpy_setup_neighbors(dpg_bumpy_handle s, const dpg_neighbor_config *cfg,
                                         dpg_neighbor_info *info) {
    if (!s || !cfg) return set_err(DPG_ERR_ARG, "null argument");
    if (!s->have_state) return set_err(DPG_ERR_STATE, "set the bodies first");
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
        s->cap = std::max(1, s->nb - 1);
        s->cutoff = 10.0 * std::sqrt(s->h.b.p.box[0] * s->h.b.p.box[0] + s->h.b.p.box[1] * s->h.b.p.box[1]);
        s->nthr2 = s->cutoff * s->cutoff;
    }
    s->h.b.p.cap = -1;  // force allocation
    s->h.x.capv = -1;
    TRY(alloc_lists(s, s->cap, s->capv));
    CK(cudaMemsetAsync(s->h.b.w.count, 0, 4 * (size_t)s->nb, s->stream));
    CK(cudaMemsetAsync(s->h.x.vcount, 0, 4 * (size_t)s->nv, s->stream));
    CK(cudaMemsetAsync(s->h.b.w.pos_n, 0, 16 * (size_t)s->nb, s->stream));
    CK(cudaMemsetAsync(s->h.b.w.pos_c, 0, 16 * (size_t)s->nb, s->stream));
    if (s->method == DPG_NEIGH_CELL) {
        if (s->cell_buf) { CK(cudaStreamSynchronize(s->stream)); CK(cudaFree(s->cell_buf)); s->cell_buf = nullptr; }
        size_t nc = (size_t)s->ncells + 1;
        CK(cudaMalloc((void **)&s->cell_buf, 3 * nc * 4));
        CK(cudaMemsetAsync(s->cell_buf, 0, 3 * nc * 4, s->stream));
        TRY(put(s, &s->d->b.w.cell_cnt, s->cell_buf));
        TRY(put(s, &s->d->b.w.cell_cur, s->cell_buf + nc));
        TRY(put(s, &s->d->b.w.cell_start, s->cell_buf + 2 * nc));
        LAUNCH(kb_index_vertices, s->gw(s->nb), kTPB, s->d);  // static vertex index = iota
    }
    DevParams &p = s->h.b.p;
    p.method = s->method; p.ncd = s->ncd; p.ncells = s->ncells; p.cap = s->cap;
    p.cutoff2 = s->cutoff * s->cutoff; p.cell_size = s->cs; p.nthr2 = s->nthr2; p.cthr2 = s->cthr2;
    mixed_grid_update(p);
    CK(cudaMemcpyAsync(&s->d->b.p, &p, sizeof(DevParams), cudaMemcpyHostToDevice, s->stream));
    TRY(put(s, &s->d->x.vcut2, s->vcutoff * s->vcutoff));
    TRY(put(s, &s->d->x.vpcut2, s->vpcutoff * s->vpcutoff));
    TRY(pull(s));
    TRY(put(s, &s->d->x.vlist_built, s->hs->n_rebuilds));
    TRY(rebuild_now(s, s->method == DPG_NEIGH_CELL ? 2 : 1));
    s->have_neighbors = true;
    TRY(vrefresh(s));
    LAUNCH(kb_force_acc, s->gw(s->nb), kTPB, s->d, 0);
    CK(cudaStreamSynchronize(s->stream));
    if (info) return dpg_bumpy_neighbor_info_get(s, info, nullptr);
    return DPG_OK;
}

static int need(BS *s) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (!s->have_neighbors) return set_err(DPG_ERR_STATE, "call dpg_bumpy_setup_neighbors first");
    return DPG_OK;
}

extern "C" int dpg_bumpy_check_neighbors(dpg_bumpy_handle s, int *rebuilt) {
    TRY(need(s));
    LAUNCH(k_decide_rebuild, 1, 1, &s->d->b);
    TRY(pull(s));
    int kind = s->hs->rebuild;
    if (rebuilt) *rebuilt = kind;
    if (kind == 0) return DPG_OK;
    TRY(enqueue_rebuild(s));
    return resolve_overflow(s);
}

extern "C" int dpg_bumpy_get_vertex_neighbors(dpg_bumpy_handle s, int32_t *list, int32_t *counts, int *cap) {
    TRY(need(s));
    if (!cap) return set_err(DPG_ERR_ARG, "cap is required");
    int cap_out = *cap;
    *cap = s->capv;
    if (!list || !counts || cap_out <= 0) return DPG_OK;
    int *dl = nullptr, *dc = nullptr;
    CK(cudaMalloc((void **)&dl, (size_t)s->nv * cap_out * 4));
    CK(cudaMalloc((void **)&dc, (size_t)s->nv * 4));
    kb_get_vnbrs<<<s->gb(s->nv), kTPB, 0, s->stream>>>(s->d, dl, dc, cap_out);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(list, dl, (size_t)s->nv * cap_out * 4, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(counts, dc, (size_t)s->nv * 4, cudaMemcpyDeviceToHost, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(dl);
    cudaFree(dc);
    if (e != cudaSuccess) return set_err(DPG_ERR_CUDA, "get_vertex_neighbors: %s", cudaGetErrorString(e));
    return DPG_OK;
}

// ---------------------------------------------------------------------------
// single operations
// ---------------------------------------------------------------------------
extern "C" int dpg_bumpy_zero_forces(dpg_bumpy_handle s) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    LAUNCH(kb_zero_force, s->gb(s->nb), kTPB, s->d);
    return DPG_OK;
}

extern "C" int dpg_bumpy_compute_forces(dpg_bumpy_handle s) {
    TRY(need(s));
    TRY(vrefresh(s));
    LAUNCH(kb_force_acc, s->gw(s->nb), kTPB, s->d, 0);
    return DPG_OK;
}

extern "C" int dpg_bumpy_kick(dpg_bumpy_handle s, double dt) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    LAUNCH(kb_kick, s->gb(s->nb), kTPB, s->d, dt);
    return DPG_OK;
}

extern "C" int dpg_bumpy_drift(dpg_bumpy_handle s, double dt) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    LAUNCH(kb_drift, s->gw(s->nb), kTPB, s->d, dt);
    return DPG_OK;
}

extern "C" int dpg_bumpy_mix(dpg_bumpy_handle s, double alpha) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    LAUNCH(kb_mix, s->gb(s->nb), kTPB, s->d, alpha);
    return DPG_OK;
}

extern "C" int dpg_bumpy_zero_velocities(dpg_bumpy_handle s) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    LAUNCH(kb_zero_vel, s->gb(s->nb), kTPB, s->d);
    return DPG_OK;
}

extern "C" int dpg_bumpy_observables(dpg_bumpy_handle s, double *pe, double *ke, double *power,
                                     double *fmax, double *tmax) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    LAUNCH(kb_observables, s->gb(s->nb), kTPB, s->d);
    TRY(pull(s));
    if (pe) *pe = s->hs->pe;
    if (ke) *ke = s->hs->ke;
    if (power) *power = s->hs->power;
    if (fmax) *fmax = std::sqrt(s->hs->fmax2);
    if (tmax) *tmax = std::sqrt(s->hx->tmax2);
    return DPG_OK;
}

extern "C" int dpg_bumpy_scale_box(dpg_bumpy_handle s, double factor) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (!(factor > 0)) return set_err(DPG_ERR_ARG, "factor must be > 0");
    LAUNCH(kb_scale, s->gw(s->nb), kTPB, s->d, factor);
    double l = std::pow(barea(s), 1.0 / 2);
    double nl = l * factor;
    s->h.b.p.box[0] = nl;
    s->h.b.p.box[1] = nl;
    if (s->ncd > 0) { s->cs = nl / s->ncd; s->h.b.p.cell_size = s->cs; }
    mixed_grid_update(s->h.b.p);
    CK(cudaMemcpyAsync(&s->d->b.p, &s->h.b.p, sizeof(DevParams), cudaMemcpyHostToDevice, s->stream));
    return DPG_OK;
}

// ---------------------------------------------------------------------------
// device-resident loops
// ---------------------------------------------------------------------------
static cudaGraphNode_t addk(cudaGraph_t g, cudaGraphNode_t dep, void *fn, int blocks, int threads,
                            void **args, cudaError_t *err) {
    cudaKernelNodeParams kp = {};
    kp.func = fn;
    kp.gridDim = dim3(blocks);
    kp.blockDim = dim3(threads);
    kp.kernelParams = args;
    cudaGraphNode_t node = nullptr;
    cudaError_t e = cudaGraphAddKernelNode(&node, g, dep ? &dep : nullptr, dep ? 1 : 0, &kp);
    if (e != cudaSuccess && *err == cudaSuccess) *err = e;
    return node;
}

// kind 0 FIRE, 1 NVE
static int enqueue_iteration(BS *s, int kind) {
    if (kind == 0) LAUNCH(kb_fire_move, s->gw(s->nb), kTPB, s->d);
    else LAUNCH(kb_nve_first, s->gw(s->nb), kTPB, s->d, 0.5 * s->loop_dt, s->loop_dt);
    TRY(enqueue_rebuild(s));
    if (kind == 0) LAUNCH(kb_fire_force, s->gw(s->nb), kTPB, s->d, 0, s->loop_tmax);
    else LAUNCH(kb_nve_second, s->gw(s->nb), kTPB, s->d, 0.5 * s->loop_dt);
    return DPG_OK;
}

static int build_graph(BS *s, int kind) {
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
    cudaGraph_t body = err == cudaSuccess ? wp.conditional.phGraph_out[0] : nullptr;
    if (err == cudaSuccess) err = cudaGraphConditionalHandleCreate(&hrb, body, 0, 0);
    double dth = 0.5 * s->loop_dt, dt = s->loop_dt, tmax = s->loop_tmax;
    int mode0 = 0;
    BumpySys *bp = s->d;
    DevSys *dp = &s->d->b;
    void *a_b[] = {&bp};
    void *a_d[] = {&dp};
    void *a_n1[] = {&bp, &dth, &dt};
    void *a_n2[] = {&bp, &dth};
    void *a_ff[] = {&bp, &mode0, &tmax};
    int GW = s->gw(s->nb), GB = s->gb(s->nb);
    cudaGraphNode_t last = nullptr;
    if (err == cudaSuccess)
        last = kind == 0 ? addk(body, nullptr, (void *)kb_fire_move, GW, kTPB, a_b, &err)
                         : addk(body, nullptr, (void *)kb_nve_first, GW, kTPB, a_n1, &err);
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
        if (s->method == DPG_NEIGH_CELL) {
            prev = addk(ib, prev, (void *)k_cell_index, GB, kTPB, a_d, &err);
            prev = addk(ib, prev, (void *)k_cell_scan, 1, kScanTPB, a_d, &err);
            prev = addk(ib, prev, (void *)k_cell_scatter, GB, kTPB, a_d, &err);
            prev = addk(ib, prev, (void *)k_cell_sort, s->gb(s->ncells), kTPB, a_d, &err);
            prev = addk(ib, prev, (void *)kb_reorder_bodies, GB, kTPB, a_b, &err);
            prev = addk(ib, prev, (void *)kb_scan_starts, 1, kScanTPB, a_b, &err);
            prev = addk(ib, prev, (void *)kb_reorder_vertices, GW, kTPB, a_b, &err);
            prev = addk(ib, prev, (void *)k_nlist_cell, GB, kTPB, a_d, &err);
        } else {
            prev = addk(ib, prev, (void *)k_nlist_all, GB, kTPB, a_d, &err);
        }
        prev = addk(ib, prev, (void *)kb_vlist, GW, kTPB, a_b, &err);
        last = kind == 0 ? addk(body, inode, (void *)kb_fire_force, GW, kTPB, a_ff, &err)
                         : addk(body, inode, (void *)kb_nve_second, GW, kTPB, a_n2, &err);
        last = addk(body, last, (void *)k_loop_guard, 1, 1, a_d, &err);
    }
    if (err == cudaSuccess) err = cudaGraphInstantiate(&s->loop_exec[kind], g, 0);
    cudaGraphDestroy(g);
    if (err != cudaSuccess) {
        s->loop_exec[kind] = nullptr;
        return set_err(DPG_ERR_CUDA, "bumpy graph: %s", cudaGetErrorString(err));
    }
    s->h_loop[kind] = hloop;
    s->h_rb[kind] = hrb;
    return DPG_OK;
}

static int run_loop(BS *s, int kind, int *ovf) {
    *ovf = 0;
    TRY(vrefresh(s));
    if (s->mode == 2) {
        if (build_graph(s, kind) != DPG_OK) {
            s->mode = 0;
        } else {
            TRY(put(s, &s->d->b.s.h_loop, (unsigned long long)s->h_loop[kind]));
            TRY(put(s, &s->d->b.s.h_rb, (unsigned long long)s->h_rb[kind]));
            CK(cudaGraphLaunch(s->loop_exec[kind], s->stream));
            TRY(put(s, &s->d->b.s.h_loop, 0ULL));
            TRY(put(s, &s->d->b.s.h_rb, 0ULL));
            TRY(pull(s));
            if (s->hs->flags & kOverflow) *ovf = 1;
            return DPG_OK;
        }
    }
    for (;;) {
        for (int i = 0; i < 32; i++) TRY(enqueue_iteration(s, kind));
        TRY(pull(s));
        if (s->hs->flags & kOverflow) { *ovf = 1; return DPG_OK; }
        if (s->hs->flags) return DPG_OK;
    }
}

static int finish_after_overflow(BS *s, int kind) {
    TRY(resolve_overflow(s));
    if (kind == 0) LAUNCH(kb_fire_force, s->gw(s->nb), kTPB, s->d, 0, s->loop_tmax);
    else LAUNCH(kb_nve_second, s->gw(s->nb), kTPB, s->d, 0.5 * s->loop_dt);
    return pull(s);
}

extern "C" int dpg_bumpy_nve_steps(dpg_bumpy_handle s, double dt, int64_t n_steps) {
    TRY(need(s));
    if (n_steps <= 0) return DPG_OK;
    if (s->loop_dt != dt) { free_graphs(s); s->loop_dt = dt; }
    TRY(put(s, &s->d->b.s.flags, 0));
    TRY(put(s, &s->d->b.s.nve_steps_done, 0LL));
    TRY(put(s, &s->d->b.s.max_steps, (long long)n_steps));
    for (int attempt = 0; attempt < 64; attempt++) {
        TRY(put(s, &s->d->b.s.guard, 0LL));
        TRY(put(s, &s->d->b.s.guard_limit, (long long)n_steps + 4));
        int ovf = 0;
        TRY(run_loop(s, 1, &ovf));
        if (ovf) TRY(finish_after_overflow(s, 1));
        if (s->hs->nve_steps_done >= n_steps) break;
        if (s->hs->flags & kError) return set_err(DPG_ERR_STATE, "NVE loop guard tripped");
        TRY(put(s, &s->d->b.s.flags, 0));
    }
    TRY(pull(s));
    if (s->hs->nve_steps_done != n_steps) return set_err(DPG_ERR_STATE, "bumpy NVE loop incomplete");
    TRY(put(s, &s->d->b.s.flags, 0));
    return DPG_OK;
}

extern "C" int dpg_bumpy_fire_init(dpg_bumpy_handle s, double alpha, double dt) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    TRY(pull(s));
    DevState st = *s->hs;
    st.f_alpha = alpha; st.f_alpha0 = alpha; st.f_dt = dt;
    st.f_dtmax = 10.0 * dt; st.f_dtmin = 0.001 * dt;
    st.f_ngood = 0; st.f_nbad = 0; st.f_stopped = 0; st.f_converged = 0; st.fire_uphill = 0;
    CK(cudaMemcpyAsync(&s->d->b.s, &st, sizeof(DevState), cudaMemcpyHostToDevice, s->stream));
    return DPG_OK;
}

extern "C" int dpg_bumpy_fire_step(dpg_bumpy_handle s, int *stopped) {
    TRY(need(s));
    TRY(put(s, &s->d->b.s.flags, 0));
    LAUNCH(kb_fire_power_decide, s->gb(s->nb), kTPB, s->d);
    LAUNCH(kb_fire_move, s->gw(s->nb), kTPB, s->d);
    TRY(enqueue_rebuild(s));
    TRY(resolve_overflow(s));
    TRY(vrefresh(s));
    LAUNCH(kb_fire_force, s->gw(s->nb), kTPB, s->d, 2, 0.0);
    TRY(pull(s));
    if (stopped) *stopped = s->hs->f_stopped;
    TRY(put(s, &s->d->b.s.flags, 0));
    return DPG_OK;
}

extern "C" int dpg_bumpy_set_mixed_switch(dpg_bumpy_handle s, double switch_fmax) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (s->prm.precision != DPG_MIXED) return set_err(DPG_ERR_STATE, "not a DPG_MIXED system");
    if (!(switch_fmax >= 0)) return set_err(DPG_ERR_ARG, "switch_fmax must be >= 0");
    s->switch_fmax = switch_fmax;
    return DPG_OK;
}

extern "C" int dpg_bumpy_fire_minimize(dpg_bumpy_handle s, const dpg_fire_params *p, double tmax,
                                       dpg_fire_result *r) {
    TRY(need(s));
    if (!p || p->max_steps <= 0) return set_err(DPG_ERR_ARG, "bad FIRE parameters");
    if (s->loop_tmax != tmax) { free_graphs(s); s->loop_tmax = tmax; }
    TRY(dpg_bumpy_fire_init(s, p->alpha_init, p->dt));
    TRY(pull(s));
    DevState st = *s->hs;
    st.flags = 0; st.iter = 0; st.max_steps = p->max_steps; st.result_step = 0;
    st.pe_target = p->avg_pe_target; st.pe_diff_target = p->avg_pe_diff_target;
    st.fmax_target = p->fmax_target; st.dof = (double)s->nb;
    st.guard = 0; st.guard_limit = p->max_steps + 4; st.h_loop = 0; st.h_rb = 0;
    st.fp64_now = 0; st.switch_fmax = s->switch_fmax; st.best_f2 = INFINITY; st.best_it = 0;
    CK(cudaMemcpyAsync(&s->d->b.s, &st, sizeof(DevState), cudaMemcpyHostToDevice, s->stream));
    LAUNCH(kb_zero_vel, s->gb(s->nb), kTPB, s->d);
    LAUNCH(k_decide_rebuild, 1, 1, &s->d->b);
    TRY(enqueue_rebuild(s));
    TRY(resolve_overflow(s));
    TRY(vrefresh(s));
    LAUNCH(kb_fire_force, s->gw(s->nb), kTPB, s->d, 1, tmax);
    for (int guard = 0; guard < 64; guard++) {
        TRY(pull(s));
        if (s->hs->flags & kDone) break;
        int ovf = 0;
        TRY(run_loop(s, 0, &ovf));
        if (ovf) TRY(finish_after_overflow(s, 0));
        if (s->hs->flags & kDone) break;
        TRY(put(s, &s->d->b.s.guard, 0LL));
        TRY(put(s, &s->d->b.s.flags, s->hs->flags & kDone));
    }
    TRY(pull(s));
    if (!(s->hs->flags & kDone)) return set_err(DPG_ERR_STATE, "bumpy FIRE loop did not finish");
    LAUNCH(kb_zero_vel, s->gb(s->nb), kTPB, s->d);
    LAUNCH(kb_observables, s->gb(s->nb), kTPB, s->d);
    TRY(pull(s));
    TRY(put(s, &s->d->b.s.fp64_now, 0));  // later calls start in FP32 again
    if (r) {
        r->steps = s->hs->result_step;
        r->stopped = s->hs->f_stopped;
        r->converged = s->hs->f_converged;
        r->avg_pe = s->hs->pe / (double)s->nb;
        r->max_force = std::sqrt(s->hs->fmax2);
        r->alpha = s->hs->f_alpha;
        r->dt = s->hs->f_dt;
    }
    TRY(put(s, &s->d->b.s.flags, 0));
    return DPG_OK;
}

// ---------------------------------------------------------------------------
// Adam, damping, walls, stress, contacts, snapshots
// ---------------------------------------------------------------------------
extern "C" int dpg_bumpy_adam_init(dpg_bumpy_handle s) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    // every moment and the twins the translational ones swap with start at zero
    const DevView &v = s->h.b.v;
    double2 *bufs[4] = {v.m1, v.m2, v.m1_t, v.m2_t};
    for (double2 *b : bufs) CK(cudaMemsetAsync(b, 0, 16 * (size_t)s->nb, s->stream));
    CK(cudaMemsetAsync(s->h.x.m1a, 0, 8 * (size_t)s->nb, s->stream));
    CK(cudaMemsetAsync(s->h.x.m2a, 0, 8 * (size_t)s->nb, s->stream));
    s->adam_ready = true;
    return DPG_OK;
}

extern "C" int dpg_bumpy_adam_step(dpg_bumpy_handle s, int64_t step, double alpha, double b1,
                                   double b2, double eps) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (!s->adam_ready) return set_err(DPG_ERR_STATE, "call dpg_bumpy_adam_init first");
    const double c1 = 1 - std::pow(b1, step + 1), c2 = 1 - std::pow(b2, step + 1);
    LAUNCH(kb_adam, s->gw(s->nb), kTPB, s->d, alpha, b1, b2, c1, c2, eps);
    return DPG_OK;
}

// minimizeAdam (src/routines/minimization.cu:3-33) over Adam::minimize
// (src/integrator/adam.cu:11-17): zero, neighbour check, forces, Adam step,
// then the PE test on the host, as the reference (its bias corrections are
// host scalars)
extern "C" int dpg_bumpy_adam_minimize(dpg_bumpy_handle s, double alpha, double b1, double b2,
                                       double eps, double pe_target, double pe_diff_target,
                                       int64_t max_steps, int64_t *steps) {
    TRY(need(s));
    TRY(dpg_bumpy_adam_init(s));
    const double dof = (double)((int64_t)s->nb * (s->prm.rotation ? 3 : 2));
    double last = 0.0;
    int64_t step = 0;
    while (step < max_steps) {
        TRY(dpg_bumpy_zero_forces(s));
        TRY(dpg_bumpy_check_neighbors(s, nullptr));
        TRY(dpg_bumpy_compute_forces(s));
        TRY(dpg_bumpy_adam_step(s, step, alpha, b1, b2, eps));
        double pe = 0.0;
        TRY(dpg_bumpy_observables(s, &pe, nullptr, nullptr, nullptr, nullptr));
        const double avg = pe / dof, diff = std::fabs(avg / last - 1);
        last = avg;
        if (diff < pe_diff_target || avg < pe_target) break;
        step++;
    }
    if (steps) *steps = step;
    return DPG_OK;
}

extern "C" int dpg_bumpy_grad_desc_step(dpg_bumpy_handle s, double alpha) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    LAUNCH(kb_grad_desc, s->gw(s->nb), kTPB, s->d, alpha);
    return DPG_OK;
}

// GradDesc::step (src/integrator/grad_desc.cu:11-17) with the rigid step
extern "C" int dpg_bumpy_grad_desc_steps(dpg_bumpy_handle s, double alpha, int64_t n_steps) {
    TRY(need(s));
    for (int64_t t = 0; t < n_steps; t++) {
        TRY(dpg_bumpy_zero_forces(s));
        TRY(dpg_bumpy_check_neighbors(s, nullptr));
        TRY(dpg_bumpy_compute_forces(s));
        TRY(dpg_bumpy_grad_desc_step(s, alpha));
    }
    return DPG_OK;
}

extern "C" int dpg_bumpy_damped_forces(dpg_bumpy_handle s, double damping) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    LAUNCH(kb_damp, s->gb(s->nb), kTPB, s->d, damping);
    return DPG_OK;
}

extern "C" int dpg_bumpy_damped_nve_steps(dpg_bumpy_handle s, double dt, double damping,
                                          int64_t n_steps) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    TRY(put(s, &s->d->b.s.damping, damping));
    int rc = dpg_bumpy_nve_steps(s, dt, n_steps);
    int rc2 = put(s, &s->d->b.s.damping, 0.0);
    return rc != DPG_OK ? rc : rc2;
}

extern "C" int dpg_bumpy_wall_forces(dpg_bumpy_handle s, int with_pairs) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (with_pairs) {
        TRY(need(s));
        TRY(vrefresh(s));
        LAUNCH(kb_force_acc, s->gw(s->nb), kTPB, s->d, 1);
    } else {
        LAUNCH(kb_wall_only, s->gw(s->nb), kTPB, s->d);
    }
    return DPG_OK;
}

extern "C" int dpg_bumpy_nve_wall_steps(dpg_bumpy_handle s, double dt, int64_t n_steps) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    TRY(put(s, &s->d->b.s.walls, 1));
    int rc = dpg_bumpy_nve_steps(s, dt, n_steps);
    int rc2 = put(s, &s->d->b.s.walls, 0);
    return rc != DPG_OK ? rc : rc2;
}

extern "C" int dpg_bumpy_stress(dpg_bumpy_handle s, double *stress, double *pressure,
                                double *per_body) {
    TRY(need(s));
    LAUNCH(kb_stress, s->gb(s->nb), kTPB, s->d);
    if (per_body) {
        double *d0 = s->xfer;  // 4 * nb doubles fit: xfer holds 2 * max(nb, nv) double2
        LAUNCH(kb_get_stress_contacts, s->gb(s->nb), kTPB, s->d, d0, (int *)nullptr, (int *)nullptr);
        CK(cudaMemcpyAsync(per_body, d0, 32 * (size_t)s->nb, cudaMemcpyDeviceToHost, s->stream));
    }
    TRY(pull(s));
    const double *t = s->hs->stress;
    if (stress) for (int k = 0; k < 4; k++) stress[k] = t[k];
    if (pressure) *pressure = (t[0] + t[3]) / 2;
    return DPG_OK;
}

extern "C" int dpg_bumpy_contacts(dpg_bumpy_handle s, double *contacts, double *vertex_contacts,
                                  int32_t *per_body, int32_t *vertex_per_body) {
    TRY(need(s));
    LAUNCH(kb_contacts, s->gb(s->nb), kTPB, s->d);
    if (per_body || vertex_per_body) {
        int *c0 = (int *)s->xfer, *c1 = c0 + s->nb;
        LAUNCH(kb_get_stress_contacts, s->gb(s->nb), kTPB, s->d, (double *)nullptr, c0, c1);
        if (per_body) CK(cudaMemcpyAsync(per_body, c0, 4 * (size_t)s->nb, cudaMemcpyDeviceToHost, s->stream));
        if (vertex_per_body)
            CK(cudaMemcpyAsync(vertex_per_body, c1, 4 * (size_t)s->nb, cudaMemcpyDeviceToHost, s->stream));
    }
    TRY(pull(s));
    if (contacts) *contacts = s->hs->contacts;
    if (vertex_contacts) *vertex_contacts = s->hx->vcontacts;
    return DPG_OK;
}

extern "C" int dpg_bumpy_save_state(dpg_bumpy_handle s) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    LAUNCH(kb_snapshot, s->gb(std::max(s->nb, s->nv)), kTPB, s->d, 0);
    s->snap_box[0] = s->h.b.p.box[0];
    s->snap_box[1] = s->h.b.p.box[1];
    s->have_snapshot = true;
    return DPG_OK;
}

extern "C" int dpg_bumpy_restore_state(dpg_bumpy_handle s) {
    TRY(need(s));
    if (!s->have_snapshot) return set_err(DPG_ERR_STATE, "call dpg_bumpy_save_state first");
    LAUNCH(kb_snapshot, s->gb(std::max(s->nb, s->nv)), kTPB, s->d, 1);
    // Particle::setBoxSize: the box only; the cell size keeps its value
    s->h.b.p.box[0] = s->snap_box[0];
    s->h.b.p.box[1] = s->snap_box[1];
    mixed_grid_update(s->h.b.p);
    CK(cudaMemcpyAsync(&s->d->b.p, &s->h.b.p, sizeof(DevParams), cudaMemcpyHostToDevice, s->stream));
    TRY(rebuild_now(s, 1));
    return vrefresh(s);
}

extern "C" int dpg_bumpy_pair_dump(dpg_bumpy_handle s, double *const *out, int64_t *this_id,
                                   int64_t *other_id, int64_t *vertex_contacts, int where) {
    TRY(need(s));
    if (!out || !this_id || !other_id || !vertex_contacts)
        return set_err(DPG_ERR_ARG, "dpg_bumpy_pair_dump: null argument");
    if (where != DPG_HOST && where != DPG_DEVICE) return set_err(DPG_ERR_ARG, "bad where");
    const long long m = (long long)s->nb * s->cap;
    BumpyPairOut o{};
    std::vector<void *> tmp;
    auto release = [&]() { for (void *p : tmp) cudaFree(p); };
    auto dev = [&](void **p) -> int {
        cudaError_t e = cudaMalloc(p, 8 * (size_t)m);
        if (e != cudaSuccess) { release(); return set_err(DPG_ERR_CUDA, "pair dump: %s", cudaGetErrorString(e)); }
        tmp.push_back(*p);
        return DPG_OK;
    };
    for (int k = 0; k < kBumpyPairArrays; k++) {
        if (!out[k]) continue;
        if (where == DPG_DEVICE) { o.d[k] = out[k]; continue; }
        void *p = nullptr;
        TRY(dev(&p));
        o.d[k] = (double *)p;
    }
    int64_t *ids[3] = {this_id, other_id, vertex_contacts};
    long long **dst[3] = {&o.this_id, &o.other_id, &o.vcount};
    for (int k = 0; k < 3; k++) {
        if (where == DPG_DEVICE) { *dst[k] = (long long *)ids[k]; continue; }
        void *p = nullptr;
        TRY(dev(&p));
        *dst[k] = (long long *)p;
    }
    kb_pair_fill<<<(int)((m + kTPB - 1) / kTPB), kTPB, 0, s->stream>>>(o, m);
    kb_pair_dump<<<s->gb(s->nb), kTPB, 0, s->stream>>>(s->d, o);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && where == DPG_HOST) {
        for (int k = 0; k < kBumpyPairArrays && e == cudaSuccess; k++)
            if (out[k]) e = cudaMemcpyAsync(out[k], o.d[k], 8 * (size_t)m, cudaMemcpyDeviceToHost, s->stream);
        for (int k = 0; k < 3 && e == cudaSuccess; k++)
            e = cudaMemcpyAsync(ids[k], *dst[k], 8 * (size_t)m, cudaMemcpyDeviceToHost, s->stream);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    release();
    if (e != cudaSuccess) return set_err(DPG_ERR_CUDA, "pair dump: %s", cudaGetErrorString(e));
    return DPG_OK;
}

// ---------------------------------------------------------------------------
// static arrays and the box (state files)
// ---------------------------------------------------------------------------
extern "C" int dpg_bumpy_get_static(dpg_bumpy_handle s, double *radii, double *masses,
                                    int32_t *n_vertices_per_body, double *vertex_masses,
                                    double *box) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    // xfer holds max(4 nb, 2 nv) doubles: radii | masses | counts, then vertex masses
    double *d0 = s->xfer, *d1 = s->xfer + s->nb;
    int *c0 = (int *)(s->xfer + 2 * (size_t)s->nb);
    LAUNCH(kb_get_static, s->gb(std::max(s->nb, s->nv)), kTPB, s->d, radii ? d0 : nullptr,
           masses ? d1 : nullptr, n_vertices_per_body ? c0 : nullptr, (double *)nullptr);
    if (radii) CK(cudaMemcpyAsync(radii, d0, 8 * (size_t)s->nb, cudaMemcpyDeviceToHost, s->stream));
    if (masses) CK(cudaMemcpyAsync(masses, d1, 8 * (size_t)s->nb, cudaMemcpyDeviceToHost, s->stream));
    if (n_vertices_per_body)
        CK(cudaMemcpyAsync(n_vertices_per_body, c0, 4 * (size_t)s->nb, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    if (vertex_masses) {
        LAUNCH(kb_get_static, s->gb(std::max(s->nb, s->nv)), kTPB, s->d, (double *)nullptr,
               (double *)nullptr, (int *)nullptr, s->xfer);
        CK(cudaMemcpyAsync(vertex_masses, s->xfer, 8 * (size_t)s->nv, cudaMemcpyDeviceToHost, s->stream));
        CK(cudaStreamSynchronize(s->stream));
    }
    if (box) { box[0] = s->h.b.p.box[0]; box[1] = s->h.b.p.box[1]; }
    return DPG_OK;
}

extern "C" int dpg_bumpy_set_inertia(dpg_bumpy_handle s, const double *masses, const double *inertia,
                                     const double *vertex_masses) {
    if (!s || !masses || !inertia || !vertex_masses) return set_err(DPG_ERR_ARG, "null argument");
    if (!s->have_state) return set_err(DPG_ERR_STATE, "set the bodies first");
    const double *dm, *di, *dv;
    TRY(to_dev(s, masses, s->nb, 0, &dm));
    TRY(to_dev(s, inertia, s->nb, 1, &di));
    // vertex masses after the two body arrays: xfer holds 2 max(nb, nv) doubles,
    // so they go through a temporary
    double *tmp = nullptr;
    CK(cudaMalloc((void **)&tmp, 8 * (size_t)s->nv));
    cudaError_t e = cudaMemcpyAsync(tmp, vertex_masses, 8 * (size_t)s->nv, cudaMemcpyHostToDevice, s->stream);
    dv = tmp;
    if (e == cudaSuccess) {
        kb_put_mass<<<s->gb(std::max(s->nb, s->nv)), kTPB, 0, s->stream>>>(s->d, dm, di, dv);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    cudaFree(tmp);
    if (e != cudaSuccess) return set_err(DPG_ERR_CUDA, "set_inertia: %s", cudaGetErrorString(e));
    return DPG_OK;
}

// Particle::setBoxSize for rigid bodies: the box; the cell size follows the box
// as updateCellSize does when a cell list is set up
extern "C" int dpg_bumpy_set_box(dpg_bumpy_handle s, double bx, double by) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (!(bx > 0) || !(by > 0)) return set_err(DPG_ERR_ARG, "box must be > 0");
    s->h.b.p.box[0] = bx;
    s->h.b.p.box[1] = by;
    if (s->ncd > 0) { s->cs = bx / s->ncd; s->h.b.p.cell_size = s->cs; }
    mixed_grid_update(s->h.b.p);
    CK(cudaMemcpyAsync(&s->d->b.p, &s->h.b.p, sizeof(DevParams), cudaMemcpyHostToDevice, s->stream));
    return DPG_OK;
}

extern "C" int dpg_bumpy_counts(dpg_bumpy_handle s, int64_t *n_bodies, int64_t *n_vertices) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (n_bodies) *n_bodies = s->nb;
    if (n_vertices) *n_vertices = s->nv;
    return DPG_OK;
}
