// ensemble_system.cu -- host side of the batched form (dpg_ensemble_* in
// include/dpg.h): S disk systems of uneven size in shared, block-padded slot
// arrays; the whole minimisation / jamming run of all systems is one CUDA
// graph (WHILE node; the rebuild kernels sit under an IF node set by the move
// kernel when any system needs new lists).  Compiled with --fmad=false.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "host_common.h"
#include "resident_kernels.cuh"

using namespace dpg;

#define CK DPG_CK
#define TRY DPG_TRY
#define set_err dpg::set_error

struct dpg_ensemble_system {
    dpg_ensemble_params prm{};
    int S = 0, T = 0, nblocks = 0, total_cells = 0, cap = 32;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::vector<ESys> sys;      // host copy
    std::vector<int> src_index;  // slot -> input index (-1 padding)
    std::vector<long long> n;
    EDev h{};                    // host mirror of the device block
    EDev *d = nullptr;
    ESys *d_sys = nullptr;
    int *d_src = nullptr;
    std::vector<void *> allocs;
    double *xfer = nullptr;
    size_t n_total = 0;
    cudaGraphExec_t exec = nullptr;
    cudaGraphConditionalHandle h_loop = 0, h_rb = 0, h_tr = 0, h_f32 = 0, h_fhi = 0;
    bool have_state = false;
    int mode = 2;
    int form = DPG_FORM_AUTO, pthreads = 0;  // execution form and persistent block size
    int max_n = 0;
    bool split_force = false;    // grid form: FP32 and refinement force kernels apart
    long long launches = 0;      // kernel launches and graph launches issued for this ensemble
    // resident form: one stream per size class, the block -> system lists
    cudaStream_t rs_stream[8] = {};
    cudaEvent_t rs_fork = nullptr, rs_join[8] = {};
    int rs_fit[8] = {};          // clusters of each class the GPU holds at once (0: not yet asked)
    int rs_rot[8] = {};          // rotation of each class's systems between launches
    int *d_rs_blocks = nullptr;
};

typedef dpg_ensemble_system ES;

#define LAUNCH(kern, blocks, threads, ...)                        \
    do {                                                          \
        kern<<<(blocks), (threads), 0, s->stream>>>(__VA_ARGS__); \
        CK(cudaGetLastError());                                   \
        s->launches++;                                            \
    } while (0)

static int ealloc(ES *s, void **p, size_t bytes) {
    CK(cudaMalloc(p, bytes > 0 ? bytes : 16));
    CK(cudaMemsetAsync(*p, 0, bytes > 0 ? bytes : 16, s->stream));
    s->allocs.push_back(*p);
    return DPG_OK;
}

extern "C" int dpg_ensemble_destroy(dpg_ensemble s) {
    if (!s) return DPG_OK;
    if (s->stream) cudaStreamSynchronize(s->stream);
    for (int c = 0; c < 8; c++) {
        if (s->rs_stream[c]) cudaStreamDestroy(s->rs_stream[c]);
        if (s->rs_join[c]) cudaEventDestroy(s->rs_join[c]);
    }
    if (s->rs_fork) cudaEventDestroy(s->rs_fork);
    if (s->exec) cudaGraphExecDestroy(s->exec);
    for (void *p : s->allocs) cudaFree(p);
    if (s->h.nbr) cudaFree(s->h.nbr);
    if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
    delete s;
    return DPG_OK;
}

static int alloc_nbr(ES *s, int cap) {
    CK(cudaStreamSynchronize(s->stream));
    if (s->h.nbr) CK(cudaFree(s->h.nbr));
    CK(cudaMalloc((void **)&s->h.nbr, (size_t)s->T * cap * sizeof(int)));
    s->cap = cap;
    s->h.p.cap = cap;
    return DPG_OK;
}

extern "C" int dpg_ensemble_create(const dpg_ensemble_params *p, const int64_t *n_particles,
                                   const double *box, void *cuda_stream, dpg_ensemble *out) {
    if (!p || !n_particles || !box || !out) return set_err(DPG_ERR_ARG, "dpg_ensemble_create: null argument");
    if (p->n_systems <= 0 || p->n_systems > (1 << 20)) return set_err(DPG_ERR_ARG, "bad n_systems");
    if (!(p->cutoff > 0) || !(p->skin > 0)) return set_err(DPG_ERR_ARG, "cutoff and skin must be > 0");
    if (p->precision != DPG_FP64 && p->precision != DPG_MIXED) return set_err(DPG_ERR_ARG, "bad precision");
    ES *s = new ES();
    s->prm = *p;
    s->S = (int)p->n_systems;
    if (cuda_stream) s->stream = (cudaStream_t)cuda_stream;
    else {
        cudaError_t e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) { delete s; return set_err(DPG_ERR_CUDA, "stream: %s", cudaGetErrorString(e)); }
        s->own_stream = true;
    }
    const char *m = getenv("DPG_LOOP_MODE");
    if (m && (!strcmp(m, "stream") || !strcmp(m, "graph"))) s->mode = 0;
    const char *f = getenv("DPG_ENSEMBLE_FORM");
    if (f && !strcmp(f, "grid")) s->form = DPG_FORM_GRID;
    if (f && !strcmp(f, "persist")) s->form = DPG_FORM_PERSIST;
    if (f && !strcmp(f, "resident")) s->form = DPG_FORM_RESIDENT;
    // DPG_FORCE_SPLIT=1: the grid form's force pass as two kernels under IF
    // nodes (FP32 systems; refinement / FP64 systems) instead of one kernel for
    // every arithmetic.  Measured on 16 x 16384 disks, the split costs 6-8 % per
    // iteration (FP32 phase 98 vs 92 us, double-word 112 vs 104 us): the FP32
    // kernel's 80 registers (against 102) do not pay for the extra nodes.
    const char *fs = getenv("DPG_FORCE_SPLIT");
    if (fs && !strcmp(fs, "1")) s->split_force = true;
    // layout: each system padded to whole blocks; its own cell grid
    s->sys.assign(s->S, ESys{});
    int slot = 0, blk = 0, cell = 0, item = 0;
    size_t in = 0;
    for (int k = 0; k < s->S; k++) {
        if (n_particles[k] <= 0 || !(box[k] > 0)) { delete s; return set_err(DPG_ERR_ARG, "system %d: bad size or box", k); }
        ESys &y = s->sys[k];
        y.off = slot;
        y.n = (int)n_particles[k];
        y.inv_n = 1.0 / (double)y.n;
        y.blk0 = blk;
        y.nblk = (y.n + kEB - 1) / kEB;
        y.L = box[k];
        // cells at least 10% larger than the cutoff, so compression keeps them valid
        y.ncd = std::max(1, (int)std::floor(y.L / (p->cutoff * 1.1)));
        y.cell_off = cell;
        y.item_off = item;
        y.cs = y.L / y.ncd;
        y.inv_cs = y.ncd / y.L;
        y.cs_f = (float)y.cs;
        y.cs_lo = (float)(y.cs - (double)y.cs_f);
        y.jam_status = -1;
        y.L_low = y.L_high = y.L_last = -1;
        for (int i = 0; i < y.nblk * kEB; i++) s->src_index.push_back(i < y.n ? (int)(in + i) : -1);
        in += y.n;
        slot += y.nblk * kEB;
        blk += y.nblk;
        cell += y.ncd * y.ncd;
        item += y.n;
        s->n.push_back(y.n);
        s->max_n = std::max(s->max_n, y.n);
    }
    s->T = slot;
    s->nblocks = blk;
    s->total_cells = cell;
    s->n_total = in;
    int rc = DPG_OK;
    auto A = [&](void **pp, size_t b) { if (rc == DPG_OK) rc = ealloc(s, pp, b); };
    EDev &h = s->h;
    const size_t T = s->T;
    A((void **)&s->d, sizeof(EDev));
    A((void **)&s->d_sys, sizeof(ESys) * s->S);
    A((void **)&h.blk_sys, 4 * (size_t)s->nblocks);
    A((void **)&s->d_src, 4 * T);
    A((void **)&h.pos, 16 * T); A((void **)&h.vel, 16 * T); A((void **)&h.frc, 16 * T);
    A((void **)&h.pos_ref, 16 * T); A((void **)&h.pos_save, 16 * T);
    A((void **)&h.rad, 8 * T); A((void **)&h.mass, 8 * T); A((void **)&h.pe, 8 * T);
    A((void **)&h.pk, 16 * T); A((void **)&h.cellc, 4 * T);
    A((void **)&h.vel32, 8 * T); A((void **)&h.frc32, 8 * T); A((void **)&h.invm, 4 * T);
    A((void **)&h.oref, 8 * T); A((void **)&h.ctr, 16 * T); A((void **)&h.pkl, 16 * T);
    A((void **)&h.cnt, 4 * T);
    A((void **)&h.cell_cnt, 4 * ((size_t)s->total_cells + 1));
    A((void **)&h.cell_start, 4 * ((size_t)s->total_cells + 1));
    A((void **)&h.cell_cur, 4 * ((size_t)s->total_cells + 1));
    A((void **)&h.cell_items, 4 * T);
    A((void **)&h.part, 8 * 8 * (size_t)s->nblocks);
    A((void **)&s->xfer, 8 * 4 * std::max<size_t>(s->n_total, 1));
    A((void **)&s->d_rs_blocks, 4 * (size_t)s->S);
    if (rc == DPG_OK) rc = alloc_nbr(s, s->cap);
    if (rc != DPG_OK) { dpg_ensemble_destroy(s); return rc; }
    h.sys = s->d_sys;
    h.p.S = s->S; h.p.T = s->T; h.p.nblocks = s->nblocks; h.p.cap = s->cap;
    h.p.total_cells = s->total_cells;
    h.p.e_c = p->e_c; h.p.n_c = p->n_c;
    h.p.cutoff2 = p->cutoff * p->cutoff;
    h.p.cutoff2_f = (float)h.p.cutoff2;
    h.p.half_skin2 = (p->skin / 2) * (p->skin / 2);
    h.p.switch_fmax = p->precision == DPG_MIXED ? (p->switch_fmax > 0 ? p->switch_fmax : 1e-6) : 0.0;
    h.p.dw_ok = p->n_c == 2.0 ? 1 : 0;
    h.p.ec_hi = (float)p->e_c;
    h.p.ec_lo = (float)(p->e_c - (double)h.p.ec_hi);
    std::vector<int> bs(s->nblocks);
    for (int k = 0; k < s->S; k++)
        for (int b = 0; b < s->sys[k].nblk; b++) bs[s->sys[k].blk0 + b] = k;
    cudaError_t e = cudaMemcpyAsync(h.blk_sys, bs.data(), 4 * bs.size(), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->d_src, s->src_index.data(), 4 * T, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->d_sys, s->sys.data(), sizeof(ESys) * s->S, cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(s->d, &h, sizeof(EDev), cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
    if (e != cudaSuccess) { dpg_ensemble_destroy(s); return set_err(DPG_ERR_CUDA, "ensemble create: %s", cudaGetErrorString(e)); }
    *out = s;
    return DPG_OK;
}

// Slot order of each system: its particles sorted by the row-major index of
// the cell holding their position (a stable counting sort), so that
// consecutive slots -- each block of the grid form, each block of a resident
// cluster -- cover a compact stripe of the box and most of a particle's
// neighbours sit in its own block.  Input order is restored on the way out
// (e_get reads the same map).
static void order_slots(ES *s, const double *x, const double *y) {
    std::vector<int> key, start;
    size_t in = 0;
    for (int k = 0; k < s->S; k++) {
        const ESys &Y = s->sys[k];
        const int n = Y.n, nc = Y.ncd;
        const double L = Y.L, inv = nc / L;
        auto cell = [&](double v) {
            double w = v - L * std::floor(v / L);  // wrapped into [0, L)
            if (!(w >= 0.0 && w < L)) w = 0.0;      // non-finite input: any cell
            return std::min((int)(w * inv), nc - 1);
        };
        key.resize(n);
        start.assign((size_t)nc * nc + 1, 0);
        for (int i = 0; i < n; i++) {
            key[i] = cell(y[in + i]) * nc + cell(x[in + i]);
            start[key[i] + 1]++;
        }
        for (int c = 0; c < nc * nc; c++) start[c + 1] += start[c];
        for (int i = 0; i < n; i++) s->src_index[Y.off + start[key[i]]++] = (int)(in + i);
        in += n;
    }
}

extern "C" int dpg_ensemble_set_state(dpg_ensemble s, const double *x, const double *y,
                                      const double *radii, const double *masses) {
    if (!s || !x || !y || !radii || !masses) return set_err(DPG_ERR_ARG, "null argument");
    const size_t n = s->n_total;
    const double *src[4] = {x, y, radii, masses};
    order_slots(s, x, y);
    CK(cudaMemcpyAsync(s->d_src, s->src_index.data(), 4 * (size_t)s->T, cudaMemcpyHostToDevice, s->stream));
    for (int k = 0; k < 4; k++)
        CK(cudaMemcpyAsync(s->xfer + k * n, src[k], 8 * n, cudaMemcpyHostToDevice, s->stream));
    LAUNCH(e_put, (s->T + 255) / 256, 256, s->d, s->xfer, s->xfer + n, s->xfer + 2 * n, s->xfer + 3 * n, s->d_src);
    CK(cudaStreamSynchronize(s->stream));
    s->have_state = true;
    return DPG_OK;
}

extern "C" int dpg_ensemble_get_state(dpg_ensemble s, double *x, double *y, double *fx, double *fy) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    const size_t n = s->n_total;
    double *dst[4] = {x, y, fx, fy};
    LAUNCH(e_get, (s->T + 255) / 256, 256, s->d, x ? s->xfer : nullptr, y ? s->xfer + n : nullptr,
           fx ? s->xfer + 2 * n : nullptr, fy ? s->xfer + 3 * n : nullptr, s->d_src);
    for (int k = 0; k < 4; k++)
        if (dst[k]) CK(cudaMemcpyAsync(dst[k], s->xfer + k * n, 8 * n, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return DPG_OK;
}

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

// the split force pass: FP32 systems, then refinement / FP64 systems
static int enqueue_force(ES *s) {
    if (s->split_force) {
        LAUNCH(e_force_k<0>, s->nblocks, kEB, s->d);
        LAUNCH(e_force_k<1>, s->nblocks, kEB, s->d);
    } else {
        LAUNCH(e_force_k<-1>, s->nblocks, kEB, s->d);
    }
    LAUNCH(e_after_force, 1, 1, s->d);
    return DPG_OK;
}

static int enqueue_rebuild(ES *s) {
    LAUNCH(e_cell_count, s->nblocks, kEB, s->d);
    LAUNCH(e_cell_scan, s->S, kEScanTPB, s->d);
    LAUNCH(e_cell_fill, s->nblocks, kEB, s->d);
    LAUNCH(e_cell_sort, (s->total_cells + 255) / 256, 256, s->d);
    LAUNCH(e_nlist, s->nblocks, kEB, s->d);
    return DPG_OK;
}

static int enqueue_iteration(ES *s) {
    LAUNCH(e_move, s->nblocks, kEB, s->d);
    TRY(enqueue_rebuild(s));
    TRY(enqueue_force(s));
    LAUNCH(e_transition, s->nblocks, kEB, s->d);
    return DPG_OK;
}

static int build_graph(ES *s) {
    if (s->exec) return DPG_OK;
    cudaGraph_t g;
    CK(cudaGraphCreate(&g, 0));
    cudaError_t err = cudaGraphConditionalHandleCreate(&s->h_loop, g, 1, cudaGraphCondAssignDefault);
    cudaGraphNodeParams wp = {};
    wp.type = cudaGraphNodeTypeConditional;
    wp.conditional.handle = s->h_loop;
    wp.conditional.type = cudaGraphCondTypeWhile;
    wp.conditional.size = 1;
    cudaGraphNode_t wnode = nullptr;
    if (err == cudaSuccess) err = cudaGraphAddNode(&wnode, g, nullptr, nullptr, 0, &wp);
    cudaGraph_t body = err == cudaSuccess ? wp.conditional.phGraph_out[0] : nullptr;
    if (err == cudaSuccess) err = cudaGraphConditionalHandleCreate(&s->h_rb, body, 0, 0);
    if (err == cudaSuccess) err = cudaGraphConditionalHandleCreate(&s->h_tr, body, 0, 0);
    s->h_f32 = s->h_fhi = 0;
    if (err == cudaSuccess && s->split_force) err = cudaGraphConditionalHandleCreate(&s->h_f32, body, 0, 0);
    if (err == cudaSuccess && s->split_force) err = cudaGraphConditionalHandleCreate(&s->h_fhi, body, 0, 0);
    EDev *dp = s->d;
    void *a[] = {&dp};
    cudaGraphNode_t last = nullptr;
    if (err == cudaSuccess) last = addk(body, nullptr, (void *)e_move, s->nblocks, kEB, a, &err);
    cudaGraphNodeParams ip = {};
    ip.type = cudaGraphNodeTypeConditional;
    ip.conditional.handle = s->h_rb;
    ip.conditional.type = cudaGraphCondTypeIf;
    ip.conditional.size = 1;
    cudaGraphNode_t inode = nullptr;
    if (err == cudaSuccess) err = cudaGraphAddNode(&inode, body, &last, nullptr, 1, &ip);
    if (err == cudaSuccess) {
        cudaGraph_t ib = ip.conditional.phGraph_out[0];
        cudaGraphNode_t prev = nullptr;
        prev = addk(ib, prev, (void *)e_cell_count, s->nblocks, kEB, a, &err);
        prev = addk(ib, prev, (void *)e_cell_scan, s->S, kEScanTPB, a, &err);
        prev = addk(ib, prev, (void *)e_cell_fill, s->nblocks, kEB, a, &err);
        prev = addk(ib, prev, (void *)e_cell_sort, (s->total_cells + 255) / 256, 256, a, &err);
        prev = addk(ib, prev, (void *)e_nlist, s->nblocks, kEB, a, &err);
        // IF(some system's pass is FP32) { e_force_k<0> }, IF(some refinement /
        // FP64 pass) { e_force_k<1> }, then the transition condition
        cudaGraphNode_t fprev = inode;
        const cudaGraphConditionalHandle fh[2] = {s->h_f32, s->h_fhi};
        void *fk[2] = {(void *)e_force_k<0>, (void *)e_force_k<1>};
        if (!s->split_force) fprev = addk(body, inode, (void *)e_force_k<-1>, s->nblocks, kEB, a, &err);
        for (int q = 0; q < 2 && err == cudaSuccess && s->split_force; q++) {
            cudaGraphNodeParams fp = {};
            fp.type = cudaGraphNodeTypeConditional;
            fp.conditional.handle = fh[q];
            fp.conditional.type = cudaGraphCondTypeIf;
            fp.conditional.size = 1;
            cudaGraphNode_t fnode = nullptr;
            err = cudaGraphAddNode(&fnode, body, &fprev, nullptr, 1, &fp);
            if (err == cudaSuccess) addk(fp.conditional.phGraph_out[0], nullptr, fk[q], s->nblocks, kEB, a, &err);
            fprev = fnode;
        }
        last = addk(body, fprev, (void *)e_after_force, 1, 1, a, &err);
        // IF(any system queued a transition) { e_transition }
        cudaGraphNodeParams tp = {};
        tp.type = cudaGraphNodeTypeConditional;
        tp.conditional.handle = s->h_tr;
        tp.conditional.type = cudaGraphCondTypeIf;
        tp.conditional.size = 1;
        cudaGraphNode_t tnode = nullptr;
        if (err == cudaSuccess) err = cudaGraphAddNode(&tnode, body, &last, nullptr, 1, &tp);
        if (err == cudaSuccess) {
            addk(tp.conditional.phGraph_out[0], nullptr, (void *)e_transition, s->nblocks, kEB, a, &err);
            last = addk(body, tnode, (void *)e_guard, 1, 1, a, &err);
        }
    }
    if (err == cudaSuccess) err = cudaGraphInstantiate(&s->exec, g, 0);
    cudaGraphDestroy(g);
    if (err != cudaSuccess) {
        s->exec = nullptr;
        return set_err(DPG_ERR_CUDA, "ensemble graph: %s", cudaGetErrorString(err));
    }
    return DPG_OK;
}

template <class T>
static int put(ES *s, T *dev, const T &v) {
    CK(cudaMemcpyAsync(dev, &v, sizeof(T), cudaMemcpyHostToDevice, s->stream));
    return DPG_OK;
}

static int pull_dev(ES *s, EDev *out) {
    CK(cudaMemcpyAsync(out, s->d, sizeof(EDev), cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return DPG_OK;
}

static int pull_sys(ES *s) {
    CK(cudaMemcpyAsync(s->sys.data(), s->d_sys, sizeof(ESys) * s->S, cudaMemcpyDeviceToHost, s->stream));
    CK(cudaStreamSynchronize(s->stream));
    return DPG_OK;
}

static int pow2ceil(int x) { return (int)std::pow(2, std::ceil(std::log2((double)x))); }

// Run the loop until every system is done.  Overflow of a neighbour list halts
// the force pass; the host grows the lists, rebuilds them for every live system
// and finishes that iteration before resuming.
static int run(ES *s, long long guard_limit) {
    for (int attempt = 0; attempt < 64; attempt++) {
        EDev cur;
        TRY(pull_dev(s, &cur));
        if (cur.active <= 0) return DPG_OK;
        TRY(put(s, &s->d->guard, 0LL));
        TRY(put(s, &s->d->guard_limit, guard_limit));
        bool ran = false;
        if (s->mode == 2 && build_graph(s) == DPG_OK) {
            TRY(put(s, &s->d->h_loop, (unsigned long long)s->h_loop));
            TRY(put(s, &s->d->h_rb, (unsigned long long)s->h_rb));
            TRY(put(s, &s->d->h_tr, (unsigned long long)s->h_tr));
            TRY(put(s, &s->d->h_f32, (unsigned long long)s->h_f32));
            TRY(put(s, &s->d->h_fhi, (unsigned long long)s->h_fhi));
            CK(cudaGraphLaunch(s->exec, s->stream));
            s->launches++;
            TRY(put(s, &s->d->h_loop, 0ULL));
            TRY(put(s, &s->d->h_rb, 0ULL));
            TRY(put(s, &s->d->h_tr, 0ULL));
            TRY(put(s, &s->d->h_f32, 0ULL));
            TRY(put(s, &s->d->h_fhi, 0ULL));
            ran = true;
        }
        if (!ran) {
            (void)cudaGetLastError();  // a failed graph build leaves its error behind
            s->mode = 0;
            for (long long it = 0; it < guard_limit; it++) {
                TRY(enqueue_iteration(s));
                if ((it & 63) == 63) {
                    TRY(pull_dev(s, &cur));
                    if (cur.active <= 0 || cur.overflow) break;
                }
            }
        }
        TRY(pull_dev(s, &cur));
        if (cur.overflow) {
            int ncap = pow2ceil(cur.max_count);
            if ((size_t)ncap * s->T > ((size_t)1 << 31)) return set_err(DPG_ERR_OVERFLOW, "ensemble neighbour list too large");
            TRY(alloc_nbr(s, ncap));
            if (s->exec) { cudaGraphExecDestroy(s->exec); s->exec = nullptr; }
            TRY(put(s, &s->d->nbr, s->h.nbr));
            TRY(put(s, &s->d->p.cap, ncap));
            TRY(put(s, &s->d->overflow, 0));
            TRY(pull_sys(s));
            for (auto &y : s->sys) if (y.phase != kIdle) y.rebuild = 1;
            CK(cudaMemcpyAsync(s->d_sys, s->sys.data(), sizeof(ESys) * s->S, cudaMemcpyHostToDevice, s->stream));
            TRY(put(s, &s->d->n_flagged, 1));
            TRY(enqueue_rebuild(s));
            TRY(enqueue_force(s));
            LAUNCH(e_transition, s->nblocks, kEB, s->d);
            TRY(pull_dev(s, &cur));
            if (cur.overflow) continue;
            continue;
        }
        if (cur.active <= 0) return DPG_OK;
        if (cur.guard >= guard_limit) return set_err(DPG_ERR_NOT_CONVERGED, "ensemble loop budget spent");
    }
    return set_err(DPG_ERR_STATE, "ensemble loop did not finish");
}

// ---- the resident form --------------------------------------------------------
typedef void (*res_kernel_fn)(EDev *, const int *, int, long long, unsigned long long);
// Size classes (threads per block, particles per lane group, blocks per
// cluster, lanes per particle): a system goes to the first class that holds it.
struct RClass {
    int nt, ppt, c, g;
    res_kernel_fn fn;
    int per_block() const { return nt / g * ppt; }
    int capacity() const { return nt / g * ppt * c; }
};
// Measured on one GB300 (double-word FIRE iterations of 4 / 48 systems):
// lanes per particle and larger blocks for the small systems (N = 128: 5.4 vs
// 9.4 us per iteration with 4 particles per thread), clusters of 8 blocks for
// the largest (N = 4096 alone: 18.8 vs 30.0 us on 4 blocks of 4 particles per
// thread), 2 particles per thread where many large systems share the GPU
// (N = 2048, 48 systems: 24.9 vs 30.6 us).
// The last class holds up to 16384 disks: 8-block clusters of 512 threads x 4
// particles (2048 disks and ~146 KB of shared memory a block).
constexpr int kNClass = 8;
#define RC(NT, PPT, C, G) {NT, PPT, C, G, e_res<NT, PPT, C, G>}
static const RClass kRClasses[kNClass] = {RC(256, 1, 1, 4), RC(256, 1, 1, 2), RC(256, 1, 1, 1),
                                          RC(512, 1, 1, 1), RC(512, 1, 2, 1), RC(256, 2, 4, 1),
                                          RC(256, 2, 8, 1), RC(512, 4, 8, 1)};
#undef RC

static int res_class_of(int n) {
    for (int c = 0; c < kNClass; c++)
        if (n <= kRClasses[c].capacity()) return c;
    return -1;
}

// largest cell count of the systems of class c
static int res_ncmax(const ES *s, int c) {
    int m = 1;
    for (const auto &y : s->sys)
        if (res_class_of(y.n) == c) m = std::max(m, y.ncd * y.ncd);
    return m;
}

static int res_smem_limit() {
    int dev = 0, v = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess) return 0;
    return v;
}

// the resident form holds every system: sizes and shared memory within limits
static bool res_fits(const ES *s) {
    if (s->max_n > kResMaxN) return false;
    const size_t lim = (size_t)res_smem_limit();
    for (int c = 0; c < kNClass; c++) {
        const size_t b = res_smem_bytes(kRClasses[c].per_block(), kRClasses[c].capacity(), res_ncmax(s, c));
        if (b + 4096 > lim) return false;  // room for the kernel's static shared memory
    }
    return true;
}


// one cluster of K.c blocks per system, nb systems
static cudaLaunchConfig_t res_config(const RClass &K, int nb, size_t smem, cudaStream_t st,
                                     cudaLaunchAttribute *attr) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(nb * K.c);
    cfg.blockDim = dim3(K.nt);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = K.c;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cfg;
}

// Launch every class that has live systems, each on its own stream (forked
// from and joined back into the ensemble's stream).  slice_ns bounds a launch.
// A launch carries at most as many systems of a class as the GPU holds
// clusters of it at once (cudaOccupancyMaxActiveClusters): more would run as a
// second wave after the first wave's time slice, on a mostly idle GPU.  The
// class's systems take turns, rotating between launches.
static int launch_resident(ES *s, long long budget, unsigned long long slice_ns, int *launched) {
    *launched = 0;
    std::vector<int> order[kNClass];
    for (int k = 0; k < s->S; k++) {
        const ESys &y = s->sys[k];
        if (y.phase == kIdle) continue;
        order[res_class_of(y.n)].push_back(k);
    }
    std::vector<int> flat;
    int first[kNClass];
    size_t smem[kNClass];
    int ncmax[kNClass];
    for (int c = 0; c < kNClass; c++) {
        first[c] = (int)flat.size();
        if (order[c].empty()) continue;
        const RClass &K = kRClasses[c];
        ncmax[c] = res_ncmax(s, c);
        smem[c] = res_smem_bytes(K.per_block(), K.capacity(), ncmax[c]);
        CK(cudaFuncSetAttribute((const void *)K.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem[c]));
        if (!s->rs_fit[c]) {
            cudaLaunchAttribute attr[1];
            const cudaLaunchConfig_t cfg = res_config(K, (int)order[c].size(), smem[c], s->stream, attr);
            int fit = 0;
            if (cudaOccupancyMaxActiveClusters(&fit, (const void *)K.fn, &cfg) != cudaSuccess || fit <= 0) {
                (void)cudaGetLastError();
                fit = 1 << 30;  // unknown: no cap
            }
            s->rs_fit[c] = fit;
        }
        // largest systems first: they start before the small ones fill the SMs
        std::sort(order[c].begin(), order[c].end(), [&](int a, int b) {
            return s->sys[a].n != s->sys[b].n ? s->sys[a].n > s->sys[b].n : a < b;
        });
        const int nb = (int)order[c].size();
        if (nb > s->rs_fit[c]) {
            const int rot = s->rs_rot[c] % nb;
            std::rotate(order[c].begin(), order[c].begin() + rot, order[c].end());
            order[c].resize(s->rs_fit[c]);
            s->rs_rot[c] = (int)(((long long)rot + s->rs_fit[c]) % nb);
        }
        flat.insert(flat.end(), order[c].begin(), order[c].end());
    }
    if (flat.empty()) return DPG_OK;
    CK(cudaMemcpyAsync(s->d_rs_blocks, flat.data(), 4 * flat.size(), cudaMemcpyHostToDevice, s->stream));
    if (!s->rs_fork) CK(cudaEventCreateWithFlags(&s->rs_fork, cudaEventDisableTiming));
    CK(cudaEventRecord(s->rs_fork, s->stream));
    for (int c = 0; c < kNClass; c++) {
        const int nb = (int)order[c].size();
        if (!nb) continue;
        if (!s->rs_stream[c]) {
            CK(cudaStreamCreateWithFlags(&s->rs_stream[c], cudaStreamNonBlocking));
            CK(cudaEventCreateWithFlags(&s->rs_join[c], cudaEventDisableTiming));
        }
        const RClass &K = kRClasses[c];
        res_kernel_fn kern = K.fn;
        CK(cudaStreamWaitEvent(s->rs_stream[c], s->rs_fork, 0));
        cudaLaunchAttribute attr[1];
        const cudaLaunchConfig_t cfg = res_config(K, nb, smem[c], s->rs_stream[c], attr);
        const int *blocks = s->d_rs_blocks + first[c];
        EDev *dev = s->d;
        CK(cudaLaunchKernelEx(&cfg, kern, dev, blocks, ncmax[c], budget, slice_ns));
        s->launches++;
        CK(cudaEventRecord(s->rs_join[c], s->rs_stream[c]));
        CK(cudaStreamWaitEvent(s->stream, s->rs_join[c], 0));
        (*launched)++;
    }
    return DPG_OK;
}

static int grow_lists(ES *s, const EDev &cur) {
    int ncap = 1;
    while (ncap < cur.max_count) ncap <<= 1;
    if ((size_t)ncap * s->T > ((size_t)1 << 31)) return set_err(DPG_ERR_OVERFLOW, "ensemble neighbour list too large");
    TRY(alloc_nbr(s, ncap));
    if (s->exec) { cudaGraphExecDestroy(s->exec); s->exec = nullptr; }
    TRY(put(s, &s->d->nbr, s->h.nbr));
    TRY(put(s, &s->d->p.cap, ncap));
    TRY(put(s, &s->d->overflow, 0));
    TRY(pull_sys(s));
    for (auto &y : s->sys) if (y.phase != kIdle) y.rebuild = 1;
    CK(cudaMemcpyAsync(s->d_sys, s->sys.data(), sizeof(ESys) * s->S, cudaMemcpyHostToDevice, s->stream));
    return DPG_OK;
}

// Relaunch the resident kernels until every system is done.  Each launch runs
// for at most kSlice of device time per block (so the classes' launches end
// together and the host sees progress); termination is the device state
// machine's (every minimisation has a step cap, jamming a compression cap);
// the host stops with an error when some system's FIRE passes in this run
// exceed guard_limit or a launch makes no progress.
static int run_resident(ES *s, long long guard_limit) {
    const unsigned long long kSlice = 200ull * 1000 * 1000;  // 0.2 s
    const long long kChunk = 1LL << 24;
    std::vector<long long> base(s->S, -1);
    long long last_sum = -1;
    for (int launches = 0; launches < (1 << 22); launches++) {
        EDev cur;
        TRY(pull_dev(s, &cur));
        if (cur.overflow) {
            TRY(grow_lists(s, cur));
            last_sum = -1;
            continue;
        }
        if (cur.active <= 0) return DPG_OK;
        TRY(pull_sys(s));
        long long most = 0, sum = 0;
        for (int k = 0; k < s->S; k++) {
            const long long f = s->sys[k].fire_total;
            if (base[k] < 0) base[k] = f;
            most = std::max(most, f - base[k]);
            sum += f;
        }
        if (most > guard_limit) return set_err(DPG_ERR_NOT_CONVERGED, "ensemble loop budget spent");
        if (sum == last_sum) return set_err(DPG_ERR_STATE, "resident launch made no progress");
        last_sum = sum;
        int nl = 0;
        TRY(launch_resident(s, kChunk, kSlice, &nl));
        if (!nl) return DPG_OK;
    }
    return set_err(DPG_ERR_STATE, "ensemble loop did not finish");
}

// ---- the persistent form ----------------------------------------------------
// AUTO runs the resident form when it holds every system (at most 16384
// particles each, shared memory within the device limit), else the grid form.
// Measured on one GB300, FIRE of 16 x 16384 disks to max|F| <= 1e-13: resident
// 4.86 solves/s, grid 1.50, persistent below 0.4; for 32 systems of 64-4096
// disks the grid form ran 3.5e8 particle-iterations/s against the persistent
// form's 3.0e8 (512-thread blocks).  dpg_ensemble_autotune measures and may
// choose any of them.
static int form_of(const ES *s) {
    if (s->form != DPG_FORM_AUTO) return s->form;
    return res_fits(s) ? DPG_FORM_RESIDENT : DPG_FORM_GRID;
}

static int threads_of(const ES *s) {
    if (s->pthreads) return s->pthreads;
    return s->max_n <= 512 ? 128 : (s->max_n <= 4096 ? 256 : 512);
}

static int launch_persist(ES *s, int nt, long long budget) {
    switch (nt) {
    case 128: LAUNCH(e_persist<128>, s->S, 128, s->d, budget); break;
    case 256: LAUNCH(e_persist<256>, s->S, 256, s->d, budget); break;
    case 512: LAUNCH(e_persist<512>, s->S, 512, s->d, budget); break;
    default: return set_err(DPG_ERR_ARG, "persistent form: threads must be 128, 256 or 512");
    }
    return DPG_OK;
}

// Relaunch the persistent kernel until every system is done: each launch runs
// at most kChunk iterations per system (launches stay well under a second or
// two); a neighbour-list overflow ends the launch, the host grows the lists
// and every live system rebuilds its lists at its next iteration.
static int run_persist(ES *s, long long guard_limit) {
    const long long kChunk = 1LL << 17;
    const int nt = threads_of(s);
    long long spent = 0;
    for (int launches = 0; launches < (1 << 22); launches++) {
        EDev cur;
        TRY(pull_dev(s, &cur));
        if (cur.overflow) {
            int ncap = pow2ceil(cur.max_count);
            if ((size_t)ncap * s->T > ((size_t)1 << 31)) return set_err(DPG_ERR_OVERFLOW, "ensemble neighbour list too large");
            TRY(alloc_nbr(s, ncap));
            if (s->exec) { cudaGraphExecDestroy(s->exec); s->exec = nullptr; }
            TRY(put(s, &s->d->nbr, s->h.nbr));
            TRY(put(s, &s->d->p.cap, ncap));
            TRY(put(s, &s->d->overflow, 0));
            TRY(pull_sys(s));
            for (auto &y : s->sys) if (y.phase != kIdle) y.rebuild = 1;
            CK(cudaMemcpyAsync(s->d_sys, s->sys.data(), sizeof(ESys) * s->S, cudaMemcpyHostToDevice, s->stream));
            continue;
        }
        if (cur.active <= 0) return DPG_OK;
        if (spent >= guard_limit) return set_err(DPG_ERR_NOT_CONVERGED, "ensemble loop budget spent");
        const long long chunk = std::min(kChunk, guard_limit - spent);
        TRY(launch_persist(s, nt, chunk));
        spent += chunk;
    }
    return set_err(DPG_ERR_STATE, "ensemble loop did not finish");
}

extern "C" int dpg_ensemble_launch_count(dpg_ensemble s, int64_t *count) {
    if (!s || !count) return set_err(DPG_ERR_ARG, "null argument");
    *count = s->launches;
    return DPG_OK;
}

extern "C" int dpg_ensemble_set_form(dpg_ensemble s, int form, int threads) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (form != DPG_FORM_AUTO && form != DPG_FORM_GRID && form != DPG_FORM_PERSIST &&
        form != DPG_FORM_RESIDENT)
        return set_err(DPG_ERR_ARG, "bad form");
    if (form == DPG_FORM_RESIDENT && !res_fits(s))
        return set_err(DPG_ERR_ARG, "resident form: systems of at most %d particles whose cell lists fit "
                                    "shared memory", kResMaxN);
    if (threads != 0 && threads != 128 && threads != 256 && threads != 512)
        return set_err(DPG_ERR_ARG, "threads must be 0, 128, 256 or 512");
    s->form = form;
    s->pthreads = threads;
    return DPG_OK;
}

// per-system FIRE / jamming state reset and parameters upload (no launches)
static int prepare(ES *s, const dpg_fire_params *fp, int jam, const dpg_jam_params *jp, int res = 0) {
    if (!s->have_state) return set_err(DPG_ERR_STATE, "set the state first");
    TRY(pull_sys(s));
    EParams &p = s->h.p;
    p.alpha0 = fp->alpha_init; p.dt0 = fp->dt;
    p.pe_target = fp->avg_pe_target; p.pe_diff_target = fp->avg_pe_diff_target;
    p.fmax_target = fp->fmax_target; p.max_steps = fp->max_steps;
    p.fmax_cert2 = (0.99 * fp->fmax_target) * (0.99 * fp->fmax_target);
    p.jam = jam;
    p.res = res;
    if (jp) {
        p.p_low = jp->pressure_low; p.p_high = jp->pressure_high;
        p.compression_rate = jp->compression_rate; p.length_tol = jp->length_tolerance;
        p.decompress = jp->decompress_factor; p.max_compressions = jp->max_compression_steps;
    }
    for (auto &y : s->sys) {
        y.phase = kSetup; y.rebuild = 1; y.done = 0;
        y.prec = (p.switch_fmax > 0 && y.ncd >= 3) ? 0 : 1;
        y.dt = p.dt0; y.alpha = p.alpha0; y.ngood = 0; y.nbad = 0; y.uphill = 0; y.stopped = 0;
        y.converged = 0; y.iter = 0; y.fire_total = 0; y.pending = kActNone; y.minimizations = 0;
        y.jam_stage = 0; y.jam_status = -1; y.jam_step = 0;
        y.L_low = y.L_high = y.L_last = -1; y.L_saved = -1; y.scale = 1.0; y.rebuilds = 0;
        y.ticket_a = y.ticket_b = 0;
        y.best_f2 = INFINITY; y.best_it = 0; y.vel_f32 = 0; y.fp64_total = 0; y.dw_total = 0;
        y.resume = 0;
        y.res_valid = 0;
        y.verify = 0;
        y.dw_scale = 0.9;
        y.fprec = y.prec;
    }
    CK(cudaMemcpyAsync(s->d_sys, s->sys.data(), sizeof(ESys) * s->S, cudaMemcpyHostToDevice, s->stream));
    CK(cudaMemcpyAsync(&s->d->p, &p, sizeof(EParams), cudaMemcpyHostToDevice, s->stream));
    TRY(put(s, &s->d->active, s->S));
    TRY(put(s, &s->d->n_flagged, 0));
    TRY(put(s, &s->d->n_pending, 0));
    TRY(put(s, &s->d->overflow, 0));
    TRY(put(s, &s->d->ticket, 0u));
    TRY(put(s, &s->d->max_count, 0));
    // velocities start at zero (minimizeFire's setVelocitiesToZero)
    CK(cudaMemsetAsync(s->h.vel, 0, 16 * (size_t)s->T, s->stream));
    CK(cudaMemsetAsync(s->h.vel32, 0, 8 * (size_t)s->T, s->stream));
    return DPG_OK;
}

static int start(ES *s, const dpg_fire_params *fp, int jam, const dpg_jam_params *jp) {
    const int form = form_of(s);
    TRY(prepare(s, fp, jam, jp, form == DPG_FORM_RESIDENT));
    long long budget = jam ? (long long)4e9 : fp->max_steps * 2 + 16;
    if (form == DPG_FORM_PERSIST) TRY(run_persist(s, budget));
    else if (form == DPG_FORM_RESIDENT) TRY(run_resident(s, budget));
    else TRY(run(s, budget));
    TRY(pull_sys(s));
    return DPG_OK;
}

static void fill_results(ES *s, dpg_ensemble_result *r) {
    if (!r) return;
    for (int k = 0; k < s->S; k++) {
        const ESys &y = s->sys[k];
        dpg_ensemble_result &o = r[k];
        o.avg_pe = y.pe / y.n;
        o.max_force = std::sqrt(y.fmax2);
        o.pressure = y.virial / (4.0 * y.L * y.L);
        o.box_length = y.L;
        o.contacts = y.contacts;
        o.fire_steps = y.fire_total;
        o.minimizations = y.minimizations;
        o.rebuilds = y.rebuilds;
        o.fp64_steps = y.fp64_total;
        o.dw_steps = y.dw_total;
        o.status = y.jam_status;
        o.converged = y.converged;
        o.packing_fraction = 0.0;  // filled by the caller, who knows the radii
    }
}

extern "C" int dpg_ensemble_fire_minimize(dpg_ensemble s, const dpg_fire_params *p, dpg_ensemble_result *r) {
    if (!s || !p) return set_err(DPG_ERR_ARG, "null argument");
    if (p->max_steps <= 0) return set_err(DPG_ERR_ARG, "max_steps must be > 0");
    TRY(start(s, p, 0, nullptr));
    fill_results(s, r);
    return DPG_OK;
}

extern "C" int dpg_ensemble_jam(dpg_ensemble s, const dpg_jam_params *p, dpg_ensemble_result *r) {
    if (!s || !p) return set_err(DPG_ERR_ARG, "null argument");
    TRY(start(s, &p->fire, 1, p));
    fill_results(s, r);
    return DPG_OK;
}

extern "C" int dpg_ensemble_compute_forces(dpg_ensemble s, int precision, dpg_ensemble_result *r) {
    if (!s) return set_err(DPG_ERR_ARG, "null handle");
    if (precision != DPG_FP64 && precision != DPG_MIXED && precision != DPG_DWORD)
        return set_err(DPG_ERR_ARG, "bad precision");
    if (precision == DPG_DWORD && s->h.p.dw_ok == 0)
        return set_err(DPG_ERR_ARG, "double-word pairs need harmonic contacts (n_c = 2)");
    const dpg_fire_params fp = {0.1, 1e-2, 0.0, 0.0, 1, 0.0};
    for (int attempt = 0; attempt < 8; attempt++) {
        TRY(prepare(s, &fp, 0, nullptr));
        for (auto &y : s->sys) {
            y.prec = y.ncd < 3 ? 1 : (precision == DPG_MIXED ? 0 : (precision == DPG_DWORD ? 2 : 1));
            y.fprec = y.prec;
        }
        CK(cudaMemcpyAsync(s->d_sys, s->sys.data(), sizeof(ESys) * s->S, cudaMemcpyHostToDevice, s->stream));
        TRY(put(s, &s->d->n_flagged, 1));
        TRY(enqueue_rebuild(s));
        TRY(enqueue_force(s));
        EDev cur;
        TRY(pull_dev(s, &cur));
        if (!cur.overflow) {
            TRY(pull_sys(s));
            fill_results(s, r);
            return DPG_OK;
        }
        int ncap = pow2ceil(cur.max_count);
        if ((size_t)ncap * s->T > ((size_t)1 << 31)) return set_err(DPG_ERR_OVERFLOW, "ensemble neighbour list too large");
        TRY(alloc_nbr(s, ncap));
        if (s->exec) { cudaGraphExecDestroy(s->exec); s->exec = nullptr; }
        TRY(put(s, &s->d->nbr, s->h.nbr));
        TRY(put(s, &s->d->p.cap, ncap));
        TRY(put(s, &s->d->overflow, 0));
    }
    return set_err(DPG_ERR_OVERFLOW, "ensemble neighbour list did not settle");
}

extern "C" int dpg_ensemble_profile_loop(dpg_ensemble s, const dpg_fire_params *p, int iters,
                                         double *avg_us, int64_t *counts) {
    if (!s || !p || !avg_us || iters <= 0) return set_err(DPG_ERR_ARG, "null argument or iters <= 0");
    TRY(prepare(s, p, 0, nullptr));
    std::vector<cudaEvent_t> ev(5 * (size_t)iters);
    for (auto &e : ev) CK(cudaEventCreate(&e));
    int rc = DPG_OK;
    for (int i = 0; i < iters && rc == DPG_OK; i++) {
        cudaEventRecord(ev[5 * i + 0], s->stream);
        LAUNCH(e_move, s->nblocks, kEB, s->d);
        cudaEventRecord(ev[5 * i + 1], s->stream);
        rc = enqueue_rebuild(s);
        cudaEventRecord(ev[5 * i + 2], s->stream);
        TRY(enqueue_force(s));
        cudaEventRecord(ev[5 * i + 3], s->stream);
        LAUNCH(e_transition, s->nblocks, kEB, s->d);
        cudaEventRecord(ev[5 * i + 4], s->stream);
    }
    cudaError_t e = cudaStreamSynchronize(s->stream);
    double acc[4] = {0, 0, 0, 0};
    if (rc == DPG_OK && e == cudaSuccess) {
        for (int i = 0; i < iters; i++)
            for (int k = 0; k < 4; k++) {
                float ms = 0;
                cudaEventElapsedTime(&ms, ev[5 * i + k], ev[5 * i + k + 1]);
                acc[k] += ms * 1e3;
            }
    }
    for (auto &x : ev) cudaEventDestroy(x);
    if (rc != DPG_OK) return rc;
    if (e != cudaSuccess) return set_err(DPG_ERR_CUDA, "profile: %s", cudaGetErrorString(e));
    for (int k = 0; k < 4; k++) avg_us[k] = acc[k] / iters;
    TRY(pull_sys(s));
    if (counts) {
        long long rb = 0, fire = 0;
        for (auto &y : s->sys) { rb += y.rebuilds; fire += y.fire_total; }
        counts[0] = iters;
        counts[1] = rb;
        counts[2] = fire;
    }
    return DPG_OK;
}

// ---------------------------------------------------------------------------
// autotuner
// ---------------------------------------------------------------------------
static int set_skin(ES *s, double skin) {
    const double cutoff = s->prm.cutoff - (s->prm.skin - skin);
    s->h.p.cutoff2 = cutoff * cutoff;
    s->h.p.cutoff2_f = (float)s->h.p.cutoff2;
    s->h.p.half_skin2 = (skin / 2) * (skin / 2);
    CK(cudaMemcpyAsync(&s->d->p, &s->h.p, sizeof(EParams), cudaMemcpyHostToDevice, s->stream));
    return DPG_OK;
}

// one trial: FIRE from the saved positions for `iters` iterations; returns
// particle-iterations per second (device time between events)
static int trial(ES *s, const double2 *saved, const dpg_fire_params *p, int iters, int form, int nt,
                 double skin, double *rate) {
    CK(cudaMemcpyAsync(s->h.pos, saved, 16 * (size_t)s->T, cudaMemcpyDeviceToDevice, s->stream));
    TRY(set_skin(s, skin));
    dpg_fire_params q = *p;
    q.max_steps = iters;
    q.avg_pe_target = 0.0;
    q.avg_pe_diff_target = 0.0;
    q.fmax_target = 0.0;
    const int f0 = s->form, t0 = s->pthreads;
    s->form = form;
    s->pthreads = nt;
    TRY(prepare(s, &q, 0, nullptr, form == DPG_FORM_RESIDENT));
    cudaEvent_t a, b;
    CK(cudaEventCreate(&a));
    CK(cudaEventCreate(&b));
    CK(cudaEventRecord(a, s->stream));
    const long long g = (long long)iters * 2 + 16;
    int rc = form == DPG_FORM_PERSIST ? run_persist(s, g)
             : (form == DPG_FORM_RESIDENT ? run_resident(s, g) : run(s, g));
    cudaEventRecord(b, s->stream);
    cudaEventSynchronize(b);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    s->form = f0;
    s->pthreads = t0;
    TRY(rc);
    TRY(pull_sys(s));
    double work = 0.0;
    for (const auto &y : s->sys) work += (double)y.n * (double)y.fire_total;
    *rate = ms > 0 ? work / (ms * 1e-3) : 0.0;
    return DPG_OK;
}

extern "C" int dpg_ensemble_autotune(dpg_ensemble s, const dpg_fire_params *p, int iters,
                                     dpg_ensemble_tuning *out) {
    if (!s || !p || iters <= 0) return set_err(DPG_ERR_ARG, "null argument or iters <= 0");
    if (!s->have_state) return set_err(DPG_ERR_STATE, "set the state first");
    double2 *saved = nullptr;
    CK(cudaMalloc((void **)&saved, 16 * (size_t)s->T));
    cudaError_t ce = cudaMemcpyAsync(saved, s->h.pos, 16 * (size_t)s->T, cudaMemcpyDeviceToDevice, s->stream);
    if (ce != cudaSuccess) { cudaFree(saved); return set_err(DPG_ERR_CUDA, "autotune: %s", cudaGetErrorString(ce)); }
    struct Cand { int form, nt; double skin, rate; };
    std::vector<Cand> cands;
    const double skins[3] = {1.0, 0.75, 0.5};
    for (double f : skins) {
        cands.push_back({DPG_FORM_GRID, 0, s->prm.skin * f, 0.0});
        for (int nt : {128, 256, 512}) cands.push_back({DPG_FORM_PERSIST, nt, s->prm.skin * f, 0.0});
        if (res_fits(s)) cands.push_back({DPG_FORM_RESIDENT, 0, s->prm.skin * f, 0.0});
    }
    int rc = DPG_OK;
    double warm = 0.0;
    // untimed first pass of each form (graph instantiation, module loading)
    rc = trial(s, saved, p, 4, DPG_FORM_GRID, 0, s->prm.skin, &warm);
    if (rc == DPG_OK) rc = trial(s, saved, p, 4, DPG_FORM_PERSIST, 256, s->prm.skin, &warm);
    if (rc == DPG_OK && res_fits(s)) rc = trial(s, saved, p, 4, DPG_FORM_RESIDENT, 0, s->prm.skin, &warm);
    for (auto &c : cands) {
        if (rc != DPG_OK) break;
        rc = trial(s, saved, p, iters, c.form, c.nt, c.skin, &c.rate);
    }
    // restore the positions and keep the fastest candidate
    cudaMemcpyAsync(s->h.pos, saved, 16 * (size_t)s->T, cudaMemcpyDeviceToDevice, s->stream);
    cudaStreamSynchronize(s->stream);
    cudaFree(saved);
    if (rc != DPG_OK) {
        set_skin(s, s->prm.skin);  // a failed trial leaves the given skin in place
        return rc;
    }
    size_t best = 0;
    for (size_t k = 1; k < cands.size(); k++)
        if (cands[k].rate > cands[best].rate) best = k;
    s->form = cands[best].form;
    s->pthreads = cands[best].nt;
    const double skin = cands[best].skin;
    s->prm.cutoff -= s->prm.skin - skin;
    s->prm.skin = skin;
    TRY(set_skin(s, skin));
    if (out) {
        out->form = s->form;
        out->threads = s->form == DPG_FORM_PERSIST ? threads_of(s) : 0;
        out->skin = skin;
        out->n_candidates = (int)cands.size();
        for (size_t k = 0; k < cands.size() && k < 16; k++) {
            out->cand_form[k] = cands[k].form;
            out->cand_threads[k] = cands[k].nt;
            out->cand_skin[k] = cands[k].skin;
            out->cand_rate[k] = cands[k].rate;
        }
    }
    return DPG_OK;
}
