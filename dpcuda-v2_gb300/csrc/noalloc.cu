// noalloc.cu -- disk forces and energies from positions and radii without any
// device allocation.
//
// Some callers cannot call cudaMalloc: an application that hands all device
// memory to its own fixed pool up front has none left for a library to take,
// and a real-time loop cannot afford the allocator's locks and the device
// synchronisation that cudaMalloc and cudaFree may imply.  For them this file
// offers one entry point, dpg_disk_forces_noalloc, that computes the same
// harmonic forces as dpg_setup_neighbors + dpg_compute_forces but keeps its
// cell-list scratch in the file-scope array below, sized for at most
// kMaxParticles particles and kMaxCells cells.  Every GPU that loads the
// library holds that array (about 1 MiB) until the process exits.
//
// Host code must not pass the array's name to a kernel (in host code it is a
// host-side stand-in, not a device address); the device address is looked up
// with cudaGetSymbolAddress, with the device current, on a device's first
// call, and again whenever the device's context has changed since (after
// cudaDeviceReset the module is loaded anew and the array may move).  Make the
// first call on each device before any stream capture.  All calls share the
// one array, so calls whose kernels overlap on the GPU (two streams at once)
// race; serialise them.  Each call clears the counters it needs before use.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "disk_kernels.cuh"
#include "host_common.h"

namespace {

constexpr int kMaxParticles = 65536;
constexpr int kMaxCells = 65536;
constexpr int kMaxDevices = 64;

// counts[kMaxCells + 1] | starts[kMaxCells + 1] | cursors[kMaxCells + 1] |
// items[kMaxParticles] | cell of each particle[kMaxParticles]
constexpr size_t kScratchInts = 3 * (size_t)(kMaxCells + 1) + 2 * (size_t)kMaxParticles;
static __device__ __align__(256) int g_noalloc_scratch[kScratchInts];

struct NaArgs {
    const double *x, *y, *r;
    double *fx, *fy, *pe;
    int n, ncd;
    double bx, by, cs, e_c, n_c;
    int *cnt, *start, *cur, *items, *cell;
};

__global__ void na_clear(NaArgs a) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c <= a.ncd * a.ncd) { a.cnt[c] = 0; a.cur[c] = 0; }
}

__global__ void na_count(NaArgs a) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    int c = dpg::cell_coord(a.x[i], a.cs, a.ncd) + dpg::cell_coord(a.y[i], a.cs, a.ncd) * a.ncd;
    a.cell[i] = c;
    atomicAdd(&a.cnt[c], 1);
}

__global__ void __launch_bounds__(1024) na_scan(NaArgs a) {
    __shared__ int wsum[32];
    __shared__ int carry_s;
    const int nc = a.ncd * a.ncd;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int carry = 0;
    for (int base = 0; base < nc; base += 1024) {
        int idx = base + threadIdx.x;
        int v = idx < nc ? a.cnt[idx] : 0;
        int incl = v;
        for (int off = 1; off < 32; off <<= 1) {
            int t = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += t;
        }
        if (lane == 31) wsum[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            int w = wsum[lane], wi = w;
            for (int off = 1; off < 32; off <<= 1) {
                int t = __shfl_up_sync(0xffffffffu, wi, off);
                if (lane >= off) wi += t;
            }
            wsum[lane] = wi - w;
            if (lane == 31) carry_s = wi;
        }
        __syncthreads();
        if (idx < nc) a.start[idx] = carry + wsum[wid] + incl - v;
        carry += carry_s;
        __syncthreads();
    }
    if (threadIdx.x == 0) a.start[nc] = carry;
}

__global__ void na_fill(NaArgs a) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    int c = a.cell[i];
    a.items[a.start[c] + atomicAdd(&a.cur[c], 1)] = i;
}

// ascending particle order inside each cell so the force sums are reproducible
__global__ void na_sort(NaArgs a) {
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= a.ncd * a.ncd) return;
    int b = a.start[c], e = a.start[c + 1];
    for (int k = b + 1; k < e; k++) {
        int key = a.items[k], j = k - 1;
        while (j >= b && a.items[j] > key) { a.items[j + 1] = a.items[j]; j--; }
        a.items[j + 1] = key;
    }
}

// forces from the 3x3 cells (all pairs when the grid is coarser than 3 cells)
__global__ void na_force(NaArgs a) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.n) return;
    const double xi = a.x[i], yi = a.y[i], ri = a.r[i];
    double ax = 0.0, ay = 0.0, en = 0.0;
    auto visit = [&](int j) {
        if (j == i) return;
        double fx, fy;
        en += dpg::disk_pair(xi, yi, ri, a.x[j], a.y[j], a.r[j], a.bx, a.by, a.e_c, a.n_c, fx, fy);
        ax += fx;
        ay += fy;
    };
    if (a.ncd >= 3) {
        int c = a.cell[i], cx = c % a.ncd, cy = c / a.ncd;
        for (int oy = -1; oy <= 1; oy++)
            for (int ox = -1; ox <= 1; ox++) {
                int g = dpg::pmod(cx + ox, a.ncd) + dpg::pmod(cy + oy, a.ncd) * a.ncd;
                for (int k = a.start[g]; k < a.start[g + 1]; k++) visit(a.items[k]);
            }
    } else {
        for (int j = 0; j < a.n; j++) visit(j);
    }
    a.fx[i] = ax;
    a.fy[i] = ay;
    a.pe[i] = en;
}

std::mutex g_lock;
int *g_scratch_addr[kMaxDevices] = {nullptr};
unsigned long long g_scratch_ctx[kMaxDevices] = {0};  // context the address belongs to

// Unique id of the calling thread's current context (driver entry points
// fetched through the runtime, so the library needs no link to libcuda);
// 0 when there is none or it cannot be read.
unsigned long long current_context_id() {
    static PFN_cuCtxGetCurrent_v4000 get_current = nullptr;
    static PFN_cuCtxGetId_v12000 get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = (PFN_cuCtxGetCurrent_v4000)f;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = (PFN_cuCtxGetId_v12000)f;
    });
    CUcontext c = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c) return 0;
    if (get_id(c, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the scratch array on the current device: looked up on the
// device's first call and again when its context changed (a reset reloads the
// module); the lookup itself makes the device's context current.
int scratch_for_current_device(int **out) {
    int dev = 0;
    DPG_CK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return dpg::set_error(DPG_ERR_ARG, "device index out of range");
    std::lock_guard<std::mutex> g(g_lock);
    const unsigned long long ctx = current_context_id();
    if (!g_scratch_addr[dev] || ctx == 0 || ctx != g_scratch_ctx[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            return dpg::set_error(DPG_ERR_CUDA, "cudaGetSymbolAddress(scratch): %s", cudaGetErrorString(e));
        g_scratch_addr[dev] = (int *)p;
        g_scratch_ctx[dev] = current_context_id();
    }
    *out = g_scratch_addr[dev];
    return DPG_OK;
}

}  // namespace

extern "C" int dpg_disk_forces_noalloc(const double *x, const double *y, const double *radii,
                                       int64_t n, double box_x, double box_y, double e_c,
                                       double n_c, double max_diameter, double *fx, double *fy,
                                       double *pe, void *cuda_stream) {
    if (!x || !y || !radii || !fx || !fy || !pe)
        return dpg::set_error(DPG_ERR_ARG, "dpg_disk_forces_noalloc: null pointer");
    if (n <= 0 || n > kMaxParticles)
        return dpg::set_error(DPG_ERR_ARG, "dpg_disk_forces_noalloc: n must be in [1, %d]", kMaxParticles);
    if (!(box_x > 0) || !(box_y > 0) || !(max_diameter > 0))
        return dpg::set_error(DPG_ERR_ARG, "dpg_disk_forces_noalloc: box and max_diameter must be > 0");
    if (box_x != box_y) return dpg::set_error(DPG_ERR_ARG, "dpg_disk_forces_noalloc: square boxes only");
    // cells no smaller than the largest contact distance
    const double per_side = std::floor(box_x / max_diameter);
    if (per_side * per_side > (double)kMaxCells)
        return dpg::set_error(DPG_ERR_ARG,
                              "dpg_disk_forces_noalloc: %.0f x %.0f cells exceed the %d-cell scratch "
                              "(box / max_diameter must stay below %d)",
                              per_side, per_side, kMaxCells, 257);
    long long ncd = (long long)per_side;
    if (ncd < 3) ncd = 1;
    int *base = nullptr;
    DPG_TRY(scratch_for_current_device(&base));
    NaArgs a;
    a.x = x; a.y = y; a.r = radii; a.fx = fx; a.fy = fy; a.pe = pe;
    a.n = (int)n; a.ncd = (int)ncd; a.bx = box_x; a.by = box_y; a.cs = box_x / ncd;
    a.e_c = e_c; a.n_c = n_c;
    a.cnt = base;
    a.start = base + (kMaxCells + 1);
    a.cur = base + 2 * (kMaxCells + 1);
    a.items = base + 3 * (kMaxCells + 1);
    a.cell = a.items + kMaxParticles;
    cudaStream_t st = (cudaStream_t)cuda_stream;
    const int nb = (int)((n + 255) / 256), cb = (int)((ncd * ncd + 1 + 255) / 256);
    if (ncd >= 3) {  // the all-pairs case (fewer than 3 cells a side) needs no cell list
        na_clear<<<cb, 256, 0, st>>>(a);
        na_count<<<nb, 256, 0, st>>>(a);
        na_scan<<<1, 1024, 0, st>>>(a);
        na_fill<<<nb, 256, 0, st>>>(a);
        na_sort<<<cb, 256, 0, st>>>(a);
    }
    na_force<<<nb, 256, 0, st>>>(a);
    DPG_CK(cudaGetLastError());
    return DPG_OK;
}
