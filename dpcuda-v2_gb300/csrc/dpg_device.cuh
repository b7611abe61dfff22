// dpg_device.cuh -- device-resident system layout shared by the kernels.
//
// One system lives in HBM as:
//   params  (DevParams)  written by the host when the box / neighbour setup changes
//   view    (DevView)    pointers to the CURRENT buffers; the cell reorder writes the
//                        gathered data into the alternate buffers and swaps the
//                        pointers here on the device, so no host round trip (and no
//                        CUDA-graph re-capture) is needed when particles are re-sorted
//   state   (DevState)   scalars owned by the device: displacement maxima, rebuild
//                        decision, FIRE state, reduction results, stop flags
// Particle data are SoA over particles with x,y interleaved as double2 so each
// particle's position / velocity / force is one coalesced 16-byte access.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <cmath>

namespace dpg {

constexpr int kTPB = 256;      // threads per block for per-particle kernels
constexpr int kScanTPB = 1024; // single-block cell-count scan

enum StopBits : int {
    kDone = 1,       // loop finished (converged, stopped or out of steps)
    kOverflow = 2,   // neighbour count exceeded capacity: halt until the host grows it
    kError = 4,
};

struct DevParams {
    int n;
    int method;   // DPG_NEIGH_*
    int ncd;      // cells per dimension
    int ncells;
    int cap;      // neighbour capacity per particle
    int precision;
    double box[2];
    double e_c, n_c;
    double cutoff2;     // neighbour cutoff squared
    double cell_size;
    double nthr2, cthr2;  // rebuild thresholds (squared)
    double inv_area;
    // mixed form (precision DPG_MIXED): a grid of mg_m[d] cells of size
    // mg_cs[d] per axis; each particle keeps an FP32 offset from the centre
    // of its grid cell and the cell's wrapped coordinates (pk)
    int mg_m[2];
    double mg_cs[2], mg_inv[2];
    float mg_cs_f[2];
};

struct DevView {
    double2 *pos, *vel, *frc;
    double *rad, *mass;
    int *sidx;  // static index of the particle in each slot
    double2 *pos_t, *vel_t, *frc_t;
    double *rad_t, *mass_t;
    int *sidx_t;
    double2 *m1, *m2, *m1_t, *m2_t;  // Adam moments and their swap twins
    int *nbr;                        // neighbour list, column-major [cap][n]
    float4 *pk;                      // mixed form: {offset x, offset y, radius, cell code}
};

struct DevState {
    double max_nd2, max_cd2;  // max squared displacement since the last list / cell build
    int rebuild;              // 0 none, 1 neighbour list, 2 cell list + neighbour list
    int max_count;
    int flags;                // StopBits
    int fire_uphill;          // apply the FIRE "uphill" branch at the next move
    long long n_rebuilds, n_cell_rebuilds;
    // results of the last reductions
    double pe, ke, power, fmax2, fsum_x, fsum_y;
    double stress[4];
    double contacts;
    // FIRE (include/integrator/fire.h:15-35)
    double f_alpha, f_alpha0, f_dt, f_dtmax, f_dtmin;
    long long f_ngood, f_nbad;
    int f_stopped;
    int f_converged;
    // minimizeFire loop (src/routines/minimization.cu:75-112)
    double last_avg_pe, pe_target, pe_diff_target, fmax_target, dof;
    long long iter, max_steps, result_step;
    long long nve_steps_done;
    double damping;           // DampedNVE coefficient (0 in plain NVE)
    int walls;                // NVE::wall_step: wall forces added before the pair forces
    int pad3;
    // mixed form: FP64 pair arithmetic once fp64_now is set (FIRE refinement)
    int fp64_now;
    int pad2;
    double switch_fmax, best_f2;
    long long best_it;
    // loop guard: the WHILE body ends with k_loop_guard, which stops the loop
    // when a flag is raised or after guard_limit iterations, whatever else happens
    long long guard, guard_limit;
    // conditional-node handles of the running graph (0 outside a graph)
    unsigned long long h_loop, h_rb;
    unsigned int ticket;  // last-block-done counter
    unsigned int pad;
};

struct DevScratch {
    double2 *pos_n, *pos_c;  // positions at the last neighbour / cell build
    double *pe;
    int *count;              // neighbour counts
    int *cell_raw;           // cell of each particle before the sort
    int *cell_of;            // cell of each particle in sorted order
    int *cell_cnt, *cell_cur, *cell_start, *perm;
    double *partials;        // per-block reduction partials
    int max_blocks;
    // snapshot (setLastState)
    double2 *s_pos, *s_vel, *s_frc;
    double *s_rad, *s_mass;
    int *s_sidx;
    double s_box[2];
};

struct DevSys {
    DevParams p;
    DevView v;
    DevState s;
    DevScratch w;
};

// ---- shared arithmetic (reference order, see oracle/dpg_oracle.c) ----------

// minimum image: include/particles/base/kernels.cuh:65-72, d - L * round(d / L).
// For |d| < L/4 the quotient rounds to +-0, so the result is d (or +0 for
// d = -0): returning d + 0.0 there is bit-identical and skips the FP64
// division, which is expensive on GB300's FP64 pipe.
__device__ __forceinline__ double pbc_dist(double a, double b, double L) {
    double d = a - b;
    if (fabs(d) < 0.25 * L) return d + 0.0;
    return d - L * round(d / L);
}

// include/particles/base/kernels.cuh:53-55
__device__ __forceinline__ int pmod(int a, int b) { return (a % b + b) % b; }

// getPBCCellIndex: include/particles/base/kernels.cuh:285-301
__device__ __forceinline__ int cell_coord(double p, double cs, int ncd) {
    long long idx = __double2ll_rd(p / cs);
    long long m = idx % ncd;
    return (int)(idx >= 0 ? m : (m + ncd) % ncd);
}

// ---- mixed form: FP32 offsets from grid-cell centres -------------------------
// grid cell counts: cells of about 2 length units, at least 3 a side (fixed at
// creation); the cell size follows the box
inline void mixed_grid_init(DevParams &p) {
    for (int d = 0; d < 2; d++) {
        double m = std::floor(p.box[d] / 2.0);
        p.mg_m[d] = (int)(m < 3.0 ? 3.0 : (m > 65535.0 ? 65535.0 : m));
    }
}

inline void mixed_grid_update(DevParams &p) {
    for (int d = 0; d < 2; d++) {
        if (p.mg_m[d] <= 0) continue;
        p.mg_cs[d] = p.box[d] / p.mg_m[d];
        p.mg_inv[d] = p.mg_m[d] / p.box[d];
        p.mg_cs_f[d] = (float)p.mg_cs[d];
    }
}

__device__ __forceinline__ int wrap_cell(long long c, int m) {
    long long r = c % m;
    return (int)(r < 0 ? r + m : r);
}

// offset of x from the centre of its cell of the mixed grid, radius, and the
// cell's wrapped coordinates packed as cx | cy << 16
__device__ __forceinline__ float4 mixed_pack(const DevParams &p, double2 x, double r) {
    double fx = floor(x.x * p.mg_inv[0]), fy = floor(x.y * p.mg_inv[1]);
    int wx = wrap_cell((long long)fx, p.mg_m[0]), wy = wrap_cell((long long)fy, p.mg_m[1]);
    float4 k;
    k.x = (float)(x.x - (fx + 0.5) * p.mg_cs[0]);
    k.y = (float)(x.y - (fy + 0.5) * p.mg_cs[1]);
    k.z = (float)r;
    k.w = __int_as_float(wx | (wy << 16));
    return k;
}

// FP32 harmonic pair force on a from b: displacement (o_a - o_b) + dc * cell
// size, with the periodic wrap done on the integer cell difference dc
__device__ __forceinline__ float mixed_pair(const DevParams &p, float4 a, float4 b, float e_c,
                                            float n_c, float &fx, float &fy) {
    int ca = __float_as_int(a.w), cb = __float_as_int(b.w);
    int dcx = (ca & 0xffff) - (cb & 0xffff), dcy = (ca >> 16) - (cb >> 16);
    const int mx = p.mg_m[0], my = p.mg_m[1];
    if (dcx > mx / 2) dcx -= mx; else if (dcx < -(mx / 2)) dcx += mx;
    if (dcy > my / 2) dcy -= my; else if (dcy < -(my / 2)) dcy += my;
    float dx = (a.x - b.x) + (float)dcx * p.mg_cs_f[0];
    float dy = (a.y - b.y) + (float)dcy * p.mg_cs_f[1];
    float rs = a.z + b.z;
    float d2 = dx * dx + dy * dy;
    fx = 0.f;
    fy = 0.f;
    if (d2 >= rs * rs) return 0.f;
    float d = sqrtf(d2);
    float ov = 1.0f - d / rs;
    float ovp = n_c == 2.0f ? ov : powf(ov, n_c - 1.0f);
    float fm = e_c * ovp / (rs * d);
    fx = fm * dx;
    fy = fm * dy;
    return e_c * ov * ovp / (2.0f * n_c);
}

// ---- block reductions with a deterministic order ---------------------------

template <int K>
__device__ __forceinline__ void warp_sum(double (&v)[K]) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int k = 0; k < K; k++) v[k] += __shfl_down_sync(0xffffffffu, v[k], off);
}

template <int K>
__device__ __forceinline__ void warp_max(double (&v)[K]) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int k = 0; k < K; k++) v[k] = fmax(v[k], __shfl_down_sync(0xffffffffu, v[k], off));
}

// Reduce K values over the block (ops[k]: 0 = sum, 1 = max).  Thread 0 gets the result.
template <int K, typename T>
__device__ __forceinline__ void block_reduce(T (&v)[K], const int (&ops)[K], T *sm) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    // warp tree (shfl_down), then warp results in order; ops are compile-time
    // constants at every call site, so only the needed operation is emitted
#pragma unroll
    for (int off = 16; off > 0; off >>= 1)
#pragma unroll
        for (int k = 0; k < K; k++) {
            T o = __shfl_down_sync(0xffffffffu, v[k], off);
            v[k] = ops[k] ? (v[k] > o ? v[k] : o) : v[k] + o;
        }
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; k++) sm[wid * K + k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            T a = sm[k];
            for (int w = 1; w < nw; w++) {
                T b = sm[w * K + k];
                a = ops[k] ? (a > b ? a : b) : a + b;
            }
            v[k] = a;
        }
    }
    __syncthreads();
}

// Grid-wide reduction by "last block done": every block publishes its partials,
// the last block to arrive reduces them in a fixed order.  Returns true on
// thread 0 of the last block, with the totals in v.  All threads of every
// block must call it.
template <int K>
__device__ bool grid_reduce(double (&v)[K], const int (&ops)[K], DevSys *ds) {
    __shared__ double sm[32 * K];
    __shared__ int am_last;
    block_reduce<K>(v, ops, sm);
    const int G = gridDim.x;
    double *part = ds->w.partials;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) part[k * G + blockIdx.x] = v[k];
        __threadfence();
        unsigned t = atomicAdd(&ds->s.ticket, 1u);
        am_last = (t == (unsigned)G - 1);
    }
    __syncthreads();
    if (!am_last) return false;
    __threadfence();
    double a[K];
#pragma unroll
    for (int k = 0; k < K; k++) a[k] = ops[k] ? -INFINITY : 0.0;
    // batches of 8 independent loads per thread (the latency of one L2 round
    // trip per batch), combined in ascending block order
    const int bd = blockDim.x;
    for (int b0 = threadIdx.x; b0 < G; b0 += 8 * bd) {
        double x[8][K];
#pragma unroll
        for (int u = 0; u < 8; u++)
#pragma unroll
            for (int k = 0; k < K; k++) {
                int b = b0 + u * bd;
                x[u][k] = b < G ? __ldcg(&part[k * G + b]) : (ops[k] ? -INFINITY : 0.0);
            }
#pragma unroll
        for (int u = 0; u < 8; u++)
#pragma unroll
            for (int k = 0; k < K; k++) {
                if (b0 + u * bd >= G) continue;
                a[k] = ops[k] ? fmax(a[k], x[u][k]) : a[k] + x[u][k];
            }
    }
    block_reduce<K>(a, ops, sm);
    if (threadIdx.x == 0) {
        ds->s.ticket = 0;
#pragma unroll
        for (int k = 0; k < K; k++) v[k] = a[k];
        return true;
    }
    return false;
}

// Same arrival protocol with no data: true on thread 0 of the last block.
__device__ __forceinline__ bool grid_last_block(DevSys *ds) {
    __shared__ int am_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned t = atomicAdd(&ds->s.ticket, 1u);
        am_last = (t == gridDim.x - 1);
        if (am_last) ds->s.ticket = 0;
    }
    __syncthreads();
    return am_last && threadIdx.x == 0;
}

}  // namespace dpg
