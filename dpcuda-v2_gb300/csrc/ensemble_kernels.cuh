// ensemble_kernels.cuh -- the batched form: many independent disk systems of
// uneven size advanced together, every kernel launch covering all of them.
//
// Layout.  System s owns the slot range [off[s], off[s] + n[s]) of the shared
// per-slot arrays; ranges are padded to whole blocks, so every block belongs to
// exactly one system and per-system reductions are deterministic (block
// partials, then the last block of the system to finish sums them in a fixed
// order, with a compensated (Kahan) sum).  Slots are never re-sorted: each
// system has its own cell grid, rebuilt into per-cell item lists whenever that
// system's neighbour list is rebuilt.
//
// Precision.  Each system carries prec = 0 (FP32 pairs), 2 (double-word FP32
// pairs, the refinement) or 1 (FP64):
//  - mixed: positions are FP64; for the pair loop each particle also keeps an
//    FP32 offset from the centre of its cell (|offset| < 1.3 units, so the
//    offset carries ~6e-8 absolute precision) and its cell coordinates; a pair
//    displacement is (o_i - o_j) + dc * cell_size in FP32 with the periodic
//    wrap done on the integer cell coordinates, the pair force is FP32, and
//    the per-particle sums are FP64.  One 16-byte load per neighbour.
//  - FP64: the reference's pair arithmetic (disk_pair).
//  Mixed systems switch to FP64 when max|F| falls below switch_fmax, or when
//  it stops falling (the FP32 noise floor, ~1e-7 x the contact stiffness),
//  for the final refinement.
//
// Control.  Per-system FIRE state, convergence tests and the pressure-band
// jamming state machine (scripts/runArthurJamWithFire.cpp) live on the device;
// finished systems are masked out.  One CUDA-graph WHILE loop drives
// move -> IF(any rebuild){cells, lists} -> force -> transition -> guard.
#pragma once
#include "disk_kernels.cuh"

namespace dpg {
namespace {

constexpr int kEB = 128;  // threads per block (slot ranges are padded to this)
// a mixed system within 100x of switch_fmax whose max|F| has not dropped by
// 10% for this many iterations has reached the FP32 noise floor and switches
// to FP64 pair arithmetic (far above it, FIRE's max|F| may plateau for
// thousands of iterations while the packing rearranges)
constexpr long long kStallIters = 2000;

enum EPhase : int { kIdle = 0, kSetup = 1, kMinimize = 2 };
enum EAction : int { kActNone = 0, kActDecompress = 1, kActCompress = 2, kActRevertScale = 3 };

struct ESys {
    // geometry
    int off, n, blk0, nblk;
    int ncd, cell_off;       // cell grid (ncd x ncd) and its first global cell
    int item_off;            // first slot of its cell items (systems packed in order)
    double L, cs, inv_cs;
    float cs_f, cs_lo;       // cs as a double word: cs_f + cs_lo
    // loop
    int phase, rebuild, prec, done;
    int vel_f32;             // velocities live in vel32 (set at the FP32 -> FP64 switch)
    int uphill, stopped, converged, pending;
    long long iter, fire_total, rebuilds, fp64_total, dw_total;
    double dt, alpha, last_avg_pe;
    long long ngood, nbad;
    // results of the last force pass
    double pe, power, fmax2, virial, contacts, max_d2;
    // mixed phase: lowest max|F|^2 so far and the iteration it was reached
    double best_f2;
    long long best_it;
    // jamming (scripts/runArthurJamWithFire.cpp:36-106)
    int jam_stage;           // 0 decompressing, 1 compressing
    int jam_status;          // 0 final state, 1 length tolerance, 2 out of steps, -1 running
    long long jam_step;
    double L_low, L_high, L_last, L_saved, scale, pressure;
    int minimizations;
    unsigned ticket_a, ticket_b;
    int resume;              // persistent form: the last launch stopped after a list overflow
                             // (move done, lists to rebuild, then the force pass)
    int res_valid;           // resident form: pk / pkl hold the exact double-word offsets
                             // written back by its last launch
    int verify;              // resident form: the next pass is an FP64 force pass at the
                             // current positions, 1 = check max|F| (back to double words if
                             // it fails), 2 = final measurement of a finished minimisation
    double dw_scale;         // resident form: double-word exit at dw_scale * fmax_target
    double inv_n;            // 1 / n (the epilogue multiplies; FP64 division is slow)
    int fprec;               // grid form: the arithmetic of this iteration's force pass
                             // (set by the move, so a switch made by one force kernel
                             // does not give the system a second pass in the other)
};

struct EParams {
    int S, T, nblocks, cap, total_cells;
    double e_c, n_c;
    double cutoff2, half_skin2;
    float cutoff2_f;
    // FIRE
    double alpha0, dt0, pe_target, pe_diff_target, fmax_target, switch_fmax;
    int dw_ok;               // double-word refinement available (harmonic contacts, n_c = 2)
    float ec_hi, ec_lo;      // e_c as a double word
    long long max_steps;
    // jamming
    int jam;                 // 0: plain minimisation, 1: jamming protocol
    double p_low, p_high, compression_rate, length_tol, decompress;
    long long max_compressions;
    int res;                 // resident form: FP64 passes only verify double-word states
    double fmax_cert2;       // (0.99 fmax_target)^2: an FP64 pass certifies max|F| with a 1 %
                             // margin, so the reference arithmetic (IEEE division and square
                             // root where these passes use Newton steps; ulp-level force
                             // differences) also finds max|F| <= fmax_target
};

struct EDev {
    EParams p;
    ESys *sys;
    int *blk_sys;            // block -> system
    int *slot_sys;           // slot -> system (-1 padding)
    double2 *pos, *vel, *frc, *pos_ref, *pos_save;
    double *rad, *mass, *pe, *vir;
    float2 *vel32, *frc32;   // FP32 phase: velocities and forces
    float *invm;             // 1 / mass
    float4 *pk;              // {offset x, offset y, radius, cell code}, offsets from ctr
    float4 *pkl;             // low words of the offsets and radius (double-word refinement)
    float2 *oref;            // offsets at the last list build (FP32 displacement test)
    double2 *ctr;            // centre of the particle's (unwrapped) cell at the last build
    int *cellc;              // wrapped cell code (cx | cy << 16) of each slot
    int *nbr, *cnt;          // neighbour list [cap][T], counts
    int *cell_cnt, *cell_start, *cell_cur, *cell_items;
    double *part;            // [nblocks][8] block partials
    int n_flagged, max_count, overflow, active;
    int n_pending;           // systems with a transition queued by the last force pass
    unsigned ticket;
    long long guard, guard_limit;
    unsigned long long h_loop, h_rb, h_tr;
    unsigned long long h_f32, h_fhi;  // graph IF nodes of the two force kernels
    int n_f32, n_fhi;                 // live systems whose pass is FP32 / refinement or FP64
};

__device__ __forceinline__ int code_of(int cx, int cy) { return cx | (cy << 16); }
__device__ __forceinline__ int code_x(int c) { return c & 0xffff; }
__device__ __forceinline__ int code_y(int c) { return c >> 16; }

// Per-system reduction by "last block of the system done": every block of the
// system publishes its block partials; the last block to arrive reduces them
// with all of its threads (thread t takes blocks t, t + blockDim, ... with a
// compensated (Kahan) running sum, then a fixed-order tree over the threads),
// so the result is deterministic and costs one L2 round trip, not one per
// block.  Block partials are reduced in T (FP32 in the FP32 phase, whose
// per-particle values are FP32 anyway), the per-system totals in FP64.
// Returns true on thread 0 of that block, with the totals in out (ops[k]:
// 0 = sum, 1 = max of non-negative values).  Every thread of every block must
// call it.
template <int K, typename T>
__device__ bool sys_reduce_t(EDev *e, ESys &s, T (&v)[K], const int (&ops)[K], unsigned *ticket,
                             double (&out)[K]) {
    __shared__ T sm[32 * K];
    __shared__ double smd[32 * K];
    __shared__ int last;
    block_reduce<K, T>(v, ops, sm);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) e->part[(size_t)blockIdx.x * 8 + k] = (double)v[k];
        __threadfence();
        unsigned t = atomicAdd(ticket, 1u);
        last = (t == (unsigned)s.nblk - 1);
        if (last) *ticket = 0;
    }
    __syncthreads();
    if (!last) return false;
    __threadfence();
    double a[K], c[K];
#pragma unroll
    for (int k = 0; k < K; k++) { a[k] = 0.0; c[k] = 0.0; }
    for (int b = threadIdx.x; b < s.nblk; b += blockDim.x) {
        const double *pp = &e->part[(size_t)(s.blk0 + b) * 8];
#pragma unroll
        for (int k = 0; k < K; k++) {
            double x = __ldcg(&pp[k]);
            if (ops[k]) {
                a[k] = fmax(a[k], x);
            } else {
                double y = x - c[k];
                double t = a[k] + y;
                c[k] = (t - a[k]) - y;
                a[k] = t;
            }
        }
    }
    block_reduce<K, double>(a, ops, smd);
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) out[k] = a[k];
        return true;
    }
    return false;
}

// FP64 values in and out (v holds the totals on the returning thread)
template <int K>
__device__ bool sys_reduce(EDev *e, ESys &s, double (&v)[K], const int (&ops)[K], unsigned *ticket) {
    return sys_reduce_t<K, double>(e, s, v, ops, ticket, v);
}

__device__ __forceinline__ bool grid_last(EDev *e) {
    __shared__ int last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned t = atomicAdd(&e->ticket, 1u);
        last = (t == gridDim.x - 1);
        if (last) e->ticket = 0;
    }
    __syncthreads();
    return last && threadIdx.x == 0;
}

// ---- FIRE decision (src/integrator/fire.cu:13-34), per system -----------------
__device__ void e_fire_decide(const EParams &p, ESys &s, double power) {
    if (power > 0) {
        s.ngood++;
        s.nbad = 0;
        if (s.ngood > 5) {
            s.dt = fmin(s.dt * 1.1, 10.0 * p.dt0);
            s.alpha *= 0.99;
        }
        s.uphill = 0;
    } else {
        s.ngood = 0;
        s.nbad++;
        if (s.nbad > 10) {
            s.stopped = 1;
            s.uphill = 0;
            return;
        }
        s.dt = fmax(s.dt * 0.5, 0.001 * p.dt0);
        s.alpha = p.alpha0;
        s.uphill = 1;
    }
}

// ---- double-FP32 ("double-word") arithmetic for the refinement stage ----------
// A value is hi + lo with |lo| <= ulp(hi) / 2 (~48 significant bits), computed
// on the FP32 pipe, which GB300 runs ~64x faster than FP64.  Building blocks:
// Knuth's TwoSum and Fast2Sum, the FMA-based TwoProduct, and the double-word
// sum / product / quotient / square root of Joldes, Muller and Popescu, "Tight
// and rigorous error bounds for basic building blocks of double-word
// arithmetic" (ACM TOMS 44(2), 2017), relative errors of a few 2^-48.
struct dw {
    float hi, lo;
};

__device__ __forceinline__ dw two_sum(float a, float b) {
    float s = __fadd_rn(a, b), bb = __fsub_rn(s, a);
    float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    return {s, e};
}
__device__ __forceinline__ dw fast_two_sum(float a, float b) {  // |a| >= |b|
    float s = __fadd_rn(a, b);
    return {s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ dw dw_add(dw x, dw y) {
    dw s = two_sum(x.hi, y.hi), t = two_sum(x.lo, y.lo);
    float c = __fadd_rn(s.lo, t.hi);
    dw v = fast_two_sum(s.hi, c);
    float w = __fadd_rn(t.lo, v.lo);
    return fast_two_sum(v.hi, w);
}
__device__ __forceinline__ dw dw_neg(dw x) { return {-x.hi, -x.lo}; }
__device__ __forceinline__ dw dw_mul(dw x, dw y) {
    float ch = __fmul_rn(x.hi, y.hi);
    float cl = __fmaf_rn(x.hi, y.hi, -ch);
    float tl = __fmul_rn(x.hi, y.lo);
    cl = __fadd_rn(cl, __fmaf_rn(x.lo, y.hi, tl));
    return fast_two_sum(ch, cl);
}
__device__ __forceinline__ dw dw_mul_f(dw x, float y) {
    float ch = __fmul_rn(x.hi, y);
    float cl = __fmaf_rn(x.hi, y, -ch);
    cl = __fmaf_rn(x.lo, y, cl);
    return fast_two_sum(ch, cl);
}
__device__ __forceinline__ dw dw_div(dw x, dw y) {
    float q = __fdiv_rn(x.hi, y.hi);
    dw r = dw_add(x, dw_neg(dw_mul_f(y, q)));  // remainder x - q y
    float q2 = __fdiv_rn(r.hi, y.hi);
    return fast_two_sum(q, q2);
}
__device__ __forceinline__ dw dw_sqrt(dw x) {
    float s = __fsqrt_rn(x.hi);
    float p = __fmul_rn(s, s), pe = __fmaf_rn(s, s, -p);
    float r = __fadd_rn(__fsub_rn(__fsub_rn(x.hi, p), pe), x.lo);
    return fast_two_sum(s, __fdiv_rn(r, __fmul_rn(2.0f, s)));
}
__device__ __forceinline__ bool dw_ge(dw a, dw b) { return a.hi > b.hi || (a.hi == b.hi && a.lo >= b.lo); }
__device__ __forceinline__ double dw_to_double(dw a) { return (double)a.hi + (double)a.lo; }

// split an FP64 value into a double word
__device__ __forceinline__ dw dw_from_double(double v) {
    float h = (float)v;
    return {h, (float)(v - (double)h)};
}

// ---- FP64 reciprocal and reciprocal square root for the refinement stage ----
// Newton-Raphson iteration on an FP32 estimate: y <- y (1.5 - 0.5 x y^2) for
// x^-1/2 and y <- y (2 - x y) for x^-1; each step doubles the number of
// correct bits, so two steps from the 2^-23 FP32 seed reach FP64 precision.
// Valid for x in the FP32 normal range (contact distances and radius sums).
__device__ __forceinline__ double rsqrt_newton(double x) {
    double y = (double)rsqrtf((float)x);
    y = y * (1.5 - 0.5 * x * y * y);
    y = y * (1.5 - 0.5 * x * y * y);
    return y;
}

__device__ __forceinline__ double rcp_newton(double x) {
    double y = (double)(1.0f / (float)x);
    y = y * (2.0 - x * y);
    y = y * (2.0 - x * y);
    return y;
}

// FIRE mix (per-particle norms, src/particles/base/kernels.cu:91-112) with
// |v| / |F| from the Newton reciprocal square root; the FP64 square root is
// kept only for |v|^2 below the FP32 normal range
__device__ __forceinline__ double2 fire_mix_newton(double2 v, double2 f, double alpha) {
    const double fn2 = f.x * f.x + f.y * f.y, vn2 = v.x * v.x + v.y * v.y;
    double mix = 0.0;
    if (fn2 > 1e-32) {  // |F| > 1e-16
        const double vn = vn2 > 1e-36 ? vn2 * rsqrt_newton(vn2) : sqrt(vn2);
        mix = vn * rsqrt_newton(fn2) * alpha;
    } else {
        v = make_double2(0.0, 0.0);
    }
    return make_double2(v.x * (1 - alpha) + f.x * mix, v.y * (1 - alpha) + f.y * mix);
}

// ---- move -------------------------------------------------------------------
// FIRE mix in FP32 (per-particle norms, src/particles/base/kernels.cu:91-112)
__device__ __forceinline__ float2 fire_mix_f(float2 v, float2 f, float alpha) {
    float fn = sqrtf(f.x * f.x + f.y * f.y), vn = sqrtf(v.x * v.x + v.y * v.y);
    float mix = 0.f;
    if (fn > 1e-16f) {
        mix = vn / fn * alpha;
    } else {
        v = make_float2(0.f, 0.f);
    }
    return make_float2(v.x * (1.f - alpha) + f.x * mix, v.y * (1.f - alpha) + f.y * mix);
}

// FIRE move of slot i.  FP32 phase: velocities, forces, the kick and the mix
// in FP32; FP64 only for the position sums and the offsets from the cell
// centre.  FP64 phase: the reference arithmetic.  Returns the squared
// displacement since the last list build in vf (FP32 phases) or v (FP64).
__device__ __forceinline__ void e_move_one(EDev *e, const ESys &s, int i, double &v0, float &vf0) {
        double2 x = e->pos[i];
        const double2 c = e->ctr[i];
        if (s.prec != 1) {
            const float dt = (float)s.dt, alpha = (float)s.alpha;
            float2 u = e->vel32[i];
            const float2 f = e->frc32[i];
            if (s.uphill) {
                const float back = -0.5f * dt;
                x.x += (double)(u.x * back);
                x.y += (double)(u.y * back);
                u = make_float2(0.f, 0.f);
            }
            const float h = 0.5f * dt * e->invm[i];
            u.x += f.x * h;
            u.y += f.y * h;
            u = fire_mix_f(u, f, alpha);
            e->vel32[i] = u;
            x.x += (double)(u.x * dt);
            x.y += (double)(u.y * dt);
            e->pos[i] = x;
            const double ox = x.x - c.x, oy = x.y - c.y;
            const float2 o = make_float2((float)ox, (float)oy);
            *reinterpret_cast<float2 *>(&e->pk[i]) = o;
            if (s.prec == 2)  // low words for the double-word pair arithmetic
                *reinterpret_cast<float2 *>(&e->pkl[i]) =
                    make_float2((float)(ox - (double)o.x), (float)(oy - (double)o.y));
            const float2 r = e->oref[i];
            const float ddx = o.x - r.x, ddy = o.y - r.y;
            vf0 = ddx * ddx + ddy * ddy;
        } else {
            const double dt = s.dt, alpha = s.alpha;
            double2 u, f = e->frc[i];
            if (s.vel_f32) {
                const float2 w = e->vel32[i];
                u = make_double2(w.x, w.y);
            } else {
                u = e->vel[i];
            }
            if (s.uphill) {
                double back = -dt / 2.0;
                x.x = x.x + u.x * back;
                x.y = x.y + u.y * back;
                u = make_double2(0.0, 0.0);
            }
            double dtm = (0.5 * dt) * rcp_newton(e->mass[i]);
            u.x = u.x + f.x * dtm;
            u.y = u.y + f.y * dtm;
            u = fire_mix_newton(u, f, alpha);
            x.x = x.x + u.x * dt;
            x.y = x.y + u.y * dt;
            e->vel[i] = u;
            e->pos[i] = x;
            *reinterpret_cast<float2 *>(&e->pk[i]) = make_float2((float)(x.x - c.x), (float)(x.y - c.y));
            double2 r = e->pos_ref[i];
            double ddx = x.x - r.x, ddy = x.y - r.y;
            v0 = ddx * ddx + ddy * ddy;
        }
}

// per-system result of a move pass
__device__ __forceinline__ void e_move_sys(const EParams &p, ESys &s, double max_d2) {
    s.max_d2 = max_d2;
    if (s.max_d2 > p.half_skin2) s.rebuild = 1;
    if (s.prec == 1) s.vel_f32 = 0;  // every thread has read vel32 by now
}

__global__ void __launch_bounds__(kEB) e_move(EDev *e) {
    const int sid = e->blk_sys[blockIdx.x];
    ESys &s = e->sys[sid];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool live = s.phase == kMinimize;
    const bool f32 = s.prec != 1;
    double v[1] = {0.0};
    float vf[1] = {0.f};
    if (live && i < s.off + s.n) e_move_one(e, s, i, v[0], vf[0]);
    const int ops[1] = {1};
    double tot[1];
    const bool last = f32 ? sys_reduce_t<1, float>(e, s, vf, ops, &s.ticket_a, tot)
                          : sys_reduce_t<1, double>(e, s, v, ops, &s.ticket_a, tot);
    if (last) {
        if (live) e_move_sys(e->p, s, tot[0]);
        s.fprec = s.prec;
        if (s.rebuild && s.phase != kIdle) atomicAdd(&e->n_flagged, 1);
        if (s.phase != kIdle) atomicAdd(s.prec == 0 ? &e->n_f32 : &e->n_fhi, 1);
    }
    if (grid_last(e)) {
        int any = e->n_flagged > 0;
        if (e->h_rb) cudaGraphSetConditional(e->h_rb, any ? 1u : 0u);
        // launch only the force kernels some system needs this iteration
        if (e->h_f32) cudaGraphSetConditional(e->h_f32, e->n_f32 > 0 ? 1u : 0u);
        if (e->h_fhi) cudaGraphSetConditional(e->h_fhi, e->n_fhi > 0 ? 1u : 0u);
        e->n_f32 = 0;
        e->n_fhi = 0;
    }
}

// ---- per-system cell lists and neighbour lists -------------------------------
__device__ __forceinline__ bool flagged(const ESys &s) { return s.rebuild && s.phase != kIdle; }

__device__ __forceinline__ int wrap_int(long long c, int ncd) {
    long long m = c % ncd;
    return (int)(m < 0 ? m + ncd : m);
}

// cell of slot i, its centre, packed offsets; counts it in its cell
__device__ __forceinline__ void e_cell_count_one(EDev *e, const ESys &s, int i) {
    double2 x = e->pos[i];
    double fx = floor(x.x * s.inv_cs), fy = floor(x.y * s.inv_cs);
    int cx = wrap_int((long long)fx, s.ncd), cy = wrap_int((long long)fy, s.ncd);
    int code = code_of(cx, cy);
    e->cellc[i] = code;
    double2 c = make_double2((fx + 0.5) * s.cs, (fy + 0.5) * s.cs);
    e->ctr[i] = c;
    const double ox = x.x - c.x, oy = x.y - c.y, r = e->rad[i];
    const float hx = (float)ox, hy = (float)oy, hr = (float)r;
    e->pk[i] = make_float4(hx, hy, hr, __int_as_float(code));
    e->pkl[i] = make_float4((float)(ox - (double)hx), (float)(oy - (double)hy), (float)(r - (double)hr), 0.f);
    atomicAdd(&e->cell_cnt[s.cell_off + cx + cy * s.ncd], 1);
}

__global__ void __launch_bounds__(kEB) e_cell_count(EDev *e) {
    const int sid = e->blk_sys[blockIdx.x];
    const ESys &s = e->sys[sid];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (!flagged(s) || i >= s.off + s.n) return;
    e_cell_count_one(e, s, i);
}

// exclusive scan of one system's cell counts per block (blockIdx.x = system);
// a system's items start at its item_off, so systems need no carry between them
// Exclusive scan of one system's cell counts by one block (any multiple of 32
// threads up to 1024); the system's items start at its item_off, so systems
// need no carry between them.  Every thread of the block must call it.
__device__ __forceinline__ void e_cell_scan_block(EDev *e, const ESys &s) {
    __shared__ int wsum[32];
    __shared__ int carry_s;
    const int nc = s.ncd * s.ncd, c0 = s.cell_off;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int carry = s.item_off;
    for (int base = 0; base < nc; base += blockDim.x) {
        int idx = base + threadIdx.x;
        int a = idx < nc ? __ldcg(&e->cell_cnt[c0 + idx]) : 0;
        int incl = a;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += y;
        }
        if (lane == 31) wsum[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            int w = lane < nw ? wsum[lane] : 0, wi = w;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, wi, off);
                if (lane >= off) wi += y;
            }
            if (lane < nw) wsum[lane] = wi - w;
            if (lane == 31) carry_s = wi;
        }
        __syncthreads();
        if (idx < nc) e->cell_start[c0 + idx] = carry + wsum[wid] + incl - a;
        carry += carry_s;
        __syncthreads();
    }
    // end of the last cell = start of the next system's items (sentinel)
    if (threadIdx.x == 0) e->cell_start[c0 + nc] = s.item_off + s.n;
}

constexpr int kEScanTPB = 256;
__global__ void __launch_bounds__(kEScanTPB) e_cell_scan(EDev *e) {
    const ESys &s = e->sys[blockIdx.x];
    if (!flagged(s)) return;
    e_cell_scan_block(e, s);
}

__device__ __forceinline__ void e_cell_fill_one(EDev *e, const ESys &s, int i) {
    int c = e->cellc[i];
    int g = s.cell_off + code_x(c) + code_y(c) * s.ncd;
    int slot = e->cell_start[g] + atomicAdd(&e->cell_cur[g], 1);
    e->cell_items[slot] = i;
}

__global__ void __launch_bounds__(kEB) e_cell_fill(EDev *e) {
    const int sid = e->blk_sys[blockIdx.x];
    const ESys &s = e->sys[sid];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (!flagged(s) || i >= s.off + s.n) return;
    e_cell_fill_one(e, s, i);
}

// ascending slot order inside cell g (deterministic lists); clears its counters
__device__ __forceinline__ void e_cell_sort_one(EDev *e, int g) {
    int b = e->cell_start[g], en = e->cell_start[g + 1];
    int *it = e->cell_items;
    for (int k = b + 1; k < en; k++) {
        int key = it[k];
        int j = k - 1;
        while (j >= b && it[j] > key) { it[j + 1] = it[j]; j--; }
        it[j + 1] = key;
    }
    e->cell_cnt[g] = 0;
    e->cell_cur[g] = 0;
}

__global__ void e_cell_sort(EDev *e) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= e->p.total_cells) return;
    e_cell_sort_one(e, g);
}

// neighbour list of slot i; returns its length
__device__ __forceinline__ int e_nlist_one(EDev *e, const ESys &s, int i) {
    int cnt = 0;
    {
        const int T = e->p.T, cap = e->p.cap, ncd = s.ncd;
        const double L = s.L, c2 = e->p.cutoff2;
        double2 xi = e->pos[i];
        int c = e->cellc[i];
        int cx = code_x(c), cy = code_y(c);
        if (ncd >= 3 && s.cs * s.cs >= c2) {
            // FP32 distances from the cell-centre offsets, with a 1e-4 relative
            // margin on the cutoff: the list may hold a few extra pairs, never
            // miss one (offsets carry ~1e-7 absolute rounding)
            const float4 a = e->pk[i];
            const float c2f = e->p.cutoff2_f * 1.0001f, cs = s.cs_f;
            for (int oy = -1; oy <= 1; oy++) {
                int yy = pmod(cy + oy, ncd);
                for (int ox = -1; ox <= 1; ox++) {
                    int g = s.cell_off + pmod(cx + ox, ncd) + yy * ncd;
                    const float sx = (float)ox * cs, sy = (float)oy * cs;
                    for (int k = e->cell_start[g]; k < e->cell_start[g + 1]; k++) {
                        int j = e->cell_items[k];
                        if (j == i) continue;
                        float4 b = e->pk[j];
                        float dx = (a.x - b.x) - sx, dy = (a.y - b.y) - sy;
                        if (dx * dx + dy * dy < c2f) {
                            if (cnt < cap) e->nbr[(size_t)cnt * T + i] = j;
                            cnt++;
                        }
                    }
                }
            }
        } else {  // grid too coarse for a 3x3 stencil: all pairs of the system
            for (int j = s.off; j < s.off + s.n; j++) {
                if (j == i) continue;
                double2 xj = e->pos[j];
                double dx = pbc_dist(xi.x, xj.x, L), dy = pbc_dist(xi.y, xj.y, L);
                if (dx * dx + dy * dy < c2) {
                    if (cnt < cap) e->nbr[(size_t)cnt * T + i] = j;
                    cnt++;
                }
            }
        }
        e->cnt[i] = cnt;
        e->pos_ref[i] = xi;
        const float4 k = e->pk[i];
        e->oref[i] = make_float2(k.x, k.y);
    }
    return cnt;
}

// per-system result of a list build (longest list mx); false on overflow
__device__ __forceinline__ bool e_nlist_sys(EDev *e, ESys &s, int mx) {
    atomicMax(&e->max_count, mx);
    s.rebuild = 0;
    s.rebuilds++;
    if (mx > e->p.cap) {
        atomicExch(&e->overflow, 1);
        return false;
    }
    return true;
}

__global__ void __launch_bounds__(kEB) e_nlist(EDev *e) {
    const int sid = e->blk_sys[blockIdx.x];
    ESys &s = e->sys[sid];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool on = flagged(s);
    int cnt = 0;
    if (on && i < s.off + s.n) cnt = e_nlist_one(e, s, i);
    double v[1] = {(double)cnt};
    const int ops[1] = {1};
    if (sys_reduce<1>(e, s, v, ops, &s.ticket_b)) {
        if (on) e_nlist_sys(e, s, (int)v[0]);
    }
    if (grid_last(e)) e->n_flagged = 0;
}

// ---- forces -------------------------------------------------------------------
// FP32 pair force from offsets: displacement (o_i - o_j) + dc * cs with the
// periodic wrap applied to the integer cell difference.
__device__ __forceinline__ void pair_f32(const float4 a, const float4 b, int ncd, float cs,
                                        float e_c, float n_c, float &fx, float &fy, float &en,
                                        float &w, int &contact) {
    int ca = __float_as_int(a.w), cb = __float_as_int(b.w);
    int dcx = code_x(ca) - code_x(cb), dcy = code_y(ca) - code_y(cb);
    if (dcx > ncd / 2) dcx -= ncd; else if (dcx < -(ncd / 2)) dcx += ncd;
    if (dcy > ncd / 2) dcy -= ncd; else if (dcy < -(ncd / 2)) dcy += ncd;
    float dx = (a.x - b.x) + (float)dcx * cs;
    float dy = (a.y - b.y) + (float)dcy * cs;
    float rs = a.z + b.z;
    float d2 = dx * dx + dy * dy;
    fx = 0.f; fy = 0.f; en = 0.f; w = 0.f; contact = 0;
    if (d2 >= rs * rs) return;
    float d = sqrtf(d2);
    float ov = 1.0f - d / rs;
    float ovp = n_c == 2.0f ? ov : powf(ov, n_c - 1.0f);
    float fm = e_c * ovp / (rs * d);
    fx = fm * dx;
    fy = fm * dy;
    en = e_c * ov * ovp / (2.0f * n_c);
    w = fx * dx + fy * dy;
    contact = 1;
}

// Per-system epilogue of a force pass (thread 0 of the system's last block):
// minimizeFire tests, the mixed-precision switch, the next FIRE decision and
// the jamming state machine (scripts/runArthurJamWithFire.cpp:36-106).
__device__ void e_finish(EDev *e, ESys &s, bool primary = true);

// primary: this copy of the system state performs the global side effects
// (a cluster of the resident form keeps one identical copy per block)
__device__ void e_force_epilogue(EDev *e, ESys &s, const double (&v)[5], bool setup,
                                 bool primary = true) {
    const EParams &p = e->p;
    // ---- per-system epilogue: minimizeFire tests and the next FIRE decision ----
    s.pe = v[0];
    s.power = v[1];
    s.fmax2 = v[2];
    s.virial = v[3];
    s.contacts = v[4];
    // no FP64 division or square root on this per-iteration path (both are long
    // instruction sequences on GB300's FP64 pipe): averages by 1/n, max|F|
    // tests on squares, relative energy changes by cross-multiplication
    const double avg = s.pe * s.inv_n;
    s.fire_total++;
    if (s.prec == 1) s.fp64_total++;
    else if (s.prec == 2) s.dw_total++;
    bool finished = false;
    if (setup) {
        s.last_avg_pe = avg;
        s.phase = kMinimize;
        s.iter = 0;
        s.best_f2 = s.fmax2;
        s.best_it = 0;
        e_fire_decide(p, s, s.power);
        return;
    }
    const double f2 = s.fmax2;
    const int pass_prec = s.prec;  // the arithmetic of this force pass
    // mixed systems hand over to the refinement at switch_fmax, when FIRE
    // keeps going uphill, or when max|F| stalls near the threshold: first to
    // double-word FP32 pairs, then, at the target, to FP64, which verifies the
    // residual (only an FP64 state passes the stop tests)
    if (s.prec != 1) {
        if (s.fmax2 < 0.81 * s.best_f2) {
            s.best_f2 = s.fmax2;
            s.best_it = s.iter;
        }
        const double exit_f = s.prec == 0 ? p.switch_fmax
                                          : (p.fmax_target > 0 ? p.fmax_target * (p.res ? s.dw_scale : 1.0)
                                                               : 1e-10);
        // (in the resident form a double-word system leaves only through its FP64
        // check: its noise floor, ~1e-14 of the contact force, is far below any
        // plateau of FIRE near jamming, and uphill runs there are FIRE's own)
        const bool dw_res = p.res && s.prec == 2;
        const bool stalled = !dw_res && f2 < 1e4 * exit_f * exit_f && s.iter - s.best_it > kStallIters;
        // a PE-change stop (pe_diff_target > 0) is only decided in FP64: once
        // the double-word energy has stopped changing at its own precision
        // (1e-12 relative), hand over so the FP64 test can fire
        const bool pe_flat = s.prec == 2 && p.pe_diff_target > 0 &&
                             fabs(avg - s.last_avg_pe) < 1e-12 * s.last_avg_pe;
        const bool at_exit = f2 <= exit_f * exit_f;
        if (at_exit || (s.nbad > 5 && !dw_res) || stalled || pe_flat) {
            if (s.prec == 0 && p.dw_ok) {
                s.prec = 2;
                s.best_f2 = s.fmax2;
                s.best_it = s.iter;
            } else if (p.res && s.prec == 2 && at_exit && p.fmax_target > 0 && !pe_flat) {
                s.verify = 1;  // resident form: an FP64 pass checks this state next
            } else {
                s.prec = 1;
                s.vel_f32 = 1;  // the next move takes the FP32 velocities over
            }
        }
    }
    const long long it = s.iter;
    const bool decompressing = p.jam && s.jam_stage == 0;
    const double pe_t = decompressing ? 1e-16 : p.pe_target;
    const double pe_dt = decompressing ? 0.0 : p.pe_diff_target;
    // |avg / last - 1| < pe_dt, for last >= 0
    const bool pe_still = pe_dt > 0 && fabs(avg - s.last_avg_pe) < pe_dt * s.last_avg_pe;
    s.last_avg_pe = avg;
    if (avg < pe_t || (pass_prec == 1 && pe_still)) finished = true;
    else if (p.fmax_target > 0 && f2 <= p.fmax_cert2 && pass_prec == 1) finished = true;
    else if (it + 1 >= p.max_steps) finished = true;
    else {
        s.iter = it + 1;
        e_fire_decide(p, s, s.power);
        if (s.stopped) finished = true;
    }
    if (!finished) return;
    if (p.res && pass_prec != 1) {
        // resident form: every finished minimisation ends with an FP64 pass at
        // its final positions, whose totals are the reported ones
        s.verify = 2;
        return;
    }
    e_finish(e, s, primary);
}

// A minimisation finished (the last force pass's totals are in s): the
// jamming state machine decides the next transition.
__device__ void e_finish(EDev *e, ESys &s, bool primary) {
    const EParams &p = e->p;
    s.converged = 1;
    s.minimizations++;
    if (!p.jam) {
        s.phase = kIdle;
        s.done = 1;
        if (primary) atomicSub(&e->active, 1);
        return;
    }
    // ---- jamming state machine (scripts/runArthurJamWithFire.cpp:36-106) ----
    // pressure with v = 0: sum_ij r_ij . f_ij / (4 A)
    double A = s.L * s.L;
    s.pressure = s.virial / (4.0 * A);
    double L = s.L;
    if (s.jam_stage == 0) {  // decompress until P < p_low
        if (s.pressure < p.p_low) {
            s.jam_stage = 1;
            // the compression loop starts with a minimisation of this state
            s.pending = kActCompress;
            s.scale = 1.0;
        } else {
            s.pending = kActDecompress;
            s.scale = p.decompress;
        }
        return;
    }
    double L_prior = L;
    double Lnew = L;
    if (s.pressure < p.p_low) {
        s.L_low = L;
        s.L_saved = L;  // the transition kernel saves positions
        s.L_last = L;
        if (s.L_high != -1) { Lnew = (s.L_high + s.L_low) / 2; s.L_high = -1; }
        else Lnew = L * p.compression_rate;
        s.pending = kActCompress;
    } else if (s.pressure > p.p_high) {
        s.L_high = L;
        L_prior = s.L_last;
        Lnew = (s.L_high + s.L_low) / 2;
        s.pending = kActRevertScale;
    } else if (s.contacts > 2.0 * s.n) {
        s.jam_status = 0;
    } else {
        s.pending = kActCompress;  // inside the band without enough contacts: minimise again
    }
    if (s.jam_status < 0 && s.L_low > 0 && s.L_high > 0 && fabs(s.L_low / s.L_high - 1) < p.length_tol)
        s.jam_status = 1;
    if (s.jam_status < 0 && ++s.jam_step >= p.max_compressions) s.jam_status = 2;
    if (s.jam_status >= 0) {
        s.pending = kActNone;
        s.phase = kIdle;
        s.done = 1;
        if (primary) atomicSub(&e->active, 1);
        return;
    }
    s.scale = Lnew / L_prior;
}

// Force pass of slot i (+ the kick unless setup): writes the forces and returns
// its terms: 0 PE, 1 power, 2 |F|^2, 3 virial, 4 contacts, in vf (FP32 phase)
// or v (refinement and FP64).  PH: 0 = FP32 pairs only, 1 = double-word or FP64
// pairs only (the split force kernels, each compiled without the other's
// paths), -1 = whatever the system's precision says.
template <int PH>
__device__ __forceinline__ void e_force_one_t(EDev *e, const ESys &s, int i, bool setup,
                                              double (&v)[5], float (&vf)[5]) {
    const EParams &p = e->p;
    const int prec = PH == 0 ? 0 : (PH == 1 ? (s.prec == 2 ? 2 : 1) : s.prec);
    const bool f32 = prec == 0;
    {
        const int T = p.T;
        int cnt = min(e->cnt[i], p.cap);
        double ax = 0.0, ay = 0.0, en = 0.0, wv = 0.0, nc = 0.0;
        const float4 a = e->pk[i];
        if (prec != 1) {
            int ncount = 0;
            if (prec == 0) {
                // FP32 pair terms summed in FP32 over runs of 8 neighbours, FP64 across runs;
                // the 8 indices and offsets of a run are loaded before any is used
                const float ecf = (float)p.e_c, ncf = (float)p.n_c;
                for (int k0 = 0; k0 < cnt; k0 += 8) {
                    float sx = 0.f, sy = 0.f, se = 0.f, sw = 0.f;
                    int jj[8];
                    float4 bb[8];
#pragma unroll
                    for (int u = 0; u < 8; u++) jj[u] = k0 + u < cnt ? __ldg(&e->nbr[(size_t)(k0 + u) * T + i]) : i;
#pragma unroll
                    for (int u = 0; u < 8; u++) bb[u] = e->pk[jj[u]];
#pragma unroll
                    for (int u = 0; u < 8; u++) {
                        if (k0 + u >= cnt) break;
                        float fx, fy, ef, wf;
                        int ct;
                        pair_f32(a, bb[u], s.ncd, s.cs_f, ecf, ncf, fx, fy, ef, wf, ct);
                        sx += fx;
                        sy += fy;
                        se += ef;
                        sw += wf;
                        ncount += ct;
                    }
                    ax += (double)sx;
                    ay += (double)sy;
                    en += (double)se;
                    wv += (double)sw;
                }
            } else {
                // double-word FP32 pairs for the contacts the FP32 offsets cannot rule out
                const float4 al = e->pkl[i];
                const dw xi = {a.x, al.x}, yi = {a.y, al.y}, ri = {a.z, al.z};
                const dw csd = {s.cs_f, s.cs_lo}, ec = {p.ec_hi, p.ec_lo};
                dw sx = {0.f, 0.f}, sy = {0.f, 0.f}, se = {0.f, 0.f};
                float sw = 0.f;
                const int ca = __float_as_int(a.w);
                // runs of 4 neighbours: indices, then packed offsets, then the
                // low words of the candidates, each batch of loads issued together
                for (int k0 = 0; k0 < cnt; k0 += 4) {
                    int jj[4];
                    float4 bb[4], bl[4];
                    int dcx[4], dcy[4];
                    unsigned cand = 0u;
#pragma unroll
                    for (int u = 0; u < 4; u++) jj[u] = k0 + u < cnt ? __ldg(&e->nbr[(size_t)(k0 + u) * T + i]) : i;
#pragma unroll
                    for (int u = 0; u < 4; u++) bb[u] = e->pk[jj[u]];
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        const int cb = __float_as_int(bb[u].w);
                        int cx = code_x(ca) - code_x(cb), cy = code_y(ca) - code_y(cb);
                        if (cx > s.ncd / 2) cx -= s.ncd; else if (cx < -(s.ncd / 2)) cx += s.ncd;
                        if (cy > s.ncd / 2) cy -= s.ncd; else if (cy < -(s.ncd / 2)) cy += s.ncd;
                        dcx[u] = cx;
                        dcy[u] = cy;
                        const float dxf = (a.x - bb[u].x) + (float)cx * s.cs_f;
                        const float dyf = (a.y - bb[u].y) + (float)cy * s.cs_f;
                        const float rsf = a.z + bb[u].z;
                        if (k0 + u < cnt && dxf * dxf + dyf * dyf < rsf * rsf * 1.0001f) cand |= 1u << u;
                    }
#pragma unroll
                    for (int u = 0; u < 4; u++)
                        if (cand & (1u << u)) bl[u] = e->pkl[jj[u]];
#pragma unroll
                    for (int u = 0; u < 4; u++) {
                        if (!(cand & (1u << u))) continue;
                        const float4 b = bb[u];
                        dw dx = dw_add(dw_add(xi, dw_neg(dw{b.x, bl[u].x})), dw_mul_f(csd, (float)dcx[u]));
                        dw dy = dw_add(dw_add(yi, dw_neg(dw{b.y, bl[u].y})), dw_mul_f(csd, (float)dcy[u]));
                        dw rs = dw_add(ri, dw{b.z, bl[u].z});
                        dw d2 = dw_add(dw_mul(dx, dx), dw_mul(dy, dy));
                        if (dw_ge(d2, dw_mul(rs, rs))) continue;
                        dw d = dw_sqrt(d2);
                        dw ov = dw_add(dw{1.f, 0.f}, dw_neg(dw_div(d, rs)));
                        dw fm = dw_div(dw_mul(ec, ov), dw_mul(rs, d));
                        sx = dw_add(sx, dw_mul(fm, dx));
                        sy = dw_add(sy, dw_mul(fm, dy));
                        se = dw_add(se, dw_mul_f(dw_mul(ec, dw_mul(ov, ov)), 0.25f));
                        sw += fm.hi * (dx.hi * dx.hi + dy.hi * dy.hi);
                        ncount++;
                    }
                }
                ax = dw_to_double(sx);
                ay = dw_to_double(sy);
                en = dw_to_double(se);
                wv = (double)sw;
            }
            const float2 fv = make_float2((float)ax, (float)ay);
            e->frc[i] = make_double2(ax, ay);
            e->frc32[i] = fv;
            float2 u = e->vel32[i];
            if (!setup) {
                const float h = 0.5f * (float)s.dt * e->invm[i];
                u.x += fv.x * h;
                u.y += fv.y * h;
                e->vel32[i] = u;
            }
            if (f32) {
                vf[0] = (float)en;
                vf[1] = fv.x * u.x + fv.y * u.y;
                vf[2] = fv.x * fv.x + fv.y * fv.y;
                vf[3] = (float)wv;
                vf[4] = (float)ncount;
            } else {
                v[0] = en;
                v[1] = ax * (double)u.x + ay * (double)u.y;
                v[2] = ax * ax + ay * ay;
                v[3] = wv;
                v[4] = (double)ncount;
            }
        } else {
            // FP64 pair arithmetic for pairs that the FP32 offsets cannot rule
            // out (a 1e-4 relative margin on the contact distance)
            const double2 xi = e->pos[i];
            const double ri = e->rad[i];
            for (int k = 0; k < cnt; k++) {
                int j = __ldg(&e->nbr[(size_t)k * T + i]);
                if (s.ncd >= 3) {
                    const float4 b = e->pk[j];
                    int ca = __float_as_int(a.w), cb = __float_as_int(b.w);
                    int dcx = code_x(ca) - code_x(cb), dcy = code_y(ca) - code_y(cb);
                    if (dcx > s.ncd / 2) dcx -= s.ncd; else if (dcx < -(s.ncd / 2)) dcx += s.ncd;
                    if (dcy > s.ncd / 2) dcy -= s.ncd; else if (dcy < -(s.ncd / 2)) dcy += s.ncd;
                    const float dxf = (a.x - b.x) + (float)dcx * s.cs_f;
                    const float dyf = (a.y - b.y) + (float)dcy * s.cs_f;
                    const float rsf = a.z + b.z;
                    if (dxf * dxf + dyf * dyf >= rsf * rsf * 1.0001f) continue;
                }
                double2 xj = e->pos[j];
                double dx = pbc_dist(xi.x, xj.x, s.L), dy = pbc_dist(xi.y, xj.y, s.L);
                double rs = ri + e->rad[j];
                double d2 = dx * dx + dy * dy;
                if (d2 >= rs * rs) continue;
                // 1/d and 1/rs by Newton-Raphson from FP32 estimates: two steps
                // take the 2^-23 seed to FP64 precision (quadratic convergence)
                const double id = rsqrt_newton(d2), irs = rcp_newton(rs);
                double d = d2 * id;
                double ov = 1.0 - d * irs;
                double ovp = p.n_c == 2.0 ? ov : pow(ov, p.n_c - 1);
                double fm = p.e_c * ovp * irs * id;
                double fx = fm * dx, fy = fm * dy;
                ax += fx;
                ay += fy;
                en += p.e_c * ov * ovp / (2.0 * p.n_c);
                wv += fx * dx + fy * dy;
                nc += 1.0;
            }
            double2 f = make_double2(ax, ay);
            e->frc[i] = f;
            double2 u = e->vel[i];
            if (!setup) {
                double dtm = (0.5 * s.dt) * rcp_newton(e->mass[i]);
                u.x = u.x + f.x * dtm;
                u.y = u.y + f.y * dtm;
                e->vel[i] = u;
            }
            v[0] = en;
            v[1] = f.x * u.x + f.y * u.y;
            v[2] = f.x * f.x + f.y * f.y;
            v[3] = wv;
            v[4] = nc;
        }
    }
}

__device__ __forceinline__ void e_force_one(EDev *e, const ESys &s, int i, bool setup,
                                            double (&v)[5], float (&vf)[5]) {
    e_force_one_t<-1>(e, s, i, setup, v, vf);
}

// The force pass of the grid form, split by arithmetic: e_force_k<0> takes the
// systems whose pass is FP32 (fprec 0), e_force_k<1> those in the double-word
// refinement or FP64 (every block of the other systems leaves at once), so the
// FP32 kernel carries only the FP32 path's registers (the combined kernel held
// 102-108 registers a thread in every phase).  The second kernel sets the
// transition node's condition.
// PH = -1: one kernel for every arithmetic (the systems' own precision).
template <int PH>
__global__ void __launch_bounds__(kEB, PH == 0 ? 6 : 5) e_force_k(EDev *e) {
    if (e->overflow) return;  // lists truncated: the host grows them and reruns this pass
    const int sid = e->blk_sys[blockIdx.x];
    ESys &s = e->sys[sid];
    const bool mine = PH < 0 || ((PH == 0) == (s.fprec == 0));
    if (mine) {
        const int i = blockIdx.x * blockDim.x + threadIdx.x;
        const bool live = s.phase != kIdle;
        const bool setup = s.phase == kSetup;
        // partials: 0 PE, 1 power, 2 max|F|^2, 3 virial, 4 contacts (FP32 block
        // sums in the FP32 phase; FP64 in the refinement, whose energies are exact
        // to ~1e-14 and are the ones reported)
        double v[5] = {0, 0, 0, 0, 0};
        float vf[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
        if (live && i < s.off + s.n) e_force_one_t<PH>(e, s, i, setup, v, vf);
        const int ops[5] = {0, 0, 1, 0, 0};
        double tot[5];
        const bool f32 = PH == 0 || (PH < 0 && s.fprec == 0);
        const bool last = f32 ? sys_reduce_t<5, float>(e, s, vf, ops, &s.ticket_a, tot)
                              : sys_reduce_t<5, double>(e, s, v, ops, &s.ticket_a, tot);
        if (last && live) {
            e_force_epilogue(e, s, tot, setup);
            if (s.pending != kActNone) atomicAdd(&e->n_pending, 1);
        }
    }
}

// sets the transition node's condition after the force kernels (one thread)
__global__ void e_after_force(EDev *e) {
    if (e->h_tr) cudaGraphSetConditional(e->h_tr, e->n_pending > 0 ? 1u : 0u);
}

// ---- transitions between minimisations (save / restore / scale, FIRE reset) ----
__device__ __forceinline__ void e_transition_one(EDev *e, const ESys &s, int act, int i) {
    double2 x = e->pos[i];
    if (act == kActCompress && s.pressure < e->p.p_low && s.jam_stage == 1 && s.L_saved == s.L)
        e->pos_save[i] = x;  // write_restart_file("last_state")
    if (act == kActRevertScale) x = e->pos_save[i];  // load("last_state")
    x.x *= s.scale;
    x.y *= s.scale;
    e->pos[i] = x;
    e->vel[i] = make_double2(0.0, 0.0);
    e->vel32[i] = make_float2(0.f, 0.f);
}

// per-system part of a transition: new box and cell size, FIRE reset, setup pass next
__device__ __forceinline__ void e_transition_sys(const EParams &p, ESys &s, int act) {
    double L0 = act == kActRevertScale ? s.L_last : s.L;
    s.L = L0 * s.scale;
    s.cs = s.L / s.ncd;
    s.inv_cs = s.ncd / s.L;
    s.cs_f = (float)s.cs;
    s.cs_lo = (float)(s.cs - (double)s.cs_f);
    s.pending = kActNone;
    s.phase = kSetup;
    s.rebuild = 1;
    s.dt = p.dt0;
    s.alpha = p.alpha0;
    s.ngood = 0;
    s.nbad = 0;
    s.stopped = 0;
    s.uphill = 0;
    s.converged = 0;
    s.iter = 0;
    s.prec = (p.switch_fmax > 0 && s.ncd >= 3) ? 0 : 1;
    s.vel_f32 = 0;
    s.verify = 0;
    s.dw_scale = 0.9;
}

__global__ void __launch_bounds__(kEB) e_transition(EDev *e) {
    if (e->overflow) return;
    const int sid = e->blk_sys[blockIdx.x];
    ESys &s = e->sys[sid];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int act = s.pending;
    if (act != kActNone && i < s.off + s.n) e_transition_one(e, s, act, i);
    double v[1] = {0.0};
    const int ops[1] = {0};
    if (sys_reduce<1>(e, s, v, ops, &s.ticket_b) && act != kActNone) e_transition_sys(e->p, s, act);
    if (grid_last(e)) e->n_pending = 0;
}

// ---- the persistent form: one block per system --------------------------------
// Every iteration of a system (move, list rebuild, force pass with its FIRE /
// jamming epilogue, transition) runs inside one block with __syncthreads()
// between the stages and the system's state in shared memory, so a whole
// minimisation or jamming run costs no kernel launches and no grid-wide
// synchronisation.  Small systems (the jamming ensemble's 64-4096 disks) are
// latency-bound in the grid form, where each stage is a launch over all
// systems and every iteration waits for the slowest; here each system runs at
// its own pace.  The launch ends when every system is done, after iter_budget
// iterations, or when a neighbour list overflows (the host grows the lists and
// relaunches; the overflowing system resumes at its list build).  Per-slot
// arithmetic is the grid form's; reductions run over the block (each thread's
// slots in order, then the block tree), so totals round differently from the
// grid form's block partials.  Blocks never wait on one another.
template <int NT>
__global__ void __launch_bounds__(NT) e_persist(EDev *e, long long iter_budget) {
    __shared__ ESys s;
    __shared__ float smf[32 * 5];
    __shared__ double smd[32 * 5];
    __shared__ int smi[32];
    __shared__ int stop;
    const int sid = blockIdx.x;
    if (threadIdx.x == 0) s = e->sys[sid];
    __syncthreads();
    const EParams &p = e->p;
    const int i0 = s.off + threadIdx.x, i1 = s.off + s.n;
    long long it = 0;
    while (s.phase != kIdle && it < iter_budget) {
        // another system's list overflowed: stop at this iteration boundary
        // (read once by thread 0, so every thread takes the same branch)
        if (threadIdx.x == 0) stop = *(volatile int *)&e->overflow;
        __syncthreads();
        if (stop) break;
        // ---- move (FIRE step of src/integrator/fire.cu:29-40)
        if (!s.resume && s.phase == kMinimize) {
            const int ops[1] = {1};
            if (s.prec != 1) {
                float m[1] = {0.f};
                for (int i = i0; i < i1; i += NT) {
                    double dv = 0.0;
                    float df = 0.f;
                    e_move_one(e, s, i, dv, df);
                    m[0] = fmaxf(m[0], df);
                }
                block_reduce<1, float>(m, ops, smf);
                if (threadIdx.x == 0) e_move_sys(p, s, (double)m[0]);
            } else {
                double m[1] = {0.0};
                for (int i = i0; i < i1; i += NT) {
                    double dv = 0.0;
                    float df = 0.f;
                    e_move_one(e, s, i, dv, df);
                    m[0] = fmax(m[0], dv);
                }
                block_reduce<1, double>(m, ops, smd);
                if (threadIdx.x == 0) e_move_sys(p, s, m[0]);
            }
            __syncthreads();
        }
        // ---- cell list and neighbour list of this system
        if (s.rebuild) {
            for (int i = i0; i < i1; i += NT) e_cell_count_one(e, s, i);
            __syncthreads();
            e_cell_scan_block(e, s);
            __syncthreads();
            for (int i = i0; i < i1; i += NT) e_cell_fill_one(e, s, i);
            __syncthreads();
            const int nc = s.ncd * s.ncd;
            for (int c = threadIdx.x; c < nc; c += NT) e_cell_sort_one(e, s.cell_off + c);
            __syncthreads();
            int m[1] = {0};
            const int ops[1] = {1};
            for (int i = i0; i < i1; i += NT) m[0] = max(m[0], e_nlist_one(e, s, i));
            block_reduce<1, int>(m, ops, smi);
            if (threadIdx.x == 0) s.resume = e_nlist_sys(e, s, m[0]) ? 0 : 1;
            __syncthreads();
            if (s.resume) break;
        }
        // ---- force pass (+ kick) and the per-system epilogue
        {
            const bool setup = s.phase == kSetup;
            const int ops[5] = {0, 0, 1, 0, 0};
            double tot[5] = {0, 0, 0, 0, 0};
            if (s.prec == 0) {
                float a[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
                for (int i = i0; i < i1; i += NT) {
                    double v[5] = {0, 0, 0, 0, 0};
                    float vf[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
                    e_force_one(e, s, i, setup, v, vf);
                    a[0] += vf[0];
                    a[1] += vf[1];
                    a[2] = fmaxf(a[2], vf[2]);
                    a[3] += vf[3];
                    a[4] += vf[4];
                }
                block_reduce<5, float>(a, ops, smf);
#pragma unroll
                for (int k = 0; k < 5; k++) tot[k] = (double)a[k];
            } else {
                double a[5] = {0, 0, 0, 0, 0};
                for (int i = i0; i < i1; i += NT) {
                    double v[5] = {0, 0, 0, 0, 0};
                    float vf[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
                    e_force_one(e, s, i, setup, v, vf);
                    a[0] += v[0];
                    a[1] += v[1];
                    a[2] = fmax(a[2], v[2]);
                    a[3] += v[3];
                    a[4] += v[4];
                }
                block_reduce<5, double>(a, ops, smd);
#pragma unroll
                for (int k = 0; k < 5; k++) tot[k] = a[k];
            }
            if (threadIdx.x == 0) e_force_epilogue(e, s, tot, setup);
            __syncthreads();
        }
        // ---- transition between minimisations (jamming protocol)
        if (s.pending != kActNone) {
            const int act = s.pending;
            for (int i = i0; i < i1; i += NT) e_transition_one(e, s, act, i);
            __syncthreads();
            if (threadIdx.x == 0) e_transition_sys(p, s, act);
            __syncthreads();
        }
        it++;
    }
    __syncthreads();
    if (threadIdx.x == 0) e->sys[sid] = s;
}

// WHILE-body guard: continue while any system is active and the budget lasts
__global__ void e_guard(EDev *e) {
    long long g = ++e->guard;
    int go = (e->active > 0) && (g < e->guard_limit) && !e->overflow;
    if (e->h_loop) cudaGraphSetConditional(e->h_loop, go ? 1u : 0u);
}

// ---- transfers ------------------------------------------------------------------
__global__ void e_put(EDev *e, const double *x, const double *y, const double *r, const double *m,
                      const int *src_index) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= e->p.T) return;
    int k = src_index[i];
    if (k < 0) {
        e->pos[i] = make_double2(0.0, 0.0);
        e->rad[i] = 0.0;
        e->mass[i] = 1.0;
        return;
    }
    e->pos[i] = make_double2(x[k], y[k]);
    e->rad[i] = r[k];
    e->mass[i] = m[k];
    e->invm[i] = (float)(1.0 / m[k]);
    e->vel[i] = make_double2(0.0, 0.0);
    e->frc[i] = make_double2(0.0, 0.0);
    e->vel32[i] = make_float2(0.f, 0.f);
    e->frc32[i] = make_float2(0.f, 0.f);
}

__global__ void e_get(EDev *e, double *x, double *y, double *fx, double *fy, const int *src_index) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= e->p.T) return;
    int k = src_index[i];
    if (k < 0) return;
    double2 p = e->pos[i], f = e->frc[i];
    if (x) x[k] = p.x;
    if (y) y[k] = p.y;
    if (fx) fx[k] = f.x;
    if (fy) fy[k] = f.y;
}

}  // namespace
}  // namespace dpg
