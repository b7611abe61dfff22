// disk_kernels.cuh -- plain FP64 kernels for soft disks (the drop-in form).
//
// Compiled with --fmad=false: every multiply and add is rounded separately, in
// the reference's operation order, so per-particle results are bit-identical
// to the reference kernels (src/particles/base/kernels.cu,
// src/particles/disk/kernels.cu).  Explicit fma() calls appear only where the
// reference itself calls fma (Adam).
//
// Every kernel takes the device-resident DevSys and reads the current buffer
// pointers from it, so launch arguments never go stale inside a CUDA graph.
#pragma once
#include "dpg_device.cuh"

namespace dpg {
namespace {  // kernels have internal linkage: each translation unit owns its copy

constexpr int kMixed = 1;  // DevParams.precision of the mixed form (DPG_MIXED)

__device__ __forceinline__ bool halted(const DevSys *ds) { return ds->s.flags != 0; }

// harmonic (power-law) contact of particle i with j, force on i:
// include/particles/base/kernels.cuh:154-183
__device__ __forceinline__ double disk_pair(double xi, double yi, double ri, double xj, double yj,
                                            double rj, double bx, double by, double e_c,
                                            double n_c, double &fx, double &fy) {
    double dx = pbc_dist(xi, xj, bx);
    double dy = pbc_dist(yi, yj, by);
    double rs = ri + rj;
    double d2 = dx * dx + dy * dy;
    if (d2 >= rs * rs) { fx = 0.0; fy = 0.0; return 0.0; }
    double d = sqrt(d2);
    double ov = 1.0 - (d / rs);
    double ovp, energy;
    if (n_c == 2.0) {  // pow(ov, 1) == ov, and x / 4 == x * 0.25 exactly
        ovp = ov;
        energy = e_c * ov * ovp * 0.25;
    } else {
        ovp = pow(ov, n_c - 1);
        energy = e_c * ov * ovp / (2.0 * n_c);
    }
    double fm = e_c * ovp / (rs * d);
    fx = fm * dx;
    fy = fm * dy;
    return energy;
}

// sum of pair forces / energies over particle i's neighbour row
// (kernelCalcDiskForces, src/particles/disk/kernels.cu:11-57)
__device__ __forceinline__ void disk_force_sum(const DevSys *__restrict__ ds, int i, double2 pi,
                                               double ri, const double2 *__restrict__ pos,
                                               const double *__restrict__ rad,
                                               const int *__restrict__ nbr, double &ax, double &ay,
                                               double &en) {
    const int n = ds->p.n;
    const double bx = ds->p.box[0], by = ds->p.box[1], e_c = ds->p.e_c, n_c = ds->p.n_c;
    int cnt = ds->w.count[i];
    if (cnt > ds->p.cap) cnt = ds->p.cap;
    ax = 0.0; ay = 0.0; en = 0.0;
    for (int k = 0; k < cnt; k++) {
        int j = __ldg(&nbr[(size_t)k * n + i]);
        double2 pj = pos[j];
        double fx, fy;
        double e = disk_pair(pi.x, pi.y, ri, pj.x, pj.y, __ldg(&rad[j]), bx, by, e_c, n_c, fx, fy);
        ax += fx;
        ay += fy;
        en += e;
    }
}

// The same sum with G threads per particle (G a power of two <= 32, groups
// aligned inside a warp): lane `sub` of the group evaluates neighbour slots
// sub, sub + G, ...; the pair terms are then shuffled so that every lane of
// the group adds them in slot order 0, 1, 2, ..., the order of the sequential
// loop above, so the result is bit-identical to disk_force_sum.  Small systems
// get G times more warps in flight to hide the FP64 divide / sqrt latency.
// Every lane of the warp must call this (shuffles); `valid` is false for lanes
// past the last particle.
template <int G>
__device__ __forceinline__ void disk_force_sum_g(const DevSys *__restrict__ ds, int i, bool valid,
                                                 double &ax, double &ay, double &en) {
    const int n = ds->p.n;
    const double bx = ds->p.box[0], by = ds->p.box[1], e_c = ds->p.e_c, n_c = ds->p.n_c;
    const double2 *__restrict__ pos = ds->v.pos;
    const double *__restrict__ rad = ds->v.rad;
    const int *__restrict__ nbr = ds->v.nbr;
    int cnt = 0;
    double2 pi = make_double2(0.0, 0.0);
    double ri = 0.0;
    if (valid) {
        cnt = ds->w.count[i];
        if (cnt > ds->p.cap) cnt = ds->p.cap;
        pi = pos[i];
        ri = rad[i];
    }
    const int lane = threadIdx.x & 31, sub = lane & (G - 1), lead = lane - sub;
    const int rounds = __reduce_max_sync(0xffffffffu, (unsigned)((cnt + G - 1) / G));
    ax = 0.0; ay = 0.0; en = 0.0;
    for (int r = 0; r < rounds; r++) {
        const int k = r * G + sub;
        double fx = 0.0, fy = 0.0, e = 0.0;
        if (k < cnt) {
            int j = __ldg(&nbr[(size_t)k * n + i]);
            double2 pj = pos[j];
            e = disk_pair(pi.x, pi.y, ri, pj.x, pj.y, __ldg(&rad[j]), bx, by, e_c, n_c, fx, fy);
        }
#pragma unroll
        for (int t = 0; t < G; t++) {
            double gx = __shfl_sync(0xffffffffu, fx, lead + t);
            double gy = __shfl_sync(0xffffffffu, fy, lead + t);
            double ge = __shfl_sync(0xffffffffu, e, lead + t);
            if (r * G + t < cnt) {
                ax += gx;
                ay += gy;
                en += ge;
            }
        }
    }
}

// Mixed form: FP32 pair forces from the packed offsets, summed in FP32 over
// runs of 8 neighbours and in FP64 across runs and for the particle total.
__device__ __forceinline__ void disk_force_sum_mixed(const DevSys *__restrict__ ds, int i,
                                                     double &ax, double &ay, double &en) {
    const int n = ds->p.n;
    const float4 *__restrict__ pk = ds->v.pk;
    const int *__restrict__ nbr = ds->v.nbr;
    const float e_c = (float)ds->p.e_c, n_c = (float)ds->p.n_c;
    int cnt = ds->w.count[i];
    if (cnt > ds->p.cap) cnt = ds->p.cap;
    const float4 a = pk[i];
    ax = 0.0; ay = 0.0; en = 0.0;
    for (int k0 = 0; k0 < cnt; k0 += 8) {
        float sx = 0.f, sy = 0.f, se = 0.f;
        const int k1 = min(cnt, k0 + 8);
        for (int k = k0; k < k1; k++) {
            int j = __ldg(&nbr[(size_t)k * n + i]);
            float fx, fy;
            se += mixed_pair(ds->p, a, pk[j], e_c, n_c, fx, fy);
            sx += fx;
            sy += fy;
        }
        ax += (double)sx;
        ay += (double)sy;
        en += (double)se;
    }
}

// Pair sum of particle i for a force kernel with G threads per particle; the
// mixed instantiation (M) uses FP32 pairs until the FIRE refinement switches
// the system to FP64 (DevState.fp64_now).  All lanes of the warp call it.
template <int G, bool M>
__device__ __forceinline__ void force_sum(const DevSys *__restrict__ ds, int i, bool valid,
                                          double &ax, double &ay, double &en) {
    ax = 0.0; ay = 0.0; en = 0.0;
    if (M && !ds->s.fp64_now) {
        if (valid) disk_force_sum_mixed(ds, i, ax, ay, en);
        return;
    }
    if (G == 1) {
        if (valid) {
            const double2 *__restrict__ pos = ds->v.pos;
            disk_force_sum(ds, i, pos[i], ds->v.rad[i], pos, ds->v.rad, ds->v.nbr, ax, ay, en);
        }
    } else {
        disk_force_sum_g<G>(ds, i, valid, ax, ay, en);
    }
}

// mixed disk systems only (rigid-body systems keep their vertex offsets in
// BumpyExt and leave the body DevParams at FP64)
__device__ __forceinline__ void mixed_update(DevSys *ds, int i, double2 p) {
    if (ds->p.precision == kMixed && ds->v.pk) ds->v.pk[i] = mixed_pack(ds->p, p, ds->v.rad[i]);
}

// mixed form: offsets of every particle from the current positions
__global__ void k_mixed_refresh(DevSys *ds) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ds->p.n) return;
    ds->v.pk[i] = mixed_pack(ds->p, ds->v.pos[i], ds->v.rad[i]);
}

// device-side neighbour rebuild decision: checkForCellListUpdate /
// checkForVerletListUpdate (src/particles/base/particle.cu:1141-1161), tolerance 3
__device__ __forceinline__ int rebuild_decision(const DevSys *ds, double max_nd2, double max_cd2) {
    const double tol = 3.0;
    if (ds->p.method == 2) return 0;
    if (ds->p.method == 1) return (tol * max_nd2 > ds->p.nthr2) ? 1 : 0;
    if (tol * max_cd2 > ds->p.cthr2) return 2;
    if (tol * max_nd2 > ds->p.nthr2) return 1;
    return 0;
}

// ============================================================================
//  Single operations (drop-in path)
// ============================================================================

// kernelUpdateVelocities: src/particles/base/kernels.cu:117-139
__global__ void k_kick(DevSys *ds, double dt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ds->p.n) return;
    double2 *vel = ds->v.vel;
    double2 v = vel[i], f = ds->v.frc[i];
    double dtm = dt / ds->v.mass[i];
    v.x = v.x + f.x * dtm;
    v.y = v.y + f.y * dtm;
    vel[i] = v;
}

// kernelUpdatePositions: src/particles/base/kernels.cu:48-81.  The reference's
// per-particle displacement arrays are only ever max-reduced, so the maxima
// are kept instead (grid reduction into DevState).
__global__ void k_drift(DevSys *ds, double dt) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[2] = {0.0, 0.0};
    if (i < ds->p.n) {
        double2 *pos = ds->v.pos;
        double2 p = pos[i], u = ds->v.vel[i];
        p.x = p.x + u.x * dt;
        p.y = p.y + u.y * dt;
        pos[i] = p;
        double2 a = ds->w.pos_n[i], c = ds->w.pos_c[i];
        double dxn = p.x - a.x, dyn = p.y - a.y, dxc = p.x - c.x, dyc = p.y - c.y;
        v[0] = dxn * dxn + dyn * dyn;
        v[1] = dxc * dxc + dyc * dyc;
    }
    const int ops[2] = {1, 1};
    if (grid_reduce<2>(v, ops, ds)) { ds->s.max_nd2 = v[0]; ds->s.max_cd2 = v[1]; }
}

// kernelMixVelocitiesAndForces (per-particle FIRE mix): src/particles/base/kernels.cu:91-112
__device__ __forceinline__ double2 fire_mix(double2 v, double2 f, double alpha) {
    double fn = sqrt(f.x * f.x + f.y * f.y);
    double vn = sqrt(v.x * v.x + v.y * v.y);
    double mix = 0.0;
    if (fn > 1e-16) {
        mix = vn / fn * alpha;
    } else {
        v.x = 0.0; v.y = 0.0; mix = 0.0;
    }
    double2 o;
    o.x = v.x * (1 - alpha) + f.x * mix;
    o.y = v.y * (1 - alpha) + f.y * mix;
    return o;
}

__global__ void k_mix(DevSys *ds, double alpha) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ds->p.n) return;
    ds->v.vel[i] = fire_mix(ds->v.vel[i], ds->v.frc[i], alpha);
}

__global__ void k_zero_vel(DevSys *ds) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ds->p.n) return;
    ds->v.vel[i] = make_double2(0.0, 0.0);
}

// kernelZeroForceAndPotentialEnergy: src/particles/base/kernels.cu:150-161
__global__ void k_zero_force(DevSys *ds) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ds->p.n) return;
    ds->v.frc[i] = make_double2(0.0, 0.0);
    ds->w.pe[i] = 0.0;
}

// kernelCalcDiskForces (+= semantics): src/particles/disk/kernels.cu:11-57
template <int G, bool M>
__global__ void k_force_acc(DevSys *ds) {
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = gid / G;
    double ax, ay, en;
    if (G == 1) {
        if (i >= ds->p.n) return;
        if (ds->w.count[i] == 0) return;
        force_sum<1, M>(ds, i, true, ax, ay, en);
    } else {
        force_sum<G, M>(ds, i, i < ds->p.n, ax, ay, en);
        if (i >= ds->p.n || (gid & (G - 1)) != 0) return;
        if (ds->w.count[i] == 0) return;
    }
    double2 *frc = ds->v.frc;
    double2 f = frc[i];
    f.x += ax;
    f.y += ay;
    frc[i] = f;
    ds->w.pe[i] += en;
}

// ---- pair and Hessian dump -----------------------------------------------------
struct PairOut {
    double *d[16];  // see dpg_pair_dump in include/dpg.h for the order
    long long *this_id, *other_id;
};

// the fills of Disk::calculateForceDistancePairs (src/particles/disk/disk.cu:229-247)
__global__ void k_pair_fill(PairOut o, long long m) {
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m) return;
    const double fill[16] = {-1, 0, 0, -1, -1, -1, -1, -1, 0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
    for (int k = 0; k < 16; k++)
        if (o.d[k]) o.d[k][q] = fill[k];
    o.this_id[q] = -1;
    o.other_id[q] = -1;
}

// kernelCalcDiskForceDistancePairs (src/particles/disk/kernels.cu:73-175):
// entry [slot * cap + k] for the k-th neighbour of the particle in slot i
__global__ void k_pair_dump(DevSys *ds, PairOut o) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = ds->p.n, cap = ds->p.cap;
    if (i >= n) return;
    int cnt = ds->w.count[i];
    if (cnt == 0) return;
    if (cnt > cap) cnt = cap;
    const double2 *pos = ds->v.pos;
    const double *rad = ds->v.rad;
    const double2 pi = pos[i];
    const double ri = rad[i];
    const double bx = ds->p.box[0], by = ds->p.box[1], e_c = ds->p.e_c, n_c = ds->p.n_c;
    for (int k = 0; k < cnt; k++) {
        const int j = ds->v.nbr[(size_t)k * n + i];
        const double2 pj = pos[j];
        const double rj = rad[j];
        double fx, fy;
        const double e = disk_pair(pi.x, pi.y, ri, pj.x, pj.y, rj, bx, by, e_c, n_c, fx, fy);
        const long long q = (long long)i * cap + k;
        const double dx = pbc_dist(pi.x, pj.x, bx), dy = pbc_dist(pi.y, pj.y, by);
        if (o.d[0]) o.d[0][q] = e;
        if (o.d[1]) o.d[1][q] = fx;
        if (o.d[2]) o.d[2][q] = fy;
        if (o.d[3]) o.d[3][q] = dx;
        if (o.d[4]) o.d[4][q] = dy;
        o.this_id[q] = ds->v.sidx[i];
        o.other_id[q] = ds->v.sidx[j];
        const double dist = sqrt(dx * dx + dy * dy);
        if (o.d[5]) o.d[5][q] = dist - (ri + rj);
        if (o.d[6]) o.d[6][q] = ri + rj;
        if (o.d[7]) o.d[7][q] = atan2(dy, dx);
        if (dist < ri + rj) {
            const double radsum = ri + rj;
            const double t_ij = -e_c / radsum * (1 - dist / radsum);
            const double c_ij = e_c / (radsum * radsum);
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
#pragma unroll
            for (int c = 0; c < 4; c++) {
                if (o.d[8 + c]) o.d[8 + c][q] += hij[c];
                if (o.d[12 + c]) o.d[12 + c][q] += hii[c];
            }
        }
    }
}

// calcWallInteraction (include/particles/base/kernels.cuh:185-235): hard walls
// at 0 and L on both axes, terms in the reference's order (left, right,
// bottom, top); returns the energy, force in (fx, fy) summed from 0
__device__ __forceinline__ double wall_force(const DevParams &p, double2 x, double rad,
                                             double &fx, double &fy) {
    const double dist[4] = {x.x, p.box[0] - x.x, x.y, p.box[1] - x.y};
    const bool near[4] = {x.x < rad, x.x > p.box[0] - rad, x.y < rad, x.y > p.box[1] - rad};
    double en = 0.0;
    fx = 0.0;
    fy = 0.0;
#pragma unroll
    for (int w = 0; w < 4; w++) {
        if (!near[w]) continue;
        const double ov = rad - dist[w];
        if (!(ov > 0)) continue;
        const double q = ov / rad;
        const double ovp = p.n_c - 1 == 1.0 ? q : pow(q, p.n_c - 1);
        const double f = p.e_c * ovp / rad;
        if (w == 0) fx += f;
        else if (w == 1) fx -= f;
        else if (w == 2) fy += f;
        else fy -= f;
        en += p.e_c * ov * ovp / (p.n_c * rad);
    }
    return en;
}

// kernelCalcDiskWallForces (+= semantics): src/particles/disk/kernels.cu:59-71
__global__ void k_wall_force(DevSys *ds) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ds->p.n) return;
    double fx, fy;
    double en = wall_force(ds->p, ds->v.pos[i], ds->v.rad[i], fx, fy);
    double2 f = ds->v.frc[i];
    f.x += fx;
    f.y += fy;
    ds->v.frc[i] = f;
    ds->w.pe[i] += en;
}

// kernelCalculateDampedForces: src/particles/base/kernels.cu:83-89
__global__ void k_damp(DevSys *ds, double gamma) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ds->p.n) return;
    double2 f = ds->v.frc[i], u = ds->v.vel[i];
    f.x -= gamma * u.x;
    f.y -= gamma * u.y;
    ds->v.frc[i] = f;
}

// kernelGradDescStep: src/particles/base/kernels.cu:613-637, with the
// displacement maxima kept as in k_drift
__global__ void k_grad_desc(DevSys *ds, double alpha) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[2] = {0.0, 0.0};
    if (i < ds->p.n) {
        double2 *pos = ds->v.pos;
        double2 p = pos[i], f = ds->v.frc[i];
        p.x = p.x + alpha * f.x;
        p.y = p.y + alpha * f.y;
        pos[i] = p;
        double2 a = ds->w.pos_n[i], c = ds->w.pos_c[i];
        double dxn = p.x - a.x, dyn = p.y - a.y, dxc = p.x - c.x, dyc = p.y - c.y;
        v[0] = dxn * dxn + dyn * dyn;
        v[1] = dxc * dxc + dyc * dyc;
    }
    const int ops[2] = {1, 1};
    if (grid_reduce<2>(v, ops, ds)) { ds->s.max_nd2 = v[0]; ds->s.max_cd2 = v[1]; }
}

// PE and KE totals (kernelCalculateTranslationalKineticEnergy + reductions,
// src/particles/base/kernels.cu:163-180, src/particles/base/particle.cu:1074-1080),
// FIRE power P = F.v (src/particles/base/particle.cu:993-1009), max|F|^2 and sum F.
__global__ void k_observables(DevSys *ds) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[6] = {0, 0, 0, 0, 0, 0};
    if (i < ds->p.n) {
        double2 u = ds->v.vel[i], f = ds->v.frc[i];
        double m = ds->v.mass[i];
        double v2 = u.x * u.x + u.y * u.y;
        v[0] = ds->w.pe[i];
        v[1] = 0.5 * m * v2;
        v[2] = f.x * u.x + f.y * u.y;
        v[3] = f.x * f.x + f.y * f.y;
        v[4] = f.x;
        v[5] = f.y;
    }
    const int ops[6] = {0, 0, 0, 1, 0, 0};
    if (grid_reduce<6>(v, ops, ds)) {
        ds->s.pe = v[0]; ds->s.ke = v[1]; ds->s.power = v[2]; ds->s.fmax2 = v[3];
        ds->s.fsum_x = v[4]; ds->s.fsum_y = v[5];
    }
}

// kernelCalcDiskStressTensor: src/particles/disk/kernels.cu:203-252 (summed)
__global__ void k_stress(DevSys *ds) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[4] = {0, 0, 0, 0};
    const int n = ds->p.n;
    if (i < n) {
        const double2 *__restrict__ pos = ds->v.pos;
        const double *__restrict__ rad = ds->v.rad;
        const int *__restrict__ nbr = ds->v.nbr;
        const double bx = ds->p.box[0], by = ds->p.box[1], e_c = ds->p.e_c, n_c = ds->p.n_c;
        double2 pi = pos[i], u = ds->v.vel[i];
        double m = ds->v.mass[i], ri = rad[i];
        double axx = m * u.x * u.x, axy = m * u.x * u.y, ayx = axy, ayy = m * u.y * u.y;
        int cnt = min(ds->w.count[i], ds->p.cap);
        for (int k = 0; k < cnt; k++) {
            int j = nbr[(size_t)k * n + i];
            double2 pj = pos[j];
            double dx = pbc_dist(pi.x, pj.x, bx), dy = pbc_dist(pi.y, pj.y, by);
            double fx, fy;
            disk_pair(pi.x, pi.y, ri, pj.x, pj.y, rad[j], bx, by, e_c, n_c, fx, fy);
            axx += dx * fx / 2;
            axy += dx * fy / 2;
            ayx += dy * fx / 2;
            ayy += dy * fy / 2;
        }
        double area = ds->p.box[0] * ds->p.box[1];
        v[0] = axx / area; v[1] = axy / area; v[2] = ayx / area; v[3] = ayy / area;
    }
    const int ops[4] = {0, 0, 0, 0};
    if (grid_reduce<4>(v, ops, ds))
        for (int k = 0; k < 4; k++) ds->s.stress[k] = v[k];
}

// kernelCountDiskContacts: src/particles/disk/kernels.cu:177-201 (summed)
__global__ void k_contacts(DevSys *ds) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[1] = {0.0};
    const int n = ds->p.n;
    if (i < n) {
        const double2 *__restrict__ pos = ds->v.pos;
        const double *__restrict__ rad = ds->v.rad;
        double2 pi = pos[i];
        int cnt = min(ds->w.count[i], ds->p.cap), c = 0;
        for (int k = 0; k < cnt; k++) {
            int j = ds->v.nbr[(size_t)k * n + i];
            double2 pj = pos[j];
            double dx = pbc_dist(pi.x, pj.x, ds->p.box[0]), dy = pbc_dist(pi.y, pj.y, ds->p.box[1]);
            if (sqrt(dx * dx + dy * dy) < rad[i] + rad[j]) c++;
        }
        v[0] = (double)c;
    }
    const int ops[1] = {0};
    if (grid_reduce<1>(v, ops, ds)) ds->s.contacts = v[0];
}

// kernelAdamStep: src/particles/base/kernels.cu:550-611
__global__ void k_adam(DevSys *ds, double alpha, double b1, double b2, double c1, double c2,
                       double eps) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[2] = {0.0, 0.0};
    if (i < ds->p.n) {
        double2 f = ds->v.frc[i], m1 = ds->v.m1[i], m2 = ds->v.m2[i];
        m1.x = fma(b1, m1.x, (b1 - 1) * f.x);
        m1.y = fma(b1, m1.y, (b1 - 1) * f.y);
        m2.x = fma(b2, m2.x, (1 - b2) * f.x * f.x);
        m2.y = fma(b2, m2.y, (1 - b2) * f.y * f.y);
        double mhx = m1.x / c1, mhy = m1.y / c1, vhx = m2.x / c2, vhy = m2.y / c2;
        double ux = -alpha * mhx / (sqrt(vhx) + eps);
        double uy = -alpha * mhy / (sqrt(vhy) + eps);
        double2 *pos = ds->v.pos;
        double2 p = pos[i];
        p.x += ux;
        p.y += uy;
        pos[i] = p;
        double2 a = ds->w.pos_n[i], c = ds->w.pos_c[i];
        double dxn = p.x - a.x, dyn = p.y - a.y, dxc = p.x - c.x, dyc = p.y - c.y;
        v[0] = dxn * dxn + dyn * dyn;
        v[1] = dxc * dxc + dyc * dyc;
        ds->v.m1[i] = m1;
        ds->v.m2[i] = m2;
    }
    const int ops[2] = {1, 1};
    if (grid_reduce<2>(v, ops, ds)) { ds->s.max_nd2 = v[0]; ds->s.max_cd2 = v[1]; }
}

// scalePositions / scalePositionsFull (src/particles/base/particle.cu:1066-1072)
__global__ void k_scale_pos(DevSys *ds, double f) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ds->p.n) return;
    double2 p = ds->v.pos[i];
    p.x *= f;
    p.y *= f;
    ds->v.pos[i] = p;
}

// ============================================================================
//  Neighbour rebuild (each kernel does nothing unless DevState.rebuild asks)
// ============================================================================

__global__ void k_set_rebuild(DevSys *ds, int kind) { ds->s.rebuild = kind; }

// host-independent decision from the stored displacement maxima
__global__ void k_decide_rebuild(DevSys *ds) {
    if (halted(ds)) { ds->s.rebuild = 0; return; }
    ds->s.rebuild = rebuild_decision(ds, ds->s.max_nd2, ds->s.max_cd2);
}

// kernelGetCellIndexForParticle (src/particles/base/kernels.cu:309-330) + counts
__global__ void k_cell_index(DevSys *ds) {
    if (ds->s.rebuild != 2) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ds->p.n) return;
    double2 p = ds->v.pos[i];
    const int ncd = ds->p.ncd;
    const double cs = ds->p.cell_size;
    int c = cell_coord(p.x, cs, ncd) + cell_coord(p.y, cs, ncd) * ncd;
    ds->w.cell_raw[i] = c;
    atomicAdd(&ds->w.cell_cnt[c], 1);
}

// exclusive scan of the per-cell counts into CSR starts (one block)
__global__ void __launch_bounds__(kScanTPB) k_cell_scan(DevSys *ds) {
    if (ds->s.rebuild != 2) return;
    __shared__ int wsum[kScanTPB / 32];
    __shared__ int carry_s;
    const int ncells = ds->p.ncells;
    const int *cnt = ds->w.cell_cnt;
    int *start = ds->w.cell_start;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int carry = 0;
    for (int base = 0; base < ncells; base += 4 * kScanTPB) {
        int idx = base + 4 * threadIdx.x;
        int a[4];
#pragma unroll
        for (int k = 0; k < 4; k++) a[k] = (idx + k < ncells) ? cnt[idx + k] : 0;
        int t = a[0] + a[1] + a[2] + a[3];
        int incl = t;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += y;
        }
        if (lane == 31) wsum[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            int w = wsum[lane];
            int wi = w;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, wi, off);
                if (lane >= off) wi += y;
            }
            wsum[lane] = wi - w;  // exclusive warp offsets
            if (lane == 31) carry_s = wi;
        }
        __syncthreads();
        int ex = carry + wsum[wid] + incl - t;
#pragma unroll
        for (int k = 0; k < 4; k++) {
            if (idx + k < ncells) start[idx + k] = ex;
            ex += a[k];
        }
        carry += carry_s;
        __syncthreads();
    }
    if (threadIdx.x == 0) start[ncells] = carry;
}

__global__ void k_cell_scatter(DevSys *ds) {
    if (ds->s.rebuild != 2) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ds->p.n) return;
    int c = ds->w.cell_raw[i];
    int slot = ds->w.cell_start[c] + atomicAdd(&ds->w.cell_cur[c], 1);
    ds->w.perm[slot] = i;
}

// Within each cell, restore ascending particle order: the result is the
// permutation of a stable sort by cell (thrust::sort_by_key in
// src/particles/base/particle.cu:1293).  Also clears the counters.
__global__ void k_cell_sort(DevSys *ds) {
    if (ds->s.rebuild != 2) return;
    int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ds->p.ncells) return;
    int b = ds->w.cell_start[c], e = ds->w.cell_start[c + 1];
    int *perm = ds->w.perm;
    for (int k = b + 1; k < e; k++) {
        int key = perm[k];
        int j = k - 1;
        while (j >= b && perm[j] > key) { perm[j + 1] = perm[j]; j--; }
        perm[j + 1] = key;
    }
    ds->w.cell_cnt[c] = 0;
    ds->w.cell_cur[c] = 0;
}

// kernelReorderParticleData (src/particles/base/kernels.cu:508-543) into the
// alternate buffers, then (last block) swap current/alternate on the device.
// The Adam moments are swapped with their twins without a gather, as the
// reference does (src/particles/base/particle.cu:1302-1303).
__global__ void k_reorder(DevSys *ds) {
    if (ds->s.rebuild != 2) return;
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s < ds->p.n) {
        int o = ds->w.perm[s];
        const DevView &v = ds->v;
        double2 p = v.pos[o];
        v.pos_t[s] = p;
        v.vel_t[s] = v.vel[o];
        v.frc_t[s] = v.frc[o];
        v.rad_t[s] = v.rad[o];
        v.mass_t[s] = v.mass[o];
        v.sidx_t[s] = v.sidx[o];
        ds->w.cell_of[s] = ds->w.cell_raw[o];
        ds->w.pos_c[s] = p;
    }
    if (grid_last_block(ds)) {
        DevView &v = ds->v;
        double2 *t2;
        double *t1;
        int *ti;
        t2 = v.pos; v.pos = v.pos_t; v.pos_t = t2;
        t2 = v.vel; v.vel = v.vel_t; v.vel_t = t2;
        t2 = v.frc; v.frc = v.frc_t; v.frc_t = t2;
        t1 = v.rad; v.rad = v.rad_t; v.rad_t = t1;
        t1 = v.mass; v.mass = v.mass_t; v.mass_t = t1;
        ti = v.sidx; v.sidx = v.sidx_t; v.sidx_t = ti;
        t2 = v.m1; v.m1 = v.m1_t; v.m1_t = t2;
        t2 = v.m2; v.m2 = v.m2_t; v.m2_t = t2;
        ds->s.max_cd2 = 0.0;
        ds->s.n_cell_rebuilds++;
    }
}

__device__ __forceinline__ void finish_list_build(DevSys *ds, int cnt) {
    double v[1] = {(double)cnt};
    const int ops[1] = {1};
    if (grid_reduce<1>(v, ops, ds)) {
        int mx = (int)v[0];
        ds->s.max_count = mx;
        if (mx > ds->p.cap) ds->s.flags |= kOverflow;
        ds->s.max_nd2 = 0.0;
        ds->s.n_rebuilds++;
        ds->s.rebuild = 0;
    }
}

// kernelUpdateCellNeighborList: src/particles/base/kernels.cu:440-505
// (3x3 cells, dy outer / dx inner, ascending slot inside each cell).
__global__ void k_nlist_cell(DevSys *ds) {
    if (ds->s.rebuild == 0) return;
    const int n = ds->p.n;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    int cnt = 0;
    if (i < n) {
        const double2 *__restrict__ pos = ds->v.pos;
        const int *__restrict__ cstart = ds->w.cell_start;
        int *__restrict__ nbr = ds->v.nbr;
        const int ncd = ds->p.ncd, cap = ds->p.cap;
        const double bx = ds->p.box[0], by = ds->p.box[1], c2 = ds->p.cutoff2;
        double2 pi = pos[i];
        int c = ds->w.cell_of[i];
        int cx = c % ncd, cy = c / ncd;
        for (int oy = -1; oy <= 1; oy++) {
            int yy = pmod(cy + oy, ncd);
            for (int ox = -1; ox <= 1; ox++) {
                int nc = pmod(cx + ox, ncd) + yy * ncd;
                int b = cstart[nc], e = cstart[nc + 1];
                for (int j = b; j < e; j++) {
                    if (j == i) continue;
                    double2 pj = pos[j];
                    double dx = pbc_dist(pi.x, pj.x, bx), dy = pbc_dist(pi.y, pj.y, by);
                    if (dx * dx + dy * dy < c2) {
                        if (cnt < cap) nbr[(size_t)cnt * n + i] = j;
                        cnt++;
                    }
                }
            }
        }
        ds->w.count[i] = cnt;
        ds->w.pos_n[i] = pi;
        mixed_update(ds, i, pi);
    }
    finish_list_build(ds, cnt);
}

// kernelUpdateNeighborList (all pairs, methods "verlet" / "all"):
// src/particles/base/kernels.cu:256-293.  j tiles staged in shared memory.
__global__ void k_nlist_all(DevSys *ds) {
    if (ds->s.rebuild == 0) return;
    __shared__ double2 tile[kTPB];
    const int n = ds->p.n;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double2 *__restrict__ pos = ds->v.pos;
    int *__restrict__ nbr = ds->v.nbr;
    const int cap = ds->p.cap;
    const double bx = ds->p.box[0], by = ds->p.box[1], c2 = ds->p.cutoff2;
    double2 pi = (i < n) ? pos[i] : make_double2(0.0, 0.0);
    int cnt = 0;
    for (int base = 0; base < n; base += kTPB) {
        int j0 = base + threadIdx.x;
        if (j0 < n) tile[threadIdx.x] = pos[j0];
        __syncthreads();
        int lim = min(kTPB, n - base);
        if (i < n) {
            for (int t = 0; t < lim; t++) {
                int j = base + t;
                if (j == i) continue;
                double2 pj = tile[t];
                double dx = pbc_dist(pi.x, pj.x, bx), dy = pbc_dist(pi.y, pj.y, by);
                if (dx * dx + dy * dy < c2) {
                    if (cnt < cap) nbr[(size_t)cnt * n + i] = j;
                    cnt++;
                }
            }
        }
        __syncthreads();
    }
    if (i < n) {
        ds->w.count[i] = cnt;
        ds->w.pos_n[i] = pi;
        mixed_update(ds, i, pi);
    }
    finish_list_build(ds, cnt);
}

// ============================================================================
//  Fused loops
// ============================================================================

// NVE::step first half (src/integrator/nve.cu:16-17): kick dt/2, drift dt,
// displacement maxima and the rebuild decision.
__global__ void k_nve_first(DevSys *ds, double dt_half, double dt) {
    if (halted(ds)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[2] = {0.0, 0.0};
    if (i < ds->p.n) {
        double2 *vel = ds->v.vel, *pos = ds->v.pos;
        double2 u = vel[i], f = ds->v.frc[i], p = pos[i];
        double dtm = dt_half / ds->v.mass[i];
        u.x = u.x + f.x * dtm;
        u.y = u.y + f.y * dtm;
        vel[i] = u;
        p.x = p.x + u.x * dt;
        p.y = p.y + u.y * dt;
        pos[i] = p;
        mixed_update(ds, i, p);
        double2 a = ds->w.pos_n[i], c = ds->w.pos_c[i];
        double dxn = p.x - a.x, dyn = p.y - a.y, dxc = p.x - c.x, dyc = p.y - c.y;
        v[0] = dxn * dxn + dyn * dyn;
        v[1] = dxc * dxc + dyc * dyc;
    }
    const int ops[2] = {1, 1};
    if (grid_reduce<2>(v, ops, ds)) {
        ds->s.max_nd2 = v[0];
        ds->s.max_cd2 = v[1];
        int rb = rebuild_decision(ds, v[0], v[1]);
        ds->s.rebuild = rb;
        if (ds->s.h_rb) cudaGraphSetConditional(ds->s.h_rb, rb != 0);
    }
}

// NVE::step second half (src/integrator/nve.cu:21-24): zero, forces, kick dt/2.
template <int G, bool M>
__global__ void k_nve_second(DevSys *ds, double dt_half) {
    if (halted(ds)) return;
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = gid / G;
    double ax, ay, en;
    force_sum<G, M>(ds, i, i < ds->p.n, ax, ay, en);
    if (i < ds->p.n && (gid & (G - 1)) == 0) {
        double2 *vel = ds->v.vel;
        double2 u = vel[i];
        double2 f;
        const double g = ds->s.damping;
        double pe0 = 0.0;
        if (ds->s.walls) {
            // NVE::wall_step (src/integrator/nve.cu:33-35): zero, wall forces,
            // then += the pair sum unless the particle has no neighbours
            double wx, wy;
            const double ew = wall_force(ds->p, ds->v.pos[i], ds->v.rad[i], wx, wy);
            f = make_double2(0.0 + wx, 0.0 + wy);
            pe0 = 0.0 + ew;
            if (ds->w.count[i] != 0) { f.x += ax; f.y += ay; pe0 += en; }
        } else if (g != 0.0) {
            // DampedNVE::step (src/integrator/damped_nve.cu:22-23): F = 0 - g v,
            // then += the pair sum unless the particle has no neighbours
            f = make_double2(0.0 - g * u.x, 0.0 - g * u.y);
            if (ds->w.count[i] != 0) { f.x += ax; f.y += ay; }
        } else {
            f = make_double2(0.0 + ax, 0.0 + ay);
        }
        ds->v.frc[i] = f;
        ds->w.pe[i] = ds->s.walls ? pe0 : 0.0 + en;
        double dtm = dt_half / ds->v.mass[i];
        u.x = u.x + f.x * dtm;
        u.y = u.y + f.y * dtm;
        vel[i] = u;
    }
    if (grid_last_block(ds)) {
        if (++ds->s.nve_steps_done >= ds->s.max_steps) ds->s.flags |= kDone;
    }
}

// ---- FIRE -------------------------------------------------------------------

// Fire::step prologue (src/integrator/fire.cu:13-34): decide dt / alpha from
// the power of the state the next step starts from.
__device__ void fire_decide(DevSys *ds, double power) {
    DevState &s = ds->s;
    if (power > 0) {
        s.f_ngood++;
        s.f_nbad = 0;
        if (s.f_ngood > 5) {
            s.f_dt = fmin(s.f_dt * 1.1, s.f_dtmax);
            s.f_alpha *= 0.99;
        }
        s.fire_uphill = 0;
    } else {
        s.f_ngood = 0;
        s.f_nbad++;
        if (s.f_nbad > 10) {
            s.f_stopped = 1;
            s.fire_uphill = 0;
            s.flags |= kDone;
            return;
        }
        s.f_dt = fmax(s.f_dt * 0.5, s.f_dtmin);
        s.f_alpha = s.f_alpha0;
        s.fire_uphill = 1;
    }
}

// FIRE move: uphill rollback (x -= v dt/2, v = 0), kick dt/2, per-particle
// mix, drift dt (src/integrator/fire.cu:29-40), displacement maxima and the
// rebuild decision.
__global__ void k_fire_move(DevSys *ds) {
    if (halted(ds)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double dt = ds->s.f_dt, alpha = ds->s.f_alpha;
    const int up = ds->s.fire_uphill;
    double v[2] = {0.0, 0.0};
    if (i < ds->p.n) {
        double2 *vel = ds->v.vel, *pos = ds->v.pos;
        double2 u = vel[i], f = ds->v.frc[i], p = pos[i];
        if (up) {
            double back = -dt / 2.0;
            p.x = p.x + u.x * back;
            p.y = p.y + u.y * back;
            u = make_double2(0.0, 0.0);
        }
        double dtm = (dt / 2.0) / ds->v.mass[i];
        u.x = u.x + f.x * dtm;
        u.y = u.y + f.y * dtm;
        u = fire_mix(u, f, alpha);
        vel[i] = u;
        p.x = p.x + u.x * dt;
        p.y = p.y + u.y * dt;
        pos[i] = p;
        mixed_update(ds, i, p);
        double2 a = ds->w.pos_n[i], c = ds->w.pos_c[i];
        double dxn = p.x - a.x, dyn = p.y - a.y, dxc = p.x - c.x, dyc = p.y - c.y;
        v[0] = dxn * dxn + dyn * dyn;
        v[1] = dxc * dxc + dyc * dyc;
    }
    const int ops[2] = {1, 1};
    if (grid_reduce<2>(v, ops, ds)) {
        ds->s.max_nd2 = v[0];
        ds->s.max_cd2 = v[1];
        int rb = rebuild_decision(ds, v[0], v[1]);
        ds->s.rebuild = rb;
        if (ds->s.h_rb) cudaGraphSetConditional(ds->s.h_rb, rb != 0);
    }
}

// FIRE force phase: forces (overwrite), kick dt/2, then on the last block the
// minimizeFire convergence tests (src/routines/minimization.cu:96-106) and the
// next step's Fire::step decision.  mode 0 = loop iteration, 1 = setup
// (forces only: minimizeFire's initial force call and last_avg_pe), 2 = a
// single Fire::step (no convergence test, decision for the next step only).
template <int G, bool M>
__global__ void k_fire_force(DevSys *ds, int mode) {
    if (halted(ds)) return;
    const int gid = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = gid / G;
    double v[3] = {0.0, 0.0, 0.0};
    double ax, ay, en;
    force_sum<G, M>(ds, i, i < ds->p.n, ax, ay, en);
    if (i < ds->p.n && (gid & (G - 1)) == 0) {
        double2 f = make_double2(0.0 + ax, 0.0 + ay);
        ds->v.frc[i] = f;
        ds->w.pe[i] = 0.0 + en;
        double2 *vel = ds->v.vel;
        double2 u = vel[i];
        if (mode != 1) {
            double dtm = (ds->s.f_dt / 2.0) / ds->v.mass[i];
            u.x = u.x + f.x * dtm;
            u.y = u.y + f.y * dtm;
            vel[i] = u;
        }
        v[0] = 0.0 + en;
        v[1] = f.x * u.x + f.y * u.y;
        v[2] = f.x * f.x + f.y * f.y;
    }
    const int ops[3] = {0, 0, 1};
    if (!grid_reduce<3>(v, ops, ds)) return;
    DevState &s = ds->s;
    s.pe = v[0];
    s.power = v[1];
    s.fmax2 = v[2];
    double avg = v[0] / s.dof;
    if (mode == 1) {
        s.last_avg_pe = avg;
        fire_decide(ds, v[1]);
        if (s.f_stopped) { s.result_step = 0; s.flags |= kDone; }
        return;
    }
    if (mode == 2) return;
    double diff = fabs(avg / s.last_avg_pe - 1);
    s.last_avg_pe = avg;
    long long it = s.iter;
    // mixed form: FP32 pairs until max|F| reaches switch_fmax, FIRE keeps going
    // uphill, or max|F| stops falling within 100x of switch_fmax (FP32 noise
    // floor); FP64 pairs after, and only an FP64 state may pass the PE-change
    // and max|F| tests
    bool fp64 = true;
    if (M && !s.fp64_now) {
        if (v[2] < 0.81 * s.best_f2) { s.best_f2 = v[2]; s.best_it = it; }
        const double fm = sqrt(v[2]);
        if (fm <= s.switch_fmax || s.f_nbad > 5 || (fm < 100.0 * s.switch_fmax && it - s.best_it > 2000))
            s.fp64_now = 1;
        fp64 = false;
    }
    if ((fp64 && diff < s.pe_diff_target) || avg < s.pe_target) {
        s.result_step = it; s.f_converged = 1; s.flags |= kDone; return;
    }
    if (fp64 && s.fmax_target > 0 && sqrt(v[2]) <= s.fmax_target) {
        s.result_step = it; s.f_converged = 1; s.flags |= kDone; return;
    }
    if (it + 1 >= s.max_steps) { s.result_step = s.max_steps; s.flags |= kDone; return; }
    s.iter = it + 1;
    fire_decide(ds, v[1]);
    if (s.f_stopped) { s.result_step = it + 1; s.f_converged = 1; s.flags |= kDone; }
}

// Fire::step prologue for a single step: P = F.v over the grid, then decide.
__global__ void k_fire_power_decide(DevSys *ds) {
    if (halted(ds)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[1] = {0.0};
    if (i < ds->p.n) {
        double2 u = ds->v.vel[i], f = ds->v.frc[i];
        v[0] = f.x * u.x + f.y * u.y;
    }
    const int ops[1] = {0};
    if (grid_reduce<1>(v, ops, ds)) {
        ds->s.power = v[0];
        fire_decide(ds, v[0]);
    }
}

// Last node of every WHILE body: continue only while no flag is raised and
// the iteration budget is not spent.  Guarantees the loop terminates.
__global__ void k_loop_guard(DevSys *ds) {
    DevState &s = ds->s;
    long long g = ++s.guard;
    int go = (s.flags == 0) && (g < s.guard_limit);
    if (!go && s.flags == 0) s.flags |= kError;
    if (s.h_loop) cudaGraphSetConditional(s.h_loop, go ? 1u : 0u);
}

// ============================================================================
//  State transfer (static order <-> sorted slots)
// ============================================================================

// which: 0 pos, 1 vel, 2 frc ; xy from separate x / y arrays in static order
__global__ void k_put_xy(DevSys *ds, int which, const double *x, const double *y) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ds->p.n) return;
    int k = ds->v.sidx[i];
    double2 *dst = which == 0 ? ds->v.pos : (which == 1 ? ds->v.vel : ds->v.frc);
    double2 o = dst[i];
    if (x) o.x = x[k];
    if (y) o.y = y[k];
    dst[i] = o;
}

// which: 0 rad, 1 mass
__global__ void k_put_scalar(DevSys *ds, int which, const double *a) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ds->p.n) return;
    int k = ds->v.sidx[i];
    (which == 0 ? ds->v.rad : ds->v.mass)[i] = a[k];
}

// which: 0 pos, 1 vel, 2 frc
__global__ void k_get_xy(DevSys *ds, int which, double *x, double *y) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ds->p.n) return;
    int k = ds->v.sidx[i];
    const double2 *src = which == 0 ? ds->v.pos : (which == 1 ? ds->v.vel : ds->v.frc);
    double2 o = src[i];
    if (x) x[k] = o.x;
    if (y) y[k] = o.y;
}

// which: 0 radii, 1 masses (static order out)
__global__ void k_get_scalar(DevSys *ds, int which, double *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ds->p.n) return;
    out[ds->v.sidx[i]] = (which == 0 ? ds->v.rad : ds->v.mass)[i];
}

__global__ void k_get_pe(DevSys *ds, double *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ds->p.n) return;
    out[ds->v.sidx[i]] = ds->w.pe[i];
}

__global__ void k_iota_sidx(DevSys *ds) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ds->p.n) return;
    ds->v.sidx[i] = i;
}

// neighbour rows in static indices, row-major [n][cap_out], -1 padded
__global__ void k_get_nbrs(DevSys *ds, int *list, int *counts, int cap_out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = ds->p.n;
    if (i >= n) return;
    const int *sidx = ds->v.sidx;
    int k = sidx[i];
    int cnt = ds->w.count[i];
    counts[k] = cnt;
    int lim = min(cnt, min(cap_out, ds->p.cap));
    for (int t = 0; t < cap_out; t++)
        list[(size_t)k * cap_out + t] = t < lim ? sidx[ds->v.nbr[(size_t)t * n + i]] : -1;
}

__global__ void k_get_cells(DevSys *ds, long long *cell_index, long long *cell_start,
                            long long *static_index) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < ds->p.n) {
        if (cell_index) cell_index[i] = ds->w.cell_of[i];
        if (static_index) static_index[i] = ds->v.sidx[i];
    }
    if (cell_start && i <= ds->p.ncells) {
        int b = ds->w.cell_start[i];
        if (i == ds->p.ncells) cell_start[i] = b;
        else cell_start[i] = (ds->w.cell_start[i + 1] > b) ? b : -1;
    }
}

// setLastState (dir = 0) / revertToLastStateVariables (dir = 1)
__global__ void k_snapshot(DevSys *ds, int dir) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= ds->p.n) return;
    DevView &v = ds->v;
    DevScratch &w = ds->w;
    if (dir == 0) {
        w.s_pos[i] = v.pos[i]; w.s_vel[i] = v.vel[i]; w.s_frc[i] = v.frc[i];
        w.s_rad[i] = v.rad[i]; w.s_mass[i] = v.mass[i]; w.s_sidx[i] = v.sidx[i];
    } else {
        v.pos[i] = w.s_pos[i]; v.vel[i] = w.s_vel[i]; v.frc[i] = w.s_frc[i];
        v.rad[i] = w.s_rad[i]; v.mass[i] = w.s_mass[i]; v.sidx[i] = w.s_sidx[i];
    }
}

}  // namespace
}  // namespace dpg
