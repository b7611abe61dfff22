// bumpy_kernels.cuh -- plain FP64 kernels for rigid bumpy bodies (rigid bodies
// made of vertex disks on a circle), the drop-in form of
// src/particles/rigid_bumpy/{rigid_bumpy.cu,kernels.cu}.
//
// Layout: BumpySys embeds the disk DevSys as its first member, with the BODIES
// in the disk slots (pos, vel, frc, rad, mass, sidx, body neighbour list, cell
// list), so the disk cell-list and body neighbour kernels run unchanged on the
// bodies.  BumpyExt adds the rotational body fields and the vertices; vertices
// of a body are contiguous ([start[b], start[b] + nvb[b])) and move as a block
// when bodies are re-sorted, like the reference.
//
// Vertex work runs warp-per-body: lane l owns vertices start + l, start + l +
// 32, ...; a body's force, torque and energy are summed over its vertices in
// vertex order with warp shuffles, which reproduces the reference's sequential
// per-body sum (kernelCalcRigidBumpyParticleForces1) bit for bit.
// Compiled with --fmad=false (reference operation order).
#pragma once
#include "disk_kernels.cuh"

namespace dpg {
namespace {  // kernels have internal linkage: each translation unit owns its copy

struct BumpyExt {
    int nv, capv, rotation, max_vcount;
    double rv, vcut2, vpcut2;
    double *w, *th, *tq, *I;  // angular velocity, angle, torque, moment of inertia
    int *nvb, *start;
    double *w_t, *th_t, *tq_t, *I_t;
    int *nvb_t, *start_t;
    double2 *vpos, *vpos_t;
    double *vmass, *vmass_t;
    int *vbody, *vbody_t, *svidx, *svidx_t;
    int *o2n;                // old -> new body slot during a re-sort
    int *vnbr, *vcount;      // vertex neighbour list, column-major [capv][nv]
    float4 *vpk;             // mixed form: packed FP32 vertex offsets (see mixed_pack)
    int mixed;               // 1: FP32 vertex pairs (the body DevParams stay FP64)
    long long vlist_built;   // n_rebuilds value at the last vertex-list build
    double tmax2, power_rot;
    // snapshot of the rotational state (setLastState)
    double *s_w, *s_th, *s_tq;
    double2 *s_vpos;
    int *s_nvb, *s_start, *s_vbody, *s_svidx;
    // per slot, never re-sorted (like the reference's angle_delta and angular
    // Adam moments): the last angle increment and the angular Adam moments
    double *adelta, *m1a, *m2a;
    // per-body results of the stress and contact passes (body-slot order)
    double *stress_b;   // [4][nb]: xx, xy, yx, yy
    int *ccount, *vccount;
    double vcontacts;
};

struct BumpySys {
    DevSys b;  // must stay first: BumpySys* is passed as DevSys* to the disk kernels
    BumpyExt x;
};

constexpr int kWarpsPerBlock = kTPB / 32;

// calcTorque: include/particles/base/kernels.cuh:237-241
__device__ __forceinline__ double torque_of(double fx, double fy, double px, double py, double cx,
                                           double cy) {
    double dx = px - cx, dy = py - cy;
    return fy * dx - fx * dy;
}

// ---- body kick: kernelUpdateRigidVelocities (kernels.cu:123-150) -----------
__device__ __forceinline__ void body_kick(BumpySys *bs, int b, double dt) {
    DevSys &d = bs->b;
    double2 v = d.v.vel[b], f = d.v.frc[b];
    double m = d.v.mass[b];
    double w = bs->x.w[b];
    if (bs->x.rotation) w += bs->x.tq[b] * dt / bs->x.I[b];
    else w = 0.0;
    v.x += f.x * dt / m;
    v.y += f.y * dt / m;
    d.v.vel[b] = v;
    bs->x.w[b] = w;
}

__global__ void kb_kick(BumpySys *bs, double dt) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= bs->b.p.n) return;
    body_kick(bs, b, dt);
}

// ---- body + vertex move: kernelUpdateRigidPositions + kernelTranslateAndRotateVertices1
// (kernels.cu:21-78,152-201), one warp per body.  Returns the squared
// displacements from the neighbour / cell reference positions (lane 0).
__device__ __forceinline__ void body_move(BumpySys *bs, int b, int lane, double dt, double &nd2,
                                          double &cd2) {
    DevSys &d = bs->b;
    BumpyExt &x = bs->x;
    double2 p = d.v.pos[b], u = d.v.vel[b];
    double ang = x.th[b], w = x.w[b];
    double ddx = u.x * dt, ddy = u.y * dt, dth = w * dt;
    double nx = p.x + ddx, ny = p.y + ddy;
    __syncwarp();
    if (lane == 0) {
        d.v.pos[b] = make_double2(nx, ny);
        x.th[b] = ang + dth;
        x.adelta[b] = dth;
        double2 a = d.w.pos_n[b], c = d.w.pos_c[b];
        double a1 = nx - a.x, a2 = ny - a.y, c1 = nx - c.x, c2 = ny - c.y;
        nd2 = a1 * a1 + a2 * a2;
        cd2 = c1 * c1 + c2 * c2;
    }
    double ca = cos(dth), sa = sin(dth);
    const int f = x.start[b], nvb = x.nvb[b];
    for (int k = lane; k < nvb; k += 32) {
        double2 q = x.vpos[f + k];
        double rx = q.x - p.x, ry = q.y - p.y;
        double rxr = rx * ca - ry * sa, ryr = rx * sa + ry * ca;
        double2 nq = make_double2(nx + rxr, ny + ryr);
        x.vpos[f + k] = nq;
        if (x.mixed) x.vpk[f + k] = mixed_pack(d.p, nq, x.rv);
    }
}

__global__ void kb_drift(BumpySys *bs, double dt) {
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    double v[2] = {0.0, 0.0};
    if (b < bs->b.p.n) body_move(bs, b, lane, dt, v[0], v[1]);
    const int ops[2] = {1, 1};
    if (grid_reduce<2>(v, ops, &bs->b)) { bs->b.s.max_nd2 = v[0]; bs->b.s.max_cd2 = v[1]; }
}

// ---- forces: kernelCalcRigidBumpyForces1 + kernelCalcRigidBumpyParticleForces1
// (kernels.cu:366-442) fused, one warp per body.  Outputs the body sums (every
// lane holds the same values).  walls: kernelCalcRigidBumpyWallForces
// (kernels.cu:348-362) first, as NVE::wall_step calls it before the pairs, so
// a vertex carries (0 + wall) + pair sum.
__device__ __forceinline__ void body_forces(const BumpySys *__restrict__ bs, int b, int lane,
                                            bool walls, double &bfx, double &bfy, double &btq,
                                            double &bpe) {
    const DevSys &d = bs->b;
    const BumpyExt &x = bs->x;
    const int nv = x.nv, capv = x.capv;
    const double bx = d.p.box[0], by = d.p.box[1], e_c = d.p.e_c, n_c = d.p.n_c, rv = x.rv;
    const double2 c = d.v.pos[b];
    const int f = x.start[b], nvb = x.nvb[b];
    const bool mixed = x.mixed && !d.s.fp64_now;
    bfx = 0.0; bfy = 0.0; btq = 0.0; bpe = 0.0;
    for (int base = 0; base < nvb; base += 32) {
        int k = base + lane;
        double vfx = 0.0, vfy = 0.0, vtq = 0.0, vpe = 0.0;
        if (k < nvb) {
            int v = f + k;
            double2 q = x.vpos[v];
            int cnt = min(x.vcount[v], capv);
            double ax = 0.0, ay = 0.0, en = 0.0;
            if (mixed) {  // FP32 vertex pairs; torque and body sums stay FP64
                const float4 a = x.vpk[v];
                float sx = 0.f, sy = 0.f, se = 0.f;
                for (int t = 0; t < cnt; t++) {
                    int u = __ldg(&x.vnbr[(size_t)t * nv + v]);
                    float fx, fy;
                    se += mixed_pair(d.p, a, x.vpk[u], (float)e_c, (float)n_c, fx, fy);
                    sx += fx;
                    sy += fy;
                }
                ax = (double)sx;
                ay = (double)sy;
                en = (double)se;
            } else {
                for (int t = 0; t < cnt; t++) {
                    int u = __ldg(&x.vnbr[(size_t)t * nv + v]);
                    double2 o = x.vpos[u];
                    double fx, fy;
                    double e = disk_pair(q.x, q.y, rv, o.x, o.y, rv, bx, by, e_c, n_c, fx, fy);
                    ax += fx;
                    ay += fy;
                    en += e;
                }
            }
            if (walls) {
                double wx, wy;
                const double we = wall_force(d.p, q, rv, wx, wy);
                vfx = 0.0 + wx;
                vfy = 0.0 + wy;
                vtq = 0.0 + torque_of(wx, wy, q.x, q.y, c.x, c.y);
                vpe = 0.0 + we;
            }
            if (cnt > 0) {
                vfx = vfx + ax;
                vfy = vfy + ay;
                vtq = vtq + torque_of(ax, ay, q.x, q.y, c.x, c.y);
                vpe = vpe + en;
            }
        }
        int lim = min(32, nvb - base);
        for (int l = 0; l < lim; l++) {
            bfx += __shfl_sync(0xffffffffu, vfx, l);
            bfy += __shfl_sync(0xffffffffu, vfy, l);
            btq += __shfl_sync(0xffffffffu, vtq, l);
            bpe += __shfl_sync(0xffffffffu, vpe, l);
        }
    }
}

// mixed form: packed offsets of every vertex from the current vertex positions
__global__ void kb_mixed_refresh(BumpySys *bs) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= bs->x.nv) return;
    bs->x.vpk[v] = mixed_pack(bs->b.p, bs->x.vpos[v], bs->x.rv);
}

// drop-in calculateForces (+= into the body arrays); walls = 1: calculateWallForces
// then calculateForces
__global__ void kb_force_acc(BumpySys *bs, int walls) {
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (b >= bs->b.p.n) return;
    double fx, fy, tq, pe;
    body_forces(bs, b, lane, walls != 0, fx, fy, tq, pe);
    if (lane == 0) {
        double2 f = bs->b.v.frc[b];
        f.x += fx;
        f.y += fy;
        bs->b.v.frc[b] = f;
        bs->x.tq[b] += tq;
        bs->b.w.pe[b] += pe;
    }
}

// zeroForceAndPotentialEnergy (rigid_bumpy.cu:1378-1381); vertex arrays are not kept
__global__ void kb_zero_force(BumpySys *bs) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= bs->b.p.n) return;
    bs->b.v.frc[b] = make_double2(0.0, 0.0);
    bs->x.tq[b] = 0.0;
    bs->b.w.pe[b] = 0.0;
}

// kernelMixRigidVelocitiesAndForces (kernels.cu:89-121)
__device__ __forceinline__ void body_mix(BumpySys *bs, int b, double alpha) {
    double2 f = bs->b.v.frc[b], v = bs->b.v.vel[b];
    double fn = sqrt(f.x * f.x + f.y * f.y), vn = sqrt(v.x * v.x + v.y * v.y), mix = 0.0;
    if (fn > 1e-16) mix = vn / fn * alpha;
    else { v.x = 0.0; v.y = 0.0; }
    double w = bs->x.w[b], t = bs->x.tq[b];
    double tn = fabs(t), wn = fabs(w), tmix = 0.0;
    if (tn > 1e-16) tmix = wn / tn * alpha;
    else { w = 0.0; tmix = 0.0; }
    double2 o;
    o.x = v.x * (1 - alpha) + f.x * mix;
    o.y = v.y * (1 - alpha) + f.y * mix;
    bs->b.v.vel[b] = o;
    bs->x.w[b] = w * (1 - alpha) + t * tmix;
}

__global__ void kb_mix(BumpySys *bs, double alpha) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= bs->b.p.n) return;
    body_mix(bs, b, alpha);
}

__global__ void kb_zero_vel(BumpySys *bs) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= bs->b.p.n) return;
    bs->b.v.vel[b] = make_double2(0.0, 0.0);
    bs->x.w[b] = 0.0;
}

// PE, KE (kernelCalculateTranslationalAndRotationalKineticEnergy, kernels.cu:254-269),
// FIRE power incl. the rotational part (rigid_bumpy.cu:1181-1190), max|F|^2, max tau^2
__global__ void kb_observables(BumpySys *bs) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    double v[5] = {0, 0, 0, 0, 0};
    if (b < bs->b.p.n) {
        double2 u = bs->b.v.vel[b], f = bs->b.v.frc[b];
        double m = bs->b.v.mass[b], w = bs->x.w[b], t = bs->x.tq[b];
        v[0] = bs->b.w.pe[b];
        v[1] = bs->x.rotation ? 0.5 * m * (u.x * u.x + u.y * u.y) + 0.5 * bs->x.I[b] * w * w
                              : 0.5 * m * (u.x * u.x + u.y * u.y);
        v[2] = f.x * u.x + f.y * u.y + t * w;
        v[3] = f.x * f.x + f.y * f.y;
        v[4] = t * t;
    }
    const int ops[5] = {0, 0, 0, 1, 1};
    if (grid_reduce<5>(v, ops, &bs->b)) {
        bs->b.s.pe = v[0]; bs->b.s.ke = v[1]; bs->b.s.power = v[2]; bs->b.s.fmax2 = v[3];
        bs->x.tmax2 = v[4];
    }
}

// ---- vertex neighbour list: kernelUpdateVertexNeighborList (kernels.cu:870-922),
// warp per body so the walk over the body's neighbour bodies is uniform.
// Runs only when the body list was rebuilt since the last vertex build.
__global__ void kb_vlist(BumpySys *bs) {
    if (bs->b.s.n_rebuilds == bs->x.vlist_built) return;
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    const DevSys &d = bs->b;
    BumpyExt &x = bs->x;
    int mxc = 0;
    if (b < d.p.n) {
        const int nb = d.p.n, nv = x.nv, capv = x.capv;
        const double bx = d.p.box[0], by = d.p.box[1], c2 = x.vcut2, pc2 = x.vpcut2;
        const int f = x.start[b], nvb = x.nvb[b];
        const int ncnt = min(d.w.count[b], d.p.cap);
        for (int base = 0; base < nvb; base += 32) {
            int k = base + lane;
            if (k >= nvb) break;
            int v = f + k;
            double2 q = x.vpos[v];
            int cnt = 0;
            for (int t = 0; t < ncnt; t++) {
                int ob = d.v.nbr[(size_t)t * nb + b];
                double2 oc = d.v.pos[ob];
                double ex = pbc_dist(q.x, oc.x, bx), ey = pbc_dist(q.y, oc.y, by);
                if (!(ex * ex + ey * ey < pc2)) continue;
                int of = x.start[ob], on = x.nvb[ob];
                for (int u = of; u < of + on; u++) {
                    double2 o = x.vpos[u];
                    double gx = pbc_dist(q.x, o.x, bx), gy = pbc_dist(q.y, o.y, by);
                    if (gx * gx + gy * gy < c2) {
                        if (cnt < capv) x.vnbr[(size_t)cnt * nv + v] = u;
                        cnt++;
                    }
                }
            }
            x.vcount[v] = cnt;
            mxc = max(mxc, cnt);
            if (x.mixed) x.vpk[v] = mixed_pack(d.p, q, x.rv);
        }
    }
    double val[1] = {(double)mxc};
    const int ops[1] = {1};
    if (grid_reduce<1>(val, ops, &bs->b)) {
        int m = (int)val[0];
        x.max_vcount = m;
        if (m > x.capv) bs->b.s.flags |= kOverflow;
        x.vlist_built = bs->b.s.n_rebuilds;
    }
}

// ---- re-sort of bodies and their vertex blocks:
// RigidBumpy::reorderParticleData (rigid_bumpy.cu:1303-1376, kernels.cu:796-868)
__global__ void kb_reorder_bodies(BumpySys *bs) {
    if (bs->b.s.rebuild != 2) return;
    int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= bs->b.p.n) return;
    DevSys &d = bs->b;
    BumpyExt &x = bs->x;
    int o = d.w.perm[s];
    x.o2n[o] = s;
    double2 p = d.v.pos[o];
    d.v.pos_t[s] = p;
    d.v.vel_t[s] = d.v.vel[o];
    d.v.frc_t[s] = d.v.frc[o];
    d.v.rad_t[s] = d.v.rad[o];
    d.v.mass_t[s] = d.v.mass[o];
    d.v.sidx_t[s] = d.v.sidx[o];
    x.w_t[s] = x.w[o];
    x.th_t[s] = x.th[o];
    x.tq_t[s] = x.tq[o];
    x.I_t[s] = x.I[o];
    x.nvb_t[s] = x.nvb[o];
    d.w.cell_of[s] = d.w.cell_raw[o];
    d.w.pos_c[s] = p;
}

// exclusive scan of the re-sorted vertex counts into the new block starts (one block)
__global__ void __launch_bounds__(kScanTPB) kb_scan_starts(BumpySys *bs) {
    if (bs->b.s.rebuild != 2) return;
    __shared__ int wsum[kScanTPB / 32];
    __shared__ int carry_s;
    const int nb = bs->b.p.n;
    const int *cnt = bs->x.nvb_t;
    int *start = bs->x.start_t;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int carry = 0;
    for (int base = 0; base < nb; base += kScanTPB) {
        int idx = base + threadIdx.x;
        int a = idx < nb ? cnt[idx] : 0;
        int incl = a;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off) incl += y;
        }
        if (lane == 31) wsum[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            int w = wsum[lane], wi = w;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                int y = __shfl_up_sync(0xffffffffu, wi, off);
                if (lane >= off) wi += y;
            }
            wsum[lane] = wi - w;
            if (lane == 31) carry_s = wi;
        }
        __syncthreads();
        if (idx < nb) start[idx] = carry + wsum[wid] + incl - a;
        carry += carry_s;
        __syncthreads();
    }
}

// move every vertex block to its body's new start (warp per new body), then
// swap current / alternate buffers on the device (last block)
__global__ void kb_reorder_vertices(BumpySys *bs) {
    if (bs->b.s.rebuild != 2) return;
    const int lane = threadIdx.x & 31;
    const int s = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    DevSys &d = bs->b;
    BumpyExt &x = bs->x;
    if (s < d.p.n) {
        int o = d.w.perm[s];
        int of = x.start[o], nf = x.start_t[s], n = x.nvb_t[s];
        for (int k = lane; k < n; k += 32) {
            x.vpos_t[nf + k] = x.vpos[of + k];
            x.vmass_t[nf + k] = x.vmass[of + k];
            x.svidx_t[nf + k] = x.svidx[of + k];
            x.vbody_t[nf + k] = s;
        }
    }
    if (grid_last_block(&bs->b)) {
        DevView &v = d.v;
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
        t1 = x.w; x.w = x.w_t; x.w_t = t1;
        t1 = x.th; x.th = x.th_t; x.th_t = t1;
        t1 = x.tq; x.tq = x.tq_t; x.tq_t = t1;
        t1 = x.I; x.I = x.I_t; x.I_t = t1;
        ti = x.nvb; x.nvb = x.nvb_t; x.nvb_t = ti;
        ti = x.start; x.start = x.start_t; x.start_t = ti;
        t2 = x.vpos; x.vpos = x.vpos_t; x.vpos_t = t2;
        t1 = x.vmass; x.vmass = x.vmass_t; x.vmass_t = t1;
        ti = x.vbody; x.vbody = x.vbody_t; x.vbody_t = ti;
        ti = x.svidx; x.svidx = x.svidx_t; x.svidx_t = ti;
        d.s.max_cd2 = 0.0;
        d.s.n_cell_rebuilds++;
    }
}

// ---- fused loops ------------------------------------------------------------

// NVE::step first half with the rigid overrides: kick dt/2, move dt
__global__ void kb_nve_first(BumpySys *bs, double dt_half, double dt) {
    if (halted(&bs->b)) return;
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    double v[2] = {0.0, 0.0};
    if (b < bs->b.p.n) {
        if (lane == 0) body_kick(bs, b, dt_half);
        __syncwarp();
        body_move(bs, b, lane, dt, v[0], v[1]);
    }
    const int ops[2] = {1, 1};
    if (grid_reduce<2>(v, ops, &bs->b)) {
        DevSys *ds = &bs->b;
        ds->s.max_nd2 = v[0];
        ds->s.max_cd2 = v[1];
        int rb = rebuild_decision(ds, v[0], v[1]);
        ds->s.rebuild = rb;
        if (ds->s.h_rb) cudaGraphSetConditional(ds->s.h_rb, rb != 0);
    }
}

// second half: forces (overwrite) + kick dt/2
__global__ void kb_nve_second(BumpySys *bs, double dt_half) {
    if (halted(&bs->b)) return;
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (b < bs->b.p.n) {
        double fx, fy, tq, pe;
        body_forces(bs, b, lane, bs->b.s.walls != 0, fx, fy, tq, pe);
        if (lane == 0) {
            const double g = bs->b.s.damping;
            if (g != 0.0) {
                // DampedNVE::step (src/integrator/damped_nve.cu:22-23) with
                // kernelCalculateRigidDampedForces (kernels.cu:80-87): body
                // F = 0 - g v, tau = 0 - g omega, then += the vertex sums
                const double2 u = bs->b.v.vel[b];
                const double w = bs->x.w[b];
                bs->b.v.frc[b] = make_double2((0.0 - g * u.x) + fx, (0.0 - g * u.y) + fy);
                bs->x.tq[b] = (0.0 - g * w) + tq;
            } else {
                bs->b.v.frc[b] = make_double2(0.0 + fx, 0.0 + fy);
                bs->x.tq[b] = 0.0 + tq;
            }
            bs->b.w.pe[b] = 0.0 + pe;
            body_kick(bs, b, dt_half);
        }
    }
    if (grid_last_block(&bs->b)) {
        if (++bs->b.s.nve_steps_done >= bs->b.s.max_steps) bs->b.s.flags |= kDone;
    }
}

// FIRE move (src/integrator/fire.cu:29-40 with the rigid overrides)
__global__ void kb_fire_move(BumpySys *bs) {
    DevSys *ds = &bs->b;
    if (halted(ds)) return;
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    const double dt = ds->s.f_dt, alpha = ds->s.f_alpha;
    const int up = ds->s.fire_uphill;
    double v[2] = {0.0, 0.0};
    if (b < ds->p.n) {
        if (up) {
            double t0, t1;
            body_move(bs, b, lane, -dt / 2.0, t0, t1);
            __syncwarp();
            if (lane == 0) {
                ds->v.vel[b] = make_double2(0.0, 0.0);
                bs->x.w[b] = 0.0;
            }
        }
        __syncwarp();
        if (lane == 0) {
            body_kick(bs, b, dt / 2.0);
            body_mix(bs, b, alpha);
        }
        __syncwarp();
        body_move(bs, b, lane, dt, v[0], v[1]);
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

// FIRE force phase (see k_fire_force for the modes); the stop test uses
// max|F_b| <= fmax_target and max|tau_b| <= tmax_target.
__global__ void kb_fire_force(BumpySys *bs, int mode, double tmax_target) {
    DevSys *ds = &bs->b;
    if (halted(ds)) return;
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    if (b < ds->p.n) {
        double fx, fy, tq, pe;
        body_forces(bs, b, lane, false, fx, fy, tq, pe);
        if (lane == 0) {
            double2 f = make_double2(0.0 + fx, 0.0 + fy);
            ds->v.frc[b] = f;
            bs->x.tq[b] = 0.0 + tq;
            ds->w.pe[b] = 0.0 + pe;
            if (mode != 1) body_kick(bs, b, ds->s.f_dt / 2.0);
            double2 u = ds->v.vel[b];
            double w = bs->x.w[b], t = bs->x.tq[b];
            v[0] = 0.0 + pe;
            v[1] = f.x * u.x + f.y * u.y + t * w;
            v[2] = f.x * f.x + f.y * f.y;
            v[3] = t * t;
        }
    }
    const int ops[4] = {0, 0, 1, 1};
    if (!grid_reduce<4>(v, ops, ds)) return;
    DevState &s = ds->s;
    s.pe = v[0];
    s.power = v[1];
    s.fmax2 = v[2];
    bs->x.tmax2 = v[3];
    double avg = v[0] / s.dof;
    if (mode == 1) {
        s.last_avg_pe = avg;
        fire_decide(ds, v[1]);
        return;
    }
    if (mode == 2) return;
    double diff = fabs(avg / s.last_avg_pe - 1);
    s.last_avg_pe = avg;
    long long it = s.iter;
    // mixed form: FP32 vertex pairs until the switch (as k_fire_force), then FP64
    bool fp64 = true;
    if (bs->x.mixed && !s.fp64_now) {
        double g2 = fmax(v[2], v[3]);
        if (g2 < 0.81 * s.best_f2) { s.best_f2 = g2; s.best_it = it; }
        const double gm = sqrt(g2);
        if (gm <= s.switch_fmax || s.f_nbad > 5 || (gm < 100.0 * s.switch_fmax && it - s.best_it > 2000))
            s.fp64_now = 1;
        fp64 = false;
    }
    if ((fp64 && diff < s.pe_diff_target) || avg < s.pe_target) {
        s.result_step = it; s.f_converged = 1; s.flags |= kDone; return;
    }
    if (fp64 && s.fmax_target > 0 && sqrt(v[2]) <= s.fmax_target && sqrt(v[3]) <= tmax_target) {
        s.result_step = it; s.f_converged = 1; s.flags |= kDone; return;
    }
    if (it + 1 >= s.max_steps) { s.result_step = s.max_steps; s.flags |= kDone; return; }
    s.iter = it + 1;
    fire_decide(ds, v[1]);
    if (s.f_stopped) { s.result_step = it + 1; s.f_converged = 1; s.flags |= kDone; }
}

// FIRE power incl. rotation, then the Fire::step decision (single-step API)
__global__ void kb_fire_power_decide(BumpySys *bs) {
    DevSys *ds = &bs->b;
    if (halted(ds)) return;
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    double v[1] = {0.0};
    if (b < ds->p.n) {
        double2 u = ds->v.vel[b], f = ds->v.frc[b];
        v[0] = f.x * u.x + f.y * u.y + bs->x.tq[b] * bs->x.w[b];
    }
    const int ops[1] = {0};
    if (grid_reduce<1>(v, ops, ds)) {
        ds->s.power = v[0];
        fire_decide(ds, v[0]);
    }
}

// ---- initialisation and transfers -------------------------------------------

// kernelInitializeVerticesOnParticles (kernels.cu:1137-1162), warp per body
__global__ void kb_init_vertices(BumpySys *bs) {
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (b >= bs->b.p.n) return;
    BumpyExt &x = bs->x;
    double2 c = bs->b.v.pos[b];
    double ang = x.th[b], r = bs->b.v.rad[b];
    int nvb = x.nvb[b], f = x.start[b];
    double inc = 2 * 3.14159265358979323846 / nvb;
    double ir = r - x.rv;
    for (int i = lane; i < nvb; i += 32) {
        double a = i * inc + ang;
        x.vpos[f + i] = make_double2(c.x + ir * cos(a), c.y + ir * sin(a));
    }
}

// vertex -> body index and block starts from the counts (host-computed starts)
__global__ void kb_index_vertices(BumpySys *bs) {
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (b >= bs->b.p.n) return;
    BumpyExt &x = bs->x;
    int f = x.start[b], n = x.nvb[b];
    for (int k = lane; k < n; k += 32) {
        x.vbody[f + k] = b;
        x.svidx[f + k] = f + k;
    }
}

// RigidBumpy::setMass: vertex masses m/nv and I = sum m_v |v - c|^2
// (rigid_bumpy.cu:1068-1080, kernels.cu:1164-1189), warp per body
__global__ void kb_set_mass(BumpySys *bs, double mass) {
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (b >= bs->b.p.n) return;
    BumpyExt &x = bs->x;
    int f = x.start[b], n = x.nvb[b];
    double2 c = bs->b.v.pos[b];
    if (lane == 0) bs->b.v.mass[b] = mass;
    double mv = mass / (double)n;
    for (int k = lane; k < n; k += 32) x.vmass[f + k] = mv;
    double acc = 0.0;
    for (int base = 0; base < n; base += 32) {
        int k = base + lane;
        double term = 0.0;
        if (k < n) {
            double2 q = x.vpos[f + k];
            double rx = q.x - c.x, ry = q.y - c.y;
            term = mv * (rx * rx + ry * ry);
        }
        int lim = min(32, n - base);
        for (int l = 0; l < lim; l++) acc += __shfl_sync(0xffffffffu, term, l);
    }
    if (lane == 0) x.I[b] = acc;
}

// radii, masses, vertex counts and vertex masses in static (vertex) order
__global__ void kb_get_static(BumpySys *bs, double *rad, double *mass, int *nvb, double *vmass) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < bs->b.p.n) {
        const int k = bs->b.v.sidx[i];
        if (rad) rad[k] = bs->b.v.rad[i];
        if (mass) mass[k] = bs->b.v.mass[i];
        if (nvb) nvb[k] = bs->x.nvb[i];
    }
    if (vmass && i < bs->x.nv) vmass[bs->x.svidx[i]] = bs->x.vmass[i];
}

// body masses, moments of inertia and vertex masses from static-order arrays
// (the values a state directory holds, as loadDataFromPath sets them)
__global__ void kb_put_mass(BumpySys *bs, const double *mass, const double *inertia,
                            const double *vmass) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < bs->b.p.n) {
        const int k = bs->b.v.sidx[i];
        bs->b.v.mass[i] = mass[k];
        bs->x.I[i] = inertia[k];
    }
    if (i < bs->x.nv) bs->x.vmass[i] = vmass[bs->x.svidx[i]];
}

// which: 0 angle, 1 angular velocity, 2 torque ; static order in/out
__global__ void kb_put_body_scalar(BumpySys *bs, int which, const double *a) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= bs->b.p.n) return;
    int k = bs->b.v.sidx[b];
    double *dst = which == 0 ? bs->x.th : (which == 1 ? bs->x.w : bs->x.tq);
    dst[b] = a[k];
}

__global__ void kb_get_body_scalar(BumpySys *bs, int which, double *a) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= bs->b.p.n) return;
    int k = bs->b.v.sidx[b];
    const double *src = which == 0 ? bs->x.th : (which == 1 ? bs->x.w : (which == 2 ? bs->x.tq : bs->x.I));
    a[k] = src[b];
}

__global__ void kb_put_vertices(BumpySys *bs, const double *px, const double *py) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= bs->x.nv) return;
    int k = bs->x.svidx[v];
    bs->x.vpos[v] = make_double2(px[k], py[k]);
}

__global__ void kb_get_vertices(BumpySys *bs, double *px, double *py) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= bs->x.nv) return;
    int k = bs->x.svidx[v];
    double2 q = bs->x.vpos[v];
    if (px) px[k] = q.x;
    if (py) py[k] = q.y;
}

__global__ void kb_get_vnbrs(BumpySys *bs, int *list, int *counts, int cap_out) {
    int v = blockIdx.x * blockDim.x + threadIdx.x;
    const int nv = bs->x.nv;
    if (v >= nv) return;
    const int *svidx = bs->x.svidx;
    int k = svidx[v];
    int cnt = bs->x.vcount[v];
    counts[k] = cnt;
    int lim = min(cnt, min(cap_out, bs->x.capv));
    for (int t = 0; t < cap_out; t++)
        list[(size_t)k * cap_out + t] = t < lim ? svidx[bs->x.vnbr[(size_t)t * nv + v]] : -1;
}

// scalePositionsFull: kernelScalePositions (kernels.cu:1308-1333), warp per body
__global__ void kb_scale(BumpySys *bs, double f) {
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (b >= bs->b.p.n) return;
    double2 p = bs->b.v.pos[b];
    double nx = p.x * f, ny = p.y * f;
    __syncwarp();
    if (lane == 0) bs->b.v.pos[b] = make_double2(nx, ny);
    int s0 = bs->x.start[b], n = bs->x.nvb[b];
    for (int k = lane; k < n; k += 32) {
        double2 q = bs->x.vpos[s0 + k];
        q.x += (nx - p.x);
        q.y += (ny - p.y);
        bs->x.vpos[s0 + k] = q;
    }
}

// ---- kernelCalculateRigidDampedForces (kernels.cu:80-87) ---------------------
__global__ void kb_damp(BumpySys *bs, double g) {
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= bs->b.p.n) return;
    double2 f = bs->b.v.frc[b], u = bs->b.v.vel[b];
    f.x -= g * u.x;
    f.y -= g * u.y;
    bs->b.v.frc[b] = f;
    bs->x.tq[b] -= g * bs->x.w[b];
}

// ---- calculateWallForces_onlyWallContacts (rigid_bumpy.cu:1495-1499): the wall
// terms of every vertex (kernelCalcRigidBumpyWallForces, kernels.cu:348-362)
// summed per body in vertex order (kernelCalcRigidBumpyParticleForces1), += into
// the body arrays; one warp per body
__global__ void kb_wall_only(BumpySys *bs) {
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    if (b >= bs->b.p.n) return;
    const DevSys &d = bs->b;
    const BumpyExt &x = bs->x;
    const double2 c = d.v.pos[b];
    const int f = x.start[b], nvb = x.nvb[b];
    double bfx = 0.0, bfy = 0.0, btq = 0.0, bpe = 0.0;
    for (int base = 0; base < nvb; base += 32) {
        int k = base + lane;
        double vfx = 0.0, vfy = 0.0, vtq = 0.0, vpe = 0.0;
        if (k < nvb) {
            const double2 q = x.vpos[f + k];
            double wx, wy;
            const double we = wall_force(d.p, q, x.rv, wx, wy);
            vfx = 0.0 + wx;
            vfy = 0.0 + wy;
            vtq = 0.0 + torque_of(wx, wy, q.x, q.y, c.x, c.y);
            vpe = 0.0 + we;
        }
        int lim = min(32, nvb - base);
        for (int l = 0; l < lim; l++) {
            bfx += __shfl_sync(0xffffffffu, vfx, l);
            bfy += __shfl_sync(0xffffffffu, vfy, l);
            btq += __shfl_sync(0xffffffffu, vtq, l);
            bpe += __shfl_sync(0xffffffffu, vpe, l);
        }
    }
    if (lane == 0) {
        double2 g = bs->b.v.frc[b];
        g.x += bfx;
        g.y += bfy;
        bs->b.v.frc[b] = g;
        bs->x.tq[b] += btq;
        bs->b.w.pe[b] += bpe;
    }
}

// ---- RigidBumpy::updatePositionsAdam: kernelRigidBumpyAdamStep then
// kernelTranslateAndRotateVertices1 (rigid_bumpy.cu:1473-1486, kernels.cu:1004-1093,
// 152-201), one warp per body.  The translational moments live in DevView (m1,
// m2: swapped with their twins on a re-sort, never gathered), the angular ones
// stay with the slot.  With rotation off the angle is left alone and the
// vertices turn by the slot's last angle increment, as the reference's stale
// angle_delta does (0 after any kick, which zeroes omega without rotation).
__global__ void kb_adam(BumpySys *bs, double alpha, double b1, double b2, double c1, double c2,
                        double eps) {
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    double v[2] = {0.0, 0.0};
    if (b < bs->b.p.n) {
        DevSys &d = bs->b;
        BumpyExt &x = bs->x;
        const double2 f = d.v.frc[b], p = d.v.pos[b];
        double2 m1 = d.v.m1[b], m2 = d.v.m2[b];
        const double t = x.tq[b], ang = x.th[b], adel = x.adelta[b];
        double m1a = x.m1a[b], m2a = x.m2a[b];
        m1.x = fma(b1, m1.x, (b1 - 1) * f.x);
        m1.y = fma(b1, m1.y, (b1 - 1) * f.y);
        m1a = fma(b1, m1a, (b1 - 1) * t);
        m2.x = fma(b2, m2.x, (1 - b2) * f.x * f.x);
        m2.y = fma(b2, m2.y, (1 - b2) * f.y * f.y);
        m2a = fma(b2, m2a, (1 - b2) * t * t);
        const double ux = -alpha * (m1.x / c1) / (sqrt(m2.x / c2) + eps);
        const double uy = -alpha * (m1.y / c1) / (sqrt(m2.y / c2) + eps);
        const double ua = -alpha * (m1a / c1) / (sqrt(m2a / c2) + eps);
        const double nx = p.x + ux, ny = p.y + uy;
        const double dth = x.rotation ? ua : adel;
        __syncwarp();
        if (lane == 0) {
            d.v.pos[b] = make_double2(nx, ny);
            if (x.rotation) {
                x.th[b] = ang + ua;
                x.adelta[b] = ua;
            }
            d.v.m1[b] = m1;
            d.v.m2[b] = m2;
            x.m1a[b] = m1a;
            x.m2a[b] = m2a;
            const double2 a = d.w.pos_n[b], c = d.w.pos_c[b];
            const double a1 = nx - a.x, a2 = ny - a.y, e1 = nx - c.x, e2 = ny - c.y;
            v[0] = a1 * a1 + a2 * a2;
            v[1] = e1 * e1 + e2 * e2;
        }
        const double ca = cos(dth), sa = sin(dth);
        const int f0 = x.start[b], nvb = x.nvb[b];
        for (int k = lane; k < nvb; k += 32) {
            const double2 q = x.vpos[f0 + k];
            const double rx = q.x - p.x, ry = q.y - p.y;
            const double rxr = rx * ca - ry * sa, ryr = rx * sa + ry * ca;
            const double2 nq = make_double2(nx + rxr, ny + ryr);
            x.vpos[f0 + k] = nq;
            if (x.mixed) x.vpk[f0 + k] = mixed_pack(d.p, nq, x.rv);
        }
    }
    const int ops[2] = {1, 1};
    if (grid_reduce<2>(v, ops, &bs->b)) { bs->b.s.max_nd2 = v[0]; bs->b.s.max_cd2 = v[1]; }
}

// ---- rigid gradient descent (no reference kernel: the reference's GradDesc on
// rigid bodies runs the disk kernelGradDescStep, src/particles/base/kernels.cu:
// 613-637, on the body centres only).  x += alpha F as that kernel, theta +=
// alpha tau with rotation, vertices translated and rotated with the body as in
// kernelTranslateAndRotateVertices1; one warp per body.
__global__ void kb_grad_desc(BumpySys *bs, double alpha) {
    const int lane = threadIdx.x & 31;
    const int b = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5);
    double v[2] = {0.0, 0.0};
    if (b < bs->b.p.n) {
        DevSys &d = bs->b;
        BumpyExt &x = bs->x;
        const double2 f = d.v.frc[b], p = d.v.pos[b];
        const double ang = x.th[b];
        const double nx = p.x + alpha * f.x, ny = p.y + alpha * f.y;
        const double dth = x.rotation ? alpha * x.tq[b] : 0.0;
        __syncwarp();
        if (lane == 0) {
            d.v.pos[b] = make_double2(nx, ny);
            if (x.rotation) x.th[b] = ang + dth;
            const double2 a = d.w.pos_n[b], c = d.w.pos_c[b];
            const double a1 = nx - a.x, a2 = ny - a.y, e1 = nx - c.x, e2 = ny - c.y;
            v[0] = a1 * a1 + a2 * a2;
            v[1] = e1 * e1 + e2 * e2;
        }
        const double ca = cos(dth), sa = sin(dth);
        const int f0 = x.start[b], nvb = x.nvb[b];
        for (int k = lane; k < nvb; k += 32) {
            const double2 q = x.vpos[f0 + k];
            const double rx = q.x - p.x, ry = q.y - p.y;
            const double2 nq = make_double2(nx + (rx * ca - ry * sa), ny + (rx * sa + ry * ca));
            x.vpos[f0 + k] = nq;
            if (x.mixed) x.vpk[f0 + k] = mixed_pack(d.p, nq, x.rv);
        }
    }
    const int ops[2] = {1, 1};
    if (grid_reduce<2>(v, ops, &bs->b)) { bs->b.s.max_nd2 = v[0]; bs->b.s.max_cd2 = v[1]; }
}

// ---- kernelCalcRigidBumpyStressTensor (kernels.cu:705-789): one thread per
// body in the reference's accumulation order (per vertex: the kinetic term with
// omega x r through atan2 / sin / cos when omega != 0, then half the virial of
// each listed vertex of another body), divided by the box area.  Per-body
// values go to stress_b, the component sums to DevState.stress.
__global__ void kb_stress(BumpySys *bs) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    double v[4] = {0.0, 0.0, 0.0, 0.0};
    const DevSys &d = bs->b;
    const BumpyExt &x = bs->x;
    const int nb = d.p.n;
    if (b < nb) {
        const int nv = x.nv, capv = x.capv;
        const double bx = d.p.box[0], by = d.p.box[1], e_c = d.p.e_c, n_c = d.p.n_c, rv = x.rv;
        const double2 c = d.v.pos[b], u = d.v.vel[b];
        const double w = x.w[b];
        double axx = 0.0, axy = 0.0, ayx = 0.0, ayy = 0.0;
        const int f0 = x.start[b], nvb = x.nvb[b];
        for (int k = 0; k < nvb; k++) {
            const int vv = f0 + k;
            const double2 q = x.vpos[vv];
            const double mv = x.vmass[vv];
            const double rx = q.x - c.x, ry = q.y - c.y;
            const double prad = sqrt(rx * rx + ry * ry);
            double wx = u.x, wy = u.y;
            if (w != 0.0) {
                const double a = atan2(ry, rx);
                wx -= sin(a) * w * prad;
                wy += cos(a) * w * prad;
            }
            axx += mv * wx * wx;
            axy += mv * wx * wy;
            ayx += mv * wy * wx;
            ayy += mv * wy * wy;
            const int cnt = min(x.vcount[vv], capv);
            for (int t = 0; t < cnt; t++) {
                const int o = x.vnbr[(size_t)t * nv + vv];
                if (o == vv || x.vbody[o] == b) continue;
                const double2 op = x.vpos[o];
                const double dx = pbc_dist(q.x, op.x, bx), dy = pbc_dist(q.y, op.y, by);
                double fx, fy;
                disk_pair(q.x, q.y, rv, op.x, op.y, rv, bx, by, e_c, n_c, fx, fy);
                axx += dx * fx / 2;
                axy += dx * fy / 2;
                ayx += dy * fx / 2;
                ayy += dy * fy / 2;
            }
        }
        const double area = bx * by;
        v[0] = axx / area;
        v[1] = axy / area;
        v[2] = ayx / area;
        v[3] = ayy / area;
        for (int k = 0; k < 4; k++) x.stress_b[(size_t)k * nb + b] = v[k];
    }
    const int ops[4] = {0, 0, 0, 0};
    if (grid_reduce<4>(v, ops, &bs->b))
        for (int k = 0; k < 4; k++) bs->b.s.stress[k] = v[k];
}

// ---- kernelCountRigidBumpyContacts (kernels.cu:924-997): per body, the
// neighbour bodies with at least one overlapping vertex pair, and per such
// neighbour the overlapping partners of the first vertex (in body vertex
// order) that has one.  Totals (getContactCount and the vertex count) go to
// DevState.contacts and BumpyExt.vcontacts.
__global__ void kb_contacts(BumpySys *bs) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    double v[2] = {0.0, 0.0};
    const DevSys &d = bs->b;
    const BumpyExt &x = bs->x;
    const int nb = d.p.n;
    if (b < nb) {
        const int nv = x.nv, capv = x.capv;
        const double bx = d.p.box[0], by = d.p.box[1], rs = 2 * x.rv;
        const int nn = min(d.w.count[b], d.p.cap), f0 = x.start[b], nvb = x.nvb[b];
        int nc = 0, nvc = 0;
        for (int k = 0; k < nn; k++) {
            const int ob = d.v.nbr[(size_t)k * nb + b];
            if (ob == b) continue;
            bool contact = false;
            for (int i = 0; i < nvb; i++) {
                const int vv = f0 + i;
                const double2 q = x.vpos[vv];
                const int cnt = min(x.vcount[vv], capv);
                for (int t = 0; t < cnt; t++) {
                    const int o = x.vnbr[(size_t)t * nv + vv];
                    if (o == vv || x.vbody[o] != ob) continue;
                    const double2 op = x.vpos[o];
                    const double dx = pbc_dist(q.x, op.x, bx), dy = pbc_dist(q.y, op.y, by);
                    if (sqrt(dx * dx + dy * dy) < rs) {
                        if (!contact) nc++;
                        nvc++;
                        contact = true;
                    }
                }
                if (contact) break;
            }
        }
        x.ccount[b] = nc;
        x.vccount[b] = nvc;
        v[0] = (double)nc;
        v[1] = (double)nvc;
    }
    const int ops[2] = {0, 0};
    if (grid_reduce<2>(v, ops, &bs->b)) {
        bs->b.s.contacts = v[0];
        bs->x.vcontacts = v[1];
    }
}

// ---- RigidBumpy::calculateForceDistancePairs (rigid_bumpy.cu:1383-1459) with
// kernelCalcRigidBumpyForceDistancePairs (kernels.cu:482-703): one thread per
// body in the reference's order; entry [slot * cap + k] for the k-th listed
// neighbour body.  Array order: see dpg_bumpy_pair_dump in include/dpg.h.
constexpr int kBumpyPairArrays = 30;
constexpr double kPi = 3.14159265358979323846;

struct BumpyPairOut {
    double *d[kBumpyPairArrays];
    long long *this_id, *other_id, *vcount;
};

__global__ void kb_pair_fill(BumpyPairOut o, long long m) {
    long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= m) return;
    // the resizeAndFill values of calculateForceDistancePairs
#pragma unroll
    for (int k = 0; k < kBumpyPairArrays; k++) {
        const double f = (k == 0 || (k >= 3 && k <= 10)) ? -1.0 : 0.0;
        if (o.d[k]) o.d[k][q] = f;
    }
    o.this_id[q] = -1;
    o.other_id[q] = -1;
    o.vcount[q] = -1;
}

__global__ void kb_pair_dump(BumpySys *bs, BumpyPairOut o) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const DevSys &d = bs->b;
    const BumpyExt &x = bs->x;
    const int nb = d.p.n, cap = d.p.cap;
    if (b >= nb) return;
    const int nn = min(d.w.count[b], cap);
    if (nn == 0) return;
    const int nv = x.nv, capv = x.capv;
    const double bx = d.p.box[0], by = d.p.box[1], e_c = d.p.e_c, n_c = d.p.n_c, rv = x.rv;
    const double rs = rv * 2.0;
    const double2 c = d.v.pos[b];
    const double thi = x.th[b], rad = d.v.rad[b];
    const int f0 = x.start[b], nvb = x.nvb[b];
    for (int k = 0; k < nn; k++) {
        const int ob = d.v.nbr[(size_t)k * nb + b];
        if (ob == b) continue;
        const double2 oc = d.v.pos[ob];
        const double thj = x.th[ob], orad = d.v.rad[ob];
        const int of = x.start[ob], onvb = x.nvb[ob];
        double fx = 0.0, fy = 0.0, en = 0.0, vov = 0.0;
        long long vci = 0;
        double hij[9], hii[9];
#pragma unroll
        for (int e = 0; e < 9; e++) { hij[e] = 0.0; hii[e] = 0.0; }
        for (int u = 0; u < nvb; u++) {
            const int v = f0 + u;
            const double2 q = x.vpos[v];
            const double phu = (double)(u * 2) * kPi / (double)nvb;
            const double rdx = q.x - c.x, rdy = q.y - c.y;
            const double Ri = sqrt(rdx * rdx + rdy * rdy);
            bool contact = false;
            const int cnt = min(x.vcount[v], capv);
            for (int t = 0; t < cnt; t++) {
                const int w = x.vnbr[(size_t)t * nv + v];
                if (w == v || x.vbody[w] != ob) continue;
                const double2 wp = x.vpos[w];
                const int iv = w - of;
                const double phv = (double)(iv * 2) * kPi / (double)onvb;
                const double odx = wp.x - oc.x, ody = wp.y - oc.y;
                const double Rj = sqrt(odx * odx + ody * ody);
                double tfx, tfy;
                const double te = disk_pair(q.x, q.y, rv, wp.x, wp.y, rv, bx, by, e_c, n_c, tfx, tfy);
                en += te;
                fx += tfx;
                fy += tfy;
                if (te > 0.0) {
                    contact = true;
                    const double dx = pbc_dist(q.x, wp.x, bx), dy = pbc_dist(q.y, wp.y, by);
                    vov += rs - sqrt(dx * dx + dy * dy);
                    const double dist = sqrt(dx * dx + dy * dy);
                    const double tij = -e_c / rs * (1 - dist / rs);
                    const double cij = e_c / (rs * rs);
                    const double si = sin(thi + phu), ci = cos(thi + phu);
                    const double sj = sin(thj + phv), cj = cos(thj + phv);
                    for (int a = 0; a < 3; a++) {
                        for (int cc = 0; cc < 3; cc++) {
                            const double dia_x = (double)(a == 0) - Ri * si * (double)(a == 2);
                            const double dia_y = (double)(a == 1) + Ri * ci * (double)(a == 2);
                            const double djb_x = -1.0 * ((double)(cc == 0) - Rj * sj * (double)(cc == 2));
                            const double djb_y = -1.0 * ((double)(cc == 1) + Rj * cj * (double)(cc == 2));
                            const double qia = dx * dia_x + dy * dia_y;
                            const double qjb = dx * djb_x + dy * djb_y;
                            const double dqjb = (dia_x * djb_x + dia_y * djb_y) / dist;
                            hij[a * 3 + cc] += cij * qia * qjb / (dist * dist) +
                                               tij * (dqjb - qia * qjb / (dist * dist * dist));
                            const double dib_x = (double)(cc == 0) - Ri * si * (double)(cc == 2);
                            const double dib_y = (double)(cc == 1) + Ri * ci * (double)(cc == 2);
                            const double d2x = -Ri * ci * (double)(a == 2) * (double)(cc == 2);
                            const double d2y = -Ri * si * (double)(a == 2) * (double)(cc == 2);
                            const double qib = dx * dib_x + dy * dib_y;
                            const double dqib = (dia_x * dib_x + dx * d2x + dia_y * dib_y + dy * d2y) / dist;
                            hii[a * 3 + cc] += cij * qia * qib / (dist * dist) +
                                               tij * (dqib - qia * qib / (dist * dist * dist));
                        }
                    }
                }
            }
            if (contact) vci++;
        }
        const long long qi = (long long)b * cap + k;
        const double xd = pbc_dist(c.x, oc.x, bx), yd = pbc_dist(c.y, oc.y, by);
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
#pragma unroll
        for (int e = 0; e < 12; e++)
            if (o.d[e]) o.d[e][qi] = vals[e];
#pragma unroll
        for (int e = 0; e < 9; e++) {
            if (o.d[12 + e]) o.d[12 + e][qi] += hij[e];
            if (o.d[21 + e]) o.d[21 + e][qi] += hii[e];
        }
        o.this_id[qi] = d.v.sidx[b];
        o.other_id[qi] = d.v.sidx[ob];
        o.vcount[qi] = vci;
    }
}

// per-body stress components [4][nb] and contact counts in static order
__global__ void kb_get_stress_contacts(BumpySys *bs, double *stress, int *cc, int *vcc) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    const int nb = bs->b.p.n;
    if (b >= nb) return;
    const int k = bs->b.v.sidx[b];
    if (stress)
        for (int c = 0; c < 4; c++) stress[(size_t)c * nb + k] = bs->x.stress_b[(size_t)c * nb + b];
    if (cc) cc[k] = bs->x.ccount[b];
    if (vcc) vcc[k] = bs->x.vccount[b];
}

// ---- RigidBumpy::setLastState (dir 0) / revertToLastStateVariables (dir 1)
// (rigid_bumpy.cu:1144-1179 over particle.cu:956-985): slot-by-slot copies of
// the body and vertex arrays the reference keeps; moments of inertia, vertex
// masses, Adam moments and cell arrays are not part of the snapshot.
__global__ void kb_snapshot(BumpySys *bs, int dir) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    DevView &v = bs->b.v;
    DevScratch &w = bs->b.w;
    BumpyExt &x = bs->x;
    if (i < bs->b.p.n) {
        if (dir == 0) {
            w.s_pos[i] = v.pos[i]; w.s_vel[i] = v.vel[i]; w.s_frc[i] = v.frc[i];
            w.s_rad[i] = v.rad[i]; w.s_mass[i] = v.mass[i]; w.s_sidx[i] = v.sidx[i];
            x.s_w[i] = x.w[i]; x.s_th[i] = x.th[i]; x.s_tq[i] = x.tq[i];
            x.s_nvb[i] = x.nvb[i]; x.s_start[i] = x.start[i];
        } else {
            v.pos[i] = w.s_pos[i]; v.vel[i] = w.s_vel[i]; v.frc[i] = w.s_frc[i];
            v.rad[i] = w.s_rad[i]; v.mass[i] = w.s_mass[i]; v.sidx[i] = w.s_sidx[i];
            x.w[i] = x.s_w[i]; x.th[i] = x.s_th[i]; x.tq[i] = x.s_tq[i];
            x.nvb[i] = x.s_nvb[i]; x.start[i] = x.s_start[i];
        }
    }
    if (i < x.nv) {
        if (dir == 0) {
            x.s_vpos[i] = x.vpos[i]; x.s_vbody[i] = x.vbody[i]; x.s_svidx[i] = x.svidx[i];
        } else {
            x.vpos[i] = x.s_vpos[i]; x.vbody[i] = x.s_vbody[i]; x.svidx[i] = x.s_svidx[i];
        }
    }
}

}  // namespace
}  // namespace dpg
