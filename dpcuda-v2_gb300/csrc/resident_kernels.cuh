// resident_kernels.cuh -- the resident form of the batched loop: each system
// is held on one SM for a whole minimisation or jamming run.
//
// The grid form pays several kernel launches and grid-wide reductions per FIRE
// iteration (~60 us at any size), and the jamming protocol of
// scripts/runArthurJamWithFire.cpp takes millions of FIRE iterations per system
// (many minimisations near jamming run to the 1e5-step cap), so small systems
// are bound by that per-iteration floor.  Here one CTA owns one system for the
// whole launch:
//   - the particles' packed offsets (read by every neighbour, every iteration)
//     and the cell lists live in shared memory;
//   - the particles a thread owns (slot t, t + NT, ..., PPT of them) keep their
//     velocity, force and last-build offset in registers;
//   - positions are the FP64 centre of the particle's cell (fixed between list
//     builds) plus a double-word FP32 offset (hi + lo, ~48 bits, ~1e-15 absolute
//     for |offset| ~ 1): the drift x += v dt is a double-word + FP32 sum on the
//     FP32 pipe, so an FP32 or double-word iteration executes no FP64
//     instruction per particle (GB300 runs FP64 at 1/64 of the FP32 rate);
//   - FP64 positions are materialised (centre + hi + lo) only at list builds,
//     transitions between minimisations, FP64 passes and the end of a launch;
//   - FP64 pair arithmetic only measures: a double-word state whose max|F| is
//     within the target gets one FP64 force pass at unchanged positions, which
//     either certifies it or sends the system back to double words with a
//     tighter threshold, and every finished minimisation is measured by one FP64
//     pass (its reported energy, max|F|, pressure and contacts are FP64).
// Stages are separated by __syncthreads(); per-system totals are block
// reductions in a fixed order; the per-system FIRE decision, convergence tests,
// precision switch and jamming state machine are the grid form's
// (e_force_epilogue, e_finish, e_transition_sys).  A launch ends when every
// system of the launch is done, after a per-system iteration budget, after a
// time slice (%globaltimer, so concurrently resident systems hand the SMs back
// together), or when some system's neighbour list overflows the shared
// capacity; the state is written back exactly (double-word offsets included),
// so where a launch ends does not change any result.  Blocks never wait on one
// another.
//
// Size classes: a system of a class runs on a thread-block cluster of C
// blocks of NT threads, each thread owning PPT particles; block r of the
// cluster owns the particles [r M, (r + 1) M), M = NT * PPT, and holds their
// packed offsets in its shared memory.  Neighbours owned by another block of
// the cluster are read from its shared memory (distributed shared memory);
// every block keeps an identical copy of the system state and of the cell
// list, per-system totals are exchanged between the blocks and summed in
// block order, so every copy takes the same decisions (only block 0 performs
// the global side effects).  The host launches each class on its own stream
// so the classes run side by side.
#pragma once
#include <cooperative_groups.h>

#include "ensemble_kernels.cuh"

namespace dpg {
namespace {

constexpr int kResMaxN = 16384;  // largest system the resident form holds

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// double word + FP32 (Joldes, Muller & Popescu, Algorithm 4 "DWPlusFP")
__device__ __forceinline__ dw dw_add_f(dw a, float b) {
    dw s = two_sum(a.hi, b);
    const float v = __fadd_rn(a.lo, s.lo);
    return fast_two_sum(s.hi, v);
}

// exact product of two FP32 numbers as a double word (FMA)
__device__ __forceinline__ dw two_prod(float a, float b) {
    const float p = __fmul_rn(a, b);
    return {p, __fmaf_rn(a, b, -p)};
}

__device__ __forceinline__ float2 split_lo(double ox, double oy, float hx, float hy) {
    return make_float2((float)(ox - (double)hx), (float)(oy - (double)hy));
}

// shared-memory layout of one block of a resident system (dynamic shared memory)
struct RLayout {
    float4 *pk;               // [m] own particles {offset hi x, offset hi y, radius hi, cell code}
    float4 *pkl;              // [m] own particles {offset lo x, offset lo y, radius lo, 0}
    int *cstart;              // [ncmax + 1] first item of each cell (the whole system)
    int *ccur;                // [ncmax] counts, then fill cursors
    unsigned short *citem;    // [nsys] particle (system index) of each cell item
};

// m: particles per block, nsys: particles per system (C m)
__host__ __device__ inline size_t res_smem_bytes(int m, int nsys, int ncmax) {
    return (size_t)32 * m + (size_t)4 * (2 * (size_t)ncmax + 1) + (size_t)2 * nsys + 16;
}

__device__ __forceinline__ RLayout res_layout(float4 *base, int m, int ncmax) {
    RLayout L;
    L.pk = base;
    L.pkl = base + m;
    L.cstart = reinterpret_cast<int *>(base + 2 * m);
    L.ccur = L.cstart + ncmax + 1;
    L.citem = reinterpret_cast<unsigned short *>(L.ccur + ncmax);
    return L;
}

// packed offsets of particle j (system index) of a cluster of C blocks of M
// particles each: block j / M holds them
template <int C, int M>
__device__ __forceinline__ const float4 *res_pk_of(const RLayout &L, int j) {
    if constexpr (C == 1) {
        return L.pk + j;
    } else {
        const int q = j / M;
        return cooperative_groups::this_cluster().map_shared_rank(L.pk, q) + (j - q * M);
    }
}
template <int C, int M>
__device__ __forceinline__ const float4 *res_pkl_of(const RLayout &L, int j) {
    if constexpr (C == 1) {
        return L.pkl + j;
    } else {
        const int q = j / M;
        return cooperative_groups::this_cluster().map_shared_rank(L.pkl, q) + (j - q * M);
    }
}

// FP64 position of own particle lo (block-local index) from its cell centre
// and double-word offset
__device__ __forceinline__ double2 res_position(const RLayout &L, const double2 c, int lo) {
    const float4 a = L.pk[lo], b = L.pkl[lo];
    return make_double2(c.x + ((double)a.x + (double)b.x), c.y + ((double)a.y + (double)b.y));
}

// Block reduction of one double-word sum and four FP32 values (0 sum, 1 max,
// 2 sum, 3 sum) in a fixed order: warp trees, then warp results in order by
// thread 0, which gets the totals.  One barrier.
template <int NT>
__device__ __forceinline__ void res_reduce(dw &pe, float (&v)[4], dw *smw, float *smv) {
    constexpr int NW = NT / 32;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        dw o = {__shfl_down_sync(0xffffffffu, pe.hi, off), __shfl_down_sync(0xffffffffu, pe.lo, off)};
        pe = dw_add(pe, o);
        const float a0 = __shfl_down_sync(0xffffffffu, v[0], off);
        const float a1 = __shfl_down_sync(0xffffffffu, v[1], off);
        const float a2 = __shfl_down_sync(0xffffffffu, v[2], off);
        const float a3 = __shfl_down_sync(0xffffffffu, v[3], off);
        v[0] += a0;
        v[1] = fmaxf(v[1], a1);
        v[2] += a2;
        v[3] += a3;
    }
    if (lane == 0) {
        smw[wid] = pe;
#pragma unroll
        for (int k = 0; k < 4; k++) smv[wid * 4 + k] = v[k];
    }
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int w = 1; w < NW; w++) {
            pe = dw_add(pe, smw[w]);
            v[0] += smv[w * 4 + 0];
            v[1] = fmaxf(v[1], smv[w * 4 + 1]);
            v[2] += smv[w * 4 + 2];
            v[3] += smv[w * 4 + 3];
        }
    }
}

// FIRE mix with per-particle norms (src/particles/base/kernels.cu:91-112) in
// FP32 from the hardware reciprocal square root: |v| / |F| = sqrt(v2 / F2)
// (the mixing weight carries no precision requirement)
__device__ __forceinline__ float2 res_fire_mix(float2 v, float2 f, float alpha) {
    const float fn2 = f.x * f.x + f.y * f.y, vn2 = v.x * v.x + v.y * v.y;
    float mix = 0.f;
    if (fn2 > 1e-32f) {
        mix = sqrtf(vn2 * __frcp_rn(fn2)) * alpha;
    } else {
        v = make_float2(0.f, 0.f);
    }
    return make_float2(v.x * (1.f - alpha) + f.x * mix, v.y * (1.f - alpha) + f.y * mix);
}

// periodic cell difference of two packed cell codes
__device__ __forceinline__ void res_dcell(int ca, int cb, int ncd, int &dcx, int &dcy) {
    dcx = code_x(ca) - code_x(cb);
    dcy = code_y(ca) - code_y(cb);
    if (dcx > ncd / 2) dcx -= ncd; else if (dcx < -(ncd / 2)) dcx += ncd;
    if (dcy > ncd / 2) dcy -= ncd; else if (dcy < -(ncd / 2)) dcy += ncd;
}

// ---- FP32 pair terms of own particle lo (slot i) from the shared offsets -------
// (neighbour lists are written by the running launch: plain, coherent loads)
template <int C, int M, int G>
__device__ __forceinline__ void res_forces_f32(const EDev *e, const ESys &s, const RLayout &L, int lo,
                                               int i, float &ax, float &ay, float &en, float &wv,
                                               int &ncount) {
    const int T = e->p.T, cnt = min(e->cnt[i], e->p.cap), off = s.off;
    const float ecf = (float)e->p.e_c, ncf = (float)e->p.n_c;
    const float4 a = L.pk[lo];
    ax = 0.f; ay = 0.f; en = 0.f; wv = 0.f; ncount = 0;
    const int g = threadIdx.x % G;
    for (int k0 = g; k0 < cnt; k0 += 8 * G) {
        int jj[8];
#pragma unroll
        for (int u = 0; u < 8; u++) jj[u] = k0 + u * G < cnt ? e->nbr[(size_t)(k0 + u * G) * T + i] - off : 0;
#pragma unroll
        for (int u = 0; u < 8; u++) {
            if (k0 + u * G >= cnt) break;
            float fx, fy, ef, wf;
            int ct;
            pair_f32(a, *res_pk_of<C, M>(L, jj[u]), s.ncd, s.cs_f, ecf, ncf, fx, fy, ef, wf, ct);
            ax += fx;
            ay += fy;
            en += ef;
            wv += wf;
            ncount += ct;
        }
    }
}

// ---- double-word pair terms of own particle lo (full double-word path) --------
// Pairs the hi offsets rule out (a 1e-4 relative margin on the contact
// distance) are skipped; the rest run in double-word arithmetic.  The energy is
// a double word (the energy-change stop test needs it).
template <int C, int M, int G>
__device__ __forceinline__ void res_forces_dw(const EDev *e, const ESys &s, const RLayout &L, int lo,
                                              int i, dw &sx, dw &sy, dw &se, float &sw, int &ncount) {
    const int T = e->p.T, cnt = min(e->cnt[i], e->p.cap), off = s.off;
    const float4 a = L.pk[lo], al = L.pkl[lo];
    const dw xi = {a.x, al.x}, yi = {a.y, al.y}, ri = {a.z, al.z};
    const dw csd = {s.cs_f, s.cs_lo}, ec = {e->p.ec_hi, e->p.ec_lo};
    const int ca = __float_as_int(a.w), ncd = s.ncd;
    sx = {0.f, 0.f}; sy = {0.f, 0.f}; se = {0.f, 0.f}; sw = 0.f; ncount = 0;
    const int g = threadIdx.x % G;
    for (int k0 = g; k0 < cnt; k0 += 4 * G) {
        int jj[4];
#pragma unroll
        for (int u = 0; u < 4; u++) jj[u] = k0 + u * G < cnt ? e->nbr[(size_t)(k0 + u * G) * T + i] - off : 0;
#pragma unroll
        for (int u = 0; u < 4; u++) {
            if (k0 + u * G >= cnt) break;
            const float4 b = *res_pk_of<C, M>(L, jj[u]);
            int dcx, dcy;
            res_dcell(ca, __float_as_int(b.w), ncd, dcx, dcy);
            const float dxf = (a.x - b.x) + (float)dcx * s.cs_f;
            const float dyf = (a.y - b.y) + (float)dcy * s.cs_f;
            const float rsf = a.z + b.z;
            if (dxf * dxf + dyf * dyf >= rsf * rsf * 1.0001f) continue;
            const float4 bl = *res_pkl_of<C, M>(L, jj[u]);
            dw dx = dw_add(dw_add(xi, dw_neg(dw{b.x, bl.x})), dw_mul_f(csd, (float)dcx));
            dw dy = dw_add(dw_add(yi, dw_neg(dw{b.y, bl.y})), dw_mul_f(csd, (float)dcy));
            dw rs = dw_add(ri, dw{b.z, bl.z});
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
}

// ---- double-word pair terms with a shorter tail (harmonic contacts) ----------
// The overlap enters the force only through sigma^2 - d^2 = (sigma - d)(sigma + d),
// so the contact is resolved to double-word precision there (sigma^2 - d^2 of
// two double words, absolute error ~1e-14), and the rest of the harmonic force
// F = e_c (sigma^2 - d^2) / (sigma^2 d (sigma + d)) dr needs only a relative
// precision of ~1e-12, which one error-free correction of each FP32 step gives
// (d by one Newton step on the FP32 square root, the quotient by one residual
// step).  Forces are accumulated with compensated sums; the energy
// e_c / 4 ((sigma^2 - d^2) / (sigma (sigma + d)))^2 and the virial in FP32
// (relative 1e-7; the energy-change stop test uses the full double-word path).
template <int C, int M, int G>
__device__ __forceinline__ void res_forces_dwf(const EDev *e, const ESys &s, const RLayout &L, int lo,
                                               int i, dw &sx, dw &sy, float &se, float &sw,
                                               int &ncount) {
    const int T = e->p.T, cnt = min(e->cnt[i], e->p.cap), off = s.off;
    const float4 a = L.pk[lo], al = L.pkl[lo];
    const float csh = s.cs_f, csl = s.cs_lo, ech = e->p.ec_hi, ecl = e->p.ec_lo;
    const int ca = __float_as_int(a.w), ncd = s.ncd;
    float fxh = 0.f, fxl = 0.f, fyh = 0.f, fyl = 0.f;
    se = 0.f; sw = 0.f; ncount = 0;
    const int g = threadIdx.x % G;
    for (int k0 = g; k0 < cnt; k0 += 4 * G) {
        int jj[4];
#pragma unroll
        for (int u = 0; u < 4; u++) jj[u] = k0 + u * G < cnt ? e->nbr[(size_t)(k0 + u * G) * T + i] - off : 0;
#pragma unroll
        for (int u = 0; u < 4; u++) {
            if (k0 + u * G >= cnt) break;
            const float4 b = *res_pk_of<C, M>(L, jj[u]);
            int dcx, dcy;
            res_dcell(ca, __float_as_int(b.w), ncd, dcx, dcy);
            const float cx = (float)dcx, cy = (float)dcy;
            const float dxf = (a.x - b.x) + cx * csh;
            const float dyf = (a.y - b.y) + cy * csh;
            const float rsf = a.z + b.z;
            if (dxf * dxf + dyf * dyf >= rsf * rsf * 1.0001f) continue;
            const float4 bl = *res_pkl_of<C, M>(L, jj[u]);
            // displacement as double words
            const dw tx = two_sum(a.x, -b.x), px = two_prod(cx, csh), ux = two_sum(tx.hi, px.hi);
            const dw dx = two_sum(ux.hi, tx.lo + px.lo + ux.lo + (al.x - bl.x) + cx * csl);
            const dw ty = two_sum(a.y, -b.y), py = two_prod(cy, csh), uy = two_sum(ty.hi, py.hi);
            const dw dy = two_sum(uy.hi, ty.lo + py.lo + uy.lo + (al.y - bl.y) + cy * csl);
            // d^2 and sigma^2
            const dw p1 = two_prod(dx.hi, dx.hi), p2 = two_prod(dy.hi, dy.hi), q = two_sum(p1.hi, p2.hi);
            const dw d2 = fast_two_sum(q.hi, q.lo + p1.lo + p2.lo + 2.f * (dx.hi * dx.lo + dy.hi * dy.lo));
            dw sg = two_sum(a.z, b.z);
            sg = fast_two_sum(sg.hi, sg.lo + al.z + bl.z);
            dw s2 = two_prod(sg.hi, sg.hi);
            s2 = fast_two_sum(s2.hi, s2.lo + 2.f * sg.hi * sg.lo);
            if (dw_ge(d2, s2)) continue;
            // sigma^2 - d^2
            const dw dt = two_sum(s2.hi, -d2.hi);
            const dw del = two_sum(dt.hi, dt.lo + (s2.lo - d2.lo));
            // d by one Newton step on the FP32 square root
            const float dh = __fsqrt_rn(d2.hi);
            const float rr = __fmaf_rn(-dh, dh, d2.hi) + d2.lo;
            const dw dd = fast_two_sum(dh, __fdividef(rr, 2.f * dh));
            // D = sigma^2 d (sigma + d), numerator e_c (sigma^2 - d^2)
            dw S = two_sum(sg.hi, dd.hi);
            S = fast_two_sum(S.hi, S.lo + sg.lo + dd.lo);
            const dw D = dw_mul(dw_mul(s2, dd), S);
            const dw num = dw_mul(dw{ech, ecl}, del);
            // fm = num / D with one residual step
            const float inv = __frcp_rn(D.hi);
            const float q0 = __fmul_rn(num.hi, inv);
            const dw pq = two_prod(q0, D.hi);
            const float rsd = ((num.hi - pq.hi) - pq.lo + num.lo) - q0 * D.lo;
            const float q1 = __fmul_rn(rsd, inv);
            // F = fm dr, compensated accumulation
            const float gx = __fmul_rn(q0, dx.hi), gy = __fmul_rn(q0, dy.hi);
            const float gxl = __fmaf_rn(q0, dx.hi, -gx) + q1 * dx.hi + q0 * dx.lo;
            const float gyl = __fmaf_rn(q0, dy.hi, -gy) + q1 * dy.hi + q0 * dy.lo;
            const dw ax = two_sum(fxh, gx), ay = two_sum(fyh, gy);
            fxh = ax.hi;
            fxl += ax.lo + gxl;
            fyh = ay.hi;
            fyl += ay.lo + gyl;
            const float ov = __fdividef(del.hi, sg.hi * S.hi);
            se += 0.25f * ech * ov * ov;
            sw += gx * dx.hi + gy * dy.hi;
            ncount++;
        }
    }
    sx = two_sum(fxh, fxl);
    sy = two_sum(fyh, fyl);
}

// ---- FP64 pair terms of own particle lo (the reference arithmetic on FP64
// positions; 1/d and 1/rs by Newton steps as in the grid form).  Neighbour
// positions may have been written by another block of the cluster: L2 loads.
template <int C, int M, int G>
__device__ __forceinline__ void res_forces_f64(const EDev *e, const ESys &s, const RLayout &L, int lo,
                                               int i, double &ax, double &ay, double &en, double &wv,
                                               double &nc) {
    const EParams &p = e->p;
    const int T = p.T, cnt = min(e->cnt[i], p.cap), off = s.off, ncd = s.ncd;
    const float4 a = L.pk[lo];
    const double2 xi = e->pos[i];
    const double ri = e->rad[i];
    ax = 0.0; ay = 0.0; en = 0.0; wv = 0.0; nc = 0.0;
    for (int k = threadIdx.x % G; k < cnt; k += G) {
        const int j = e->nbr[(size_t)k * T + i];
        if (ncd >= 3) {
            const float4 b = *res_pk_of<C, M>(L, j - off);
            int dcx, dcy;
            res_dcell(__float_as_int(a.w), __float_as_int(b.w), ncd, dcx, dcy);
            const float dxf = (a.x - b.x) + (float)dcx * s.cs_f;
            const float dyf = (a.y - b.y) + (float)dcy * s.cs_f;
            const float rsf = a.z + b.z;
            if (dxf * dxf + dyf * dyf >= rsf * rsf * 1.0001f) continue;
        }
        const double2 xj = __ldcg(&e->pos[j]);
        const double dx = pbc_dist(xi.x, xj.x, s.L), dy = pbc_dist(xi.y, xj.y, s.L);
        const double rs = ri + e->rad[j];
        const double d2 = dx * dx + dy * dy;
        if (d2 >= rs * rs) continue;
        const double id = rsqrt_newton(d2), irs = rcp_newton(rs);
        const double d = d2 * id;
        const double ov = 1.0 - d * irs;
        const double ovp = p.n_c == 2.0 ? ov : pow(ov, p.n_c - 1);
        const double fm = p.e_c * ovp * irs * id;
        const double fx = fm * dx, fy = fm * dy;
        ax += fx;
        ay += fy;
        en += p.e_c * ov * ovp / (2.0 * p.n_c);
        wv += fx * dx + fy * dy;
        nc += 1.0;
    }
}

// ---- neighbour list of own particle lo (system index l, slot i) ---------------
template <int C, int M>
__device__ __forceinline__ int res_nlist(EDev *e, const ESys &s, const RLayout &L, int lo, int l, int i) {
    const int T = e->p.T, cap = e->p.cap, ncd = s.ncd, off = s.off;
    int cnt = 0;
    if (ncd >= 3 && s.cs * s.cs >= e->p.cutoff2) {
        const float4 a = L.pk[lo];
        const int c = __float_as_int(a.w), cx = code_x(c), cy = code_y(c);
        // FP32 distances with a 1e-4 relative margin: a superset of the list
        const float c2f = e->p.cutoff2_f * 1.0001f, cs = s.cs_f;
        for (int oy = -1; oy <= 1; oy++) {
            const int yy = pmod(cy + oy, ncd);
            for (int ox = -1; ox <= 1; ox++) {
                const int g = pmod(cx + ox, ncd) + yy * ncd;
                const float sx = (float)ox * cs, sy = (float)oy * cs;
                const int b0 = L.cstart[g], b1 = L.cstart[g + 1];
                for (int k = b0; k < b1; k++) {
                    const int j = L.citem[k];
                    if (j == l) continue;
                    const float4 b = *res_pk_of<C, M>(L, j);
                    const float dx = (a.x - b.x) - sx, dy = (a.y - b.y) - sy;
                    if (dx * dx + dy * dy < c2f) {
                        if (cnt < cap) e->nbr[(size_t)cnt * T + i] = off + j;
                        cnt++;
                    }
                }
            }
        }
    } else {  // grid too coarse for a 3x3 stencil: all pairs of the system (FP64)
        const double2 xi = e->pos[i];
        const double c2 = e->p.cutoff2;
        for (int j = off; j < off + s.n; j++) {
            if (j == i) continue;
            const double2 xj = __ldcg(&e->pos[j]);
            const double dx = pbc_dist(xi.x, xj.x, s.L), dy = pbc_dist(xi.y, xj.y, s.L);
            if (dx * dx + dy * dy < c2) {
                if (cnt < cap) e->nbr[(size_t)cnt * T + i] = j;
                cnt++;
            }
        }
    }
    e->cnt[i] = cnt;
    return cnt;
}

// Exclusive scan of the shared cell counts (nc cells) into cstart; clears ccur.
template <int NT>
__device__ __forceinline__ void res_scan(const RLayout &L, int nc, int *wsum, int *carry_s) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    constexpr int NW = NT / 32;
    int carry = 0;
    for (int base = 0; base < nc; base += NT) {
        const int idx = base + threadIdx.x;
        const int a = idx < nc ? L.ccur[idx] : 0;
        int incl = a;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        if (lane == 31) wsum[wid] = incl;
        __syncthreads();
        if (wid == 0) {
            const int w = lane < NW ? wsum[lane] : 0;
            int wi = w;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) wi += y;
            }
            if (lane < NW) wsum[lane] = wi - w;
            if (lane == 31) *carry_s = wi;
        }
        __syncthreads();
        if (idx < nc) {
            L.cstart[idx] = carry + wsum[wid] + incl - a;
            L.ccur[idx] = 0;
        }
        carry += *carry_s;
        __syncthreads();
    }
    if (threadIdx.x == 0) L.cstart[nc] = carry;
}

// Epilogue of an FP64 pass at unchanged positions (thread 0): a finished
// minimisation (kind 2) or a double-word state whose FP64 max|F| is within the
// target finishes with these FP64 totals; otherwise the double-word loop goes
// on with its exit threshold halved.  FIRE's state is not touched: the pass is
// a measurement, not an iteration.
__device__ void res_verify_epilogue(EDev *e, ESys &s, const double (&v)[5], int kind, bool primary) {
    const EParams &p = e->p;
    s.verify = 0;
    s.fire_total++;
    s.fp64_total++;
    const double avg = v[0] * s.inv_n;
    const double pe_t = (p.jam && s.jam_stage == 0) ? 1e-16 : p.pe_target;
    if (kind == 2 || avg < pe_t || (p.fmax_target > 0 && v[2] <= p.fmax_cert2)) {
        s.pe = v[0];
        s.power = v[1];
        s.fmax2 = v[2];
        s.virial = v[3];
        s.contacts = v[4];
        e_finish(e, s, primary);
    } else {
        s.dw_scale *= 0.5;
    }
}

// per-block totals exchanged between the blocks of a cluster
struct RPart {
    dw pe;
    float v[4];
    int req;          // block 0: leave the loop after this iteration (time slice, overflow)
};
struct RPartD {
    double v[5];
    int req;
};

struct RCtl {
    int stop;         // leave the loop (uniform decision)
    int req;          // block 0's request, seen by every block after an exchange
    int wsum[32];
    int carry;
    int imax[32];
    int rb_in[8];     // rebuild requests of the cluster's blocks
    int mx_in[8];     // longest neighbour list of each block
    RPart part_in[8];
    RPartD partd_in[8];
};

// cluster-wide barrier (release / acquire; a block barrier for one block)
template <int C>
__device__ __forceinline__ void res_csync() {
    if constexpr (C == 1) __syncthreads();
    else cooperative_groups::this_cluster().sync();
}

// thread 0 writes x into slot r of field f of every block of the cluster
template <int C, typename Tv>
__device__ __forceinline__ void res_bcast(Tv *field, int r, const Tv &x) {
    if constexpr (C == 1) {
        field[r] = x;
    } else {
        auto cl = cooperative_groups::this_cluster();
#pragma unroll
        for (int q = 0; q < C; q++) cl.map_shared_rank(field, q)[r] = x;
    }
}

// sum over the G lanes of a particle (xor butterfly; every lane gets the same
// bits: TwoSum-based double-word addition is commutative)
template <int G>
__device__ __forceinline__ dw lanes_dw(dw a) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
        const dw b = {__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
        a = dw_add(a, b);
    }
    return a;
}
template <int G, typename Tv>
__device__ __forceinline__ Tv lanes_sum(Tv a) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
    return a;
}

// The resident kernel: one system per cluster of C blocks (C = 1: one block).
// Thread t is lane t % G of particle group t / G; a group owns particles
// q, q + NT / G, ... (PPT of them) and its G lanes share each particle's
// neighbour loop (slots g, g + G, ...), the lane sums meeting by shuffles; the
// group's lane 0 keeps the particle's velocity, force and last-build offset in
// registers and does the per-particle work of the move and the list build.
// sys_of_cluster[b]: the system of cluster b (one class); ncmax (cells) sizes
// the dynamic shared memory; iter_budget: most iterations per system in this
// launch; slice_ns: the launch's time slice (0 = none).
template <int NT, int PPT, int C, int G>
__global__ void __launch_bounds__(NT) e_res(EDev *e, const int *sys_of_cluster, int ncmax,
                                          long long iter_budget, unsigned long long slice_ns) {
    extern __shared__ float4 res_smem[];
    __shared__ ESys s;
    __shared__ RCtl ctl;
    __shared__ dw smw[NT / 32];
    __shared__ float smv[NT / 32 * 4];
    __shared__ double smd[32 * 5];
    constexpr int NG = NT / G;     // particle groups per block
    constexpr int M = NG * PPT;    // particles per block
    const RLayout L = res_layout(res_smem, M, ncmax);
    const int t = threadIdx.x, q = t / G;
    const bool lead = (t % G) == 0;
    const int r = C == 1 ? 0 : (int)cooperative_groups::this_cluster().block_rank();
    const bool primary = r == 0;
    const int sid = sys_of_cluster[blockIdx.x / C];
    unsigned long long t_end = 0;
    if (t == 0) {
        s = e->sys[sid];
        ctl.req = 0;
        t_end = slice_ns ? global_ns() + slice_ns : 0ull;
    }
    __syncthreads();
    const EParams &p = e->p;
    const int n = s.n, off = s.off, base = r * M;

    // ---- load own particles (lead lanes): offsets (exact double words, or split
    // from the FP64 positions), velocity, force, last-build offsets
    float2 u[PPT], fr[PPT], frl[PPT], orf[PPT];
    float im[PPT];
#pragma unroll
    for (int k = 0; k < PPT; k++) {
        const int lo = q + k * NG, l = base + lo;
        u[k] = make_float2(0.f, 0.f); fr[k] = u[k]; frl[k] = u[k]; orf[k] = u[k]; im[k] = 1.f;
        if (!lead || l >= n) continue;
        const int i = off + l;
        if (s.res_valid) {
            L.pk[lo] = e->pk[i];
            L.pkl[lo] = e->pkl[i];
        } else {
            const double2 x = e->pos[i], c = e->ctr[i];
            const double rad = e->rad[i];
            const double ox = x.x - c.x, oy = x.y - c.y;
            const float hx = (float)ox, hy = (float)oy, hr = (float)rad;
            L.pk[lo] = make_float4(hx, hy, hr, __int_as_float(e->cellc[i]));
            const float2 lw = split_lo(ox, oy, hx, hy);
            L.pkl[lo] = make_float4(lw.x, lw.y, (float)(rad - (double)hr), 0.f);
        }
        u[k] = e->vel32[i];
        fr[k] = e->frc32[i];
        orf[k] = e->oref[i];
        im[k] = e->invm[i];
    }
    res_csync<C>();

    // e->pos lags the offsets (an FP32 / double-word move since the last
    // materialisation); every thread tracks it identically
    bool pstale = false;
    long long it = 0;
    const float half_skin2_f = (float)p.half_skin2;
    // Uniform loop exit, decided by thread 0 after each epilogue (before the
    // barrier that publishes the epilogue) from the state every block shares:
    // the system is done, the budget is spent, or block 0 asked to leave (its
    // request travels with the exchanged totals; one block checks the time
    // slice and the overflow flag itself, every 32 iterations).
    auto decide_stop = [&](long long next_it) {
        int st = (s.phase == kIdle) || (next_it >= iter_budget) || ctl.req;
        if (C == 1 && !st && (next_it & 31) == 0) {
            if (*(volatile int *)&e->overflow) st = 1;
            else if (t_end && global_ns() > t_end) st = 1;
        }
        ctl.stop = st;
    };
    if (t == 0) decide_stop(0);
    __syncthreads();
    for (;;) {
        if (ctl.stop) break;
        // block 0's request to leave after this iteration (multi-block clusters)
        int req = 0;
        if (C > 1 && primary && t == 0 && (it & 31) == 31)
            req = (*(volatile int *)&e->overflow) || (t_end && global_ns() > t_end);

        if (s.verify) {
            // ---- FP64 pass at the current positions (no move, no kick)
            const int kind = s.verify;
#pragma unroll
            for (int k = 0; k < PPT; k++) {
                const int lo = q + k * NG, l = base + lo;
                if (!pstale || !lead || l >= n) break;
                const int i = off + l;
                e->pos[i] = res_position(L, e->ctr[i], lo);
            }
            pstale = false;
            if (C > 1) __threadfence();
            res_csync<C>();
            double a[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
            for (int k = 0; k < PPT; k++) {
                const int lo = q + k * NG, l = base + lo;
                const bool live = l < n;
                const int i = off + (live ? l : 0);
                double ax = 0, ay = 0, en = 0, wv = 0, nc = 0;
                if (live) res_forces_f64<C, M, G>(e, s, L, lo, i, ax, ay, en, wv, nc);
                ax = lanes_sum<G>(ax); ay = lanes_sum<G>(ay); en = lanes_sum<G>(en);
                wv = lanes_sum<G>(wv); nc = lanes_sum<G>(nc);
                if (!lead || !live) continue;
                e->frc[i] = make_double2(ax, ay);
                fr[k] = make_float2((float)ax, (float)ay);
                frl[k] = make_float2((float)(ax - (double)fr[k].x), (float)(ay - (double)fr[k].y));
                a[0] += en;
                a[1] += ax * (double)u[k].x + ay * (double)u[k].y;
                a[2] = fmax(a[2], ax * ax + ay * ay);
                a[3] += wv;
                a[4] += nc;
            }
            const int ops[5] = {0, 0, 1, 0, 0};
            block_reduce<5, double>(a, ops, smd);
            if (t == 0) {
                RPartD pd;
#pragma unroll
                for (int b = 0; b < 5; b++) pd.v[b] = a[b];
                pd.req = req;
                res_bcast<C>(ctl.partd_in, r, pd);
            }
            res_csync<C>();
            if (t == 0) {
                double tot[5];
#pragma unroll
                for (int b = 0; b < 5; b++) tot[b] = ctl.partd_in[0].v[b];
                for (int b = 1; b < C; b++) {
                    tot[0] += ctl.partd_in[b].v[0];
                    tot[1] += ctl.partd_in[b].v[1];
                    tot[2] = fmax(tot[2], ctl.partd_in[b].v[2]);
                    tot[3] += ctl.partd_in[b].v[3];
                    tot[4] += ctl.partd_in[b].v[4];
                }
                ctl.req = ctl.partd_in[0].req;
                res_verify_epilogue(e, s, tot, kind, primary);
                if (s.pending == kActNone) decide_stop(it + 1);
            }
            __syncthreads();
        } else {
            // ---- move (src/integrator/fire.cu:29-40), lead lanes
            int moved_rb = 0;
            if (!s.resume && s.phase == kMinimize) {
                int need = 0;
                if (s.prec != 1) {
                    const float dt = (float)s.dt, alpha = (float)s.alpha;
                    const bool uphill = s.uphill;
#pragma unroll
                    for (int k = 0; k < PPT; k++) {
                        const int lo = q + k * NG, l = base + lo;
                        if (!lead || l >= n) break;
                        const float4 a = L.pk[lo], al = L.pkl[lo];
                        dw ox = {a.x, al.x}, oy = {a.y, al.y};
                        float2 v = u[k];
                        const float2 f = fr[k];
                        if (uphill) {
                            const float back = -0.5f * dt;
                            ox = dw_add_f(ox, v.x * back);
                            oy = dw_add_f(oy, v.y * back);
                            v = make_float2(0.f, 0.f);
                        }
                        const float h = 0.5f * dt * im[k];
                        v.x += f.x * h;
                        v.y += f.y * h;
                        v = res_fire_mix(v, f, alpha);
                        u[k] = v;
                        ox = dw_add_f(ox, v.x * dt);
                        oy = dw_add_f(oy, v.y * dt);
                        L.pk[lo] = make_float4(ox.hi, oy.hi, a.z, a.w);
                        L.pkl[lo] = make_float4(ox.lo, oy.lo, al.z, al.w);
                        const float ddx = ox.hi - orf[k].x, ddy = oy.hi - orf[k].y;
                        need |= (ddx * ddx + ddy * ddy > half_skin2_f);
                    }
                } else {
                    const double dt = s.dt, alpha = s.alpha;
                    const bool from32 = s.vel_f32, stale = pstale;
#pragma unroll
                    for (int k = 0; k < PPT; k++) {
                        const int lo = q + k * NG, l = base + lo;
                        if (!lead || l >= n) break;
                        const int i = off + l;
                        const double2 c = e->ctr[i];
                        double2 x = stale ? res_position(L, c, lo) : e->pos[i];
                        double2 v = from32 ? make_double2(u[k].x, u[k].y) : e->vel[i];
                        // the last pass was a double-word one: its force is in registers
                        const double2 f = from32 ? make_double2((double)fr[k].x + (double)frl[k].x,
                                                                (double)fr[k].y + (double)frl[k].y)
                                                 : e->frc[i];
                        if (s.uphill) {
                            const double back = -dt / 2.0;
                            x.x = x.x + v.x * back;
                            x.y = x.y + v.y * back;
                            v = make_double2(0.0, 0.0);
                        }
                        const double dtm = (0.5 * dt) * rcp_newton(e->mass[i]);
                        v.x = v.x + f.x * dtm;
                        v.y = v.y + f.y * dtm;
                        v = fire_mix_newton(v, f, alpha);
                        x.x = x.x + v.x * dt;
                        x.y = x.y + v.y * dt;
                        e->vel[i] = v;
                        e->pos[i] = x;
                        const float4 a = L.pk[lo];
                        L.pk[lo] = make_float4((float)(x.x - c.x), (float)(x.y - c.y), a.z, a.w);
                        const double2 rf = e->pos_ref[i];
                        const double ddx = x.x - rf.x, ddy = x.y - rf.y;
                        need |= (ddx * ddx + ddy * ddy > p.half_skin2);
                    }
                    if (C > 1) __threadfence();
                }
                pstale = s.prec != 1;
                moved_rb = __syncthreads_or(need);
                if (C > 1) {
                    if (t == 0) res_bcast<C>(ctl.rb_in, r, moved_rb);
                    res_csync<C>();
                    moved_rb = 0;
#pragma unroll
                    for (int b = 0; b < C; b++) moved_rb |= ctl.rb_in[b];
                }
                if (t == 0 && s.prec == 1) s.vel_f32 = 0;
            }

            // ---- cell list (the whole system, in every block) and neighbour lists
            if (s.rebuild || moved_rb) {
                const bool stale = pstale;
                const int ncd = s.ncd, nc = ncd * ncd;
                for (int c = t; c < nc; c += NT) L.ccur[c] = 0;
#pragma unroll
                for (int k = 0; k < PPT; k++) {
                    const int lo = q + k * NG, l = base + lo;
                    if (!lead || l >= n) break;
                    const int i = off + l;
                    const double2 x = stale ? res_position(L, e->ctr[i], lo) : e->pos[i];
                    const double fx = floor(x.x * s.inv_cs), fy = floor(x.y * s.inv_cs);
                    const int cx = wrap_int((long long)fx, ncd), cy = wrap_int((long long)fy, ncd);
                    const int code = code_of(cx, cy);
                    const double2 c = make_double2((fx + 0.5) * s.cs, (fy + 0.5) * s.cs);
                    e->pos[i] = x;
                    e->pos_ref[i] = x;
                    e->ctr[i] = c;
                    e->cellc[i] = code;
                    const double ox = x.x - c.x, oy = x.y - c.y;
                    const float hx = (float)ox, hy = (float)oy;
                    const float4 a = L.pk[lo], al = L.pkl[lo];
                    L.pk[lo] = make_float4(hx, hy, a.z, __int_as_float(code));
                    const float2 lw = split_lo(ox, oy, hx, hy);
                    L.pkl[lo] = make_float4(lw.x, lw.y, al.z, 0.f);
                    orf[k] = make_float2(hx, hy);
                }
                if (C > 1) __threadfence();
                res_csync<C>();
                // count every particle of the system into its cell
                for (int j = t; j < n; j += NT) {
                    const int c = __float_as_int(res_pk_of<C, M>(L, j)->w);
                    atomicAdd(&L.ccur[code_x(c) + code_y(c) * ncd], 1);
                }
                __syncthreads();
                res_scan<NT>(L, nc, ctl.wsum, &ctl.carry);
                __syncthreads();
                for (int j = t; j < n; j += NT) {
                    const int c = __float_as_int(res_pk_of<C, M>(L, j)->w);
                    const int g = code_x(c) + code_y(c) * ncd;
                    L.citem[L.cstart[g] + atomicAdd(&L.ccur[g], 1)] = (unsigned short)j;
                }
                __syncthreads();
                // ascending particle order inside each cell: reproducible lists
                for (int c = t; c < nc; c += NT) {
                    const int b = L.cstart[c], en = L.cstart[c + 1];
                    for (int k = b + 1; k < en; k++) {
                        const unsigned short key = L.citem[k];
                        int j = k - 1;
                        while (j >= b && L.citem[j] > key) { L.citem[j + 1] = L.citem[j]; j--; }
                        L.citem[j + 1] = key;
                    }
                }
                __syncthreads();
                int mx = 0;
#pragma unroll
                for (int k = 0; k < PPT; k++) {
                    const int lo = q + k * NG, l = base + lo;
                    if (!lead || l >= n) break;
                    mx = max(mx, res_nlist<C, M>(e, s, L, lo, l, off + l));
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_down_sync(0xffffffffu, mx, o));
                if ((t & 31) == 0) ctl.imax[t >> 5] = mx;
                __syncthreads();
                if (t == 0) {
                    for (int w = 1; w < NT / 32; w++) mx = max(mx, ctl.imax[w]);
                    res_bcast<C>(ctl.mx_in, r, mx);
                }
                res_csync<C>();
                if (t == 0) {
                    mx = ctl.mx_in[0];
                    for (int b = 1; b < C; b++) mx = max(mx, ctl.mx_in[b]);
                    s.resume = e_nlist_sys(e, s, mx) ? 0 : 1;
                }
                pstale = false;
                __syncthreads();
                if (s.resume) break;  // list overflow: the host grows the lists and relaunches
            }

            // ---- force pass (+ kick unless setup) and the per-system epilogue
            {
                const bool setup = s.phase == kSetup;
                if (s.prec != 1) {
                    dw pe = {0.f, 0.f};
                    float v[4] = {0.f, 0.f, 0.f, 0.f};  // power, max|F|^2, virial, contacts
                    const float h = 0.5f * (float)s.dt;
                    const bool dwp = s.prec == 2;
                    // the energy-change stop test needs double-word energies
                    const bool short_dw = p.pe_diff_target <= 0.0;
#pragma unroll
                    for (int k = 0; k < PPT; k++) {
                        const int lo = q + k * NG, l = base + lo;
                        const bool live = l < n;
                        const int i = off + (live ? l : 0);
                        dw fx = {0.f, 0.f}, fy = {0.f, 0.f}, en = {0.f, 0.f};
                        float wv = 0.f;
                        int ncount = 0;
                        if (live) {
                            if (!dwp) {
                                float ax, ay, ef;
                                res_forces_f32<C, M, G>(e, s, L, lo, i, ax, ay, ef, wv, ncount);
                                fx.hi = ax; fy.hi = ay; en.hi = ef;
                            } else if (short_dw) {
                                float ef;
                                res_forces_dwf<C, M, G>(e, s, L, lo, i, fx, fy, ef, wv, ncount);
                                en.hi = ef;
                            } else {
                                res_forces_dw<C, M, G>(e, s, L, lo, i, fx, fy, en, wv, ncount);
                            }
                        }
                        if (G > 1) {
                            if (dwp) {
                                fx = lanes_dw<G>(fx);
                                fy = lanes_dw<G>(fy);
                                en = lanes_dw<G>(en);
                            } else {
                                fx.hi = lanes_sum<G>(fx.hi);
                                fy.hi = lanes_sum<G>(fy.hi);
                                en.hi = lanes_sum<G>(en.hi);
                            }
                            wv = lanes_sum<G>(wv);
                            ncount = lanes_sum<G>(ncount);
                        }
                        if (!lead || !live) continue;
                        pe = dw_add(pe, en);
                        const float2 f = make_float2(fx.hi, fy.hi);
                        fr[k] = f;
                        frl[k] = make_float2(fx.lo, fy.lo);
                        float2 vv = u[k];
                        if (!setup) {
                            const float hm = h * im[k];
                            vv.x += f.x * hm;
                            vv.y += f.y * hm;
                            u[k] = vv;
                        }
                        v[0] += f.x * vv.x + f.y * vv.y;
                        v[1] = fmaxf(v[1], f.x * f.x + f.y * f.y);
                        v[2] += wv;
                        v[3] += (float)ncount;
                    }
                    res_reduce<NT>(pe, v, smw, smv);
                    if (t == 0) {
                        RPart pp;
                        pp.pe = pe;
#pragma unroll
                        for (int b = 0; b < 4; b++) pp.v[b] = v[b];
                        pp.req = req;
                        res_bcast<C>(ctl.part_in, r, pp);
                    }
                    res_csync<C>();
                    if (t == 0) {
                        dw tp = ctl.part_in[0].pe;
                        float tv[4];
#pragma unroll
                        for (int b = 0; b < 4; b++) tv[b] = ctl.part_in[0].v[b];
                        for (int b = 1; b < C; b++) {
                            tp = dw_add(tp, ctl.part_in[b].pe);
                            tv[0] += ctl.part_in[b].v[0];
                            tv[1] = fmaxf(tv[1], ctl.part_in[b].v[1]);
                            tv[2] += ctl.part_in[b].v[2];
                            tv[3] += ctl.part_in[b].v[3];
                        }
                        ctl.req = ctl.part_in[0].req;
                        const double tot[5] = {(double)tp.hi + (double)tp.lo, tv[0], tv[1], tv[2], tv[3]};
                        e_force_epilogue(e, s, tot, setup, primary);
                        if (s.pending == kActNone) decide_stop(it + 1);
                    }
                } else {
                    double a[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
#pragma unroll
                    for (int k = 0; k < PPT; k++) {
                        const int lo = q + k * NG, l = base + lo;
                        const bool live = l < n;
                        const int i = off + (live ? l : 0);
                        double ax = 0, ay = 0, en = 0, wv = 0, nc = 0;
                        if (live) res_forces_f64<C, M, G>(e, s, L, lo, i, ax, ay, en, wv, nc);
                        ax = lanes_sum<G>(ax); ay = lanes_sum<G>(ay); en = lanes_sum<G>(en);
                        wv = lanes_sum<G>(wv); nc = lanes_sum<G>(nc);
                        if (!lead || !live) continue;
                        const double2 f = make_double2(ax, ay);
                        e->frc[i] = f;
                        fr[k] = make_float2((float)ax, (float)ay);
                        frl[k] = make_float2((float)(ax - (double)fr[k].x), (float)(ay - (double)fr[k].y));
                        double2 vv = e->vel[i];
                        if (!setup) {
                            const double dtm = (0.5 * s.dt) * rcp_newton(e->mass[i]);
                            vv.x = vv.x + f.x * dtm;
                            vv.y = vv.y + f.y * dtm;
                            e->vel[i] = vv;
                        }
                        a[0] += en;
                        a[1] += f.x * vv.x + f.y * vv.y;
                        a[2] = fmax(a[2], f.x * f.x + f.y * f.y);
                        a[3] += wv;
                        a[4] += nc;
                    }
                    const int ops[5] = {0, 0, 1, 0, 0};
                    block_reduce<5, double>(a, ops, smd);
                    if (t == 0) {
                        RPartD pd;
#pragma unroll
                        for (int b = 0; b < 5; b++) pd.v[b] = a[b];
                        pd.req = req;
                        res_bcast<C>(ctl.partd_in, r, pd);
                    }
                    res_csync<C>();
                    if (t == 0) {
                        double tot[5];
#pragma unroll
                        for (int b = 0; b < 5; b++) tot[b] = ctl.partd_in[0].v[b];
                        for (int b = 1; b < C; b++) {
                            tot[0] += ctl.partd_in[b].v[0];
                            tot[1] += ctl.partd_in[b].v[1];
                            tot[2] = fmax(tot[2], ctl.partd_in[b].v[2]);
                            tot[3] += ctl.partd_in[b].v[3];
                            tot[4] += ctl.partd_in[b].v[4];
                        }
                        ctl.req = ctl.partd_in[0].req;
                        e_force_epilogue(e, s, tot, setup, primary);
                        if (s.pending == kActNone) decide_stop(it + 1);
                    }
                }
                __syncthreads();
            }
        }

        // ---- transition between minimisations (jamming protocol)
        if (s.pending != kActNone) {
            const int act = s.pending;
            const bool stale = pstale;
#pragma unroll
            for (int k = 0; k < PPT; k++) {
                const int lo = q + k * NG, l = base + lo;
                if (!lead || l >= n) break;
                const int i = off + l;
                double2 x = stale ? res_position(L, e->ctr[i], lo) : e->pos[i];
                if (act == kActCompress && s.pressure < p.p_low && s.jam_stage == 1 && s.L_saved == s.L)
                    e->pos_save[i] = x;  // write_restart_file("last_state")
                if (act == kActRevertScale) x = e->pos_save[i];  // load("last_state")
                x.x *= s.scale;
                x.y *= s.scale;
                e->pos[i] = x;
                e->vel[i] = make_double2(0.0, 0.0);
                u[k] = make_float2(0.f, 0.f);
            }
            __syncthreads();
            if (t == 0) {
                e_transition_sys(p, s, act);
                decide_stop(it + 1);
            }
            pstale = false;
            __syncthreads();
        }
        it++;
    }

    // ---- write back own particles (exact double-word offsets, registers, FP64
    // positions); block 0 writes the system state
    const bool stale = pstale;
    const bool f64_last = s.prec == 1;
#pragma unroll
    for (int k = 0; k < PPT; k++) {
        const int lo = q + k * NG, l = base + lo;
        if (!lead || l >= n) break;
        const int i = off + l;
        if (stale) e->pos[i] = res_position(L, e->ctr[i], lo);
        e->pk[i] = L.pk[lo];
        e->pkl[i] = L.pkl[lo];
        e->vel32[i] = u[k];
        e->frc32[i] = fr[k];
        e->oref[i] = orf[k];
        if (!f64_last)
            e->frc[i] = make_double2((double)fr[k].x + (double)frl[k].x, (double)fr[k].y + (double)frl[k].y);
    }
    if (t == 0 && primary) {
        s.res_valid = 1;
        e->sys[sid] = s;
    }
    // no block leaves while another may still read its shared memory
    res_csync<C>();
}

}  // namespace
}  // namespace dpg
