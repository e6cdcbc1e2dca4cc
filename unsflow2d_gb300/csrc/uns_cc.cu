// uns_cc.cu -- cell-centred (CCFVM) residual-and-update hot path on GB300.
//
// Design:
//   * structure-of-arrays in HBM with small per-entity vectors: double4 for
//     the four conserved / primitive / gradient / limiter values of a cell,
//     so a gathered neighbour costs one 32-byte sector;
//   * face kernels compute every per-face quantity once (flux, spectral
//     radius, face gradient) and write it to a face array; cell kernels then
//     gather their faces from an index-sorted face list.  That is atomic-free
//     and deterministic, and the per-cell summation order is exactly the
//     reference's face-loop order (boundary faces, then interior faces, then
//     the viscous loop), so there is no colour pass and no reordering error;
//   * cell kernels fuse what the reference runs as separate cell loops
//     (con2prim + save_old + the limiter's global min/max; spectral radius
//     gather + dt + gradient + limiter; residual gather + RK stage + norm);
//   * LU-SGS forward/backward sweeps run as a list-scheduled dataflow sweep
//     over the cell DAG of the reference ordering inside one cooperative
//     launch: each warp works through its own list of (cell, pass) items and
//     waits (bounded) on the published records of the items it depends on,
//     which reproduces the sequential sweep exactly;
//   * one iteration of the main loop is captured once as a CUDA graph and
//     replayed; iteration number, CFL schedule and the convergence stop live
//     in device memory.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "uns_cc_impl.cuh"
#include "uns_common.cuh"
#include "uns_phys.cuh"
#include "uns_sched.hpp"
#include "unsflow_gpu.h"

using namespace uns;

namespace {


__device__ __forceinline__ bool stopped(const CCView& v, int inst) {
    return v.done != nullptr && ((volatile int*)v.done)[inst] != 0;
}
__device__ __forceinline__ bool stopped(const CCView& v) { return stopped(v, 0); }
__device__ __forceinline__ double cur_cfl(const CCView& v, int inst, double cfl) {
    return v.cfl_sched ? v.cfl_sched[(size_t)inst * v.cfl_stride + v.iter[inst]] : cfl;
}
// Instance of a cell / face / vertex (0 for a single case; -1 for padding).
__device__ __forceinline__ int cell_inst(const CCView& v, int i) { return v.ninst ? v.cinst[i] : 0; }
__device__ __forceinline__ int face_inst(const CCView& v, int f) { return v.ninst ? v.finst[f] : 0; }
__device__ __forceinline__ int vert_inst(const CCView& v, int k) { return v.ninst ? v.pinst[k] : 0; }
// Instance of a block of interior cells: its first cell is a real one.
__device__ __forceinline__ int block_inst(const CCView& v) { return v.ninst ? v.cinst[blockIdx.x * blockDim.x] : 0; }
__device__ __forceinline__ const Gas& gas_of(const CCView& v, int inst) { return v.ninst ? v.gas[inst] : v.g; }

// Minimum / maximum of a 64-bit key over a group of lanes (all of which call
// it with the same mask): the extreme high word, then the extreme low word
// among the lanes holding it.
__device__ __forceinline__ unsigned long long grp_min_u64(unsigned grp, unsigned long long e) {
    const unsigned hi = (unsigned)(e >> 32), lo = (unsigned)e;
    const unsigned mh = __reduce_min_sync(grp, hi);
    const unsigned ml = __reduce_min_sync(grp, hi == mh ? lo : 0xffffffffu);
    return ((unsigned long long)mh << 32) | ml;
}
__device__ __forceinline__ unsigned long long grp_max_u64(unsigned grp, unsigned long long e) {
    const unsigned hi = (unsigned)(e >> 32), lo = (unsigned)e;
    const unsigned mh = __reduce_max_sync(grp, hi);
    const unsigned ml = __reduce_max_sync(grp, hi == mh ? lo : 0u);
    return ((unsigned long long)mh << 32) | ml;
}

// ---------------------------------------------------------------- kernels
// con2prim (main.F90:62-67) + save_old (solution.F90:118-132) + the global
// min/max of every cell's primitives incl. ghosts (limiter.F90:146-149) +
// the positivity check of main.F90:384-411, fused over one pass of the cells.
enum { BEGIN_PRIM = 1, BEGIN_OLD = 2, BEGIN_MINMAX = 4, BEGIN_POS = 8 };

__global__ void __launch_bounds__(kBlock) k_begin(CCView v, int flags) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int inst = i < v.ntot ? cell_inst(v, i) : (v.ninst ? -1 : 0);
    const bool live = inst >= 0 && !stopped(v, inst);
    if (!v.ninst && !live) return;  // one case: the whole grid stops together
    unsigned long long emx[4] = {0ULL, 0ULL, 0ULL, 0ULL};
    unsigned long long emn[4] = {~0ULL, ~0ULL, ~0ULL, ~0ULL};
    bool have = false;  // the primitives below are this thread's qp (no read-back for the limiter range)
    double pr[4];
    if (live && i < v.noc) {
        const Gas& gi = gas_of(v, inst);
        double4 q = v.qc[i];
        if ((flags & BEGIN_PRIM) && v.mixed) {  // con2prim in FP32 from the rounded state
            const float E = (float)q.x, r = (float)q.y, ru = (float)q.z, rv = (float)q.w;
            const float u = ru / r, w = rv / r;
            const float p = (float)gi.gamma1 * (E - 0.5f * r * (u * u + w * w));
            v.qpf[i] = make_float4(r, u, w, p);
            v.qp[i] = make_double4(r, u, w, p);
            pr[0] = r; pr[1] = u; pr[2] = w; pr[3] = p;
            have = true;
            if (v.laminar || v.grad_type == UNS_GRAD_GGFC) v.qT[i] = (double)(p / (r * (float)gi.znd));
            if ((flags & BEGIN_POS) && (r <= 0.f || p <= 0.f)) set_err(v.err, UNS_ERR_NONPOSITIVE, i);
        } else if (flags & BEGIN_PRIM) {
            Prim P = con2prim(gi, q.x, q.y, q.z, q.w);
            v.qp[i] = make_double4(P.rho, P.u, P.v, P.p);
            v.qT[i] = P.t;
            pr[0] = P.rho; pr[1] = P.u; pr[2] = P.v; pr[3] = P.p;
            have = true;
            if ((flags & BEGIN_POS) && (P.rho <= 0.0 || P.p <= 0.0)) set_err(v.err, UNS_ERR_NONPOSITIVE, i);
        }
        if (flags & BEGIN_OLD) v.qold[i] = q;
    }
    if (flags & BEGIN_MINMAX) {
        if (live && i < v.ntot) {
            if (!have) {
                const double4 p = v.qp[i];
                pr[0] = p.x; pr[1] = p.y; pr[2] = p.z; pr[3] = p.w;
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) { emx[j] = enc_ord(pr[j]); emn[j] = emx[j]; }
        }
        if (v.ninst && blockIdx.x * blockDim.x >= v.noc) {  // ghost blocks of packed cases: per-case lane groups
            const unsigned grp = __match_any_sync(0xffffffffu, live ? inst : -1);
            unsigned long long mx[4], mn[4];
#pragma unroll
            for (int j = 0; j < 4; ++j) { mx[j] = grp_max_u64(grp, emx[j]); mn[j] = grp_min_u64(grp, emn[j]); }
            if (live && (int)(threadIdx.x & 31) == __ffs(grp) - 1)
                for (int j = 0; j < 4; ++j) {
                    atomicMax(&v.minmax[8 * inst + j], mx[j]);
                    atomicMin(&v.minmax[8 * inst + 4 + j], mn[j]);
                }
            return;
        }
#pragma unroll
        for (int j = 0; j < 4; ++j) {
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                unsigned long long t = __shfl_xor_sync(0xffffffffu, emx[j], o);
                emx[j] = t > emx[j] ? t : emx[j];
                t = __shfl_xor_sync(0xffffffffu, emn[j], o);
                emn[j] = t < emn[j] ? t : emn[j];
            }
        }
        __shared__ unsigned long long smx[kBlock / 32][4], smn[kBlock / 32][4];
        int w = threadIdx.x >> 5, l = threadIdx.x & 31;
        if (l == 0)
            for (int j = 0; j < 4; ++j) { smx[w][j] = emx[j]; smn[w][j] = emn[j]; }
        __syncthreads();
        if (threadIdx.x < 4) {  // a block of one case (padded interior blocks of packed cases too)
            const int bi = block_inst(v);
            int j = threadIdx.x;
            unsigned long long a = smx[0][j], b = smn[0][j];
            for (int k = 1; k < kBlock / 32; ++k) { a = smx[k][j] > a ? smx[k][j] : a; b = smn[k][j] < b ? smn[k][j] : b; }
            atomicMax(&v.minmax[8 * bi + j], a);
            atomicMin(&v.minmax[8 * bi + 4 + j], b);
        }
    }
}

// avg_c2v vertex part (average.F90:11-29): pseudo-Laplacian weighted mean.
__global__ void __launch_bounds__(512) k_vertex_avg(CCView v) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.nop || stopped(v, vert_inst(v, i))) return;
    if (v.mixed) {  // FP32 from the FP32 primitives; FP64 copies only where an FP64 kernel reads them
        const bool dbl = v.laminar || v.grad_type == UNS_GRAD_GGFC;
        float wt = 0.f, c0 = 0.f, c1 = 0.f, c2 = 0.f, c3 = 0.f;
        double c4 = 0.0;
        auto add = [&](int c, float w, const float4& q) {
            wt = wt + w;
            c0 = c0 + q.x * w; c1 = c1 + q.y * w; c2 = c2 + q.z * w; c3 = c3 + q.w * w;
            if (dbl) c4 = c4 + v.qT[c] * (double)w;
        };
        int k = v.v2c_off[i];
        const int k1 = v.v2c_off[i + 1];
        for (; k + 3 < k1; k += 4) {  // four cells' gathers in flight together, sums in order
            int c[4];
            float w[4];
            float4 q[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) { c[u] = __ldg(&v.v2c[k + u]); w[u] = __ldg(&v.v2c_wtf[k + u]); }
#pragma unroll
            for (int u = 0; u < 4; ++u) q[u] = v.qpf[c[u]];
#pragma unroll
            for (int u = 0; u < 4; ++u) add(c[u], w[u], q[u]);
        }
        for (; k < k1; ++k) {
            const int c = __ldg(&v.v2c[k]);
            add(c, __ldg(&v.v2c_wtf[k]), v.qpf[c]);
        }
        const float r = 1.f / wt;
        const float4 pp = make_float4(c0 * r, c1 * r, c2 * r, c3 * r);
        v.ppf[i] = pp;
        if (dbl) {
            v.pp[i] = make_double4(pp.x, pp.y, pp.z, pp.w);
            v.ppT[i] = c4 / (double)wt;
        }
        return;
    }
    double wt = 0.0, c0 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0, c4 = 0.0;
#pragma unroll 4
    for (int k = v.v2c_off[i]; k < v.v2c_off[i + 1]; ++k) {
        int c = __ldg(&v.v2c[k]);
        double w = __ldg(&v.v2c_wt[k]);
        wt = wt + w;
        double4 q = v.qp[c];
        c0 = c0 + q.x * w;
        c1 = c1 + q.y * w;
        c2 = c2 + q.z * w;
        c3 = c3 + q.w * w;
        c4 = c4 + v.qT[c] * w;
    }
    v.pp[i] = make_double4(c0 / wt, c1 / wt, c2 / wt, c3 / wt);
    v.ppT[i] = c4 / wt;
}

// avg_c2v face part (average.F90:31-36) + spectral02 face radius
// (timestep.F90:77-104).
__global__ void __launch_bounds__(kBlock) k_face_prim_spec(CCView v) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= v.nof) return;
    const int inst = face_inst(v, f);
    if (stopped(v, inst)) return;
    const Gas& g = gas_of(v, inst);
    if (v.mixed) {  // FP32; the FP64 face radius stays (the LU-SGS prep reads it)
        const int2 p = v.fpt[f];
        const float4 a = v.ppf[p.x], b = v.ppf[p.y], na = v.fnaf[f];
        const float4 q = make_float4(0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z), 0.5f * (a.w + b.w));
        v.fqf[f] = q;
        const float a0 = sqrtf((float)g.gamma * q.w / q.x);
        float ll = na.z * (fabsf(q.y * na.x + q.z * na.y) + a0);
        if (v.laminar) {
            ll = ll + (float)(g.vll * v.fmu[f]) / q.x;
            v.fq[f] = make_double4(q.x, q.y, q.z, q.w);
            v.fqT[f] = 0.5 * (v.ppT[p.x] + v.ppT[p.y]);
        }
        v.flaf[f] = ll;
        v.fla[f] = (double)ll;
        return;
    }
    int2 p = v.fpt[f];
    double4 a = v.pp[p.x], b = v.pp[p.y];
    double4 q = make_double4(0.5 * (a.x + b.x), 0.5 * (a.y + b.y), 0.5 * (a.z + b.z), 0.5 * (a.w + b.w));
    v.fq[f] = q;
    v.fqT[f] = 0.5 * (v.ppT[p.x] + v.ppT[p.y]);
    double2 n = v.fn[f];
    double a0 = sqrt(g.gamma * q.w / q.x);
    double un = q.y * n.x + q.z * n.y;
    double ll = v.farea[f] * (fabs(un) + a0);
    ll = ll + g.vll * v.fmu[f] / q.x;
    v.fla[f] = ll;
}

// Diamond-path face gradient (gradient.F90:183-261, gradtrixy :281-321).
__device__ __forceinline__ bool gradtri(const double* pr0, const double* pr1, const double* pr2, double x0, double y0,
                                        double x1, double y1, double x2, double y2, double gxo[5], double gyo[5],
                                        double& tarea) {
    const double xs[3] = {x0, x1, x2}, ys[3] = {y0, y1, y2};
    const double* prs[3] = {pr0, pr1, pr2};
    tarea = 0.0;
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        int ip1 = (i == 2) ? 0 : i + 1;
        double dx = 0.5 * (xs[ip1] + xs[i]);
        double dy = ys[ip1] - ys[i];
        tarea = tarea + dx * dy;
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) { gxo[k] = 0.0; gyo[k] = 0.0; }
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        int ip1 = (i == 2) ? 0 : i + 1;
        double dx = ys[ip1] - ys[i];
        double dy = -(xs[ip1] - xs[i]);
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            double var = 0.5 * (prs[i][k] + prs[ip1][k]);
            gxo[k] = gxo[k] + var * dx;
            gyo[k] = gyo[k] + var * dy;
        }
    }
#pragma unroll
    for (int k = 0; k < 5; ++k) { gxo[k] = gxo[k] / tarea; gyo[k] = gyo[k] / tarea; }
    return tarea > 0.0;
}

__global__ void __launch_bounds__(kBlock) k_face_ggfc(CCView v) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= v.nof || stopped(v, face_inst(v, f))) return;
    int2 nb = v.fnb[f];
    int2 p = v.fpt[f];
    double2 X1 = v.pxy[p.x], X2 = v.pxy[p.y], Ci = v.cen[nb.x], Co = v.cen[nb.y];
    double4 a = v.pp[p.x], b = v.pp[p.y], qi = v.qp[nb.x], qo = v.qp[nb.y];
    double P1[5] = {a.x, a.y, a.z, a.w, v.ppT[p.x]};
    double P2[5] = {b.x, b.y, b.z, b.w, v.ppT[p.y]};
    double QI[5] = {qi.x, qi.y, qi.z, qi.w, v.qT[nb.x]};
    double QO[5] = {qo.x, qo.y, qo.z, qo.w, v.qT[nb.y]};
    double g1x[5], g1y[5], g2x[5], g2y[5], a1, a2;
    bool ok1 = gradtri(P1, QO, P2, X1.x, X1.y, Co.x, Co.y, X2.x, X2.y, g1x, g1y, a1);
    bool ok2 = gradtri(P1, P2, QI, X1.x, X1.y, X2.x, X2.y, Ci.x, Ci.y, g2x, g2y, a2);
    if (!(ok1 && ok2)) set_err(v.err, UNS_ERR_MESH, f);
    double s = a1 + a2;
    double gx[5], gy[5];
#pragma unroll
    for (int k = 0; k < 5; ++k) {
        gx[k] = (a1 * g1x[k] + a2 * g2x[k]) / s;
        gy[k] = (a1 * g1y[k] + a2 * g2y[k]) / s;
    }
    v.fgx[f] = make_double4(gx[0], gx[1], gx[2], gx[3]);
    v.fgy[f] = make_double4(gy[0], gy[1], gy[2], gy[3]);
    v.fgT[f] = make_double2(gx[4], gy[4]);
    v.fasum[f] = s;
}

__device__ __forceinline__ void d4get(const double4& q, double o[4]) { o[0] = q.x; o[1] = q.y; o[2] = q.z; o[3] = q.w; }
__device__ __forceinline__ double4 d4(const double o[4]) { return make_double4(o[0], o[1], o[2], o[3]); }

// Per-cell gather over the index-sorted face list: spectral radius + dt
// (timestep.F90:40-49, 101-103), the cell gradient (Gradient_GG
// gradient.F90:95-156, Gradient_GG_FC :159-323, Gradient_LSQR :2-93) and
// limiter_VKN1 (limiter.F90:146-279).  Face order is the reference's loop
// order (interior faces, then boundary faces).
// CG_DIAG: also the LU-SGS diagonal and its reciprocal (with CG_DT; only an
// LU-SGS step reads them).
enum { CG_DT = 1, CG_GRAD = 2, CG_LIM = 4, CG_DIAG = 8 };

// atomicMin of an order-encoded dt into its instance's slot with one atomic
// per converged group of lanes of one instance.  Same result as one atomic
// per lane (min is exact and order-free), without 32 same-address atomics
// per warp.
__device__ __forceinline__ void warp_atomic_min_u64(const CCView& v, int inst, unsigned long long e) {
    const unsigned mask = v.ninst ? __match_any_sync(__activemask(), inst) : __activemask();
    const unsigned long long m = grp_min_u64(mask, e);
    if ((int)(threadIdx.x & 31) == __ffs(mask) - 1) atomicMin(&v.dtmin[inst], m);
}

__global__ void __launch_bounds__(kBlock) k_cell_grad(CCView v, int flags, double cfl_in) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.noc) return;
    const int inst = cell_inst(v, i);
    if (inst < 0 || stopped(v, inst)) return;
    const int k0 = v.cf_off[i], k1 = v.cf_off[i + 1];
    const double cvi = v.cv[i];
    const double rcv = (flags & (CG_DT | CG_GRAD)) ? 1.0 / cvi : 0.0;  // shared by dt/cv and the gradient
    if (flags & CG_DT) {
        double la = 0.0;
        for (int k = k0; k < k1; ++k) la = la + v.fla[v.cf[k] & FACE_MASK];
        v.la[i] = la;
        double cfl = cur_cfl(v, inst, cfl_in);
        double dt = cfl * cvi / la;
        v.dt[i] = dt;
        v.dcv[i] = div_rn_recip(dt, cvi, rcv);
        if (flags & CG_DIAG) {
            v.diag[i] = v.cv[i] / dt + 0.5 * 1.5 * la;
            v.diaginv[i] = 1.0 / v.diag[i];
        }
        warp_atomic_min_u64(v, inst, enc_ord(dt));
    }
    double gx[4], gy[4];
    if (flags & CG_GRAD) {
#pragma unroll
        for (int j = 0; j < 4; ++j) { gx[j] = 0.0; gy[j] = 0.0; }
        if (v.grad_type == UNS_GRAD_GG) {
            for (int k = k0; k < k1; ++k) {
                int e = v.cf[k], f = e & FACE_MASK;
                double2 n = v.fn[f];
                double area = v.farea[f];
                double q[4];
                d4get(v.fq[f], q);
                if (f < v.nfi) {
                    double dx = n.x * area, dy = n.y * area;
                    if (e & SIDE_BIT) {
#pragma unroll
                        for (int j = 0; j < 4; ++j) { gx[j] = gx[j] - q[j] * dx; gy[j] = gy[j] - q[j] * dy; }
                    } else {
#pragma unroll
                        for (int j = 0; j < 4; ++j) { gx[j] = gx[j] + q[j] * dx; gy[j] = gy[j] + q[j] * dy; }
                    }
                } else {
                    double dx = -n.x * area, dy = -n.y * area;
#pragma unroll
                    for (int j = 0; j < 4; ++j) { gx[j] = gx[j] + q[j] * dx; gy[j] = gy[j] + q[j] * dy; }
                }
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) {  // eight quotients by cv through its reciprocal (Markstein)
                gx[j] = div_rn_recip(gx[j], cvi, rcv);
                gy[j] = div_rn_recip(gy[j], cvi, rcv);
            }
        } else if (v.grad_type == UNS_GRAD_GGFC) {
            for (int k = k0; k < k1; ++k) {
                int f = v.cf[k] & FACE_MASK;
                double s = v.fasum[f];
                double a[4], b[4];
                d4get(v.fgx[f], a);
                d4get(v.fgy[f], b);
#pragma unroll
                for (int j = 0; j < 4; ++j) { gx[j] = gx[j] + a[j] * s; gy[j] = gy[j] + b[j] * s; }
            }
            const double var = v.cov[i], rv = 1.0 / var;
#pragma unroll
            for (int j = 0; j < 4; ++j) { gx[j] = div_rn_recip(gx[j], var, rv); gy[j] = div_rn_recip(gy[j], var, rv); }
        } else {  // LSQR
            double qi[4];
            d4get(v.qp[i], qi);
            for (int k = k0; k < k1; ++k) {
                int e = v.cf[k], f = e & FACE_MASK;
                double4 w = v.lsw[f];
                int2 nb = v.fnb[f];
                double qa[4], qb[4];
                d4get(v.qp[nb.x], qa);
                d4get(v.qp[nb.y], qb);
                if (f < v.nfi && (e & SIDE_BIT)) {
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        double var = qb[j] - qa[j];
                        gx[j] = gx[j] - var * w.z;
                        gy[j] = gy[j] - var * w.w;
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        double var = qb[j] - qa[j];
                        gx[j] = gx[j] + var * w.x;
                        gy[j] = gy[j] + var * w.y;
                    }
                }
            }
            (void)qi;
        }
        v.gx[i] = d4(gx);
        v.gy[i] = d4(gy);
    } else {
        d4get(v.gx[i], gx);
        d4get(v.gy[i], gy);
    }
    if (flags & CG_LIM) {
        double qmax[4], qmin[4], tol[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            qmax[j] = dec_ord(v.minmax[8 * inst + j]);
            qmin[j] = dec_ord(v.minmax[8 * inst + 4 + j]);
            tol[j] = 0.05 * (qmax[j] - qmin[j]);
        }
        double qi[4], umax[4], umin[4], ph[4];
        d4get(v.qp[i], qi);
        d4get(v.phi[i], ph);
#pragma unroll
        for (int j = 0; j < 4; ++j) { umax[j] = qi[j]; umin[j] = qi[j]; }
        for (int k = k0; k < k1; ++k) {
            int e = v.cf[k], f = e & FACE_MASK;
            double u[4];
            if (f < v.nfi) {
                int2 nb = v.fnb[f];
                d4get(v.qp[(e & SIDE_BIT) ? nb.x : nb.y], u);
            } else {
                int2 p = v.fpt[f];
                double4 a = v.pp[p.x], b = v.pp[p.y];
                u[0] = 0.5 * (a.x + b.x); u[1] = 0.5 * (a.y + b.y); u[2] = 0.5 * (a.z + b.z); u[3] = 0.5 * (a.w + b.w);
            }
#pragma unroll
            for (int j = 0; j < 4; ++j) { umax[j] = rmax(umax[j], u[j]); umin[j] = rmin(umin[j], u[j]); }
        }
        // phi = min(phi, phi0 of every face): the faces' ratios nr/dr are
        // compared exactly and only the smallest is divided (the minimum of
        // correctly rounded quotients is the rounded minimum), so one IEEE
        // division per variable instead of one per face and variable.
        double bn[4], bd[4];
        bool have[4] = {false, false, false, false};
        double2 c = v.cen[i];
        for (int k = k0; k < k1; ++k) {
            int f = v.cf[k] & FACE_MASK;
            double2 fc = v.fcen[f];
            double d0 = fc.x - c.x, d1 = fc.y - c.y;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                double D_L = gx[j] * d0 + gy[j] * d1;
                if (D_L > 0.0 || D_L < 0.0) {
                    double nr, dr;
                    vk_terms((D_L > 0.0 ? umax[j] : umin[j]) - qi[j], D_L, tol[j], nr, dr);
                    if (!ratio_ok(nr, dr)) {
                        ph[j] = rmin(ph[j], nr / dr);
                    } else if (!have[j] || ratio_less(nr, dr, bn[j], bd[j])) {
                        bn[j] = nr; bd[j] = dr; have[j] = true;
                    }
                } else {
                    ph[j] = rmin(ph[j], 1.0);
                }
            }
        }
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (have[j]) ph[j] = rmin(ph[j], bn[j] / bd[j]);
        v.phi[i] = d4(ph);
    }
}

// k_cell_grad in the mixed form: the same gathers, face orders and formulas
// with the gradient and the Venkatakrishnan limiter in FP32 on the FP32
// copies.  dt, la and diag come from the FP32 face radii.  The per-cell pack
// (primitives, gradient, phi) is the gradient and limiter state of record in
// this form (phi is a running minimum across iterations); k_unpack_f32
// writes it back to the FP64 arrays when a caller reads them or the handle
// leaves the form.
__global__ void __launch_bounds__(kBlock, 5) k_cell_grad_mixed(CCView v, int flags, double cfl_in) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.noc) return;
    const int inst = cell_inst(v, i);
    if (inst < 0 || stopped(v, inst)) return;
    const int k0 = v.cf_off[i], k1 = v.cf_off[i + 1];
    if (flags & CG_DT) {
        float la = 0.f;
        for (int k = k0; k < k1; ++k) la = la + v.flaf[v.cf[k] & FACE_MASK];
        const float cvf = (float)v.cv[i];
        const float dt = (float)cur_cfl(v, inst, cfl_in) * cvf / la;
        v.la[i] = (double)la;
        v.dt[i] = (double)dt;
        v.dcv[i] = (double)(dt / cvf);
        if (flags & CG_DIAG) {
            v.diag[i] = (double)(cvf / dt + 0.75f * la);
            v.diaginv[i] = 1.0 / v.diag[i];
        }
        warp_atomic_min_u64(v, inst, enc_ord((double)dt));
    }
    if (!(flags & (CG_GRAD | CG_LIM))) return;
    const float4 q4 = v.qpf[i];
    const float qi[4] = {q4.x, q4.y, q4.z, q4.w};
    float gx[4], gy[4];
    if (flags & CG_GRAD) {
#pragma unroll
        for (int j = 0; j < 4; ++j) { gx[j] = 0.f; gy[j] = 0.f; }
        if (v.grad_type == UNS_GRAD_GG) {
            for (int k = k0; k < k1; ++k) {
                int e = v.cf[k], f = e & FACE_MASK;
                const float4 na = v.fnaf[f];
                const float4 q = v.fqf[f];
                // outward from this cell: + for the `in` side of an interior face
                const float s = (f < v.nfi && !(e & SIDE_BIT)) ? 1.f : -1.f;
                const float dx = s * (na.x * na.z), dy = s * (na.y * na.z);
                gx[0] += q.x * dx; gx[1] += q.y * dx; gx[2] += q.z * dx; gx[3] += q.w * dx;
                gy[0] += q.x * dy; gy[1] += q.y * dy; gy[2] += q.z * dy; gy[3] += q.w * dy;
            }
            const float r = 1.f / (float)v.cv[i];
#pragma unroll
            for (int j = 0; j < 4; ++j) { gx[j] *= r; gy[j] *= r; }
        } else if (v.grad_type == UNS_GRAD_GGFC) {
            for (int k = k0; k < k1; ++k) {
                int f = v.cf[k] & FACE_MASK;
                const float s = (float)v.fasum[f];
                const double4 a = v.fgx[f], b = v.fgy[f];
                gx[0] += (float)a.x * s; gx[1] += (float)a.y * s; gx[2] += (float)a.z * s; gx[3] += (float)a.w * s;
                gy[0] += (float)b.x * s; gy[1] += (float)b.y * s; gy[2] += (float)b.z * s; gy[3] += (float)b.w * s;
            }
            const float r = 1.f / (float)v.cov[i];
#pragma unroll
            for (int j = 0; j < 4; ++j) { gx[j] *= r; gy[j] *= r; }
        } else {  // LSQR
            for (int k = k0; k < k1; ++k) {
                int e = v.cf[k], f = e & FACE_MASK;
                const float4 w = v.lswf[f];
                const int2 nb = v.fnb[f];
                const float4 a = v.qpf[nb.x], b = v.qpf[nb.y];
                const float d[4] = {b.x - a.x, b.y - a.y, b.z - a.z, b.w - a.w};
                if (f < v.nfi && (e & SIDE_BIT)) {
#pragma unroll
                    for (int j = 0; j < 4; ++j) { gx[j] -= d[j] * w.z; gy[j] -= d[j] * w.w; }
                } else {
#pragma unroll
                    for (int j = 0; j < 4; ++j) { gx[j] += d[j] * w.x; gy[j] += d[j] * w.y; }
                }
            }
        }
    } else {  // limiter alone: the gradient of record
        const float4 a = v.packf[4 * (size_t)i + 1], b = v.packf[4 * (size_t)i + 2];
        gx[0] = a.x; gx[1] = a.y; gx[2] = a.z; gx[3] = a.w;
        gy[0] = b.x; gy[1] = b.y; gy[2] = b.z; gy[3] = b.w;
    }
    const float4 p0 = v.packf[4 * (size_t)i + 3];
    float ph[4] = {p0.x, p0.y, p0.z, p0.w};
    if (flags & CG_LIM) {
        float tol[4], umax[4], umin[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float hi = (float)dec_ord(v.minmax[8 * inst + j]), lo = (float)dec_ord(v.minmax[8 * inst + 4 + j]);
            tol[j] = 0.05f * (hi - lo);
            tol[j] = tol[j] * tol[j];
            umax[j] = qi[j];
            umin[j] = qi[j];
        }
        for (int k = k0; k < k1; ++k) {
            int e = v.cf[k], f = e & FACE_MASK;
            float4 u;
            if (f < v.nfi) {
                const int2 nb = v.fnb[f];
                u = v.qpf[(e & SIDE_BIT) ? nb.x : nb.y];
            } else {
                u = v.fqf[f];  // the face average of avg_c2v, as limiter.F90 uses on boundary faces
            }
            umax[0] = rmax(umax[0], u.x); umin[0] = rmin(umin[0], u.x);
            umax[1] = rmax(umax[1], u.y); umin[1] = rmin(umin[1], u.y);
            umax[2] = rmax(umax[2], u.z); umin[2] = rmin(umin[2], u.z);
            umax[3] = rmax(umax[3], u.w); umin[3] = rmin(umin[3], u.w);
        }
        for (int k = k0; k < k1; ++k) {
            int e = v.cf[k], f = e & FACE_MASK;
            const float4 gd = v.fgeof[f];
            const float d0 = (e & SIDE_BIT) ? gd.z : gd.x, d1 = (e & SIDE_BIT) ? gd.w : gd.y;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float D_L = gx[j] * d0 + gy[j] * d1;
                float phi0 = 1.f;
                if (D_L != 0.f) {  // limiter.F90:286-294 with a = (umax or umin) - qi, b = D_L
                    const float a = (D_L > 0.f ? umax[j] : umin[j]) - qi[j];
                    const float nr = a * a + 2.f * a * D_L + tol[j];
                    const float dr = a * a + 2.f * D_L * D_L + a * D_L + tol[j];
                    phi0 = __fdividef(nr, dr);
                }
                ph[j] = rmin(ph[j], phi0);
            }
        }
    }
    v.packf[4 * (size_t)i] = q4;
    v.packf[4 * (size_t)i + 1] = make_float4(gx[0], gx[1], gx[2], gx[3]);
    v.packf[4 * (size_t)i + 2] = make_float4(gy[0], gy[1], gy[2], gy[3]);
    v.packf[4 * (size_t)i + 3] = make_float4(ph[0], ph[1], ph[2], ph[3]);
}

// k_face_prim_spec + k_cell_grad_mixed for the Green-Gauss gradient of an
// inviscid flow in the mixed form, as one gather per cell.  Each of the
// cell's faces is described by a cell-side record (v.sideg / v.sidei, in the
// cell's face order): the unit normal signed outward as Gradient_GG counts it,
// the centre-to-midpoint offset of this side, the cell across the face (-1 on
// a boundary) and the face's end points.  The face average and spectral
// radius are formed from the end points' vertex values with the operations of
// k_face_prim_spec (the sign of the normal drops out of |u.n|), so the
// records stream in order and the only gathers are the vertex values and the
// neighbours' primitives.  dt, the gradient, the limiter and the pack are
// those of k_cell_grad_mixed, bit for bit.
__global__ void __launch_bounds__(kBlock, 4) k_cell_grad_side(CCView v, int flags, double cfl_in) {
    // the limiter tolerances of the block's instance (blocks of cells are
    // instance-pure), decoded once per block
    __shared__ float stol[4];
    if ((flags & CG_LIM) && threadIdx.x < 4) {
        const int b = block_inst(v), j = threadIdx.x;
        const float hi = (float)dec_ord(v.minmax[8 * b + j]), lo = (float)dec_ord(v.minmax[8 * b + 4 + j]);
        const float t = 0.05f * (hi - lo);
        stol[j] = t * t;
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.noc) return;
    const int inst = cell_inst(v, i);
    if (inst < 0 || stopped(v, inst)) return;
    const Gas& g = gas_of(v, inst);
    const float gam = (float)g.gamma;
    const int k0 = v.cf_off[i], k1 = v.cf_off[i + 1];
    const float4 q4 = v.qpf[i];
    const float qi[4] = {q4.x, q4.y, q4.z, q4.w};
    float gx[4] = {0.f, 0.f, 0.f, 0.f}, gy[4] = {0.f, 0.f, 0.f, 0.f};
    float umax[4] = {qi[0], qi[1], qi[2], qi[3]}, umin[4] = {qi[0], qi[1], qi[2], qi[3]};
    float la = 0.f;
    for (int k = k0; k < k1; ++k) {
        const float4 sg = v.sideg[k];
        const int4 si = v.sidei[k];
        const float area = __int_as_float(si.w);
        const float4 a = v.ppf[si.y], b = v.ppf[si.z];
        const float4 u = si.x >= 0 ? v.qpf[si.x] : make_float4(0.f, 0.f, 0.f, 0.f);
        const float4 q = make_float4(0.5f * (a.x + b.x), 0.5f * (a.y + b.y), 0.5f * (a.z + b.z), 0.5f * (a.w + b.w));
        const float a0 = sqrtf(gam * q.w / q.x);
        la = la + area * (fabsf(q.y * sg.x + q.z * sg.y) + a0);
        const float dx = sg.x * area, dy = sg.y * area;
        gx[0] += q.x * dx; gx[1] += q.y * dx; gx[2] += q.z * dx; gx[3] += q.w * dx;
        gy[0] += q.x * dy; gy[1] += q.y * dy; gy[2] += q.z * dy; gy[3] += q.w * dy;
        const float4 w = si.x >= 0 ? u : q;  // the face average on a boundary face, as limiter.F90 uses
        umax[0] = rmax(umax[0], w.x); umin[0] = rmin(umin[0], w.x);
        umax[1] = rmax(umax[1], w.y); umin[1] = rmin(umin[1], w.y);
        umax[2] = rmax(umax[2], w.z); umin[2] = rmin(umin[2], w.z);
        umax[3] = rmax(umax[3], w.w); umin[3] = rmin(umin[3], w.w);
    }
    const float cvf = (float)v.cv[i];
    if (flags & CG_DT) {
        const float dt = (float)cur_cfl(v, inst, cfl_in) * cvf / la;
        v.la[i] = (double)la;
        v.dt[i] = (double)dt;
        v.dcv[i] = (double)(dt / cvf);
        if (flags & CG_DIAG) {
            v.diag[i] = (double)(cvf / dt + 0.75f * la);
            v.diaginv[i] = 1.0 / v.diag[i];
        }
        warp_atomic_min_u64(v, inst, enc_ord((double)dt));
    }
    {
        const float r = 1.f / cvf;
#pragma unroll
        for (int j = 0; j < 4; ++j) { gx[j] *= r; gy[j] *= r; }
    }
    const float4 p0 = v.packf[4 * (size_t)i + 3];
    float ph[4] = {p0.x, p0.y, p0.z, p0.w};
    if (flags & CG_LIM) {
        const float tol[4] = {stol[0], stol[1], stol[2], stol[3]};
        for (int k = k0; k < k1; ++k) {
            const float4 sg = v.sideg[k];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float D_L = gx[j] * sg.z + gy[j] * sg.w;
                float phi0 = 1.f;
                if (D_L != 0.f) {  // limiter.F90:286-294 with a = (umax or umin) - qi, b = D_L
                    const float a = (D_L > 0.f ? umax[j] : umin[j]) - qi[j];
                    const float nr = a * a + 2.f * a * D_L + tol[j];
                    const float dr = a * a + 2.f * D_L * D_L + a * D_L + tol[j];
                    phi0 = __fdividef(nr, dr);
                }
                ph[j] = rmin(ph[j], phi0);
            }
        }
    }
    v.packf[4 * (size_t)i] = q4;
    v.packf[4 * (size_t)i + 1] = make_float4(gx[0], gx[1], gx[2], gx[3]);
    v.packf[4 * (size_t)i + 2] = make_float4(gy[0], gy[1], gy[2], gy[3]);
    v.packf[4 * (size_t)i + 3] = make_float4(ph[0], ph[1], ph[2], ph[3]);
}

// Convective face flux (fvresidual.F90:27-171).  Boundary faces also write
// their ghost cell (farfield: Riemann state; wall: slip / no-slip mirror).
// R = double for the FP64 form, float for FP32 face arithmetic.
template <class R>
__device__ __forceinline__ bool flux_dispatch(const Gas& g, R nx, R ny, R area, V4<R>& ql, V4<R>& qr, V4<R>& F) {
    return face_flux<R>(g, nx, ny, area, ql, qr, F);
}

// Boundary face f of cell `in` (fvresidual.F90:27-101): the reconstructed
// state of the cell (the FP32 pack of record in the mixed form), the farfield
// or wall ghost from it and, for a wall, from the cell's conserved state cin;
// writes the ghost cell, the wall force and the flux, and returns the flux.
template <class R>
__device__ __forceinline__ double4 bnd_face_flux(const CCView& v, const Gas& g, int f, int in, const double cin4[4]) {
    const double2 n = v.fn[f];
    const double area = v.farea[f];
    const double2 fc = v.fcen[f];
    const double2 ci = v.cen[in];
    double qi[4], gxi[4], gyi[4], phi_i[4];
    if constexpr (std::is_same<R, float>::value) {
        const float4* A = v.packf + 4 * (size_t)in;
        const float4 a0 = A[0], a1 = A[1], a2 = A[2], a3 = A[3];
        qi[0] = a0.x; qi[1] = a0.y; qi[2] = a0.z; qi[3] = a0.w;
        gxi[0] = a1.x; gxi[1] = a1.y; gxi[2] = a1.z; gxi[3] = a1.w;
        gyi[0] = a2.x; gyi[1] = a2.y; gyi[2] = a2.z; gyi[3] = a2.w;
        phi_i[0] = a3.x; phi_i[1] = a3.y; phi_i[2] = a3.z; phi_i[3] = a3.w;
    } else {
        d4get(v.qp[in], qi);
        d4get(v.gx[in], gxi);
        d4get(v.gy[in], gyi);
        d4get(v.phi[in], phi_i);
    }
    const int bc = v.fbc[f];
    const double d0 = fc.x - ci.x, d1 = fc.y - ci.y;
    V4<double> qcl;
#pragma unroll
    for (int j = 0; j < 4; ++j) qcl[j] = qi[j] + phi_i[j] * (gxi[j] * d0 + gyi[j] * d1);
    double4 Fd = make_double4(0.0, 0.0, 0.0, 0.0);
    if (bc == 2001 || bc == 1001) {
        const V4<double> cin = {cin4[0], cin4[1], cin4[2], cin4[3]};
        CCBnd<double> b = cc_boundary<double, R>(g, bc, n.x, n.y, area, qcl, cin, g.u_inf, g.v_inf);
        if (!b.ok) set_err(v.err, UNS_ERR_NEG_SOUND_SPEED, f);
        Fd = make_double4(b.F[0], b.F[1], b.F[2], b.F[3]);
        const int out = v.fnb[f].y;
        v.qc[out] = make_double4(b.gq[0], b.gq[1], b.gq[2], b.gq[3]);
        v.qp[out] = make_double4(b.gp[0], b.gp[1], b.gp[2], b.gp[3]);
        v.qT[out] = b.gT;
        v.qpf[out] = make_float4((float)b.gp[0], (float)b.gp[1], (float)b.gp[2], (float)b.gp[3]);
        if (bc == 1001) v.fwall[f - v.nfi] = make_double2(Fd.z, Fd.w);
    }
    v.fF[f] = Fd;
    return Fd;
}

// One thread per face; the first blocks take the boundary faces, whose FP64
// ghost arithmetic is the longest per thread, so that they run beside the
// interior faces instead of after them.
template <class R>
__global__ void __launch_bounds__(512, std::is_same<R, float>::value ? 2 : 1) k_face_conv(CCView v) {
    const int bs = blockDim.x;
    const int nbb = (v.nbf + bs - 1) / bs;
    const bool bnd = (int)blockIdx.x < nbb;
    const int f = bnd ? v.nfi + blockIdx.x * bs + threadIdx.x : (blockIdx.x - nbb) * bs + threadIdx.x;
    if (f >= (bnd ? v.nof : v.nfi)) return;
    const int inst = face_inst(v, f);
    if (stopped(v, inst)) return;
    const Gas& g = gas_of(v, inst);
    const int2 nb = v.fnb[f];
    if (bnd) {
        double cin[4] = {0.0, 0.0, 0.0, 0.0};
        if (v.fbc[f] == 1001) d4get(v.qc[nb.x], cin);
        bnd_face_flux<R>(v, g, f, nb.x, cin);
        return;
    }
    if constexpr (std::is_same<R, float>::value) {  // interior face of the mixed form: FP32 packs and geometry only
        const float4* A = v.packf + 4 * (size_t)nb.x;
        const float4* B = v.packf + 4 * (size_t)nb.y;
        const float4 qa = A[0], ga = A[1], ha = A[2], pa = A[3];
        const float4 qb = B[0], gb = B[1], hb = B[2], pb = B[3];
        const float4 d = v.fgeof[f], na = v.fnaf[f];
        const float zhi = 1.f / 3.f, zlo = 1.f - 1.f / 3.f;
        const float qi[4] = {qa.x, qa.y, qa.z, qa.w}, qo[4] = {qb.x, qb.y, qb.z, qb.w};
        const float gxi[4] = {ga.x, ga.y, ga.z, ga.w}, gyi[4] = {ha.x, ha.y, ha.z, ha.w};
        const float gxo[4] = {gb.x, gb.y, gb.z, gb.w}, gyo[4] = {hb.x, hb.y, hb.z, hb.w};
        const float phi_i[4] = {pa.x, pa.y, pa.z, pa.w}, phi_o[4] = {pb.x, pb.y, pb.z, pb.w};
        V4<float> ql, qr, F;
#pragma unroll
        for (int j = 0; j < 4; ++j) {  // recon (fvresidual.F90:235-247)
            const float beta = qo[j] - qi[j];
            ql[j] = qi[j] + 0.5f * phi_i[j] * (zhi * beta + zlo * (gxi[j] * d.x + gyi[j] * d.y));
            qr[j] = qo[j] + 0.5f * phi_o[j] * (zhi * -beta + zlo * (gxo[j] * d.z + gyo[j] * d.w));
        }
        bool ok = flux_dispatch<float>(g, na.x, na.y, na.z, ql, qr, F);
        if (!ok) set_err(v.err, UNS_ERR_NEG_SOUND_SPEED, f);
        v.fF[f] = make_double4((double)F[0], (double)F[1], (double)F[2], (double)F[3]);
    } else {
        const int in = nb.x, out = nb.y;
        const double2 n = v.fn[f];
        const double area = v.farea[f];
        const double2 fc = v.fcen[f];
        const double2 ci = v.cen[in], co = v.cen[out];
        double qi[4], gxi[4], gyi[4], phi_i[4], qo[4], gxo[4], gyo[4], phi_o[4];
        d4get(v.qp[in], qi);
        d4get(v.gx[in], gxi);
        d4get(v.gy[in], gyi);
        d4get(v.phi[in], phi_i);
        d4get(v.qp[out], qo);
        d4get(v.gx[out], gxo);
        d4get(v.gy[out], gyo);
        d4get(v.phi[out], phi_o);
        const double zhi = 1.0 / 3.0;
        double dl0 = fc.x - ci.x, dl1 = fc.y - ci.y;
        double dr0 = fc.x - co.x, dr1 = fc.y - co.y;
        V4<double> ql, qr, F;
#pragma unroll
        for (int j = 0; j < 4; ++j) {  // recon (fvresidual.F90:235-247)
            double alfa = gxi[j] * dl0 + gyi[j] * dl1;
            double beta = qo[j] - qi[j];
            ql[j] = qi[j] + 0.5 * phi_i[j] * (zhi * beta + (1.0 - zhi) * alfa);
            alfa = gxo[j] * dr0 + gyo[j] * dr1;
            beta = qi[j] - qo[j];
            qr[j] = qo[j] + 0.5 * phi_o[j] * (zhi * beta + (1.0 - zhi) * alfa);
        }
        bool ok = flux_dispatch<double>(g, n.x, n.y, area, ql, qr, F);
        if (!ok) set_err(v.err, UNS_ERR_NEG_SOUND_SPEED, f);
        v.fF[f] = make_double4(F[0], F[1], F[2], F[3]);
    }
}

// Sutherland viscosity of every interior cell (viscous_flux.F90:20-22,127-141).
__global__ void __launch_bounds__(kBlock) k_cell_mul(CCView v) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.noc) return;
    const int inst = cell_inst(v, i);
    if (inst < 0 || stopped(v, inst)) return;
    const Gas& g = gas_of(v, inst);
    double4 c = v.qc[i];
    Prim P = con2prim(g, c.x, c.y, c.z, c.w);
    double num = 1.0 + g.T_infd / g.SCONST;
    double den = P.t + g.T_infd / g.SCONST;
    v.mul[i] = (num / den) * pow(P.t, 1.5);
}

// Laminar viscous face flux (viscous_flux.F90:30-76), stored as flux*area.
__global__ void __launch_bounds__(kBlock) k_face_visc(CCView v) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= v.nof) return;
    const int inst = face_inst(v, f);
    if (stopped(v, inst)) return;
    const Gas& g = gas_of(v, inst);
    int2 nb = v.fnb[f];
    double2 n = v.fn[f];
    double area = v.farea[f];
    double mu = (nb.y < v.noc) ? 0.5 * (v.mul[nb.x] + v.mul[nb.y]) : v.mul[nb.x];
    v.fmu[f] = mu;
    double4 q = v.fq[f];
    double4 a = v.fgx[f], b = v.fgy[f];
    double2 t = v.fgT[f];
    double uvel = q.y, vvel = q.z;
    double ux = a.y, uy = b.y, vx = a.z, vy = b.z, tx = t.x, ty = t.y;
    const double two = 2.0, two_third = two / 3.0;
    double tauxx = two_third * (two * ux - vy);
    double tauxy = (uy + vx);
    double tauyy = two_third * (two * vy - ux);
    double factor = (g.gamma - 1.0) * g.m_inf * g.m_inf * g.prandtl;
    double qx = -(tx / factor), qy = -(ty / factor);
    double mr = mu / g.rey;
    double f1 = mr * ((uvel * tauxx + vvel * tauxy - qx) * n.x + (uvel * tauxy + vvel * tauyy - qy) * n.y);
    double f3 = mr * (tauxx * n.x + tauxy * n.y);
    double f4 = mr * (tauxy * n.x + tauyy * n.y);
    v.fV[f] = make_double4(f1 * area, 0.0 * area, f3 * area, f4 * area);
    if (f >= v.nfi) v.fwallv[f - v.nfi] = (v.fbc[f] == 1001) ? make_double2(f3 * area, f4 * area) : make_double2(0.0, 0.0);
}

// Residual gather in the reference's accumulation order, optionally fused
// with one RK3 stage (main.F90:92-101) and the block partials of the norm.
__device__ __forceinline__ void add4(double r[4], const double4& a) { r[0] = r[0] + a.x; r[1] = r[1] + a.y; r[2] = r[2] + a.z; r[3] = r[3] + a.w; }
__device__ __forceinline__ void sub4(double r[4], const double4& a) { r[0] = r[0] - a.x; r[1] = r[1] - a.y; r[2] = r[2] - a.z; r[3] = r[3] - a.w; }

__global__ void __launch_bounds__(kBlock) k_cell_res(CCView v, int irk, int partial) {
    if (stopped(v, block_inst(v))) return;  // blocks of cells are instance-pure
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double rr = 0.0;
    if (i < v.noc && cell_inst(v, i) >= 0) {
        const int k0 = v.cf_off[i], k1 = v.cf_off[i + 1];
        double r[4] = {0.0, 0.0, 0.0, 0.0};
        for (int k = k0; k < k1; ++k) {  // boundary faces first
            int f = v.cf[k] & FACE_MASK;
            if (f >= v.nfi) add4(r, v.fF[f]);
        }
        for (int k = k0; k < k1; ++k) {  // then interior faces
            int e = v.cf[k], f = e & FACE_MASK;
            if (f < v.nfi) { if (e & SIDE_BIT) sub4(r, v.fF[f]); else add4(r, v.fF[f]); }
        }
        if (v.laminar) {
            for (int k = k0; k < k1; ++k) {
                int e = v.cf[k], f = e & FACE_MASK;
                if (f < v.nfi && (e & SIDE_BIT)) add4(r, v.fV[f]); else sub4(r, v.fV[f]);
            }
        }
        v.res[i] = d4(r);
        if (irk > 0) {
            double a = rk3_a(irk), b = rk3_b(irk);
            double dtbyarea = v.dcv[i];  // dt / cv, formed once per time step
            double o[4], c[4], q[4];
            d4get(v.qc[i], c);
            if (v.mixed && irk == 1) {  // a = 0, b = 1
#pragma unroll
                for (int j = 0; j < 4; ++j) q[j] = c[j] - dtbyarea * r[j];
            } else {
                d4get(v.qold[i], o);
#pragma unroll
                for (int j = 0; j < 4; ++j) q[j] = a * o[j] + b * (c[j] - dtbyarea * r[j]);
            }
            v.qc[i] = d4(q);
        }
        if (partial) rr = r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3];
    }
    if (partial) {
        __shared__ double s[kBlock / 32];
        rr = warp_sum(rr);
        if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = rr;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int k = 0; k < kBlock / 32; ++k) t = t + s[k];
            v.partial[blockIdx.x] = t;
        }
    }
}

// The residual gather of the mixed form: FP64 accumulation of the face
// fluxes in the cell's face order (the first face initialises the sum), the
// RK stage with fused multiply-adds, and the FP64 norm partial reduced with
// one FP64 add per cell before the warp stage (FP64 issue, not bytes, bounds
// this kernel on GB300).  walls_done: the mixed form's one-pass step, where
// k_cell_rk23_wall has already advanced the wall cells through all three
// stages; they only contribute their residual to the norm here.
__global__ void __launch_bounds__(kBlock, 8) k_cell_res_mixed(CCView v, int irk, int partial, int walls_done) {
    if (stopped(v, block_inst(v))) return;  // blocks of cells are instance-pure
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double rr = 0.0;
    if (i < v.noc && cell_inst(v, i) >= 0) {
        double r[4] = {0.0, 0.0, 0.0, 0.0};
        if (walls_done && ((__ldg(v.bcell + (i >> 5)) >> (i & 31)) & 1u)) {
            d4get(v.res[i], r);  // a wall cell: its last-stage residual (k_cell_rk23_wall)
        } else {
            const int k0 = v.cf_off[i], k1 = v.cf_off[i + 1];
            auto add = [&](int k, int e, const double4& F) {
                const int f = e & FACE_MASK;
                const bool neg = f < v.nfi && (e & SIDE_BIT);
                if (k == k0) {  // sign flip on the bits: no FP64 instruction
                    const long long m = neg ? (long long)0x8000000000000000ULL : 0LL;
                    r[0] = __longlong_as_double(__double_as_longlong(F.x) ^ m);
                    r[1] = __longlong_as_double(__double_as_longlong(F.y) ^ m);
                    r[2] = __longlong_as_double(__double_as_longlong(F.z) ^ m);
                    r[3] = __longlong_as_double(__double_as_longlong(F.w) ^ m);
                } else {
                    const double s = neg ? -1.0 : 1.0;
                    r[0] = __fma_rn(s, F.x, r[0]); r[1] = __fma_rn(s, F.y, r[1]); r[2] = __fma_rn(s, F.z, r[2]); r[3] = __fma_rn(s, F.w, r[3]);
                }
            };
            if (k1 - k0 == 3) {  // a triangle: the three fluxes' gathers in flight together, summed in order
                const int e0 = v.cf[k0], e1 = v.cf[k0 + 1], e2 = v.cf[k0 + 2];
                const double4 F0 = v.fF[e0 & FACE_MASK], F1 = v.fF[e1 & FACE_MASK], F2 = v.fF[e2 & FACE_MASK];
                add(k0, e0, F0);
                add(k0 + 1, e1, F1);
                add(k0 + 2, e2, F2);
            } else {
                for (int k = k0; k < k1; ++k) {
                    const int e = v.cf[k];
                    add(k, e, v.fF[e & FACE_MASK]);
                }
            }
            if (v.laminar) {
                for (int k = k0; k < k1; ++k) {
                    const int e = v.cf[k], f = e & FACE_MASK;
                    const double4 V = v.fV[f];
                    const double s = (f < v.nfi && (e & SIDE_BIT)) ? 1.0 : -1.0;
                    r[0] = __fma_rn(s, V.x, r[0]); r[1] = __fma_rn(s, V.y, r[1]); r[2] = __fma_rn(s, V.z, r[2]); r[3] = __fma_rn(s, V.w, r[3]);
                }
            }
            v.res[i] = d4(r);
            if (irk > 0) {
                const double D = v.dcv[i];
                double c[4], q[4];
                d4get(v.qc[i], c);
#pragma unroll
                for (int j = 0; j < 4; ++j) q[j] = __fma_rn(-D, r[j], c[j]);
                if (irk > 1) {
                    const double a = rk3_a(irk), b = rk3_b(irk);
                    double o[4];
                    d4get(v.qold[i], o);
#pragma unroll
                    for (int j = 0; j < 4; ++j) q[j] = __fma_rn(a, o[j], b * q[j]);
                }
                v.qc[i] = d4(q);
            }
        }
        if (partial) rr = __fma_rn(r[3], r[3], __fma_rn(r[2], r[2], __fma_rn(r[1], r[1], r[0] * r[0])));
    }
    if (partial) {
        __shared__ double sh[kBlock];
        sh[threadIdx.x] = rr;
        __syncthreads();
        if (threadIdx.x < 32) {
            double t = sh[threadIdx.x];
            for (int k = threadIdx.x + 32; k < kBlock; k += 32) t = t + sh[k];
            t = warp_sum(t);
            if (threadIdx.x == 0) v.partial[blockIdx.x] = t;
        }
    }
}

// RK stages 2 and 3 of an inviscid step in one pass over the cells.  Those
// stages' interior and farfield face fluxes equal the first stage's: their
// inputs -- the cells' primitives, gradient and limiter -- are formed once
// per time step (main.F90:62-84) and the farfield ghost is built from them
// alone; only a wall ghost reads the stage's conserved state (slip_wall /
// NoSlip_wall, boundCond.F90:19-81).  So a cell without a wall face keeps the
// first stage's residual in both stages, and a wall cell's residual changes
// only through its own wall faces, whose fluxes its thread recomputes from
// the cell's stage state.  Each stage update and the last stage's norm
// partial are evaluated as in the stage-by-stage sequence (k_cell_res for the
// FP64 form, k_cell_res_mixed for the mixed form), so states, residuals,
// ghosts and norms are the same bit for bit.
template <bool kMixed>
__device__ __forceinline__ void rk_update(int irk, double D, const double o[4], const double r[4], double q[4]) {
    const double a = rk3_a(irk), b = rk3_b(irk);
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        if (kMixed) q[j] = __fma_rn(a, o[j], b * __fma_rn(-D, r[j], q[j]));
        else q[j] = a * o[j] + b * (q[j] - D * r[j]);
    }
}

// The residual of wall cell i at stage state q: its wall faces' fluxes
// recomputed (ghosts, wall force and fF written), the other faces' stored;
// with recompute false every face's stored flux (the first stage's sum).
template <class R>
__device__ __forceinline__ void wall_cell_res(const CCView& v, const Gas& g, int i, const double q[4], double r[4],
                                              bool recompute = true) {
    const int k0 = v.cf_off[i], k1 = v.cf_off[i + 1];
    auto flux = [&](int f) -> double4 {
        return (recompute && f >= v.nfi && v.fbc[f] == 1001) ? bnd_face_flux<R>(v, g, f, i, q) : v.fF[f];
    };
    if constexpr (std::is_same<R, float>::value) {  // k_cell_res_mixed's order
        for (int k = k0; k < k1; ++k) {
            const int e = v.cf[k], f = e & FACE_MASK;
            const double4 F = flux(f);
            const double s = (f < v.nfi && (e & SIDE_BIT)) ? -1.0 : 1.0;
            if (k == k0) { r[0] = s * F.x; r[1] = s * F.y; r[2] = s * F.z; r[3] = s * F.w; }
            else { r[0] = __fma_rn(s, F.x, r[0]); r[1] = __fma_rn(s, F.y, r[1]); r[2] = __fma_rn(s, F.z, r[2]); r[3] = __fma_rn(s, F.w, r[3]); }
        }
    } else {  // k_cell_res's order: boundary faces first
        r[0] = r[1] = r[2] = r[3] = 0.0;
        for (int k = k0; k < k1; ++k) {
            const int f = v.cf[k] & FACE_MASK;
            if (f >= v.nfi) add4(r, flux(f));
        }
        for (int k = k0; k < k1; ++k) {
            const int e = v.cf[k], f = e & FACE_MASK;
            if (f < v.nfi) { if (e & SIDE_BIT) sub4(r, v.fF[f]); else add4(r, v.fF[f]); }
        }
    }
}

// Stages 2 and 3 of cell i (instance inst): the stage updates and, for a
// wall cell, its residual in each stage; returns the squared residual that
// the last stage's norm takes.  kFrom1 (a wall cell of the mixed form): the
// first stage too, from the stored face fluxes (k_cell_res_mixed's sum and
// update).
template <class R, bool kWall, bool kFrom1 = false>
__device__ __forceinline__ double rk23_cell(const CCView& v, int i, int inst) {
    constexpr bool kMixed = std::is_same<R, float>::value;
    double r[4], q[4], o[4];
    d4get(v.qc[i], q);
    d4get(v.qold[i], o);
    const double D = v.dcv[i];
    if constexpr (kFrom1) {
        static_assert(kMixed && kWall, "the first stage here is the mixed form's");
        wall_cell_res<R>(v, gas_of(v, inst), i, q, r, false);
#pragma unroll
        for (int j = 0; j < 4; ++j) q[j] = __fma_rn(-D, r[j], q[j]);
    } else {
        d4get(v.res[i], r);
    }
    for (int irk = 2; irk <= 3; ++irk) {
        if (kWall) wall_cell_res<R>(v, gas_of(v, inst), i, q, r);
        rk_update<kMixed>(irk, D, o, r, q);
    }
    if (kWall) v.res[i] = d4(r);
    v.qc[i] = d4(q);
    if (kMixed) return __fma_rn(r[3], r[3], __fma_rn(r[2], r[2], __fma_rn(r[1], r[1], r[0] * r[0])));
    return r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3];
}

// The wall cells (v.wcell), one per thread in one-warp blocks so that their
// long FP64 chains spread over the SMs; they run before k_cell_rk23 (FP64
// form, stages 2-3) or k_cell_res_mixed (mixed form, all three stages).
template <class R, bool kFrom1>
__global__ void __launch_bounds__(32) k_cell_rk23_wall(CCView v) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= v.nwcell) return;
    const int i = v.wcell[t];
    const int inst = cell_inst(v, i);
    if (inst < 0 || stopped(v, inst)) return;
    rk23_cell<R, true, kFrom1>(v, i, inst);
}

// The residual of every wall cell (v.wcell) from the stored face fluxes, in
// the residual gather's order (uns_cc_fvresidual's cached form).
template <class R>
__global__ void __launch_bounds__(32) k_wall_res(CCView v) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= v.nwcell) return;
    const int i = v.wcell[t];
    const int inst = cell_inst(v, i);
    if (inst < 0 || stopped(v, inst)) return;
    const double q[4] = {0.0, 0.0, 0.0, 0.0};
    double r[4];
    wall_cell_res<R>(v, gas_of(v, inst), i, q, r, false);
    v.res[i] = d4(r);
}

// Every other cell: a stream over the stored residual and states; the wall
// cells contribute the last-stage residual k_cell_rk23_wall stored.  The norm
// partial is reduced as the stage-by-stage kernels reduce it.
template <class R>
__global__ void __launch_bounds__(kBlock) k_cell_rk23(CCView v) {
    constexpr bool kMixed = std::is_same<R, float>::value;
    if (stopped(v, block_inst(v))) return;  // blocks of cells are instance-pure
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int inst = i < v.noc ? cell_inst(v, i) : -1;
    double rr = 0.0;
    if (inst >= 0) {
        if ((__ldg(v.bcell + (i >> 5)) >> (i & 31)) & 1u) {
            double r[4];
            d4get(v.res[i], r);
            if (kMixed) rr = __fma_rn(r[3], r[3], __fma_rn(r[2], r[2], __fma_rn(r[1], r[1], r[0] * r[0])));
            else rr = r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + r[3] * r[3];
        } else {
            rr = rk23_cell<R, false>(v, i, inst);
        }
    }
    if (kMixed) {  // k_cell_res_mixed's block reduction
        __shared__ double sh[kBlock];
        sh[threadIdx.x] = rr;
        __syncthreads();
        if (threadIdx.x < 32) {
            double t = sh[threadIdx.x];
            for (int k = threadIdx.x + 32; k < kBlock; k += 32) t = t + sh[k];
            t = warp_sum(t);
            if (threadIdx.x == 0) v.partial[blockIdx.x] = t;
        }
    } else if (v.wpart) {  // one partial per warp (v.ninst == 0)
        rr = warp_sum(rr);
        if ((threadIdx.x & 31) == 0) v.partial[i >> 5] = rr;
    } else {  // k_cell_res's
        __shared__ double s[kBlock / 32];
        rr = warp_sum(rr);
        if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = rr;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int k = 0; k < kBlock / 32; ++k) t = t + s[k];
            v.partial[blockIdx.x] = t;
        }
    }
}

// One Jacobi sweep of cirs (ImpResiSmoothening.F90:27-44).
__global__ void __launch_bounds__(kBlock) k_cirs(CCView v, const double4* src, double4* dst, double eps) {
    if (stopped(v)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.noc) return;
    double s[4] = {0.0, 0.0, 0.0, 0.0};
    for (int k = v.cf_off[i]; k < v.cf_off[i + 1]; ++k) {
        int e = v.cf[k], f = e & FACE_MASK;
        if (f >= v.nfi) continue;
        int2 nb = v.fnb[f];
        add4(s, src[(e & SIDE_BIT) ? nb.x : nb.y]);
    }
    double den = 1.0 / (1.0 + eps * (double)v.nc2c[i]);
    double o[4];
    d4get(v.res0[i], o);
    double r[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) r[j] = (s[j] * eps + o[j]) * den;
    dst[i] = d4(r);
}

__global__ void __launch_bounds__(kBlock) k_rk_stage(CCView v, int irk) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.noc) return;
    double a = rk3_a(irk), b = rk3_b(irk);
    double dtbyarea = v.dt[i] / v.cv[i];
    double o[4], c[4], r[4], q[4];
    d4get(v.qold[i], o);
    d4get(v.qc[i], c);
    d4get(v.res[i], r);
#pragma unroll
    for (int j = 0; j < 4; ++j) q[j] = a * o[j] + b * (c[j] - dtbyarea * r[j]);
    v.qc[i] = d4(q);
}

__global__ void __launch_bounds__(kBlock) k_res_partial(CCView v) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double rr = 0.0;
    if (i < v.noc) {
        double4 r = v.res[i];
        rr = r.x * r.x + r.y * r.y + r.z * r.z + r.w * r.w;
    }
    __shared__ double s[kBlock / 32];
    rr = warp_sum(rr);
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = rr;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < kBlock / 32; ++k) t = t + s[k];
        v.partial[blockIdx.x] = t;
    }
}

// Deterministic final sum of the block partials; in the graph path it also
// records the history, the first-iteration normalisation and the stop flag
// (solution.F90:159-166, main.F90:57).
// Block partial k: stored, or the sum of its eight warp partials in warp
// order (v.wpart), the warps past the last cell counting zero as they do in
// a block's own sum.
__device__ __forceinline__ double block_partial(const CCView& v, int k) {
    if (!v.wpart) return v.partial[k];
    const int nw = (v.noc + 31) >> 5;
    double t = 0.0;
#pragma unroll
    for (int u = 0; u < kBlock / 32; ++u) t = t + (8 * k + u < nw ? v.partial[8 * k + u] : 0.0);
    return t;
}

__global__ void __launch_bounds__(kBlock) k_res_final(CCView v, int nparts, double* out) {
    const int inst = blockIdx.x;  // one block per instance
    if (stopped(v, inst)) return;
    const int k0 = v.ninst ? v.boff[inst] : 0;
    const int n = v.ninst ? v.boff[inst + 1] - k0 : nparts;
    __shared__ double s[kBlock];
    double t = 0.0;
    // eight partials loaded together, then added in the loop's order
    int k = threadIdx.x;
    for (; k + 7 * kBlock < n; k += 8 * kBlock) {
        double p[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) p[u] = block_partial(v, k0 + k + u * kBlock);
#pragma unroll
        for (int u = 0; u < 8; ++u) t = t + p[u];
    }
    for (; k < n; k += kBlock) t = t + block_partial(v, k0 + k);
    s[threadIdx.x] = t;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) s[threadIdx.x] = s[threadIdx.x] + s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const int nc = v.ninst ? v.ncell[inst] : v.noc;
        double fres = sqrt(s[0] / (double)nc / 4.0);
        if (out) out[inst] = fres;
        if (!isfinite(fres)) set_err(v.err, UNS_ERR_NAN, inst);
        if (v.iter) {
            int it = v.iter[inst];
            v.fres_hist[(size_t)inst * v.cfl_stride + it] = fres;
            if (it == 0 && v.first_iter) v.fres1[inst] = fres;
            double f1 = v.fres1[inst];
            double nf = (f1 >= 2.220446049250313e-16) ? fres / f1 : fres;
            const double mr = v.ninst ? v.minres[inst] : v.min_res;
            if (!(nf > mr) || v.err->code != 0) {
                v.done[inst] = 1;
                if (v.err->code != 0) v.err->iter = it;
            }
            v.iter[inst] = it + 1;
            // reset the encoded reductions for the next iteration
            for (int j = 0; j < 4; ++j) { v.minmax[8 * inst + j] = 0ULL; v.minmax[8 * inst + 4 + j] = ~0ULL; }
            v.dtmin[inst] = ~0ULL;
        }
    }
}

__global__ void k_reset_minmax(CCView v) {
    const int n = v.ninst ? v.ninst : 1;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        if (stopped(v, k)) continue;
        for (int j = 0; j < 4; ++j) { v.minmax[8 * k + j] = 0ULL; v.minmax[8 * k + 4 + j] = ~0ULL; }
        v.dtmin[k] = ~0ULL;
    }
}

// Sequential wall-force sums in face order (fvresidual.F90:99-100 then
// viscous_flux.F90:73-74).
__global__ void k_forces(CCView v, double* out) {
    double fx = 0.0, fy = 0.0;
#pragma unroll 8
    for (int k = 0; k < v.nbf; ++k)  // unrolled: loads in flight together, sums in order
        if (v.fbc[v.nfi + k] == 1001) { fx = fx + v.fwall[k].x; fy = fy + v.fwall[k].y; }
    if (v.laminar)
#pragma unroll 8
        for (int k = 0; k < v.nbf; ++k)
            if (v.fbc[v.nfi + k] == 1001) { fx = fx - v.fwallv[k].x; fy = fy - v.fwallv[k].y; }
    out[0] = fx;
    out[1] = fy;
}

__global__ void k_check_pos(CCView v) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.noc || cell_inst(v, i) < 0) return;
    double4 p = v.qp[i];
    if (p.x <= 0.0 || p.w <= 0.0) set_err(v.err, UNS_ERR_NONPOSITIVE, i);
}

__global__ void k_initialize(CCView v, double4 qinf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < v.ntot) {
        const int inst = cell_inst(v, i);
        v.qc[i] = (v.ninst && inst >= 0) ? v.qinfs[inst] : qinf;
        v.qp[i] = make_double4(0.0, 0.0, 0.0, 0.0); v.qT[i] = 0.0;
        v.qpf[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    if (i < v.noc) {
        v.phi[i] = make_double4(1.0, 1.0, 1.0, 1.0);
        v.packf[4 * (size_t)i + 3] = make_float4(1.f, 1.f, 1.f, 1.f);
    }
}

// Rebuilds every FP32 copy from the FP64 state, so a handle switched to the
// mixed form between calls starts from consistent copies.
__global__ void k_mirror_f32(CCView v) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < v.ntot) {
        double4 q = v.qp[i];
        float4 qf = make_float4((float)q.x, (float)q.y, (float)q.z, (float)q.w);
        v.qpf[i] = qf;
        if (i < v.noc) {
            double4 a = v.gx[i], b = v.gy[i], c = v.phi[i];
            v.packf[4 * (size_t)i] = qf;
            v.packf[4 * (size_t)i + 1] = make_float4((float)a.x, (float)a.y, (float)a.z, (float)a.w);
            v.packf[4 * (size_t)i + 2] = make_float4((float)b.x, (float)b.y, (float)b.z, (float)b.w);
            v.packf[4 * (size_t)i + 3] = make_float4((float)c.x, (float)c.y, (float)c.z, (float)c.w);
        }
    }
    if (i < v.nof) {
        double4 q = v.fq[i];
        v.fqf[i] = make_float4((float)q.x, (float)q.y, (float)q.z, (float)q.w);
        v.flaf[i] = (float)v.fla[i];
    }
    if (i < v.nop) {
        double4 q = v.pp[i];
        v.ppf[i] = make_float4((float)q.x, (float)q.y, (float)q.z, (float)q.w);
    }
}

// The gradient and phi of record of the mixed form (the per-cell pack)
// written back to the FP64 arrays.
__global__ void k_unpack_f32(CCView v) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.noc) return;
    const float4* A = v.packf + 4 * (size_t)i;
    const float4 a = A[1], b = A[2], c = A[3];
    v.gx[i] = make_double4(a.x, a.y, a.z, a.w);
    v.gy[i] = make_double4(b.x, b.y, b.z, b.w);
    v.phi[i] = make_double4(c.x, c.y, c.z, c.w);
}

// lusgs2 sweep pieces (lusgs.F90:245-318).  The per-cell neighbour sum keeps
// the reference c2f order, so the result equals the sequential sweep.
__device__ __forceinline__ void normal_flux_d(const Gas& g, const double4& qo, const double4& dq, double nx, double ny,
                                              double area, double out[4]) {
    Prim P = con2prim(g, qo.x, qo.y, qo.z, qo.w);
    double et = P.e * P.rho;
    double un = P.u * nx + P.v * ny;
    double f1[4] = {(et + P.p) * un, P.rho * un, 0.0, 0.0};
    f1[2] = f1[1] * P.u + P.p * nx;
    f1[3] = f1[1] * P.v + P.p * ny;
    Prim Q = con2prim(g, qo.x + dq.x, qo.y + dq.y, qo.z + dq.z, qo.w + dq.w);
    et = Q.e * Q.rho;
    un = Q.u * nx + Q.v * ny;
    double f2[4] = {(et + Q.p) * un, Q.rho * un, 0.0, 0.0};
    f2[2] = f2[1] * Q.u + Q.p * nx;
    f2[3] = f2[1] * Q.v + Q.p * ny;
#pragma unroll
    for (int k = 0; k < 4; ++k) out[k] = area * (f2[k] - f1[k]);
}

// normal_flux pieces (lusgs.F90:328-359): the flux of a state along (nx, ny).
__device__ __forceinline__ void nflux_prims(const double4& w, double et, double nx, double ny, double o[4]) {
    double un = w.y * nx + w.z * ny;
    o[0] = (et + w.w) * un;
    o[1] = w.x * un;
    o[2] = o[1] * w.y + w.w * nx;
    o[3] = o[1] * w.z + w.w * ny;
}

constexpr int kSweepBlock = 128;
// One sweep block per SM: one warp per SM sub-partition, so concurrently
// active items never share an FP64 unit.
constexpr int kSweepBlocksPerSM = 1;
constexpr double kOmega = 1.5;  // lusgs.F90:229

// Per LU-SGS call: everything a sweep item needs from a face that does not
// change during the sweeps, contiguous in schedule order:
//   rec[3r]   normal_flux of qold(nb) along the cell's outward normal
//             (lusgs.F90:328-346, the flux1 part)
//   rec[3r+1] (nx, ny, area, omega * la) with the cell's outward normal
//   rec[3r+2] (qold(nb).rho, 0, nb as integer bits, 0)
__global__ void __launch_bounds__(kBlock) k_cc_sweep_prep(CCView v) {
    if (stopped(v)) return;
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= v.nrec) return;
    const int c = v.rec_face[r], nb = v.rec_nb[r];
    const double2 n = v.fn[c];
    const double nx = v.rec_flip[r] ? -n.x : n.x, ny = v.rec_flip[r] ? -n.y : n.y;
    const double4 q = v.qold[nb];
    Prim P = con2prim(v.g, q.x, q.y, q.z, q.w);
    double o[4];
    nflux_prims(make_double4(P.rho, P.u, P.v, P.p), P.e * P.rho, nx, ny, o);
    v.rec[3 * (size_t)r] = d4(o);
    v.rec[3 * (size_t)r + 1] = make_double4(nx, ny, v.farea[c], kOmega * v.fla[c]);
    v.rec[3 * (size_t)r + 2] = make_double4(q.y, 0.0, __longlong_as_double((long long)nb), 0.0);
}

// Mixed-precision sweeps (delta form): per record, in FP32, the neighbour's
// old state and primitives and the face geometry (the cell's outward normal):
//   [rho, rho*u, rho*v, E] [u, v, p, u.n] [nx, ny, area, omega*la] [1, nb, 0, 0]
__global__ void __launch_bounds__(kBlock) k_cc_sweep_prep_mixed(CCView v) {
    if (stopped(v)) return;
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= v.nrec) return;
    const int c = v.rec_face[r], nb = v.rec_nb[r];
    const double2 n = v.fn[c];
    const double nx = v.rec_flip[r] ? -n.x : n.x, ny = v.rec_flip[r] ? -n.y : n.y;
    const double4 q = v.qold[nb];
    Prim P = con2prim(v.g, q.x, q.y, q.z, q.w);
    float4* rf = reinterpret_cast<float4*>(v.rec) + 4 * (size_t)r;
    rf[0] = make_float4((float)q.y, (float)q.z, (float)q.w, (float)q.x);
    rf[1] = make_float4((float)P.u, (float)P.v, (float)P.p, (float)(P.u * nx + P.v * ny));
    rf[2] = make_float4((float)nx, (float)ny, (float)v.farea[c], (float)(kOmega * v.fla[c]));
    rf[3] = make_float4(1.f, __int_as_float(nb), 0.f, 0.f);
}

__device__ __forceinline__ double pick4(int k, double a, double b, double c, double d) {
    return k == 0 ? a : (k == 1 ? b : (k == 2 ? c : d));
}

// Lanes of a sweep item: lane = 4 * slot + k, slot = the taken face (up to 8
// per round), k = the variable.  An FP64 instruction costs its SM
// sub-partition the same whatever the number of active lanes, so each item's
// arithmetic is spread over the lanes: the four flux components of up to
// eight faces in one pass, the per-variable sums and divides in lanes 0..3,
// and the three divisions of con2prim in lanes 0, 2 and 3 at once.
struct SweepIn {
    double f1, nx, ny, area, ol, rho_old;  // the slot's record; f1 = component k
    int nb;
    double D, o, r;  // lanes 0..3: the cell's diagonal, qold and res, variable k
};

__device__ __forceinline__ void sweep_load_face(const CCView& v, int rec, int k, SweepIn& x) {
    const double4* p = v.rec + 3 * (size_t)rec;
    x.f1 = reinterpret_cast<const double*>(p)[k];
    double4 b = p[1], c = p[2];
    x.nx = b.x; x.ny = b.y; x.area = b.z; x.ol = b.w;
    x.rho_old = c.x; x.nb = (int)__double_as_longlong(c.z);
}

// The cell's own diagonal, qold and res (variable `lane`) in lanes 0..3;
// benign operands elsewhere, so the warp-wide divides meet no 0 or inf.
__device__ __forceinline__ void own_load(const CCView& v, const int4& S, int lane, double& D, double& o, double& r) {
    if (lane < 4) {
        D = v.diag[S.x];
        o = reinterpret_cast<const double*>(&v.qold[S.x])[lane];
        if (S.y == 0) r = reinterpret_cast<const double*>(&v.res[S.x])[lane];
    } else {
        D = 1.0;
        o = 1.0;
        r = 0.0;
    }
}

__device__ __forceinline__ void sweep_load(const CCView& v, const int4& S, int lane, SweepIn& x) {
    if ((lane >> 2) < S.w) sweep_load_face(v, S.z + (lane >> 2), lane & 3, x);
    own_load(v, S, lane, x.D, x.o, x.r);
}

// One unconditional read of a neighbour record, issued early; the values are
// checked (record_set) only when the item that needs them starts.
__device__ __forceinline__ void peek_neighbour(const CCView& v, size_t rs, double w[4], double dq[4]) {
    const double2* pa = reinterpret_cast<const double2*>(v.rec_a + rs);
    const double2* pb = reinterpret_cast<const double2*>(v.rec_b + rs);
    double2 x0 = ld_relaxed2(pa), x1 = ld_relaxed2(pa + 1), x2 = ld_relaxed2(pb), x3 = ld_relaxed2(pb + 1);
    w[0] = x0.x; w[1] = x0.y; w[2] = x1.x; w[3] = x1.y;
    dq[0] = x2.x; dq[1] = x2.y; dq[2] = x3.x; dq[3] = x3.y;
}

__device__ __forceinline__ bool record_set(const double w[4], const double dq[4]) {
    bool ready = true;
#pragma unroll
    for (int j = 0; j < 4; ++j) ready = ready && !is_unset(w[j]) && !is_unset(dq[j]);
    return ready;
}

// lusgs2 sweeps (lusgs.F90:245-318) as one cooperative launch.  Each warp runs
// its own list of items (cell, pass) from the host-side list schedule, in
// order, loading the next item's inputs while it works on the current one.
// Per item, for each face whose neighbour precedes the cell in this pass
// (reference c2f order): the neighbour's values come from registers when the
// warp itself computed that neighbour last, else from its record (read early
// or polled); the face term area*(F(qold+dq) - F(qold)) - omega*lam*dq is
// formed per component; lanes 0..3 add the terms in c2f order and apply the
// diagonal; the new values are spread to all lanes, which keep the
// primitives of qold + dq for the next item while lanes 0 and 1 publish the
// record.  Every operation and operand order is the reference's.
__global__ void __launch_bounds__(kSweepBlock, 1) k_lusgs(CCView v, const int* __restrict__ woff) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int gw = blockIdx.x * (kSweepBlock / 32) + wib;
    const int slot = lane >> 2, k = lane & 3;
    if (stopped(v)) return;
    const int n = v.noc;
    const double gm1 = v.g.gamma - 1.0;
    const int kbeg = woff[gw], kend = woff[gw + 1];
    if (kbeg >= kend) return;
    const int4 none = make_int4(0, 0, 0, 0);
    int4 S = v.sched[kbeg];
    int4 Sn = kbeg + 1 < kend ? v.sched[kbeg + 1] : none;
    SweepIn X = {}, Xn = {};
    sweep_load(v, S, lane, X);
    int last = -1;  // code of the warp's previous item; its values below, in every lane
    double Lrho = 0.0, Lu = 0.0, Lv = 0.0, Lp = 0.0, Le = 0.0, L0 = 0.0, L1 = 0.0, L2 = 0.0, L3 = 0.0;
    // early read of the current item's first-round neighbour record, issued
    // during the previous item (usually already published)
    double Sw[4] = {0.0, 0.0, 0.0, 0.0}, Sdq[4] = {0.0, 0.0, 0.0, 0.0};
    bool spec = false;
    for (int kk = kbeg; kk < kend; ++kk) {
        const int4 Snn = kk + 2 < kend ? v.sched[kk + 2] : none;
        const int it = S.x, pass = S.y, ntake = S.w;
        double cres = 0.0;  // lanes 0..3: sum over faces of component k
        for (int base = 0; base < ntake; base += 8) {
            SweepIn E = X;
            if (base > 0 && base + slot < ntake) sweep_load_face(v, S.z + base + slot, k, E);
            bool ok = true;
            double t = 0.0;
            if (base + slot < ntake) {
                double w[8], rho;
                if (((E.nb << 1) | pass) == last) {
                    w[0] = Lu; w[1] = Lv; w[2] = Lp; w[3] = Le; w[4] = L0; w[5] = L1; w[6] = L2; w[7] = L3;
                    rho = Lrho;
                } else if (base == 0 && spec && record_set(Sw, Sdq)) {
                    w[0] = Sw[0]; w[1] = Sw[1]; w[2] = Sw[2]; w[3] = Sw[3];
                    w[4] = Sdq[0]; w[5] = Sdq[1]; w[6] = Sdq[2]; w[7] = Sdq[3];
                    rho = E.rho_old + w[5];
                } else {
                    const size_t rs = (size_t)pass * n + E.nb;
                    ok = poll_record2(v.rec_a + rs, v.rec_b + rs, w, v.err, v.wait_cycles);
                    rho = E.rho_old + w[5];
                }
                // normal_flux (lusgs.F90:348-357) component k, then the face term
                const double u = w[0], vv = w[1], p = w[2], et = w[3];
                const double un = u * E.nx + vv * E.ny;
                const double o1 = rho * un;
                const double prod = (k == 0 ? et + p : o1) * (k == 0 ? un : (k == 2 ? u : vv));
                const double pn = p * (k == 2 ? E.nx : E.ny);
                const double o = k == 1 ? o1 : (k == 0 ? prod : prod + pn);
                t = E.area * (o - E.f1) - E.ol * pick4(k, w[4], w[5], w[6], w[7]);
            }
            if (__ballot_sync(full, !ok)) return;  // a wait gave up; the error is recorded
            const int nr = min(8, ntake - base);
            int e = 0;
            if (base == 0) { cres = zero_plus(__shfl_sync(full, t, k)); e = 1; }  // 0.0 + t0, exact
            for (; e < nr; ++e) cres = cres + __shfl_sync(full, t, 4 * e + k);
        }
        // next item's inputs (independent of the sweep), issued once this
        // item's polls are done so they do not queue ahead of them
        if (kk + 1 < kend) sweep_load(v, Sn, lane, Xn);
        double r = X.r;
        bool ok = true;
        if (pass == 1 && lane < 4) {  // own lower
            if ((it << 1) == last) r = pick4(lane, L0, L1, L2, L3);
            else ok = poll_value(reinterpret_cast<const double*>(v.rec_b + it) + lane, r, v.err, v.wait_cycles);
        }
        if (__ballot_sync(full, !ok)) return;
        // lower / upper (lusgs.F90:276-279 / 314-317), component k in lane k
        const double d = pass == 0 ? (-r - 0.5 * cres) / X.D : r - 0.5 * cres / X.D;
        const double q = X.o + d;  // qold + dq (and, after the backward sweep, the new qc)
        spec = false;
        if (kk + 1 < kend && slot < Sn.w && ((Xn.nb << 1) | Sn.y) != ((it << 1) | pass)) {
            peek_neighbour(v, (size_t)Sn.y * n + Xn.nb, Sw, Sdq);
            spec = true;
        }
        // con2prim (pri.F90:13-37): rho = q1, then E/rho, rhou/rho, rhov/rho in lanes 0, 2, 3
        const double rho = __shfl_sync(full, q, 1);
        const double quo = q / rho;
        const double E0 = __shfl_sync(full, q, 0), Q2 = __shfl_sync(full, q, 2), Q3 = __shfl_sync(full, q, 3);
        // the four products of the pressure and the record as one
        // multiplication: lane 0 e*rho, lane 1 0.5*rho, lane 2 u*u, lane 3 v*v
        // (an FP64 instruction costs the warp the same for one lane or four)
        const double ma = lane == 1 ? 0.5 : quo, mb = lane < 2 ? rho : quo;
        const double pr = ma * mb;
        const double u = __shfl_sync(full, quo, 2), vv = __shfl_sync(full, quo, 3);
        const double erho = __shfl_sync(full, pr, 0), hrho = __shfl_sync(full, pr, 1);
        const double qq = __shfl_sync(full, pr, 2) + __shfl_sync(full, pr, 3);  // u*u + v*v
        const double p = gm1 * (E0 - hrho * qq);                                  // gm1*(E - 0.5*rho*qq)
        L0 = __shfl_sync(full, d, 0);
        L1 = __shfl_sync(full, d, 1);
        L2 = __shfl_sync(full, d, 2);
        L3 = __shfl_sync(full, d, 3);
        Lrho = rho; Lu = u; Lv = vv; Lp = p; Le = erho;
        last = (it << 1) | pass;
        const size_t slotr = (size_t)pass * n + it;
        if (last == v.skip_code) {  // test hook: this item publishes nothing and hands nothing on
            last = -1;
        } else {
            // Lane 0 stores (u, v, p, e*rho), lane 1 dq, as predicated stores
            // of one instruction sequence (lane-divergent branches around the
            // stores cost the sweep's critical path more than the stores).
            double2* dst = reinterpret_cast<double2*>(lane == 0 ? v.rec_a + slotr : v.rec_b + slotr);
            const double x0 = lane == 0 ? Lu : L0, x1 = lane == 0 ? Lv : L1;
            const double x2 = lane == 0 ? Lp : L2, x3 = lane == 0 ? Le : L3;
            const int st_ab = lane < 2;
            asm volatile(
                "{\n\t.reg .pred pa;\n\t"
                "setp.ne.s32 pa, %0, 0;\n\t"
                "@pa st.relaxed.gpu.global.v2.f64 [%1], {%2, %3};\n\t"
                "@pa st.relaxed.gpu.global.v2.f64 [%4], {%5, %6};\n\t}"
                :
                : "r"(st_ab), "l"(dst), "d"(x0), "d"(x1), "l"(dst + 1), "d"(x2), "d"(x3)
                : "memory");
            if (pass == 1 && lane == 2) v.qc[it] = make_double4(E0, rho, Q2, Q3);
        }
        S = Sn;
        Sn = Snn;
        X = Xn;
    }
}

// ------------------------------------------------------------ mixed (delta form)
// The FP32 sweep cannot form F(qold + dq) - F(qold) as a difference of two
// O(1) fluxes: near convergence that difference drowns in FP32 rounding and
// the solve stalls.  It forms the change directly from dq (dflux_k), so its
// FP32 error is relative to the change itself; items publish dq only (FP32
// for the face terms, FP64 for the cell's own backward step) and form no
// primitives.
struct SweepInM {
    float rho, ru, rv, E, u, v, p, un, nx, ny, area, ol;  // the slot's record
    int nb;
    double D, o, r;  // lanes 0..3: the reciprocal of the cell's diagonal, qold and res, variable k
};

__device__ __forceinline__ void sweep_load_face_m(const CCView& v, int rec, SweepInM& x) {
    const float4* p = reinterpret_cast<const float4*>(v.rec) + 4 * (size_t)rec;
    float4 a = p[0], b = p[1], c = p[2], d = p[3];
    x.rho = a.x; x.ru = a.y; x.rv = a.z; x.E = a.w;
    x.u = b.x; x.v = b.y; x.p = b.z; x.un = b.w;
    x.nx = c.x; x.ny = c.y; x.area = c.z; x.ol = c.w;
    x.nb = __float_as_int(d.y);
}

__device__ __forceinline__ void sweep_load_m(const CCView& v, const int4& S, int lane, SweepInM& x) {
    if ((lane >> 2) < S.w) sweep_load_face_m(v, S.z + (lane >> 2), x);
    own_load(v, S, lane, x.D, x.o, x.r);
    if (lane < 4) x.D = v.diaginv[S.x];  // the FP32 sweep multiplies by the FP64 reciprocal
}

// lusgs2 sweeps in the mixed form: the schedule, lanes, hand-offs and FP64
// sums of k_lusgs, the diagonal as its FP64 reciprocal (formed with the
// diagonal, off the sweep's critical path); FP32 delta-form face terms.
__global__ void __launch_bounds__(kSweepBlock, 1) k_lusgs_mixed(CCView v, const int* __restrict__ woff) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int gw = blockIdx.x * (kSweepBlock / 32) + wib;
    const int slot = lane >> 2, k = lane & 3;
    if (stopped(v)) return;
    const int n = v.noc;
    const float gm1 = (float)(v.g.gamma - 1.0);
    const float4* recf = reinterpret_cast<const float4*>(v.rec_a);
    const int kbeg = woff[gw], kend = woff[gw + 1];
    if (kbeg >= kend) return;
    const int4 none = make_int4(0, 0, 0, 0);
    int4 S = v.sched[kbeg];
    int4 Sn = kbeg + 1 < kend ? v.sched[kbeg + 1] : none;
    SweepInM X = {}, Xn = {};
    sweep_load_m(v, S, lane, X);
    int last = -1;
    float LF[4] = {0.f, 0.f, 0.f, 0.f};             // previous item's dq (FP32)
    double L0 = 0.0, L1 = 0.0, L2 = 0.0, L3 = 0.0;  // and in FP64
    float Sf[4] = {0.f, 0.f, 0.f, 0.f};
    bool spec = false;
    for (int kk = kbeg; kk < kend; ++kk) {
        const int4 Snn = kk + 2 < kend ? v.sched[kk + 2] : none;
        const int it = S.x, pass = S.y, ntake = S.w;
        double cres = 0.0;
        for (int base = 0; base < ntake; base += 8) {
            SweepInM E = X;
            if (base > 0 && base + slot < ntake) sweep_load_face_m(v, S.z + base + slot, E);
            bool ok = true;
            double t = 0.0;
            if (base + slot < ntake) {
                float dq[4];
                if (((E.nb << 1) | pass) == last) {
                    dq[0] = LF[0]; dq[1] = LF[1]; dq[2] = LF[2]; dq[3] = LF[3];
                } else if (base == 0 && spec && set_f4(Sf)) {
                    dq[0] = Sf[0]; dq[1] = Sf[1]; dq[2] = Sf[2]; dq[3] = Sf[3];
                } else {
                    ok = poll_f4(recf + (size_t)pass * n + E.nb, dq, v.err, v.wait_cycles);
                }
                const float df = dflux_k(E, gm1, dq, k);
                const float dqk = k == 0 ? dq[0] : (k == 1 ? dq[1] : (k == 2 ? dq[2] : dq[3]));
                t = (double)(E.area * df - E.ol * dqk);
            }
            if (__ballot_sync(full, !ok)) return;
            const int nr = min(8, ntake - base);
            int e = 0;
            if (base == 0) { cres = zero_plus(__shfl_sync(full, t, k)); e = 1; }  // 0.0 + t0, exact
            for (; e < nr; ++e) cres = cres + __shfl_sync(full, t, 4 * e + k);
        }
        if (kk + 1 < kend) sweep_load_m(v, Sn, lane, Xn);
        double r = X.r;
        bool ok = true;
        if (pass == 1 && lane < 4) {  // own lower
            if ((it << 1) == last) r = pick4(lane, L0, L1, L2, L3);
            else ok = poll_value(reinterpret_cast<const double*>(v.rec_b + it) + lane, r, v.err, v.wait_cycles);
        }
        if (__ballot_sync(full, !ok)) return;
        const double d = pass == 0 ? (-r - 0.5 * cres) * X.D : r - 0.5 * cres * X.D;
        const double q = X.o + d;
        spec = false;
        if (kk + 1 < kend && slot < Sn.w && ((Xn.nb << 1) | Sn.y) != ((it << 1) | pass)) {
            peek_f4(recf + (size_t)Sn.y * n + Xn.nb, Sf);
            spec = true;
        }
        const float df = (float)d;
        LF[0] = __shfl_sync(full, df, 0);
        LF[1] = __shfl_sync(full, df, 1);
        LF[2] = __shfl_sync(full, df, 2);
        LF[3] = __shfl_sync(full, df, 3);
        L0 = __shfl_sync(full, d, 0);
        L1 = __shfl_sync(full, d, 1);
        L2 = __shfl_sync(full, d, 2);
        L3 = __shfl_sync(full, d, 3);
        const double Q0 = __shfl_sync(full, q, 0), Q1 = __shfl_sync(full, q, 1), Q2 = __shfl_sync(full, q, 2),
                     Q3 = __shfl_sync(full, q, 3);
        last = (it << 1) | pass;
        const size_t slotr = (size_t)pass * n + it;
        if (last == v.skip_code) {  // test hook: this item publishes nothing and hands nothing on
            last = -1;
        } else {
            publish_mixed(lane, reinterpret_cast<float4*>(v.rec_a) + slotr, reinterpret_cast<double2*>(v.rec_b + slotr), LF,
                          L0, L1, L2, L3);
            if (pass == 1 && lane == 2) v.qc[it] = make_double4(Q0, Q1, Q2, Q3);
        }
        S = Sn;
        Sn = Snn;
        X = Xn;
    }
}

}  // namespace

// ====================================================================== handle

namespace {

int check_dev_err(uns_cc_handle* h) {
    DevErr e;
    UNS_CUDA(cudaMemcpyAsync(&e, h->v.err, sizeof(DevErr), cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    if (e.code != 0) {
        const char* what = e.code == UNS_ERR_NEG_SOUND_SPEED ? "Roe scheme: sonic speed is negative at face "
                           : e.code == UNS_ERR_NONPOSITIVE  ? "Density/pressure is negative at cell "
                           : e.code == UNS_ERR_MESH         ? "ggfc,gradtrixy: -ve area at face "
                           : e.code == UNS_ERR_TIMEOUT      ? "bounded device wait timed out in block "
                                                            : "device error at ";
        set_last_error(std::string(what) + std::to_string(e.index));
        int code = e.code;
        DevErr z = {0, 0, 0, 0};
        UNS_CUDA(cudaMemcpyAsync(h->v.err, &z, sizeof(DevErr), cudaMemcpyHostToDevice, h->stream));
        UNS_CUDA(cudaStreamSynchronize(h->stream));
        return code;
    }
    return UNS_OK;
}

// Build the forward/backward level schedules of the lusgs2 sweeps: a cell
// waits for every interior neighbour that precedes it in sweep order.

void launch_cfg(int n, dim3& g, dim3& b) { b = dim3(kBlock); g = dim3(std::max(1, nblocks(n))); }

#define LAUNCH(kern, n, ...)                                                         \
    do {                                                                             \
        dim3 g_, b_;                                                                 \
        launch_cfg((n), g_, b_);                                                     \
        kern<<<g_, b_, 0, h->stream>>>(__VA_ARGS__);                                 \
        UNS_CUDA(cudaGetLastError());                                                \
    } while (0)

int enqueue_minmax(uns_cc_handle* h, CCView& v) {
    k_reset_minmax<<<1, 32, 0, h->stream>>>(v);
    UNS_CUDA(cudaGetLastError());
    LAUNCH(k_begin, v.ntot, v, (int)BEGIN_MINMAX);
    return UNS_OK;
}

// k_cell_grad, or its FP32 form for a handle in the mixed form.
// k_face_conv's grid: the boundary faces' blocks, then the interior faces'.
#define LAUNCH_FACE_CONV(R, v)                                                                     \
    do {                                                                                           \
        const int bs_ = (v).blk_face;                                                              \
        const int nb_ = std::max(1, ((v).nbf + bs_ - 1) / bs_ + ((v).nfi + bs_ - 1) / bs_);        \
        k_face_conv<R><<<nb_, bs_, 0, h->stream>>>(v);                                             \
        UNS_CUDA(cudaGetLastError());                                                              \
    } while (0)

// A launch over n items with block size bs.
#define LAUNCH_BS(kern, n, bs, ...)                                                                \
    do {                                                                                           \
        const int bs_ = (bs);                                                                      \
        kern<<<std::max(1, (int)(((n) + bs_ - 1) / bs_)), bs_, 0, h->stream>>>(__VA_ARGS__);       \
        UNS_CUDA(cudaGetLastError());                                                              \
    } while (0)

// Block size of a per-element kernel whose threads are independent (no
// block-level reduction): kBlock, halved down to one warp while the launch
// would have fewer than two blocks per SM, so that a small mesh spreads its
// FP64 work over every SM sub-partition instead of stacking warps on a few
// SMs (meshes above about 2 x 256 x SMs elements keep kBlock).  The
// per-element arithmetic, and so every result, is the same at any width.
inline int spread_bs(const uns_cc_handle* h, int n) {
    int bs = kBlock;
    while (bs > 32 && (n + bs - 1) / bs < 2 * h->nsm) bs >>= 1;
    return bs;
}
#define LAUNCH_SPREAD(kern, n, ...) LAUNCH_BS(kern, (n), spread_bs(h, (n)), __VA_ARGS__)

#define LAUNCH_CELL_GRAD(v, flags, cfl)                                                 \
    do {                                                                               \
        if ((v).mixed) LAUNCH(k_cell_grad_mixed, (v).noc, (v), (int)(flags), (cfl));   \
        else LAUNCH_SPREAD(k_cell_grad, (v).noc, (v), (int)(flags), (cfl));            \
    } while (0)

int enqueue_gradient(uns_cc_handle* h, CCView& v, int extra_flags, double cfl, bool do_reduce) {
    if (v.grad_type == UNS_GRAD_GGFC) LAUNCH(k_face_ggfc, v.nof, v);
    int flags = CG_GRAD | extra_flags | (v.ilimit ? CG_LIM : 0);
    if (v.ilimit && do_reduce) { int rc = enqueue_minmax(h, v); if (rc) return rc; }
    LAUNCH_CELL_GRAD(v, flags, cfl);
    return UNS_OK;
}

double epsirs_of(const uns_cc_handle* h, double cfl) {
    double r = cfl / h->P.cfl_max;
    return std::max(0.25 * (r * r - 1.0), 0.0);
}

// Whether the main loop's RK3 step runs stages 2 and 3 as one pass over the
// cells (k_cell_rk23): an inviscid flow without a smoothing sweep (a viscous
// stage recomputes the cell gradient and viscosity from the stage's state; a
// smoothing sweep replaces the residual that the pass reuses).
bool rk23_in_one_pass(const uns_cc_handle* h, const CCView& v, double cfl) {
    const double eps = v.irs ? epsirs_of(h, cfl) : 0.0;
    return h->P.time_mode == UNS_TIME_RK3 && !v.laminar && !(v.irs && eps > 0.0);
}

// Whether the step forms the face averages and radii inside the cell
// gradient pass (k_cell_grad_side): the mixed form with the Green-Gauss
// gradient of an inviscid flow under RK3 (the LU-SGS prep reads the FP64 face
// radii that k_face_prim_spec writes).
bool grad_by_sides(const uns_cc_handle* h, const CCView& v) {
    return v.mixed && v.sideg != nullptr && h->P.time_mode == UNS_TIME_RK3;
}

// uns_cc_fvresidual when only the wall ghosts can have changed since the last
// call that computed every face (same primitives, gradient and limiter; the
// reference main loop's RK stages 2 and 3): the boundary faces' fluxes and
// the wall cells' residuals; every other cell keeps the residual it has.
int enqueue_wall_res(uns_cc_handle* h, CCView& v) {
    const int nbb = (v.nbf + v.blk_face - 1) / v.blk_face;  // k_face_conv's boundary blocks come first
    if (nbb == 0) return UNS_OK;
    if (v.mixed) k_face_conv<float><<<nbb, v.blk_face, 0, h->stream>>>(v);
    else k_face_conv<double><<<nbb, v.blk_face, 0, h->stream>>>(v);
    UNS_CUDA(cudaGetLastError());
    if (v.nwcell > 0) {
        const int nb = (v.nwcell + 31) / 32;
        if (v.mixed) k_wall_res<float><<<nb, 32, 0, h->stream>>>(v);
        else k_wall_res<double><<<nb, 32, 0, h->stream>>>(v);
        UNS_CUDA(cudaGetLastError());
    }
    return UNS_OK;
}

// The wall cells' stages: 2-3 in the FP64 form, 1-3 in the mixed form.
// Whether the FP64 k_cell_rk23 of this handle runs spread over the SMs with
// per-warp norm partials: one case (no packed instances) on a small mesh.
inline bool rk23_warp_partials(const uns_cc_handle* h, const CCView& v) {
    return v.ninst == 0 && spread_bs(h, v.noc) < kBlock;
}

// k_res_final's view after the FP64 one-pass RK stages.
inline CCView final_view(const uns_cc_handle* h, const CCView& v) {
    CCView w = v;
    w.wpart = rk23_warp_partials(h, v) ? 1 : 0;
    return w;
}

int enqueue_wall_rk(uns_cc_handle* h, CCView& v) {
    if (v.nwcell == 0) return UNS_OK;
    const int nb = (v.nwcell + 31) / 32;
    if (v.mixed) k_cell_rk23_wall<float, true><<<nb, 32, 0, h->stream>>>(v);
    else k_cell_rk23_wall<double, false><<<nb, 32, 0, h->stream>>>(v);
    UNS_CUDA(cudaGetLastError());
    return UNS_OK;
}

// RK stages 2 and 3 of the FP64 form in one pass over the cells: the wall
// cells first.
int enqueue_rk23(uns_cc_handle* h, CCView& v) {
    int rc = enqueue_wall_rk(h, v);
    if (rc) return rc;
    if (rk23_warp_partials(h, v)) {
        CCView w = v;
        w.wpart = 1;
        LAUNCH_SPREAD(k_cell_rk23<double>, v.noc, w);
    } else {
        LAUNCH(k_cell_rk23<double>, v.noc, v);
    }
    return UNS_OK;
}

// fvresidual as a kernel sequence; irk > 0 fuses that RK stage into the
// residual gather (only when no smoothing sweep sits in between).
int enqueue_fvresidual(uns_cc_handle* h, CCView& v, double cfl, int irk, int partial, bool* fused) {
    if (h->P.precision == UNS_PREC_MIXED) LAUNCH_FACE_CONV(float, v);
    else LAUNCH_FACE_CONV(double, v);
    if (v.laminar) {
        LAUNCH(k_cell_mul, v.noc, v);
        if (v.grad_type != UNS_GRAD_GGFC) {
            CCView w = v;
            w.grad_type = UNS_GRAD_GGFC;
            int rc = enqueue_gradient(h, w, 0, cfl, true);
            if (rc) return rc;
        }
        LAUNCH(k_face_visc, v.nof, v);
    }
    double eps = v.irs ? epsirs_of(h, cfl) : 0.0;
    // With eps == 0 both smoothing sweeps reproduce the residual exactly
    // ((0*x + r) * 1 == r for finite x), so they are launched only for eps > 0.
    bool smooth = v.irs && eps > 0.0;
    *fused = !smooth && irk > 0;
    if (v.mixed) LAUNCH(k_cell_res_mixed, v.noc, v, *fused ? irk : 0, (partial && !smooth) ? 1 : 0, 0);
    else if ((partial && !smooth) || v.ninst) LAUNCH(k_cell_res, v.noc, v, *fused ? irk : 0, (partial && !smooth) ? 1 : 0);
    else LAUNCH_SPREAD(k_cell_res, v.noc, v, *fused ? irk : 0, 0);
    if (smooth) {
        UNS_CUDA(cudaMemcpyAsync(v.res0, v.res, sizeof(double4) * v.noc, cudaMemcpyDeviceToDevice, h->stream));
        LAUNCH(k_cirs, v.noc, v, (const double4*)v.res0, v.restmp, eps);
        LAUNCH(k_cirs, v.noc, v, (const double4*)v.restmp, v.res, eps);
        if (partial) LAUNCH(k_res_partial, v.noc, v);
    }
    return UNS_OK;
}

int enqueue_lusgs(uns_cc_handle* h, CCView& v) {
    const bool mixed = h->P.precision != UNS_PREC_FP64;  // FP32 sweep arithmetic
    if (v.nrec > 0) {
        if (mixed) LAUNCH(k_cc_sweep_prep_mixed, v.nrec, v);
        else LAUNCH(k_cc_sweep_prep, v.nrec, v);
    }
    const long long n2 = 2LL * v.noc * 2;  // double2 per record array
    if (mixed)
        k_fill_unset_f<<<std::min<long long>(nblocks(2LL * v.noc), 4096), kBlock, 0, h->stream>>>((float4*)v.rec_a,
                                                                                                   2LL * v.noc);
    else
        k_fill_unset<<<std::min<long long>(nblocks(n2), 4096), kBlock, 0, h->stream>>>((double2*)v.rec_a, n2);
    k_fill_unset<<<std::min<long long>(nblocks(n2), 4096), kBlock, 0, h->stream>>>((double2*)v.rec_b, n2);
    UNS_CUDA(cudaGetLastError());
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(h->coop_blocks);
    cfg.blockDim = dim3(kSweepBlock);
    cfg.stream = h->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (mixed) UNS_CUDA(cudaLaunchKernelEx(&cfg, k_lusgs_mixed, v, (const int*)h->woff));
    else UNS_CUDA(cudaLaunchKernelEx(&cfg, k_lusgs, v, (const int*)h->woff));
    return UNS_OK;
}

// The main-loop body (main.F90:60-115) as one kernel sequence.
int enqueue_iteration(uns_cc_handle* h, CCView& v, double cfl_for_eps) {
    int rc;
    k_reset_minmax<<<1, 32, 0, h->stream>>>(v);
    UNS_CUDA(cudaGetLastError());
    int bflags = BEGIN_PRIM | BEGIN_OLD | BEGIN_POS | (v.ilimit ? BEGIN_MINMAX : 0);
    LAUNCH(k_begin, v.ntot, v, bflags);
    LAUNCH_BS(k_vertex_avg, v.nop, v.blk_vert, v);
    const int gflags = CG_DT | CG_GRAD | (v.ilimit ? CG_LIM : 0) | (h->P.time_mode == UNS_TIME_RK3 ? 0 : CG_DIAG);
    if (grad_by_sides(h, v)) {
        LAUNCH_BS(k_cell_grad_side, v.noc, v.blk_grad, v, gflags, 0.0);
    } else {
        LAUNCH_SPREAD(k_face_prim_spec, v.nof, v);
        if (v.grad_type == UNS_GRAD_GGFC) LAUNCH(k_face_ggfc, v.nof, v);
        LAUNCH_CELL_GRAD(v, gflags, 0.0);
    }
    if (rk23_in_one_pass(h, v, cfl_for_eps) && v.mixed) {
        // Mixed form: the wall cells through all three stages, then every other
        // cell's update and the norm.  A cell without a wall face has the same
        // residual r in all three stages, and then the RK3 stages (main.F90:
        // 92-101, a = 0, 3/4, 1/3; b = 1, 1/4, 2/3) give, with D = dt/cv,
        //   q1 = qold - D r,  q2 = 3/4 qold + 1/4 (q1 - D r) = qold - D r / 2,
        //   q3 = 1/3 qold + 2/3 (q2 - D r) = qold - D r = q1
        // in exact arithmetic; this form keeps the FP64 q1 (it differs from the
        // three rounded stage updates in the last bits, far below the FP32 face
        // arithmetic).  The FP64 form evaluates both stage updates in the
        // reference's operation order (k_cell_rk23).
        LAUNCH_FACE_CONV(float, v);
        if ((rc = enqueue_wall_rk(h, v))) return rc;
        LAUNCH(k_cell_res_mixed, v.noc, v, 1, 1, 1);
    } else if (rk23_in_one_pass(h, v, cfl_for_eps)) {
        bool fused = false;
        if ((rc = enqueue_fvresidual(h, v, cfl_for_eps, 1, 0, &fused))) return rc;
        if ((rc = enqueue_rk23(h, v))) return rc;
        k_res_final<<<std::max(1, v.ninst), kBlock, 0, h->stream>>>(final_view(h, v), h->nparts, nullptr);
        UNS_CUDA(cudaGetLastError());
        return UNS_OK;
    } else if (h->P.time_mode == UNS_TIME_RK3) {
        for (int irk = 1; irk <= 3; ++irk) {
            bool fused = false;
            if ((rc = enqueue_fvresidual(h, v, cfl_for_eps, irk, irk == 3, &fused))) return rc;
            if (!fused) LAUNCH(k_rk_stage, v.noc, v, irk);
        }
    } else {
        bool fused = false;
        if ((rc = enqueue_fvresidual(h, v, cfl_for_eps, 0, 1, &fused))) return rc;
        if ((rc = enqueue_lusgs(h, v))) return rc;
    }
    k_res_final<<<std::max(1, v.ninst), kBlock, 0, h->stream>>>(v, h->nparts, nullptr);
    UNS_CUDA(cudaGetLastError());
    return UNS_OK;
}

}  // namespace

namespace uns {

int cc_check_dev_err(uns_cc_handle* h) { return check_dev_err(h); }

// The RK3 main-loop body of enqueue_iteration / enqueue_fvresidual with the
// limiter frozen (the view's ilimit cleared, so phi keeps its values) and a
// fixed CFL, calling `hook` where the adjoint records its linearisation
// points.  Residual smoothing is not part of it (the caller checks that its
// eps is 0).
int cc_record_iteration(uns_cc_handle* h, double cfl, CCRecHook hook, void* ctx) {
    CCView v = h->v;
    v.ilimit = 0;
    v.cfl_sched = nullptr;
    v.iter = nullptr;
    v.done = nullptr;
    int rc;
    LAUNCH(k_begin, v.ntot, v, (int)(BEGIN_PRIM | BEGIN_OLD | BEGIN_POS));
    LAUNCH_BS(k_vertex_avg, v.nop, v.blk_vert, v);
    LAUNCH_SPREAD(k_face_prim_spec, v.nof, v);
    if (v.grad_type == UNS_GRAD_GGFC) LAUNCH(k_face_ggfc, v.nof, v);
    LAUNCH_SPREAD(k_cell_grad, v.noc, v, (int)(CG_DT | CG_GRAD), cfl);
    if ((rc = hook(h, REC_AFTER_START, 0, ctx))) return rc;
    for (int irk = 1; irk <= 3; ++irk) {
        if ((rc = hook(h, REC_BEFORE_FACE_CONV, irk, ctx))) return rc;
        LAUNCH_FACE_CONV(double, v);
        if (v.laminar) {
            if ((rc = hook(h, REC_BEFORE_CELL_MUL, irk, ctx))) return rc;
            LAUNCH(k_cell_mul, v.noc, v);
            if (v.grad_type != UNS_GRAD_GGFC) {
                CCView w = v;
                w.grad_type = UNS_GRAD_GGFC;
                LAUNCH(k_face_ggfc, w.nof, w);
                LAUNCH_SPREAD(k_cell_grad, w.noc, w, (int)CG_GRAD, cfl);
            }
            LAUNCH(k_face_visc, v.nof, v);
            if ((rc = hook(h, REC_AFTER_FACE_VISC, irk, ctx))) return rc;
        }
        LAUNCH(k_cell_res, v.noc, v, irk, 0);
    }
    return check_dev_err(h);
}

}  // namespace uns

// Gas constants of one case: math + initialize (CCFVM/solution.F90:4-84),
// and its freestream conserved state.
static Gas make_gas(const uns_params* p, double4* qinf) {
    Gas g;
    g.gamma = 1.4;
    g.gamma1 = g.gamma - 1.0;
    double pi = 4.0 * std::atan(1.0);
    double aoa = p->aoa_deg * pi / 180.0;
    double q1 = 1.0, q2 = std::cos(aoa) * 1.0, q3 = std::sin(aoa) * 1.0;
    g.p_inf = 1.0 / (g.gamma * p->m_inf * p->m_inf);
    double q0 = g.p_inf / (g.gamma - 1.0) + 0.5;
    g.r_inf = q1;
    g.a_inf = std::sqrt(g.gamma * g.p_inf / g.r_inf);
    g.u_inf = q2 / q1;
    g.v_inf = q3 / q1;
    g.m_inf = p->m_inf;
    g.znd = 1.0 / (g.gamma * p->m_inf * p->m_inf);
    g.T_infd = 300.0;
    g.SCONST = 110.4;
    g.t_wall = p->t_wall / g.T_infd;
    g.rey = p->rey;
    g.prandtl = 0.72;
    g.vll = (p->flow_type != UNS_FLOW_INVISCID) ? 2.0 * g.gamma / (g.prandtl * p->rey * 0.25) : 0.0;
    g.mref = std::max((double)0.32f, 0.5 * p->m_inf);
    g.flux = p->flux_type;
    g.flow = p->flow_type;
    g.iwall = p->iwall;
    *qinf = make_double4(q0, q1, q2, q3);
    return g;
}

static int create_impl(const uns_cc_mesh* m, const uns_params* p, bool lusgs_schedule, uns_cc_handle** out);
static int grow_schedule(uns_cc_handle* h, int cap);
static int iterate_graph(uns_cc_handle* h, int niter, const double* cfl, int first_iter, double* fres_raw, int* done_iters);

// ====================================================================== C-ABI
extern "C" {

int uns_cc_create(const uns_cc_mesh* m, const uns_params* p, uns_cc_handle** out) {
    return create_impl(m, p, true, out);
}

}  // extern "C"

static int create_impl(const uns_cc_mesh* m, const uns_params* p, bool lusgs_schedule, uns_cc_handle** out) {
    if (!m || !p || !out) { set_last_error("uns_cc_create: null argument"); return UNS_ERR_ARG; }
    *out = nullptr;
    if (m->nop <= 0 || m->noc <= 0 || m->nfi < 0 || m->nbf < 0) { set_last_error("uns_cc_create: bad sizes"); return UNS_ERR_ARG; }
    if (p->flux_type < 0 || p->flux_type > 3 || p->grad_type < 0 || p->grad_type > 2 || p->flow_type < 0 ||
        p->flow_type > 1 || p->time_mode < 0 || p->time_mode > 1 || !(p->m_inf > 0.0) ||
        p->precision < UNS_PREC_FP64 || p->precision > UNS_PREC_MIXED_SWEEP) {
        set_last_error("uns_cc_create: bad parameters");
        return UNS_ERR_ARG;
    }
    const int nop = m->nop, noc = m->noc, nfi = m->nfi, nbf = m->nbf, nof = nfi + nbf, ntot = noc + nbf;
    // Validate indices on the host before anything reaches the device.
    for (int f = 0; f < nof; ++f) {
        bool ok = m->fin[f] >= 0 && m->fin[f] < noc && m->fp1[f] >= 0 && m->fp1[f] < nop && m->fp2[f] >= 0 && m->fp2[f] < nop;
        ok = ok && (f < nfi ? (m->fout[f] >= 0 && m->fout[f] < noc) : (m->fout[f] == noc + (f - nfi)));
        if (!ok) { set_last_error("uns_cc_create: face " + std::to_string(f) + " has an out-of-range index"); return UNS_ERR_MESH; }
    }
    for (int i = 0; i < nop; ++i)
        if (m->v2c_off[i] > m->v2c_off[i + 1]) { set_last_error("uns_cc_create: bad v2c"); return UNS_ERR_MESH; }
    for (int k = 0; k < m->v2c_off[nop]; ++k)
        if (m->v2c[k] < 0 || m->v2c[k] >= ntot) { set_last_error("uns_cc_create: v2c index out of range"); return UNS_ERR_MESH; }
    for (int i = 0; i < noc; ++i)
        for (int k = m->c2f_off[i]; k < m->c2f_off[i + 1]; ++k)
            if (m->c2f[k] < 0 || m->c2f[k] >= nof) { set_last_error("uns_cc_create: c2f index out of range"); return UNS_ERR_MESH; }

    uns_cc_handle* h = new uns_cc_handle();
    h->P = *p;
    int rc = UNS_OK;
    auto fail = [&](int code) { uns_cc_destroy(h); return code; };
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_last_error("uns_cc_create: cudaStreamCreate failed (no usable GPU?)");
        delete h;
        return UNS_ERR_CUDA;
    }
    {
        int dev = 0, nsm = 0;
        if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
            nsm > 0)
            h->nsm = nsm;
    }
    Gas& g = h->g;
    g = make_gas(p, &h->qinf);

    // Host-side derived connectivity.
    std::vector<double2> pxy(nop), cen(ntot), fn(nof), fcen(nof);
    std::vector<int2> fnb(nof), fpt(nof);
    for (int i = 0; i < nop; ++i) pxy[i] = make_double2(m->px[i], m->py[i]);
    for (int i = 0; i < ntot; ++i) cen[i] = make_double2(m->cx[i], m->cy[i]);
    for (int f = 0; f < nof; ++f) {
        fnb[f] = make_int2(m->fin[f], m->fout[f]);
        fpt[f] = make_int2(m->fp1[f], m->fp2[f]);
        fn[f] = make_double2(m->fnx[f], m->fny[f]);
        fcen[f] = make_double2(m->fcx[f], m->fcy[f]);
    }
    std::vector<int> cnt(noc + 1, 0);
    for (int f = 0; f < nof; ++f) { cnt[m->fin[f] + 1]++; if (m->fout[f] < noc) cnt[m->fout[f] + 1]++; }
    for (int i = 0; i < noc; ++i) cnt[i + 1] += cnt[i];
    std::vector<int> cf(cnt[noc]), pos(cnt.begin(), cnt.end() - 1);
    for (int f = 0; f < nof; ++f) {  // ascending face index per cell
        cf[pos[m->fin[f]]++] = f;
        if (m->fout[f] < noc) cf[pos[m->fout[f]]++] = f | SIDE_BIT;
    }
    // LSQ weights (gradient.F90:27-44, 72-78), host-side in the reference's
    // expression order (-ffp-contract=off translation unit).
    std::vector<double4> lsw(nof);
    for (int f = 0; f < nof; ++f) {
        int in = m->fin[f], o = m->fout[f];
        double xc = m->cx[in], yc = m->cy[in], xn = m->cx[o], yn = m->cy[o];
        double dx = xn - xc, dy = yn - yc;
        double r11 = m->r11[in], r12 = m->r12[in], r22 = m->r22[in];
        double alfa1 = dx / r11 / r11;
        double alfa2 = f < nfi ? (dy - dx * r12 / r11) / (r22 * r22) : (dy - dx * r12 / r11) / r22 / r22;
        double wx0 = alfa1 - alfa2 * r12 / r11, wy0 = alfa2, wx1 = 0.0, wy1 = 0.0;
        if (f < nfi) {
            dx = xc - xn; dy = yc - yn;
            r11 = m->r11[o]; r12 = m->r12[o]; r22 = m->r22[o];
            alfa1 = dx / r11 / r11;
            alfa2 = (dy - dx * r12 / r11) / (r22 * r22);
            wx1 = alfa1 - alfa2 * r12 / r11; wy1 = alfa2;
        }
        lsw[f] = make_double4(wx0, wy0, wx1, wy1);
    }
    h->lsq_r.resize((size_t)noc * 3);
    for (int i = 0; i < noc; ++i) { h->lsq_r[3 * i] = m->r11[i]; h->lsq_r[3 * i + 1] = m->r12[i]; h->lsq_r[3 * i + 2] = m->r22[i]; }
    h->fnb_host = fnb;
    // FP32 geometry of the mixed form, rounded once from the FP64 values.
    std::vector<float4> fgeof(nof), fnaf(nof), lswf(nof);
    for (int f = 0; f < nof; ++f) {
        int in = m->fin[f], o = m->fout[f];
        double xl = m->fcx[f] - m->cx[in], yl = m->fcy[f] - m->cy[in];
        double xr = f < nfi ? m->fcx[f] - m->cx[o] : 0.0, yr = f < nfi ? m->fcy[f] - m->cy[o] : 0.0;
        fgeof[f] = make_float4((float)xl, (float)yl, (float)xr, (float)yr);
        fnaf[f] = make_float4((float)m->fnx[f], (float)m->fny[f], (float)m->farea[f], 0.f);
        lswf[f] = make_float4((float)lsw[f].x, (float)lsw[f].y, (float)lsw[f].z, (float)lsw[f].w);
    }
    std::vector<int> rc2f_off(m->c2f_off, m->c2f_off + noc + 1);
    std::vector<int> rc2f(m->c2f, m->c2f + rc2f_off[noc]);

    CCView& v = h->v;
    std::memset(&v, 0, sizeof(v));
    v.nop = nop; v.noc = noc; v.nfi = nfi; v.nbf = nbf; v.nof = nof; v.ntot = ntot;
    v.g = g;
    v.grad_type = p->grad_type; v.ilimit = p->ilimit; v.irs = p->irs;
    v.laminar = p->flow_type == UNS_FLOW_LAMINAR;
    v.cfl_max = p->cfl_max; v.min_res = p->min_res;
    v.mixed = p->precision == UNS_PREC_MIXED;
    // Block sizes of the kernels without block-level reductions, from a
    // measured sweep of 64-512 on the 4.2 M-cell mixed step and the 256-case
    // batch (faces 64, vertices 256, cell gradient 128); UNS_CC_BLOCK_FACE /
    // _VERTEX (64..512) and UNS_CC_BLOCK_GRAD (64..256: a divisor of the
    // 256-cell instance-pure blocks) override them for tuning runs.
    auto block_env = [](const char* name, int def, int hi) {
        const char* e = std::getenv(name);
        const int b = e ? std::atoi(e) : def;
        return (b == 64 || b == 128 || b == 256 || b == 512) && b <= hi ? b : def;
    };
    v.blk_face = block_env("UNS_CC_BLOCK_FACE", 64, 512);
    v.blk_vert = block_env("UNS_CC_BLOCK_VERTEX", kBlock, 512);
    v.blk_grad = block_env("UNS_CC_BLOCK_GRAD", 128, kBlock);
#define UP(field, vec) if ((rc = h->upload(*(std::remove_const<std::remove_pointer<decltype(v.field)>::type>::type**)&v.field, vec.data(), vec.size()))) return fail(rc)
#define AL(field, n) if ((rc = h->alloc(v.field, (n)))) return fail(rc)
    UP(pxy, pxy); UP(cen, cen);
    { std::vector<double> t(m->cv, m->cv + noc); UP(cv, t); }
    { std::vector<double> t(m->cov, m->cov + noc); UP(cov, t); }
    UP(fnb, fnb); UP(fpt, fpt); UP(fn, fn); UP(fcen, fcen);
    { std::vector<double> t(m->farea, m->farea + nof); UP(farea, t); }
    { std::vector<int> t(m->fbc, m->fbc + nof); UP(fbc, t); }
    UP(lsw, lsw);
    { std::vector<int> t(m->nc2c, m->nc2c + noc); UP(nc2c, t); }
    UP(cf_off, cnt); UP(cf, cf);
    if (p->grad_type == UNS_GRAD_GG && p->flow_type != UNS_FLOW_LAMINAR) {  // cell-side records (k_cell_grad_side)
        std::vector<float4> sg(cf.size());
        std::vector<int4> si(cf.size());
        for (size_t k = 0; k < cf.size(); ++k) {
            const int e = cf[k], f = e & FACE_MASK;
            const bool out_side = f < nfi && (e & SIDE_BIT);
            const float s = (f < nfi && !(e & SIDE_BIT)) ? 1.f : -1.f;  // Gradient_GG's sign (boundary: -1)
            const float4 na = fnaf[f], gd = fgeof[f];
            sg[k] = make_float4(s * na.x, s * na.y, out_side ? gd.z : gd.x, out_side ? gd.w : gd.y);
            const int nbr = f < nfi ? (out_side ? m->fin[f] : m->fout[f]) : -1;
            int area_bits;
            std::memcpy(&area_bits, &na.z, sizeof(int));
            si[k] = make_int4(nbr, m->fp1[f], m->fp2[f], area_bits);
        }
        UP(sideg, sg); UP(sidei, si);
    }
    {  // wall cells: a bit per cell and their list
        std::vector<unsigned> t((noc + 31) / 32, 0u);
        std::vector<int> wc;
        for (int f = nfi; f < nof; ++f) {
            const int c = m->fin[f];
            if (m->fbc[f] == 1001 && c >= 0 && c < noc) t[c >> 5] |= 1u << (c & 31);
        }
        for (int c = 0; c < noc; ++c)
            if ((t[c >> 5] >> (c & 31)) & 1u) wc.push_back(c);
        UP(bcell, t); UP(wcell, wc);
        v.nwcell = (int)wc.size();
    }
    UP(rc2f_off, rc2f_off); UP(rc2f, rc2f);
    { std::vector<int> t(m->v2c_off, m->v2c_off + nop + 1); UP(v2c_off, t); }
    { std::vector<int> t(m->v2c, m->v2c + m->v2c_off[nop]); UP(v2c, t); }
    { std::vector<double> t(m->v2c_wt, m->v2c_wt + m->v2c_off[nop]); UP(v2c_wt, t); }
    AL(qc, ntot); AL(qp, ntot); AL(qT, ntot); AL(qold, noc); AL(res, noc); AL(res0, noc); AL(restmp, noc);
    AL(gx, noc); AL(gy, noc); AL(phi, noc); AL(dt, noc); AL(la, noc); AL(mul, ntot);
    AL(pp, nop); AL(ppT, nop); AL(fq, nof); AL(fqT, nof); AL(fla, nof); AL(fmu, nof);
    AL(fF, nof); AL(fV, nof); AL(fgx, nof); AL(fgy, nof); AL(fgT, nof); AL(fasum, nof);
    AL(fwall, nbf); AL(fwallv, nbf);
    AL(diag, noc); AL(diaginv, noc); AL(rec_a, 2 * (size_t)noc); AL(rec_b, 2 * (size_t)noc);
    UP(fgeof, fgeof); UP(fnaf, fnaf); UP(lswf, lswf);
    AL(qpf, ntot); AL(fqf, nof); AL(flaf, nof); AL(packf, 4 * (size_t)noc); AL(ppf, nop); AL(dcv, noc);
    { std::vector<float> t(m->v2c_wt, m->v2c_wt + m->v2c_off[nop]); UP(v2c_wtf, t); }
    AL(minmax, 8); AL(dtmin, 1); AL(err, 1);
    h->v.wait_cycles = kWaitCycles;
    h->v.skip_code = -1;
    h->nparts = nblocks(noc);
    AL(partial, 8 * (size_t)h->nparts);  // per-warp partials of a small mesh's spread RK pass
    if ((rc = h->alloc(h->d_scalar, 4))) return fail(rc);
    if ((rc = h->alloc(h->d_iter, 1))) return fail(rc);
    if ((rc = h->alloc(h->d_done, 1))) return fail(rc);
    if ((rc = h->alloc(h->d_fres1, 1))) return fail(rc);
    // LU-SGS warp schedule on the reference c2f lists.
    if (lusgs_schedule) {
        int maxdeg = 0;
        for (int i = 0; i < noc; ++i) maxdeg = std::max(maxdeg, m->c2f_off[i + 1] - m->c2f_off[i]);
        if (maxdeg > 32) { set_last_error("uns_cc_create: a cell has more than 32 faces"); return fail(UNS_ERR_MESH); }
        if (noc >= (1 << 30)) { set_last_error("uns_cc_create: too many cells"); return fail(UNS_ERR_MESH); }
        int dev = 0, nsm = 0, per = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_lusgs, kSweepBlock, 0) != cudaSuccess || per < 1) {
            set_last_error("uns_cc_create: cannot size the cooperative LU-SGS launch");
            return fail(UNS_ERR_CUDA);
        }
        h->coop_blocks = nsm * std::min(per, kSweepBlocksPerSM);
        // the cell across each c2f face (ghosts >= noc), and whether the face
        // normal points into the cell
        auto other = [&](int i, int f, int* flip) {
            if (m->fout[f] == i) { *flip = 1; return m->fin[f]; }
            *flip = 0;
            return m->fout[f];
        };
        std::vector<int> nbr(m->c2f_off[noc]);
        for (int i = 0; i < noc; ++i)
            for (int k = m->c2f_off[i]; k < m->c2f_off[i + 1]; ++k) {
                int fl;
                nbr[k] = other(i, m->c2f[k], &fl);
            }
        WarpSchedule ws = list_schedule(noc, m->c2f_off, nbr.data(), h->coop_blocks * (kSweepBlock / 32));
        std::vector<int4> sched(ws.items.size());
        std::vector<int> rf, rn, rl;
        for (size_t pos = 0; pos < ws.items.size(); ++pos) {
            const int it = ws.items[pos] >> 1, pass = ws.items[pos] & 1;
            const int first = (int)rf.size();
            for (int k = m->c2f_off[it]; k < m->c2f_off[it + 1]; ++k) {
                int fl, nb = other(it, m->c2f[k], &fl);
                bool take = nb >= 0 && nb < noc && (pass == 0 ? nb < it : nb > it);
                if (take) { rf.push_back(m->c2f[k]); rn.push_back(nb); rl.push_back(fl); }
            }
            sched[pos] = make_int4(it, pass, first, (int)rf.size() - first);
        }
        v.nrec = (int)rf.size();
        if ((rc = h->upload(h->woff, ws.off.data(), ws.off.size()))) return fail(rc);
        UP(sched, sched); UP(rec_face, rf); UP(rec_nb, rn); UP(rec_flip, rl);
        AL(rec, 3 * rf.size());
    }
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) { set_last_error("uns_cc_create: upload failed"); return fail(UNS_ERR_CUDA); }
    rc = uns_cc_initialize(h);
    if (rc) return fail(rc);
    *out = h;
    return UNS_OK;
#undef UP
#undef AL
}

extern "C" {

int uns_cc_destroy(uns_cc_handle* h) {
    if (!h) return UNS_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    cc_adj_free(h);
    if (h->graph) cudaGraphExecDestroy(h->graph);
    for (void* p : h->allocs) cudaFree(p);
    if (h->d_cfl) cudaFree(h->d_cfl);
    if (h->d_hist) cudaFree(h->d_hist);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return UNS_OK;
}

int uns_cc_initialize(uns_cc_handle* h) {
    if (!h) return UNS_ERR_ARG;
    ++h->flux_gen;
    CCView v = h->v;
    k_initialize<<<nblocks(v.ntot), kBlock, 0, h->stream>>>(v, h->qinf);
    UNS_CUDA(cudaGetLastError());
    UNS_CUDA(cudaMemsetAsync(v.mul, 0, sizeof(double) * v.ntot, h->stream));
    UNS_CUDA(cudaMemsetAsync(v.fmu, 0, sizeof(double) * v.nof, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    return UNS_OK;
}

int uns_cc_set_state(uns_cc_handle* h, const double* qc) {
    if (!h || !qc) return UNS_ERR_ARG;
    UNS_CUDA(cudaMemcpyAsync(h->v.qc, qc, sizeof(double4) * h->v.ntot, cudaMemcpyHostToDevice, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    return UNS_OK;
}

int uns_cc_get_state(uns_cc_handle* h, double* qc) {
    if (!h || !qc) return UNS_ERR_ARG;
    UNS_CUDA(cudaMemcpyAsync(qc, h->v.qc, sizeof(double4) * h->v.ntot, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    return UNS_OK;
}

int uns_cc_get_field(uns_cc_handle* h, int field, double* out) {
    if (!h || !out) return UNS_ERR_ARG;
    const CCView& v = h->v;
    if (v.mixed && (field == UNS_CC_GRAD || field == UNS_CC_PHI)) LAUNCH(k_unpack_f32, v.noc, v);
    // the graph step of this form forms the face radii inside k_cell_grad_side
    if (v.mixed && v.sideg && field == UNS_CC_FLA) LAUNCH_SPREAD(k_face_prim_spec, v.nof, v);
    auto d2h = [&](void* dst, const void* src, size_t bytes) {
        return cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->stream);
    };
    auto interleave = [&](const double4* a, const double* b, int n, int stride5) -> int {
        std::vector<double4> A(n);
        std::vector<double> B(n);
        UNS_CUDA(d2h(A.data(), a, sizeof(double4) * n));
        UNS_CUDA(d2h(B.data(), b, sizeof(double) * n));
        UNS_CUDA(cudaStreamSynchronize(h->stream));
        for (int i = 0; i < n; ++i) {
            double* o = out + (size_t)i * stride5;
            o[0] = A[i].x; o[1] = A[i].y; o[2] = A[i].z; o[3] = A[i].w; o[4] = B[i];
        }
        return UNS_OK;
    };
    switch (field) {
        case UNS_CC_QC: UNS_CUDA(d2h(out, v.qc, sizeof(double4) * v.ntot)); break;
        case UNS_CC_QP: return interleave(v.qp, v.qT, v.ntot, 5);
        case UNS_CC_QOLD: UNS_CUDA(d2h(out, v.qold, sizeof(double4) * v.noc)); break;
        case UNS_CC_RES: UNS_CUDA(d2h(out, v.res, sizeof(double4) * v.noc)); break;
        case UNS_CC_PHI: UNS_CUDA(d2h(out, v.phi, sizeof(double4) * v.noc)); break;
        case UNS_CC_DT: UNS_CUDA(d2h(out, v.dt, sizeof(double) * v.noc)); break;
        case UNS_CC_LA: UNS_CUDA(d2h(out, v.la, sizeof(double) * v.noc)); break;
        case UNS_CC_FLA: UNS_CUDA(d2h(out, v.fla, sizeof(double) * v.nof)); break;
        case UNS_CC_FMU: UNS_CUDA(d2h(out, v.fmu, sizeof(double) * v.nof)); break;
        case UNS_CC_MUL: UNS_CUDA(d2h(out, v.mul, sizeof(double) * v.noc)); break;
        case UNS_CC_PTPRIM: return interleave(v.pp, v.ppT, v.nop, 5);
        case UNS_CC_FQP: return interleave(v.fq, v.fqT, v.nof, 5);
        case UNS_CC_FWALL: {
            std::vector<double2> A(v.nbf), B(v.nbf);
            UNS_CUDA(d2h(A.data(), v.fwall, sizeof(double2) * v.nbf));
            UNS_CUDA(d2h(B.data(), v.fwallv, sizeof(double2) * v.nbf));
            UNS_CUDA(cudaStreamSynchronize(h->stream));
            for (int b = 0; b < v.nbf; ++b) {
                out[4 * (size_t)b] = A[b].x; out[4 * (size_t)b + 1] = A[b].y;
                out[4 * (size_t)b + 2] = v.laminar ? B[b].x : 0.0; out[4 * (size_t)b + 3] = v.laminar ? B[b].y : 0.0;
            }
            return UNS_OK;
        }
        case UNS_CC_GRAD: {
            std::vector<double4> X(v.noc), Y(v.noc);
            UNS_CUDA(d2h(X.data(), v.gx, sizeof(double4) * v.noc));
            UNS_CUDA(d2h(Y.data(), v.gy, sizeof(double4) * v.noc));
            UNS_CUDA(cudaStreamSynchronize(h->stream));
            for (int i = 0; i < v.noc; ++i) {
                double a[4] = {X[i].x, X[i].y, X[i].z, X[i].w}, b[4] = {Y[i].x, Y[i].y, Y[i].z, Y[i].w};
                for (int j = 0; j < 4; ++j) { out[(size_t)i * 8 + 2 * j] = a[j]; out[(size_t)i * 8 + 2 * j + 1] = b[j]; }
            }
            return UNS_OK;
        }
        case UNS_CC_FGRAD: {
            std::vector<double4> X(v.nof), Y(v.nof);
            std::vector<double2> T(v.nof);
            UNS_CUDA(d2h(X.data(), v.fgx, sizeof(double4) * v.nof));
            UNS_CUDA(d2h(Y.data(), v.fgy, sizeof(double4) * v.nof));
            UNS_CUDA(d2h(T.data(), v.fgT, sizeof(double2) * v.nof));
            UNS_CUDA(cudaStreamSynchronize(h->stream));
            for (int f = 0; f < v.nof; ++f) {
                double a[5] = {X[f].x, X[f].y, X[f].z, X[f].w, T[f].x}, b[5] = {Y[f].x, Y[f].y, Y[f].z, Y[f].w, T[f].y};
                for (int j = 0; j < 5; ++j) { out[(size_t)f * 10 + 2 * j] = a[j]; out[(size_t)f * 10 + 2 * j + 1] = b[j]; }
            }
            return UNS_OK;
        }
        default: set_last_error("uns_cc_get_field: unknown field"); return UNS_ERR_ARG;
    }
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    return UNS_OK;
}

int uns_cc_set_field(uns_cc_handle* h, int field, const double* in) {
    if (!h || !in) return UNS_ERR_ARG;
    ++h->flux_gen;
    CCView& v = h->v;
    switch (field) {
        case UNS_CC_QC:
            UNS_CUDA(cudaMemcpyAsync(v.qc, in, sizeof(double4) * v.ntot, cudaMemcpyHostToDevice, h->stream));
            break;
        case UNS_CC_QP: {
            std::vector<double4> A(v.ntot);
            std::vector<double> B(v.ntot);
            std::vector<float4> F(v.ntot);
            for (int i = 0; i < v.ntot; ++i) {
                const double* o = in + (size_t)i * 5;
                A[i] = make_double4(o[0], o[1], o[2], o[3]);
                B[i] = o[4];
                F[i] = make_float4((float)o[0], (float)o[1], (float)o[2], (float)o[3]);
            }
            UNS_CUDA(cudaMemcpyAsync(v.qp, A.data(), sizeof(double4) * v.ntot, cudaMemcpyHostToDevice, h->stream));
            UNS_CUDA(cudaMemcpyAsync(v.qT, B.data(), sizeof(double) * v.ntot, cudaMemcpyHostToDevice, h->stream));
            UNS_CUDA(cudaMemcpyAsync(v.qpf, F.data(), sizeof(float4) * v.ntot, cudaMemcpyHostToDevice, h->stream));
            UNS_CUDA(cudaStreamSynchronize(h->stream));
            return UNS_OK;
        }
        case UNS_CC_PHI:
            if (v.mixed) LAUNCH(k_unpack_f32, v.noc, v);
            UNS_CUDA(cudaMemcpyAsync(v.phi, in, sizeof(double4) * v.noc, cudaMemcpyHostToDevice, h->stream));
            if (v.mixed) LAUNCH(k_mirror_f32, std::max(std::max(v.ntot, v.nof), v.nop), v);
            break;
        default: set_last_error("uns_cc_set_field: field cannot be set"); return UNS_ERR_ARG;
    }
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    return UNS_OK;
}

int uns_cc_con2prim(uns_cc_handle* h) {
    if (!h) return UNS_ERR_ARG;
    ++h->flux_gen;
    CCView v = h->v;
    LAUNCH(k_begin, v.noc, v, (int)BEGIN_PRIM);
    return UNS_OK;
}

int uns_cc_avg_c2v(uns_cc_handle* h) {
    if (!h) return UNS_ERR_ARG;
    ++h->flux_gen;
    CCView v = h->v;
    LAUNCH_BS(k_vertex_avg, v.nop, v.blk_vert, v);
    LAUNCH_SPREAD(k_face_prim_spec, v.nof, v);
    return UNS_OK;
}

int uns_cc_time_step(uns_cc_handle* h, double cfl, double* dtglobal) {
    if (!h) return UNS_ERR_ARG;
    CCView v = h->v;
    h->cfl_cur = cfl;  // cirs of this iteration uses the same CFL
    k_reset_minmax<<<1, 32, 0, h->stream>>>(v);
    UNS_CUDA(cudaGetLastError());
    LAUNCH_CELL_GRAD(v, CG_DT | CG_DIAG, cfl);
    if (dtglobal) {
        unsigned long long e = 0;
        UNS_CUDA(cudaMemcpyAsync(&e, v.dtmin, 8, cudaMemcpyDeviceToHost, h->stream));
        UNS_CUDA(cudaStreamSynchronize(h->stream));
        *dtglobal = std::min(1.0e20, dec_ord(e));
    }
    return UNS_OK;
}

int uns_cc_save_old(uns_cc_handle* h) {
    if (!h) return UNS_ERR_ARG;
    CCView v = h->v;
    LAUNCH(k_begin, v.noc, v, (int)BEGIN_OLD);
    return UNS_OK;
}

int uns_cc_gradient(uns_cc_handle* h) {
    if (!h) return UNS_ERR_ARG;
    ++h->flux_gen;
    CCView v = h->v;
    return enqueue_gradient(h, v, 0, 0.0, true);
}

int uns_cc_limit(uns_cc_handle* h) {
    if (!h) return UNS_ERR_ARG;
    ++h->flux_gen;
    CCView v = h->v;
    int rc = enqueue_minmax(h, v);
    if (rc) return rc;
    LAUNCH_CELL_GRAD(v, CG_LIM, 0.0);
    return UNS_OK;
}

int uns_cc_fvresidual(uns_cc_handle* h) {
    if (!h) return UNS_ERR_ARG;
    CCView v = h->v;
    bool fused = false;
    // Since the last call that computed every face, only the conserved state
    // has changed (rk_stage, set_state): the interior and farfield fluxes read
    // the primitives, gradient and limiter alone, so only the wall faces and
    // their cells' residuals are recomputed (bit-identical to a full call).
    // Viscous fluxes read the state, and a smoothing sweep replaces the stored
    // residual: those calls compute everything.
    const bool smooth = v.irs && epsirs_of(h, h->cfl_cur) > 0.0;
    if (!v.laminar && !smooth && h->res_gen == h->flux_gen) return enqueue_wall_res(h, v);
    const int rc = enqueue_fvresidual(h, v, h->cfl_cur, 0, 0, &fused);
    if (!rc) h->res_gen = h->flux_gen;
    return rc;
}

int uns_cc_rk_stage(uns_cc_handle* h, int irk) {
    if (!h || irk < 1 || irk > 3) return UNS_ERR_ARG;
    CCView v = h->v;
    LAUNCH(k_rk_stage, v.noc, v, irk);
    return UNS_OK;
}

int uns_cc_lusgs(uns_cc_handle* h) {
    if (!h) return UNS_ERR_ARG;
    int rc = uns_cc_fvresidual(h);
    if (rc) return rc;
    CCView v = h->v;
    return enqueue_lusgs(h, v);
}

int uns_cc_check_positivity(uns_cc_handle* h, int* bad) {
    if (!h) return UNS_ERR_ARG;
    CCView v = h->v;
    int rc = check_dev_err(h);
    if (rc) { if (bad) *bad = -1; return rc; }
    LAUNCH(k_check_pos, v.noc, v);
    DevErr e;
    UNS_CUDA(cudaMemcpyAsync(&e, v.err, sizeof(DevErr), cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    if (bad) *bad = e.code == UNS_ERR_NONPOSITIVE ? e.index : -1;
    return check_dev_err(h);
}

int uns_cc_residue(uns_cc_handle* h, double* fres) {
    if (!h || !fres) return UNS_ERR_ARG;
    CCView v = h->v;
    LAUNCH(k_res_partial, v.noc, v);
    k_res_final<<<1, kBlock, 0, h->stream>>>(v, h->nparts, h->d_scalar);
    UNS_CUDA(cudaGetLastError());
    UNS_CUDA(cudaMemcpyAsync(fres, h->d_scalar, sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    return check_dev_err(h);
}

int uns_cc_forces(uns_cc_handle* h, double* fx, double* fy) {
    if (!h || !fx || !fy) return UNS_ERR_ARG;
    k_forces<<<1, 1, 0, h->stream>>>(h->v, h->d_scalar);
    UNS_CUDA(cudaGetLastError());
    double r[2];
    UNS_CUDA(cudaMemcpyAsync(r, h->d_scalar, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    *fx = r[0];
    *fy = r[1];
    return UNS_OK;
}

// One main-loop iteration of a handle captured as a graph, wired to the
// handle's device-side CFL schedule, iteration counter, history and stop flag.
static int capture_iteration(uns_cc_handle* h, int first_iter, cudaGraph_t* out) {
    CCView v = h->v;
    v.cfl_sched = h->d_cfl;
    v.cfl_stride = h->cfl_cap;
    v.iter = h->d_iter;
    v.done = h->d_done;
    v.fres_hist = h->d_hist;
    v.fres1 = h->d_fres1;
    v.first_iter = first_iter ? 1 : 0;
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    UNS_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int rc = enqueue_iteration(h, v, 0.0);
    cudaError_t ce = cudaStreamEndCapture(h->stream, out);
    if (rc) return rc;
    if (ce != cudaSuccess) { set_last_error(std::string("graph capture: ") + cudaGetErrorString(ce)); return UNS_ERR_CUDA; }
    return UNS_OK;
}

int uns_cc_iterate(uns_cc_handle* h, int niter, const double* cfl, int first_iter, double* fres_raw, int* done_iters) {
    if (!h || niter < 0 || (niter > 0 && (!cfl || !fres_raw))) return UNS_ERR_ARG;
    if (h->v.ninst) { set_last_error("uns_cc_iterate: a packed handle iterates with uns_cc_packed_iterate"); return UNS_ERR_ARG; }
    if (done_iters) *done_iters = 0;
    if (niter == 0) return UNS_OK;
    if (niter > h->cfl_cap) {
        int rc = grow_schedule(h, niter);
        if (rc) return rc;
    }
    // The smoothing sweeps are launched only while their coefficient is
    // non-zero; the schedule must agree on that for the whole chunk.
    bool any_smooth = false, all_smooth = true;
    for (int k = 0; k < niter; ++k) {
        bool s = h->P.irs && epsirs_of(h, cfl[k]) > 0.0;
        any_smooth = any_smooth || s;
        all_smooth = all_smooth && s;
    }
    if (any_smooth) {
        // Residual smoothing with a CFL above CFLmax changes the sweep
        // weights per iteration: run the chunk through the per-call path.
        double f1 = 0.0;
        int done = 0;
        for (int k = 0; k < niter; ++k) {
            int rc;
            if ((rc = uns_cc_con2prim(h)) || (rc = uns_cc_avg_c2v(h)) || (rc = uns_cc_time_step(h, cfl[k], nullptr)) ||
                (rc = uns_cc_save_old(h)) || (rc = uns_cc_gradient(h)))
                return rc;
            if (h->P.time_mode == UNS_TIME_RK3) {
                for (int irk = 1; irk <= 3; ++irk)
                    if ((rc = uns_cc_fvresidual(h)) || (rc = uns_cc_rk_stage(h, irk))) return rc;
            } else if ((rc = uns_cc_lusgs(h))) return rc;
            int bad;
            if ((rc = uns_cc_check_positivity(h, &bad))) return rc;
            if ((rc = uns_cc_residue(h, &fres_raw[k]))) return rc;
            ++done;
            if (first_iter && k == 0) f1 = fres_raw[0];
            double nf = (f1 >= 2.220446049250313e-16) ? fres_raw[k] / f1 : fres_raw[k];
            if (!(nf > h->P.min_res)) break;
        }
        if (done_iters) *done_iters = done;
        return UNS_OK;
    }
    (void)all_smooth;
    return iterate_graph(h, niter, cfl, first_iter, fres_raw, done_iters);
}

}  // extern "C"

// Device CFL schedule and residual history with room for cap iterations per
// instance; the captured iteration bakes in their addresses and stride.
static int grow_schedule(uns_cc_handle* h, int cap) {
    const size_t n = (size_t)std::max(1, h->v.ninst);
    if (h->d_cfl) cudaFree(h->d_cfl);
    if (h->d_hist) cudaFree(h->d_hist);
    h->d_cfl = nullptr; h->d_hist = nullptr;
    UNS_CUDA(cudaMalloc(&h->d_cfl, sizeof(double) * n * cap));
    UNS_CUDA(cudaMalloc(&h->d_hist, sizeof(double) * n * cap));
    h->cfl_cap = cap;
    ++h->gen;
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    return UNS_OK;
}

// The graph-replayed iterations of every instance: cfl and fres_raw are
// [instances][niter], done_iters [instances].
static int iterate_graph(uns_cc_handle* h, int niter, const double* cfl, int first_iter, double* fres_raw, int* done_iters) {
    ++h->flux_gen;
    const int n = std::max(1, h->v.ninst);
    if (niter > h->cfl_cap) {
        int rc = grow_schedule(h, niter);
        if (rc) return rc;
    }
    const size_t pitch = sizeof(double) * h->cfl_cap, row = sizeof(double) * niter;
    UNS_CUDA(cudaMemcpy2DAsync(h->d_cfl, pitch, cfl, row, row, n, cudaMemcpyHostToDevice, h->stream));
    UNS_CUDA(cudaMemsetAsync(h->d_iter, 0, sizeof(int) * n, h->stream));
    UNS_CUDA(cudaMemsetAsync(h->d_done, 0, sizeof(int) * n, h->stream));
    UNS_CUDA(cudaMemsetAsync(h->d_hist, 0, pitch * n, h->stream));
    if (!h->graph || h->graph_first != (first_iter ? 1 : 0)) {
        if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
        cudaGraph_t graph;
        int rc = capture_iteration(h, first_iter, &graph);
        if (rc) return rc;
        cudaError_t ce = cudaGraphInstantiate(&h->graph, graph, 0);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess) { set_last_error(std::string("graph instantiate: ") + cudaGetErrorString(ce)); return UNS_ERR_CUDA; }
        h->graph_first = first_iter ? 1 : 0;
    }
    for (int k = 0; k < niter; ++k) UNS_CUDA(cudaGraphLaunch(h->graph, h->stream));
    UNS_CUDA(cudaMemcpy2DAsync(fres_raw, row, h->d_hist, pitch, row, n, cudaMemcpyDeviceToHost, h->stream));
    std::vector<int> it(n, 0);
    UNS_CUDA(cudaMemcpyAsync(it.data(), h->d_iter, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    if (done_iters) std::copy(it.begin(), it.end(), done_iters);
    return check_dev_err(h);
}

extern "C" {

int uns_cc_set_wait_limit(uns_cc_handle* h, long long cycles) {
    if (!h || cycles <= 0) return UNS_ERR_ARG;
    h->v.wait_cycles = cycles;
    ++h->gen;
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    return UNS_OK;
}

int uns_cc_debug_unpublish(uns_cc_handle* h, int cell, int pass) {
    if (!h || cell < -1 || cell >= h->v.noc || pass < 0 || pass > 1) return UNS_ERR_ARG;
    h->v.skip_code = cell < 0 ? -1 : (cell << 1) | pass;
    ++h->gen;
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    return UNS_OK;
}

int uns_cc_set_precision(uns_cc_handle* h, int precision) {
    if (!h || precision < UNS_PREC_FP64 || precision > UNS_PREC_MIXED_SWEEP) return UNS_ERR_ARG;
    ++h->flux_gen;
    if (h->P.precision != precision) {
        UNS_CUDA(cudaStreamSynchronize(h->stream));
        h->P.precision = precision;
        CCView& v = h->v;
        const int was_mixed = v.mixed;
        v.mixed = precision == UNS_PREC_MIXED;
        if (v.mixed && !was_mixed) LAUNCH(k_mirror_f32, std::max(std::max(v.ntot, v.nof), v.nop), v);
        if (was_mixed && !v.mixed) LAUNCH(k_unpack_f32, v.noc, v);
        ++h->gen;
        if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    }
    return UNS_OK;
}

// ---------------------------------------------------------------- batches
// Independent instances advanced together: one CUDA graph whose parallel
// branches are the instances' captured iterations, so one launch advances
// every instance by one iteration and small meshes share the GPU.  Each
// instance keeps its own device state, CFL schedule, history and stop flag;
// an instance that has converged skips its kernels on the device.
struct uns_cc_batch {
    std::vector<uns_cc_handle*> hs;
    std::vector<int> gens;  // each handle's `gen` when the graph was built
    cudaStream_t stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    int first = -1;
};

int uns_cc_batch_create(uns_cc_handle* const* handles, int n, uns_cc_batch** out) {
    if (!handles || n <= 0 || !out) { set_last_error("uns_cc_batch_create: bad arguments"); return UNS_ERR_ARG; }
    *out = nullptr;
    std::vector<uns_cc_handle*> hs(handles, handles + n);
    std::vector<uns_cc_handle*> sorted = hs;
    std::sort(sorted.begin(), sorted.end());
    if (!sorted[0] || std::adjacent_find(sorted.begin(), sorted.end()) != sorted.end()) {
        set_last_error("uns_cc_batch_create: null or repeated handle");
        return UNS_ERR_ARG;
    }
    auto* b = new uns_cc_batch();
    b->hs = hs;
    b->gens.assign(n, -1);
    if (cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking) != cudaSuccess) {
        delete b;
        set_last_error("uns_cc_batch_create: cudaStreamCreate failed");
        return UNS_ERR_CUDA;
    }
    *out = b;
    return UNS_OK;
}

void* uns_cc_batch_stream(uns_cc_batch* b) { return b ? (void*)b->stream : nullptr; }

int uns_cc_batch_destroy(uns_cc_batch* b) {
    if (!b) return UNS_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return UNS_OK;
}

int uns_cc_batch_iterate(uns_cc_batch* b, int niter, const double* cfl, int first_iter, double* fres_raw,
                         int* done_iters) {
    if (!b || niter < 0 || (niter > 0 && (!cfl || !fres_raw || !done_iters))) return UNS_ERR_ARG;
    const int n = (int)b->hs.size();
    if (niter == 0) {
        for (int i = 0; i < n; ++i) done_iters[i] = 0;
        return UNS_OK;
    }
    for (int i = 0; i < n; ++i) {
        uns_cc_handle* h = b->hs[i];
        ++h->flux_gen;
        for (int k = 0; k < niter; ++k)
            if (h->P.irs && epsirs_of(h, cfl[(size_t)i * niter + k]) > 0.0) {
                set_last_error("uns_cc_batch_iterate: residual smoothing above CFLmax is not batched");
                return UNS_ERR_ARG;
            }
        if (niter > h->cfl_cap) {
            UNS_CUDA(cudaStreamSynchronize(h->stream));
            if (h->d_cfl) cudaFree(h->d_cfl);
            if (h->d_hist) cudaFree(h->d_hist);
            h->d_cfl = nullptr; h->d_hist = nullptr;
            UNS_CUDA(cudaMalloc(&h->d_cfl, sizeof(double) * niter));
            UNS_CUDA(cudaMalloc(&h->d_hist, sizeof(double) * niter));
            h->cfl_cap = niter;
            ++h->gen;
            if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
        }
        UNS_CUDA(cudaStreamSynchronize(h->stream));
    }
    bool rebuild = !b->exec || b->first != (first_iter ? 1 : 0);
    for (int i = 0; i < n && !rebuild; ++i) rebuild = b->gens[i] != b->hs[i]->gen;
    if (rebuild) {
        if (b->exec) { cudaGraphExecDestroy(b->exec); b->exec = nullptr; }
        cudaGraph_t parent;
        UNS_CUDA(cudaGraphCreate(&parent, 0));
        for (int i = 0; i < n; ++i) {
            cudaGraph_t child;
            int rc = capture_iteration(b->hs[i], first_iter, &child);
            if (rc) { cudaGraphDestroy(parent); return rc; }
            cudaGraphNode_t node;
            cudaError_t ce = cudaGraphAddChildGraphNode(&node, parent, nullptr, 0, child);
            cudaGraphDestroy(child);
            if (ce != cudaSuccess) {
                cudaGraphDestroy(parent);
                set_last_error(std::string("batch graph: ") + cudaGetErrorString(ce));
                return UNS_ERR_CUDA;
            }
            b->gens[i] = b->hs[i]->gen;
        }
        cudaError_t ce = cudaGraphInstantiate(&b->exec, parent, 0);
        cudaGraphDestroy(parent);
        if (ce != cudaSuccess) { set_last_error(std::string("batch graph instantiate: ") + cudaGetErrorString(ce)); return UNS_ERR_CUDA; }
        b->first = first_iter ? 1 : 0;
    }
    for (int i = 0; i < n; ++i) {
        uns_cc_handle* h = b->hs[i];
        UNS_CUDA(cudaMemcpyAsync(h->d_cfl, cfl + (size_t)i * niter, sizeof(double) * niter, cudaMemcpyHostToDevice, b->stream));
        UNS_CUDA(cudaMemsetAsync(h->d_iter, 0, sizeof(int), b->stream));
        UNS_CUDA(cudaMemsetAsync(h->d_done, 0, sizeof(int), b->stream));
        UNS_CUDA(cudaMemsetAsync(h->d_hist, 0, sizeof(double) * niter, b->stream));
    }
    for (int k = 0; k < niter; ++k) UNS_CUDA(cudaGraphLaunch(b->exec, b->stream));
    for (int i = 0; i < n; ++i) {
        uns_cc_handle* h = b->hs[i];
        UNS_CUDA(cudaMemcpyAsync(fres_raw + (size_t)i * niter, h->d_hist, sizeof(double) * niter, cudaMemcpyDeviceToHost,
                                 b->stream));
        UNS_CUDA(cudaMemcpyAsync(done_iters + i, h->d_iter, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    }
    UNS_CUDA(cudaStreamSynchronize(b->stream));
    for (int i = 0; i < n; ++i) {
        int rc = check_dev_err(b->hs[i]);
        if (rc) return rc;
    }
    return UNS_OK;
}

void* uns_cc_stream(uns_cc_handle* h) { return h ? (void*)h->stream : nullptr; }

// Launch-geometry autotuner: times k_face_conv, k_vertex_avg and (in the
// mixed Green-Gauss step) k_cell_grad_side at each candidate block size on
// the handle's own mesh and state, keeps the fastest, and re-captures the
// step with them.  The timed launches read the handle's arrays and write
// scratch copies only, so the solution, the running limiter and the device
// counters are untouched.
int uns_cc_autotune(uns_cc_handle* h, int reps, int* blocks) {
    if (!h || reps < 1) return UNS_ERR_ARG;
    ++h->flux_gen;
    const CCView& v = h->v;
    std::vector<void*> bufs;
    auto scratch = [&](size_t bytes) -> void* {
        void* q = nullptr;
        if (cudaMalloc(&q, std::max<size_t>(bytes, 16)) != cudaSuccess) return nullptr;
        bufs.push_back(q);
        return q;
    };
    auto release = [&]() { for (void* q : bufs) cudaFree(q); bufs.clear(); };
    CCView t = v;  // inputs as the handle has them, outputs redirected
    t.cfl_sched = nullptr; t.iter = nullptr; t.done = nullptr;
    bool ok = (t.fF = (double4*)scratch(sizeof(double4) * v.nof)) && (t.qc = (double4*)scratch(sizeof(double4) * v.ntot)) &&
              (t.qp = (double4*)scratch(sizeof(double4) * v.ntot)) && (t.qT = (double*)scratch(sizeof(double) * v.ntot)) &&
              (t.qpf = (float4*)scratch(sizeof(float4) * v.ntot)) && (t.fwall = (double2*)scratch(sizeof(double2) * v.nbf)) &&
              (t.err = (DevErr*)scratch(sizeof(DevErr))) && (t.ppf = (float4*)scratch(sizeof(float4) * v.nop)) &&
              (t.pp = (double4*)scratch(sizeof(double4) * v.nop)) && (t.ppT = (double*)scratch(sizeof(double) * v.nop)) &&
              (t.la = (double*)scratch(sizeof(double) * v.noc)) && (t.dt = (double*)scratch(sizeof(double) * v.noc)) &&
              (t.dcv = (double*)scratch(sizeof(double) * v.noc)) && (t.packf = (float4*)scratch(sizeof(float4) * 4 * (size_t)v.noc)) &&
              (t.dtmin = (unsigned long long*)scratch(sizeof(unsigned long long) * std::max(1, v.ninst))) &&
              (t.minmax = (unsigned long long*)scratch(sizeof(unsigned long long) * 8 * std::max(1, v.ninst)));
    if (!ok) { release(); set_last_error("uns_cc_autotune: no device memory for the scratch outputs"); return UNS_ERR_CUDA; }
    int rc = UNS_OK;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cuda = [&](cudaError_t e) { if (e != cudaSuccess && rc == UNS_OK) { rc = UNS_ERR_CUDA; set_last_error(std::string("uns_cc_autotune: ") + cudaGetErrorString(e)); } };
    cuda(cudaMemcpyAsync(t.qc, v.qc, sizeof(double4) * v.ntot, cudaMemcpyDeviceToDevice, h->stream));
    cuda(cudaMemcpyAsync(t.qp, v.qp, sizeof(double4) * v.ntot, cudaMemcpyDeviceToDevice, h->stream));
    cuda(cudaMemcpyAsync(t.qT, v.qT, sizeof(double) * v.ntot, cudaMemcpyDeviceToDevice, h->stream));
    cuda(cudaMemcpyAsync(t.qpf, v.qpf, sizeof(float4) * v.ntot, cudaMemcpyDeviceToDevice, h->stream));
    cuda(cudaMemcpyAsync(t.packf, v.packf, sizeof(float4) * 4 * (size_t)v.noc, cudaMemcpyDeviceToDevice, h->stream));
    cuda(cudaMemsetAsync(t.err, 0, sizeof(DevErr), h->stream));
    {  // a limiter range of [0, 1] for every case
        auto enc = [](double x) {  // enc_ord on the host
            unsigned long long b;
            std::memcpy(&b, &x, sizeof(b));
            return (b & 0x8000000000000000ULL) ? ~b : (b | 0x8000000000000000ULL);
        };
        std::vector<unsigned long long> mm(8 * (size_t)std::max(1, v.ninst));
        for (size_t k = 0; k < mm.size(); ++k) mm[k] = enc((k % 8) < 4 ? 1.0 : 0.0);
        cuda(cudaMemcpyAsync(t.minmax, mm.data(), sizeof(unsigned long long) * mm.size(), cudaMemcpyHostToDevice, h->stream));
        cuda(cudaStreamSynchronize(h->stream));
    }
    cuda(cudaEventCreate(&e0));
    cuda(cudaEventCreate(&e1));
    const bool sides = grad_by_sides(h, v);
    auto time_it = [&](auto&& launch) -> float {
        launch();  // warm-up
        cuda(cudaEventRecord(e0, h->stream));
        for (int r = 0; r < reps; ++r) launch();
        cuda(cudaEventRecord(e1, h->stream));
        cuda(cudaEventSynchronize(e1));
        float ms = 0.f;
        cuda(cudaEventElapsedTime(&ms, e0, e1));
        cuda(cudaGetLastError());
        return ms;
    };
    auto pick = [&](std::initializer_list<int> cand, auto&& launch_with) -> int {
        int best = 0;
        float tbest = 0.f;
        for (int bs : cand) {
            const float ms = time_it([&]() { launch_with(bs); });
            if (rc) return 0;
            if (!best || ms < tbest) { best = bs; tbest = ms; }
        }
        return best;
    };
    int bf = 0, bv = 0, bg = 0;
    if (rc == UNS_OK && v.nof > 0)
        bf = pick({64, 128, 256, 512}, [&](int bs) {
            const int nb = std::max(1, (v.nbf + bs - 1) / bs + (v.nfi + bs - 1) / bs);
            if (v.mixed) k_face_conv<float><<<nb, bs, 0, h->stream>>>(t);
            else k_face_conv<double><<<nb, bs, 0, h->stream>>>(t);
        });
    if (rc == UNS_OK && v.nop > 0)
        bv = pick({64, 128, 256, 512}, [&](int bs) { k_vertex_avg<<<(v.nop + bs - 1) / bs, bs, 0, h->stream>>>(t); });
    if (rc == UNS_OK && sides && v.noc > 0)
        bg = pick({64, 128, 256}, [&](int bs) {
            k_cell_grad_side<<<(v.noc + bs - 1) / bs, bs, 0, h->stream>>>(t, CG_DT | CG_GRAD | (v.ilimit ? CG_LIM : 0), 0.5);
        });
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    cudaStreamSynchronize(h->stream);
    release();
    if (rc) return rc;
    if (bf) h->v.blk_face = bf;
    if (bv) h->v.blk_vert = bv;
    if (bg) h->v.blk_grad = bg;
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    ++h->gen;  // the captured step changes
    if (blocks) { blocks[0] = h->v.blk_face; blocks[1] = h->v.blk_vert; blocks[2] = h->v.blk_grad; }
    return check_dev_err(h);
}

int uns_cc_profile(uns_cc_handle* h, double cfl, int reps, double* ms, const char** names, int nphase) {
    static const char* kNames[] = {"begin", "vertex_avg", "face_prim_spec", "face_ggfc", "cell_grad", "face_conv",
                                   "viscous", "cell_res", "cirs", "lusgs_sweeps", "residue", "cell_rk23"};
    const int NP = 12;
    if (!h || reps < 1 || !ms) return UNS_ERR_ARG;
    ++h->flux_gen;
    std::vector<double> acc(NP, 0.0);
    cudaEvent_t e0, e1;
    UNS_CUDA(cudaEventCreate(&e0));
    UNS_CUDA(cudaEventCreate(&e1));
    CCView v = h->v;
    int rc = UNS_OK;
    auto timed = [&](int phase, auto&& launch) -> int {
        UNS_CUDA(cudaEventRecord(e0, h->stream));
        int r = launch();
        if (r) return r;
        UNS_CUDA(cudaEventRecord(e1, h->stream));
        UNS_CUDA(cudaEventSynchronize(e1));
        float t = 0.f;
        UNS_CUDA(cudaEventElapsedTime(&t, e0, e1));
        acc[phase] += t;
        return UNS_OK;
    };
    const bool rk3 = h->P.time_mode == UNS_TIME_RK3;
    const double eps = v.irs ? epsirs_of(h, cfl) : 0.0;
    const bool smooth = v.irs && eps > 0.0;
    for (int r = 0; r < reps && !rc; ++r) {
        rc = timed(0, [&]() -> int {
            k_reset_minmax<<<1, 32, 0, h->stream>>>(v);
            UNS_CUDA(cudaGetLastError());
            LAUNCH(k_begin, v.ntot, v, BEGIN_PRIM | BEGIN_OLD | BEGIN_POS | (v.ilimit ? BEGIN_MINMAX : 0));
            return UNS_OK;
        });
        if (!rc) rc = timed(1, [&]() -> int { LAUNCH_BS(k_vertex_avg, v.nop, v.blk_vert, v); return UNS_OK; });
        const bool sides = grad_by_sides(h, v);
        if (!rc && !sides) rc = timed(2, [&]() -> int { LAUNCH_SPREAD(k_face_prim_spec, v.nof, v); return UNS_OK; });
        if (!rc && v.grad_type == UNS_GRAD_GGFC) rc = timed(3, [&]() -> int { LAUNCH(k_face_ggfc, v.nof, v); return UNS_OK; });
        if (!rc) rc = timed(4, [&]() -> int {
            const int gflags = CG_DT | CG_GRAD | (v.ilimit ? CG_LIM : 0) | (rk3 ? 0 : CG_DIAG);
            if (sides) LAUNCH_BS(k_cell_grad_side, v.noc, v.blk_grad, v, gflags, cfl);
            else LAUNCH_CELL_GRAD(v, gflags, cfl);
            return UNS_OK;
        });
        const bool one_pass = rk23_in_one_pass(h, v, cfl);
        for (int irk = 1; irk <= (rk3 && !one_pass ? 3 : 1) && !rc; ++irk) {
            rc = timed(5, [&]() -> int {
                if (h->P.precision == UNS_PREC_MIXED) LAUNCH_FACE_CONV(float, v);
                else LAUNCH_FACE_CONV(double, v);
                return UNS_OK;
            });
            if (!rc && v.laminar) rc = timed(6, [&]() -> int {
                LAUNCH(k_cell_mul, v.noc, v);
                if (v.grad_type != UNS_GRAD_GGFC) {
                    CCView w = v;
                    w.grad_type = UNS_GRAD_GGFC;
                    int r2 = enqueue_gradient(h, w, 0, cfl, true);
                    if (r2) return r2;
                }
                LAUNCH(k_face_visc, v.nof, v);
                return UNS_OK;
            });
            int fuse = (rk3 && !smooth) ? irk : 0;
            if (!rc && one_pass && v.mixed) rc = timed(11, [&]() -> int { return enqueue_wall_rk(h, v); });
            if (!rc) rc = timed(7, [&]() -> int {
                if (v.mixed) LAUNCH(k_cell_res_mixed, v.noc, v, fuse, smooth ? 0 : 1, one_pass ? 1 : 0);
                else if (!(smooth || one_pass) || v.ninst) LAUNCH(k_cell_res, v.noc, v, fuse, (smooth || one_pass) ? 0 : 1);
                else LAUNCH_SPREAD(k_cell_res, v.noc, v, fuse, 0);  // as the iteration launches it
                return UNS_OK;
            });
            if (!rc && smooth) rc = timed(8, [&]() -> int {
                UNS_CUDA(cudaMemcpyAsync(v.res0, v.res, sizeof(double4) * v.noc, cudaMemcpyDeviceToDevice, h->stream));
                LAUNCH(k_cirs, v.noc, v, (const double4*)v.res0, v.restmp, eps);
                LAUNCH(k_cirs, v.noc, v, (const double4*)v.restmp, v.res, eps);
                LAUNCH(k_res_partial, v.noc, v);
                if (rk3) LAUNCH(k_rk_stage, v.noc, v, irk);
                return UNS_OK;
            });
        }
        if (!rc && one_pass && !v.mixed) rc = timed(11, [&]() -> int { return enqueue_rk23(h, v); });
        if (!rc && !rk3) rc = timed(9, [&]() -> int { return enqueue_lusgs(h, v); });
        if (!rc) rc = timed(10, [&]() -> int {
            k_res_final<<<1, kBlock, 0, h->stream>>>(one_pass && !v.mixed ? final_view(h, v) : v, h->nparts, h->d_scalar);
            UNS_CUDA(cudaGetLastError());
            return UNS_OK;
        });
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    for (int k = 0; k < nphase; ++k) {
        ms[k] = k < NP ? acc[k] / reps : 0.0;
        if (names) names[k] = k < NP ? kNames[k] : "";
    }
    return check_dev_err(h);
}

}  // extern "C"

// ------------------------------------------------------------ packed cases
// Many independent CCFVM cases in ONE index space: the meshes are
// concatenated (points, then interior cells padded per case to a multiple of
// the block size, interior faces, boundary faces and their ghosts in case
// order), every element records its case, and the per-case constants and
// loop control become arrays.  One launch of each kernel then advances every
// case; each case's arithmetic, face orders and norm blocks are the ones it
// has alone, so it evolves bit-identically to a handle of its own.
extern "C" {

int uns_cc_create_packed(const uns_cc_mesh* meshes, const uns_params* params, int n, uns_cc_handle** out) {
    if (!meshes || !params || !out || n < 1) { set_last_error("uns_cc_create_packed: bad argument"); return UNS_ERR_ARG; }
    *out = nullptr;
    const uns_params& p0 = params[0];
    for (int i = 0; i < n; ++i) {
        const uns_params& p = params[i];
        if (p.time_mode != UNS_TIME_RK3 || p.irs != 0 || p.grad_type != p0.grad_type || p.ilimit != p0.ilimit ||
            p.flow_type != p0.flow_type || p.precision != p0.precision || p.limiter_type != p0.limiter_type) {
            set_last_error("uns_cc_create_packed: cases must share RK3 without smoothing, gradient, limiter, flow "
                           "type and precision (case " + std::to_string(i) + ")");
            return UNS_ERR_ARG;
        }
        const uns_cc_mesh& m = meshes[i];
        if (m.nop <= 0 || m.noc <= 0 || m.nfi < 0 || m.nbf < 0) { set_last_error("uns_cc_create_packed: bad sizes"); return UNS_ERR_ARG; }
    }
    std::vector<long long> C(n + 1, 0), F(n + 1, 0), B(n + 1, 0), P(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        const uns_cc_mesh& m = meshes[i];
        C[i + 1] = C[i] + ((long long)m.noc + kBlock - 1) / kBlock * kBlock;
        F[i + 1] = F[i] + m.nfi;
        B[i + 1] = B[i] + m.nbf;
        P[i + 1] = P[i] + m.nop;
    }
    if (C[n] + B[n] >= (1LL << 30) || F[n] + B[n] >= (1LL << 30)) { set_last_error("uns_cc_create_packed: too large"); return UNS_ERR_ARG; }
    const int NOC = (int)C[n], NFI = (int)F[n], NBF = (int)B[n], NOP = (int)P[n], NOF = NFI + NBF, NTOT = NOC + NBF;
    std::vector<double> px(NOP), py(NOP), cx(NTOT, 0.0), cy(NTOT, 0.0), cv(NOC, 1.0), cov(NOC, 1.0);
    std::vector<double> r11(NOC, 1.0), r12(NOC, 0.0), r22(NOC, 1.0);
    std::vector<int> nc2c(NOC, 0), fp1(NOF), fp2(NOF), fin(NOF), fout(NOF), fbc(NOF);
    std::vector<double> fnx(NOF), fny(NOF), farea(NOF), fcx(NOF), fcy(NOF);
    std::vector<int> c2f_off(NOC + 1, 0), c2f, v2c_off(NOP + 1, 0), v2c;
    std::vector<double> v2c_wt;
    std::vector<int> cinst(NTOT, -1), finst(NOF), pinst(NOP);
    for (int i = 0; i < n; ++i) {
        const uns_cc_mesh& m = meshes[i];
        const int noc = m.noc, nfi = m.nfi, nof = m.nfi + m.nbf;
        auto cell = [&](int c) { return c < noc ? (int)C[i] + c : NOC + (int)B[i] + (c - noc); };
        auto face = [&](int f) { return f < nfi ? (int)F[i] + f : NFI + (int)B[i] + (f - nfi); };
        for (int k = 0; k < m.nop; ++k) { px[P[i] + k] = m.px[k]; py[P[i] + k] = m.py[k]; pinst[P[i] + k] = i; }
        for (int c = 0; c < noc + m.nbf; ++c) { cx[cell(c)] = m.cx[c]; cy[cell(c)] = m.cy[c]; cinst[cell(c)] = i; }
        for (int c = 0; c < noc; ++c) {
            const int g = (int)C[i] + c;
            cv[g] = m.cv[c]; cov[g] = m.cov[c]; r11[g] = m.r11[c]; r12[g] = m.r12[c]; r22[g] = m.r22[c]; nc2c[g] = m.nc2c[c];
        }
        for (int f = 0; f < nof; ++f) {
            const int g = face(f);
            if (m.fin[f] < 0 || m.fin[f] >= noc || m.fp1[f] < 0 || m.fp1[f] >= m.nop || m.fp2[f] < 0 || m.fp2[f] >= m.nop ||
                (f < nfi ? (m.fout[f] < 0 || m.fout[f] >= noc) : (m.fout[f] != noc + (f - nfi)))) {
                set_last_error("uns_cc_create_packed: case " + std::to_string(i) + " face " + std::to_string(f) +
                               " has an out-of-range index");
                return UNS_ERR_MESH;
            }
            fp1[g] = (int)P[i] + m.fp1[f]; fp2[g] = (int)P[i] + m.fp2[f];
            fin[g] = cell(m.fin[f]); fout[g] = cell(m.fout[f]); fbc[g] = m.fbc[f];
            fnx[g] = m.fnx[f]; fny[g] = m.fny[f]; farea[g] = m.farea[f]; fcx[g] = m.fcx[f]; fcy[g] = m.fcy[f];
            finst[g] = i;
        }
    }
    // cell -> faces (reference c2f order) and vertex -> cells, in global order
    for (int i = 0; i < n; ++i) {
        const uns_cc_mesh& m = meshes[i];
        const int noc = m.noc, nfi = m.nfi, ntot = noc + m.nbf;
        auto face = [&](int f) { return f < nfi ? (int)F[i] + f : NFI + (int)B[i] + (f - nfi); };
        auto cell = [&](int c) { return c < noc ? (int)C[i] + c : NOC + (int)B[i] + (c - noc); };
        for (int c = 0; c < (int)(C[i + 1] - C[i]); ++c) {
            const int g = (int)C[i] + c;
            if (c < noc)
                for (int k = m.c2f_off[c]; k < m.c2f_off[c + 1]; ++k) {
                    if (m.c2f[k] < 0 || m.c2f[k] >= m.nfi + m.nbf) { set_last_error("uns_cc_create_packed: c2f index out of range"); return UNS_ERR_MESH; }
                    c2f.push_back(face(m.c2f[k]));
                }
            c2f_off[g + 1] = (int)c2f.size();
        }
        for (int k = 0; k < m.nop; ++k) {
            const int g = (int)P[i] + k;
            for (int e = m.v2c_off[k]; e < m.v2c_off[k + 1]; ++e) {
                if (m.v2c[e] < 0 || m.v2c[e] >= ntot) { set_last_error("uns_cc_create_packed: v2c index out of range"); return UNS_ERR_MESH; }
                v2c.push_back(cell(m.v2c[e]));
                v2c_wt.push_back(m.v2c_wt[e]);
            }
            v2c_off[g + 1] = (int)v2c.size();
        }
    }
    uns_cc_mesh pm;
    pm.nop = NOP; pm.noc = NOC; pm.nfi = NFI; pm.nbf = NBF;
    pm.px = px.data(); pm.py = py.data(); pm.cx = cx.data(); pm.cy = cy.data(); pm.cv = cv.data(); pm.cov = cov.data();
    pm.fp1 = fp1.data(); pm.fp2 = fp2.data(); pm.fin = fin.data(); pm.fout = fout.data(); pm.fbc = fbc.data();
    pm.fnx = fnx.data(); pm.fny = fny.data(); pm.farea = farea.data(); pm.fcx = fcx.data(); pm.fcy = fcy.data();
    pm.r11 = r11.data(); pm.r12 = r12.data(); pm.r22 = r22.data(); pm.nc2c = nc2c.data();
    pm.c2f_off = c2f_off.data(); pm.c2f = c2f.data(); pm.v2c_off = v2c_off.data(); pm.v2c = v2c.data(); pm.v2c_wt = v2c_wt.data();
    uns_cc_handle* h = nullptr;
    int rc = create_impl(&pm, &p0, false, &h);
    if (rc) return rc;
    auto fail = [&](int code) { uns_cc_destroy(h); return code; };
    // per-case constants and loop control
    std::vector<Gas> gas(n);
    std::vector<double4> qinfs(n);
    std::vector<int> boff(n + 1), ncell(n);
    std::vector<double> minres(n);
    for (int i = 0; i < n; ++i) {
        gas[i] = make_gas(&params[i], &qinfs[i]);
        boff[i] = (int)(C[i] / kBlock);
        ncell[i] = meshes[i].noc;
        minres[i] = params[i].min_res;
    }
    boff[n] = (int)(C[n] / kBlock);
    CCView& v = h->v;
#define UPP(field, vec) if ((rc = h->upload(*(std::remove_const<std::remove_pointer<decltype(v.field)>::type>::type**)&v.field, vec.data(), vec.size()))) return fail(rc)
    UPP(cinst, cinst); UPP(finst, finst); UPP(pinst, pinst); UPP(gas, gas); UPP(qinfs, qinfs);
    UPP(boff, boff); UPP(ncell, ncell); UPP(minres, minres);
#undef UPP
    if ((rc = h->alloc(v.minmax, 8 * (size_t)n)) || (rc = h->alloc(v.dtmin, (size_t)n)) || (rc = h->alloc(h->d_iter, (size_t)n)) ||
        (rc = h->alloc(h->d_done, (size_t)n)) || (rc = h->alloc(h->d_fres1, (size_t)n)))
        return fail(rc);
    v.ninst = n;
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) { set_last_error("uns_cc_create_packed: upload failed"); return fail(UNS_ERR_CUDA); }
    if ((rc = uns_cc_initialize(h))) return fail(rc);
    *out = h;
    return UNS_OK;
}

int uns_cc_packed_layout(uns_cc_handle* h, int* cell_off, int* ghost_off) {
    if (!h || !h->v.ninst || !cell_off || !ghost_off) { set_last_error("uns_cc_packed_layout: not a packed handle"); return UNS_ERR_ARG; }
    const int n = h->v.ninst;
    std::vector<int> b(n + 1), nc(n);
    UNS_CUDA(cudaMemcpyAsync(b.data(), h->v.boff, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaMemcpyAsync(nc.data(), h->v.ncell, sizeof(int) * n, cudaMemcpyDeviceToHost, h->stream));
    std::vector<int> fi(h->v.nof);
    UNS_CUDA(cudaMemcpyAsync(fi.data(), h->v.finst, sizeof(int) * h->v.nof, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    for (int i = 0; i <= n; ++i) cell_off[i] = b[i] * kBlock;
    // ghosts follow the boundary faces, which are in case order
    int k = 0;
    for (int i = 0; i < n; ++i) {
        ghost_off[i] = k;
        while (k < h->v.nbf && fi[h->v.nfi + k] == i) ++k;
    }
    ghost_off[n] = k;
    return UNS_OK;
}

int uns_cc_packed_iterate(uns_cc_handle* h, int niter, const double* cfl, int first_iter, double* fres_raw, int* done_iters) {
    if (!h || !h->v.ninst || niter < 1 || !cfl || !fres_raw) { set_last_error("uns_cc_packed_iterate: bad argument"); return UNS_ERR_ARG; }
    return iterate_graph(h, niter, cfl, first_iter, fres_raw, done_iters);
}

}  // extern "C"
