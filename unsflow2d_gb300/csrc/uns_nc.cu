// uns_nc.cu -- vertex-centred median-dual (NCFVM) residual-and-update hot
// path on GB300.
//
// Per residual evaluation (NCFVM/fvresidual.f90:4-85):
//   k_nc_grad_lim  node gather over v2v: LSQ gradient (gradient.f90:2-30),
//                  then the node's limiter (VKN limiter.f90:15-98 or Barth
//                  :192-260) from its own edges -- one pass, no scatter;
//   k_nc_edge      per edge: half-edge reconstruction, van Leer or AUSM+-up
//                  flux on the dual face, Roe-averaged spectral radius, wall
//                  / farfield closure; results go to edge arrays;
//   k_nc_node_res  node gather over v2f in edge-index order (the
//                  reference's accumulation order), time_step2, optionally
//                  fused with the RK3 stage and the residual-norm partials.
// LU-SGS (lusgs.f90:4-157) runs level-scheduled in one cooperative launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "uns_common.cuh"
#include "uns_phys.cuh"
#include "unsflow_gpu.h"

using namespace uns;

namespace {

constexpr int P2_BIT = 1 << 30;  // node is fp2 of this edge
constexpr int EDGE_MASK = P2_BIT - 1;

struct NCView {
    int nop, nof, nbnd;
    const double2* pxy;
    const double* cv;
    const int2* fpt;
    const int* fbc;
    const int* fslot;   // boundary slot of an edge, -1 inside
    const double2* fn;
    const double* farea;
    const int* v2v_off;
    const int* v2v;
    const double2* wxy;
    const int* v2f_off;
    const int* v2f;     // ascending edge index, P2_BIT when the node is fp2
    const int* rv2f_off;  // reference v2f order (LU-SGS)
    const int* rv2f;
    double4* qc;
    double4* qp;
    double4* qold;
    double4* res;
    double4* gx;
    double4* gy;
    double4* phi;
    double* dt;
    double* la;
    double* fla;
    double4* fF;     // flux * area, into fp1 (fp2 receives -fF)
    double4* bres1;  // boundary closure residual into fp1 / fp2
    double4* bres2;
    double2* bla;    // boundary closure spectral radius into fp1 / fp2
    double4* fold1;  // normalflux(qold(fp1)) on the edge (LU-SGS)
    double4* fold2;
    double4* dqc;
    double* diag;    // LU-SGS diagonal cv/dt + 0.5*omega*la (lusgs.f90:36)
    double4* pw;     // sweep-published primitives of qc: (rho, u, v, p)
    double* pe;      // and e*rho, as normalflux forms them (lusgs.f90:144-147)
    double* partial;   // [2*nblk]: sum, max
    int* partial_i;    // argmax
    DevErr* err;
    const double* cfl_sched;
    int* iter;
    int* done;
    double* fres_hist;
    double* fresi_hist;
    double* fres1;
    Gas g;
    int limiter, first_iter;
    double min_res, eps, kappa;
};

__device__ __forceinline__ bool stopped(const NCView& v) { return v.done != nullptr && *((volatile int*)v.done) != 0; }
__device__ __forceinline__ void g4(const double4& q, double o[4]) { o[0] = q.x; o[1] = q.y; o[2] = q.z; o[3] = q.w; }
__device__ __forceinline__ double4 m4(const double o[4]) { return make_double4(o[0], o[1], o[2], o[3]); }

// save_old (common.f90:88-104): con2prim + qold.
__global__ void __launch_bounds__(kBlock) k_nc_save_old(NCView v) {
    if (stopped(v)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.nop) return;
    double4 q = v.qc[i];
    Prim P = con2prim(v.g, q.x, q.y, q.z, q.w);
    v.qp[i] = make_double4(P.rho, P.u, P.v, P.p);
    v.qold[i] = q;
}

__global__ void __launch_bounds__(kBlock) k_nc_grad_lim(NCView v) {
    if (stopped(v)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.nop) return;
    double qi[4], gx[4] = {0, 0, 0, 0}, gy[4] = {0, 0, 0, 0};
    g4(v.qp[i], qi);
    for (int j = v.v2v_off[i]; j < v.v2v_off[i + 1]; ++j) {
        int c = v.v2v[j];
        double2 w = v.wxy[j];
        double qc[4];
        g4(v.qp[c], qc);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            gx[k] = gx[k] + (qc[k] - qi[k]) * w.x;
            gy[k] = gy[k] + (qc[k] - qi[k]) * w.y;
        }
    }
    v.gx[i] = m4(gx);
    v.gy[i] = m4(gy);
    // DUmax/DUmin over the node's edges (limiter.f90:24-39).
    double dmx[4], dmn[4], ph[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) { dmn[k] = v.eps; dmx[k] = -v.eps; }
    const int k0 = v.v2f_off[i], k1 = v.v2f_off[i + 1];
    for (int k = k0; k < k1; ++k) {
        int e = v.v2f[k], f = e & EDGE_MASK;
        int2 p = v.fpt[f];
        double a[4], b[4];
        g4(v.qp[p.x], a);
        g4(v.qp[p.y], b);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            double du = b[j] - a[j];
            if (e & P2_BIT) du = -du;
            dmx[j] = rmax(dmx[j], du);
            dmn[j] = rmin(dmn[j], du);
        }
    }
    g4(v.phi[i], ph);
    double2 xi = v.pxy[i];
    double sq = sqrt(v.cv[i]);
    for (int k = k0; k < k1; ++k) {
        int e = v.v2f[k], f = e & EDGE_MASK;
        int2 p = v.fpt[f];
        double2 a = v.pxy[p.x], b = v.pxy[p.y];
        double d0 = b.x - a.x, d1 = b.y - a.y;
        (void)xi;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            double s = gx[j] * d0 + gy[j] * d1;
            double phj;
            if (v.limiter == UNS_LIM_VKN) {
                double D_L = (e & P2_BIT) ? -(0.5 * s) : 0.5 * s;
                double kk = v.kappa * sq;
                double TOL = kk * kk * kk;
                double alfa = D_L > 0.0 ? dmx[j] : dmn[j];
                if (fabs(alfa) < v.eps) alfa = 0.0;
                double nr = alfa * alfa + 2.0 * D_L * alfa + TOL;
                double dr = alfa * alfa + 2.0 * D_L * D_L + D_L * alfa + TOL;
                phj = rmin(1.0, nr / dr);
            } else {  // Barth-Jespersen: reference form projects fp2 with +1/2
                const bool corrected = v.limiter == UNS_LIM_BARTH_CORRECTED;
                double D_L = 0.5 * s;
                if (corrected && (e & P2_BIT)) D_L = -D_L;
                if (D_L > 0.0) phj = rmin(1.0, dmx[j] / D_L);
                else if (D_L < 0.0) phj = rmin(1.0, dmn[j] / D_L);
                else phj = 1.0;
                if (corrected) phj = rmax(0.0, phj);
            }
            ph[j] = rmin(ph[j], phj);
        }
    }
    v.phi[i] = m4(ph);
}

template <class R>
__global__ void __launch_bounds__(kBlock) k_nc_edge(NCView v) {
    if (stopped(v)) return;
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= v.nof) return;
    int2 p = v.fpt[f];
    double2 X1 = v.pxy[p.x], X2 = v.pxy[p.y];
    double d0 = X2.x - X1.x, d1 = X2.y - X1.y;
    double q1[4], q2[4], a[4], b[4], c[4], d[4], f1[4], f2[4];
    g4(v.qp[p.x], q1); g4(v.qp[p.y], q2);
    g4(v.gx[p.x], a); g4(v.gy[p.x], b); g4(v.gx[p.y], c); g4(v.gy[p.y], d);
    g4(v.phi[p.x], f1); g4(v.phi[p.y], f2);
    V4<R> L, Rt, F;
#pragma unroll
    for (int k = 0; k < 4; ++k) {  // fvresidual.f90:576-590
        double g = a[k] * d0 + b[k] * d1;
        L[k] = (R)(q1[k] + 0.5 * g * f1[k]);
        g = c[k] * d0 + d[k] * d1;
        Rt[k] = (R)(q2[k] - 0.5 * g * f2[k]);
    }
    double2 n = v.fn[f];
    double area = v.farea[f];
    const R G = (R)v.g.gamma, G1 = (R)v.g.gamma1;
    R hl, hr;
    if (v.g.flux == UNS_FLUX_AUSM) ausm_core<R>(G, G1, (R)n.x, (R)n.y, (R)v.g.mref, L, Rt, F, hl, hr);
    else vanleer_core<R>(G, G1, (R)n.x, (R)n.y, L, Rt, F, hl, hr);
    v.fF[f] = make_double4((double)F[0] * area, (double)F[1] * area, (double)F[2] * area, (double)F[3] * area);
    // Roe-averaged spectral radius (vanleer_flux.f90:417-430).
    double rL = (double)L[0], rR = (double)Rt[0];
    double RT = sqrt(rR / rL);
    double u = ((double)L[1] + RT * (double)Rt[1]) / (1.0 + RT);
    double vv = ((double)L[2] + RT * (double)Rt[2]) / (1.0 + RT);
    double H = ((double)hl + RT * (double)hr) / (1.0 + RT);
    double aa = sqrt((v.g.gamma1) * (H - 0.5 * (u * u + vv * vv)));
    double un = fabs(u * n.x + vv * n.y);
    v.fla[f] = (un + aa) * area;
    int bc = v.fbc[f];
    if (bc != 1001 && bc != 2001) return;
    int s = v.fslot[f];
    const Gas& g = v.g;
    if (bc == 1001) {  // solid_flux (solid_flux.f90:460-475)
        double pa = 0.75 * q1[3] + 0.25 * q2[3];
        double pb = 0.25 * q1[3] + 0.75 * q2[3];
        double nx = 0.5 * (X2.y - X1.y);
        double ny = -0.5 * (X2.x - X1.x);
        double ar = sqrt(nx * nx + ny * ny);
        v.bla[s] = make_double2(sqrt(g.gamma * q1[3] / q1[0]) * ar, sqrt(g.gamma * q2[3] / q2[0]) * ar);
        v.bres1[s] = make_double4(0.0, 0.0, pa * nx, pa * ny);
        v.bres2[s] = make_double4(0.0, 0.0, pb * nx, pb * ny);
    } else {  // farfield_flux1 (farfield_flux.f90:13-95)
        double nx = -(0.5 * (X2.y - X1.y));
        double ny = 0.5 * (X2.x - X1.x);
        double dr = sqrt(nx * nx + ny * ny);
        nx = nx / dr; ny = ny / dr;
        double un_inf = g.u_inf * nx + g.v_inf * ny;
        double rho = 0.5 * (q1[0] + q2[0]), uu = 0.5 * (q1[1] + q2[1]), vq = 0.5 * (q1[2] + q2[2]), pp = 0.5 * (q1[3] + q2[3]);
        double a0 = sqrt(g.gamma * pp / rho);
        double unn = uu * nx + vq * ny;
        double Rp = unn + 2.0 * a0 / g.gamma1;
        double Rm = un_inf - 2.0 * g.a_inf / g.gamma1;
        double Unf = 0.5 * (Rp + Rm);
        double af = 0.25 * (Rp - Rm) * g.gamma1;
        double uf, vf, Sf;
        if (Unf > 0.0) { uf = uu + nx * (Unf - unn); vf = vq + ny * (Unf - unn); Sf = pp / pow(rho, g.gamma); }
        else { uf = g.u_inf + nx * (Unf - un_inf); vf = g.v_inf + ny * (Unf - un_inf); Sf = g.p_inf / pow(g.r_inf, g.gamma); }
        double rhof = pow(af * af / g.gamma / Sf, 1.0 / g.gamma1);
        double pf = rhof * af * af / g.gamma;
        double ef = pf / g.gamma1 + 0.5 * rhof * (uf * uf + vf * vf);
        double fl0 = (ef + pf) * Unf, fl1 = rhof * Unf;
        double fl2 = fl1 * uf + pf * nx, fl3 = fl1 * vf + pf * ny;
        double ar = sqrt(nx * nx + ny * ny);
        v.bla[s] = make_double2((fabs(Unf) + sqrt(g.gamma * q1[3] / q1[0])) * ar, (fabs(Unf) + sqrt(g.gamma * q2[3] / q2[0])) * ar);
        double4 r = make_double4(dr * fl0, dr * fl1, dr * fl2, dr * fl3);
        v.bres1[s] = r;
        v.bres2[s] = r;
    }
}

// Node gather in edge-index order (the reference's accumulation order):
// residual, spectral radius, time_step2 (timestep.f90:173-191), optional RK3
// stage (main.f90:325-334) and residual-norm block partials
// (common.f90:130-141: sum, max with first-index tie-break).
__global__ void __launch_bounds__(kBlock) k_nc_node_res(NCView v, double cfl_in, int irk, int partial) {
    if (stopped(v)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double fr = 0.0, frs = -1.0;
    int fri = 0x7fffffff;
    if (i < v.nop) {
        double r[4] = {0, 0, 0, 0}, la = 0.0;
        for (int k = v.v2f_off[i]; k < v.v2f_off[i + 1]; ++k) {
            int e = v.v2f[k], f = e & EDGE_MASK;
            double F[4];
            g4(v.fF[f], F);
            bool is2 = (e & P2_BIT) != 0;
#pragma unroll
            for (int j = 0; j < 4; ++j) r[j] = is2 ? r[j] - F[j] : r[j] + F[j];
            la = la + v.fla[f];
            int s = v.fslot[f];
            if (s >= 0) {
                double2 bl = v.bla[s];
                la = la + (is2 ? bl.y : bl.x);
                double B[4];
                g4(is2 ? v.bres2[s] : v.bres1[s], B);
                int bc = v.fbc[f];
                if (bc == 1001) { r[2] = r[2] + B[2]; r[3] = r[3] + B[3]; }
                else {
#pragma unroll
                    for (int j = 0; j < 4; ++j) r[j] = r[j] + B[j];
                }
            }
        }
        v.res[i] = m4(r);
        v.la[i] = la;
        double cfl = v.cfl_sched ? v.cfl_sched[*v.iter] : cfl_in;
        double dt = cfl * v.cv[i] / la;
        v.dt[i] = dt;
        v.diag[i] = v.cv[i] / dt + 0.5 * 1.5 * la;
        if (irk > 0) {
            double a = rk3_a(irk), b = rk3_b(irk);
            double dtbyarea = dt / v.cv[i];
            double o[4], c[4], q[4];
            g4(v.qold[i], o);
            g4(v.qc[i], c);
#pragma unroll
            for (int j = 0; j < 4; ++j) q[j] = a * o[j] + b * (c[j] - dtbyarea * r[j]);
            v.qc[i] = m4(q);
        }
        double t = 0.0;
#pragma unroll
        for (int j = 0; j < 4; ++j) t = t + r[j] * r[j];
        fr = t;
        frs = sqrt(t);
        fri = i;
    }
    if (!partial) return;
    __shared__ double ss[kBlock / 32], sm[kBlock / 32];
    __shared__ int si[kBlock / 32];
    double s = warp_sum(fr);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        double om = __shfl_xor_sync(0xffffffffu, frs, o);
        int oi = __shfl_xor_sync(0xffffffffu, fri, o);
        if (om > frs || (om == frs && oi < fri)) { frs = om; fri = oi; }
    }
    int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { ss[w] = s; sm[w] = frs; si[w] = fri; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0, m = -1.0;
        int mi = 0x7fffffff;
        for (int k = 0; k < kBlock / 32; ++k) {
            t = t + ss[k];
            if (sm[k] > m || (sm[k] == m && si[k] < mi)) { m = sm[k]; mi = si[k]; }
        }
        v.partial[2 * blockIdx.x] = t;
        v.partial[2 * blockIdx.x + 1] = m;
        v.partial_i[blockIdx.x] = mi;
    }
}

__global__ void __launch_bounds__(kBlock) k_nc_rk(NCView v, int irk) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.nop) return;
    double a = rk3_a(irk), b = rk3_b(irk);
    double dtbyarea = v.dt[i] / v.cv[i];
    double o[4], c[4], r[4], q[4];
    g4(v.qold[i], o); g4(v.qc[i], c); g4(v.res[i], r);
#pragma unroll
    for (int j = 0; j < 4; ++j) q[j] = a * o[j] + b * (c[j] - dtbyarea * r[j]);
    v.qc[i] = m4(q);
}

__global__ void __launch_bounds__(kBlock) k_nc_res_partial(NCView v) {
    // Same partials as k_nc_node_res, recomputed from the stored residual.
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double fr = 0.0, frs = -1.0;
    int fri = 0x7fffffff;
    if (i < v.nop) {
        double r[4];
        g4(v.res[i], r);
        double t = 0.0;
#pragma unroll
        for (int j = 0; j < 4; ++j) t = t + r[j] * r[j];
        fr = t; frs = sqrt(t); fri = i;
    }
    __shared__ double ss[kBlock / 32], sm[kBlock / 32];
    __shared__ int si[kBlock / 32];
    double s = warp_sum(fr);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        double om = __shfl_xor_sync(0xffffffffu, frs, o);
        int oi = __shfl_xor_sync(0xffffffffu, fri, o);
        if (om > frs || (om == frs && oi < fri)) { frs = om; fri = oi; }
    }
    int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { ss[w] = s; sm[w] = frs; si[w] = fri; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0, m = -1.0;
        int mi = 0x7fffffff;
        for (int k = 0; k < kBlock / 32; ++k) {
            t = t + ss[k];
            if (sm[k] > m || (sm[k] == m && si[k] < mi)) { m = sm[k]; mi = si[k]; }
        }
        v.partial[2 * blockIdx.x] = t;
        v.partial[2 * blockIdx.x + 1] = m;
        v.partial_i[blockIdx.x] = mi;
    }
}

__global__ void __launch_bounds__(kBlock) k_nc_res_final(NCView v, int nparts, double* out) {
    if (stopped(v)) return;
    __shared__ double s[kBlock], sm[kBlock];
    __shared__ int si[kBlock];
    double t = 0.0, m = -1.0;
    int mi = 0x7fffffff;
    for (int k = threadIdx.x; k < nparts; k += blockDim.x) {
        t = t + v.partial[2 * k];
        double pm = v.partial[2 * k + 1];
        int pi = v.partial_i[k];
        if (pm > m || (pm == m && pi < mi)) { m = pm; mi = pi; }
    }
    s[threadIdx.x] = t; sm[threadIdx.x] = m; si[threadIdx.x] = mi;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            s[threadIdx.x] = s[threadIdx.x] + s[threadIdx.x + w];
            double om = sm[threadIdx.x + w];
            int oi = si[threadIdx.x + w];
            if (om > sm[threadIdx.x] || (om == sm[threadIdx.x] && oi < si[threadIdx.x])) { sm[threadIdx.x] = om; si[threadIdx.x] = oi; }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double fres = sqrt(s[0] / (double)v.nop);
        double fresi = sm[0] > 0.0 ? sm[0] : 0.0;
        int iresi = sm[0] > 0.0 ? si[0] : -1;
        if (out) { out[0] = fres; out[1] = fresi; out[2] = (double)iresi; }
        if (v.iter) {
            int it = *v.iter;
            v.fres_hist[it] = fres;
            v.fresi_hist[it] = fresi;
            if (it == 0 && v.first_iter) *v.fres1 = fres;
            double f1 = *v.fres1;
            double nf = (f1 != 0.0) ? fres / f1 : fres;
            if (!(nf > v.min_res) || v.err->code != 0) {
                *v.done = 1;
                if (v.err->code != 0) v.err->iter = it;
            }
            *v.iter = it + 1;
        }
    }
}

// normalflux(qold) of both end nodes on every edge (lusgs.f90:137-155); it
// does not change during the sweeps, so it is evaluated once per edge.
__device__ __forceinline__ void normalflux_nc(const Gas& g, const double4& q, double nx, double ny, double ds, double o[4]) {
    Prim P = con2prim(g, q.x, q.y, q.z, q.w);
    double et = P.e * P.rho;
    double un = P.u * nx + P.v * ny;
    o[0] = (et + P.p) * un;
    o[1] = P.rho * un;
    o[2] = o[1] * P.u + P.p * nx;
    o[3] = o[1] * P.v + P.p * ny;
#pragma unroll
    for (int k = 0; k < 4; ++k) o[k] = o[k] * ds;
}

__global__ void __launch_bounds__(kBlock) k_nc_fold(NCView v) {
    if (stopped(v)) return;
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= v.nof) return;
    int2 p = v.fpt[f];
    double2 n = v.fn[f];
    double ds = v.farea[f], o[4];
    normalflux_nc(v.g, v.qold[p.x], n.x, n.y, ds, o);
    v.fold1[f] = m4(o);
    normalflux_nc(v.g, v.qold[p.y], n.x, n.y, ds, o);
    v.fold2[f] = m4(o);
}

// normalflux (lusgs.f90:137-155) from primitives a sweep has published.
__device__ __forceinline__ void normalflux_prims(const double4& w, double et, double nx, double ny, double ds,
                                                 double o[4]) {
    double un = w.y * nx + w.z * ny;
    o[0] = (et + w.w) * un;
    o[1] = w.x * un;
    o[2] = o[1] * w.y + w.w * nx;
    o[3] = o[1] * w.z + w.w * ny;
#pragma unroll
    for (int k = 0; k < 4; ++k) o[k] = o[k] * ds;
}

// lusgs sweeps (lusgs.f90:48-124) as a dataflow kernel.  Items are the
// forward sweep's nodes sorted by dependency level, then the backward sweep's;
// item s goes to warp s mod (warps in the grid).  A warp's lanes take the
// node's edges (reference v2f order), wait for the neighbour's completion flag
// when that neighbour precedes the node in the sweep, and form the edge term
// from the primitives the neighbour published; lane 0 adds the terms in edge
// order -- the reference's summation order -- updates the node, publishes its
// primitives (the con2prim a later normalflux of this node would do) and
// releases its flag.  Every wait targets an earlier item, and the cooperative
// launch keeps all warps resident, so the sweep always completes; each wait is
// also bounded (wait_flag).
__global__ void __launch_bounds__(kBlock) k_nc_lusgs(NCView v, const int* __restrict__ order, int nfwd, int nitems,
                                                     int* flag) {
    __shared__ double sterm[kBlock / 32][32][4];
    const double omega = 1.5;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int gw = blockIdx.x * (kBlock / 32) + wib, nw = gridDim.x * (kBlock / 32);
    if (stopped(v)) return;
    for (int s = gw; s < nitems; s += nw) {
        const int pass = s < nfwd ? 0 : 1;
        const int it = order[s];
        const int k0 = v.rv2f_off[it], deg = v.rv2f_off[it + 1] - k0;
        bool take = false, ok = true;
        double t4[4] = {0.0, 0.0, 0.0, 0.0};
        if (lane < deg) {
            int c = v.rv2f[k0 + lane];
            int2 p = v.fpt[c];
            int nb = p.y;
            double sign = 1.0;
            bool nb_is_p1 = false;
            if (nb == it) { nb = p.x; sign = -1.0; nb_is_p1 = true; }
            take = pass == 0 ? (nb < it && nb >= 0) : (nb > it && nb >= 0);
            if (take) {
                ok = wait_flag(flag + nb, pass + 1, v.err);
                if (ok) {
                    double2 n = v.fn[c];
                    double f1[4], f2[4], dq[4];
                    g4(nb_is_p1 ? v.fold1[c] : v.fold2[c], f1);
                    normalflux_prims(ldcg4(&v.pw[nb]), __ldcg(&v.pe[nb]), n.x, n.y, v.farea[c], f2);
                    g4(ldcg4(&v.dqc[nb]), dq);
                    double ol = omega * v.fla[c];
#pragma unroll
                    for (int iv = 0; iv < 4; ++iv) t4[iv] = 0.5 * (sign * (f2[iv] - f1[iv]) - ol * dq[iv]);
                }
            }
        }
        if (pass == 1 && lane == 0) ok = ok && wait_flag(flag + it, 1, v.err);  // own forward value
        if (__ballot_sync(0xffffffffu, !ok)) return;
        unsigned taken = __ballot_sync(0xffffffffu, take);
#pragma unroll
        for (int iv = 0; iv < 4; ++iv) sterm[wib][lane][iv] = t4[iv];
        __syncwarp();
        if (lane == 0) {
            double cres[4] = {0.0, 0.0, 0.0, 0.0};
            for (int j = 0; j < deg; ++j)
                if (taken & (1u << j))
#pragma unroll
                    for (int iv = 0; iv < 4; ++iv) cres[iv] = cres[iv] + sterm[wib][j][iv];
            const double D = v.diag[it];
            double d[4], o[4], r[4], q[4];
            g4(v.qold[it], o);
            if (pass == 0) {
                g4(v.res[it], r);
#pragma unroll
                for (int iv = 0; iv < 4; ++iv) d[iv] = (-r[iv] - cres[iv]) / D;
            } else {
                g4(ldcg4(&v.dqc[it]), d);
#pragma unroll
                for (int iv = 0; iv < 4; ++iv) d[iv] = d[iv] - cres[iv] / D;
            }
#pragma unroll
            for (int iv = 0; iv < 4; ++iv) q[iv] = o[iv] + d[iv];
            Prim P = con2prim(v.g, q[0], q[1], q[2], q[3]);
            stcg4(&v.dqc[it], m4(d));
            stcg4(&v.pw[it], make_double4(P.rho, P.u, P.v, P.p));
            __stcg(&v.pe[it], P.e * P.rho);
            v.qc[it] = m4(q);
            st_release(flag + it, pass + 1);
        }
        __syncwarp();
    }
}

__global__ void k_nc_initialize(NCView v, double4 qinf, double phi0) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.nop) return;
    v.qc[i] = qinf;
    v.phi[i] = make_double4(phi0, phi0, phi0, phi0);
}

void build_levels_nc(int nop, const int* v2f_off, const int* v2f, const int* fp1, const int* fp2, bool forward,
                     std::vector<int>& off, std::vector<int>& nodes) {
    std::vector<int> lev(nop, 0);
    int maxl = 0;
    for (int s = 0; s < nop; ++s) {
        int it = forward ? s : nop - 1 - s;
        int l = 0;
        for (int k = v2f_off[it]; k < v2f_off[it + 1]; ++k) {
            int c = v2f[k];
            int nb = fp2[c] == it ? fp1[c] : fp2[c];
            if (nb < 0 || nb == it) continue;
            if (forward ? nb < it : nb > it) l = std::max(l, lev[nb] + 1);
        }
        lev[it] = l;
        maxl = std::max(maxl, l);
    }
    off.assign(maxl + 2, 0);
    for (int i = 0; i < nop; ++i) off[lev[i] + 1]++;
    for (int l = 0; l <= maxl; ++l) off[l + 1] += off[l];
    nodes.assign(nop, 0);
    std::vector<int> pos(off.begin(), off.end() - 1);
    for (int i = 0; i < nop; ++i) nodes[pos[lev[i]]++] = i;
}

}  // namespace

struct uns_nc_handle {
    uns_params P;
    NCView v;
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;
    int nparts = 0;
    int* order = nullptr;   // forward items (level order) then backward items
    int* flag = nullptr;    // per-node sweep progress: 0, 1 forward done, 2 backward done
    int coop_blocks = 0;
    double4 qinf;
    cudaGraphExec_t graph = nullptr;
    int graph_first = -1;
    double* d_cfl = nullptr;
    double* d_hist = nullptr;
    double* d_histi = nullptr;
    int cfl_cap = 0;
    int* d_iter = nullptr;
    int* d_done = nullptr;
    double* d_fres1 = nullptr;
    double* d_scalar = nullptr;

    template <class T>
    int alloc(T*& p, size_t n) {
        void* q = nullptr;
        size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
        UNS_CUDA(cudaMalloc(&q, bytes));
        UNS_CUDA(cudaMemsetAsync(q, 0, bytes, stream));
        allocs.push_back(q);
        p = (T*)q;
        return UNS_OK;
    }
    template <class T>
    int upload(T*& p, const T* src, size_t n) {
        int rc = alloc(p, n);
        if (rc) return rc;
        if (n) UNS_CUDA(cudaMemcpyAsync(p, src, n * sizeof(T), cudaMemcpyHostToDevice, stream));
        return UNS_OK;
    }
};

namespace {

int check_err_nc(uns_nc_handle* h) {
    DevErr e;
    UNS_CUDA(cudaMemcpyAsync(&e, h->v.err, sizeof(DevErr), cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    if (e.code != 0) {
        set_last_error(std::string(e.code == UNS_ERR_TIMEOUT ? "bounded device wait timed out in block " : "device error at ") +
                       std::to_string(e.index));
        int code = e.code;
        DevErr z = {0, 0, 0, 0};
        UNS_CUDA(cudaMemcpyAsync(h->v.err, &z, sizeof(DevErr), cudaMemcpyHostToDevice, h->stream));
        UNS_CUDA(cudaStreamSynchronize(h->stream));
        return code;
    }
    return UNS_OK;
}

#define NLAUNCH(kern, n, ...)                                                        \
    do {                                                                             \
        kern<<<std::max(1, nblocks(n)), kBlock, 0, h->stream>>>(__VA_ARGS__);        \
        UNS_CUDA(cudaGetLastError());                                                \
    } while (0)

int enqueue_fvres_nc(uns_nc_handle* h, NCView& v, double cfl, int irk, int partial) {
    NLAUNCH(k_nc_grad_lim, v.nop, v);
    if (h->P.precision == UNS_PREC_MIXED) NLAUNCH(k_nc_edge<float>, v.nof, v);
    else NLAUNCH(k_nc_edge<double>, v.nof, v);
    NLAUNCH(k_nc_node_res, v.nop, v, cfl, irk, partial);
    return UNS_OK;
}

int launch_sweeps_nc(uns_nc_handle* h, NCView& v) {
    UNS_CUDA(cudaMemsetAsync(v.dqc, 0, sizeof(double4) * v.nop, h->stream));
    UNS_CUDA(cudaMemsetAsync(h->flag, 0, sizeof(int) * v.nop, h->stream));
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(h->coop_blocks);
    cfg.blockDim = dim3(kBlock);
    cfg.stream = h->stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    UNS_CUDA(cudaLaunchKernelEx(&cfg, k_nc_lusgs, v, (const int*)h->order, v.nop, 2 * v.nop, h->flag));
    return UNS_OK;
}

int enqueue_lusgs_nc(uns_nc_handle* h, NCView& v) {
    NLAUNCH(k_nc_fold, v.nof, v);
    return launch_sweeps_nc(h, v);
}

int enqueue_iteration_nc(uns_nc_handle* h, NCView& v) {
    int rc;
    NLAUNCH(k_nc_save_old, v.nop, v);
    if (h->P.time_mode == UNS_TIME_RK3) {
        for (int irk = 1; irk <= 3; ++irk)
            if ((rc = enqueue_fvres_nc(h, v, 0.0, irk, irk == 3))) return rc;
    } else {
        if ((rc = enqueue_fvres_nc(h, v, 0.0, 0, 1))) return rc;
        if ((rc = enqueue_lusgs_nc(h, v))) return rc;
    }
    k_nc_res_final<<<1, kBlock, 0, h->stream>>>(v, h->nparts, nullptr);
    UNS_CUDA(cudaGetLastError());
    return UNS_OK;
}

}  // namespace

extern "C" {

int uns_nc_create(const uns_nc_mesh* m, const uns_params* p, uns_nc_handle** out) {
    if (!m || !p || !out) { set_last_error("uns_nc_create: null argument"); return UNS_ERR_ARG; }
    *out = nullptr;
    if (m->nop <= 0 || m->nof <= 0 || !(p->m_inf > 0.0) || p->time_mode < 0 || p->time_mode > 1 ||
        (p->flux_type != UNS_FLUX_VANLEER && p->flux_type != UNS_FLUX_AUSM) ||
        (p->limiter_type < UNS_LIM_VKN || p->limiter_type > UNS_LIM_BARTH_CORRECTED)) {
        set_last_error("uns_nc_create: bad sizes or parameters");
        return UNS_ERR_ARG;
    }
    const int nop = m->nop, nof = m->nof;
    for (int f = 0; f < nof; ++f)
        if (m->fp1[f] < 0 || m->fp1[f] >= nop || m->fp2[f] < 0 || m->fp2[f] >= nop) {
            set_last_error("uns_nc_create: edge " + std::to_string(f) + " has an out-of-range node");
            return UNS_ERR_MESH;
        }
    for (int k = 0; k < m->v2v_off[nop]; ++k)
        if (m->v2v[k] < 0 || m->v2v[k] >= nop) { set_last_error("uns_nc_create: v2v out of range"); return UNS_ERR_MESH; }
    for (int k = 0; k < m->v2f_off[nop]; ++k)
        if (m->v2f[k] < 0 || m->v2f[k] >= nof) { set_last_error("uns_nc_create: v2f out of range"); return UNS_ERR_MESH; }
    uns_nc_handle* h = new uns_nc_handle();
    h->P = *p;
    auto fail = [&](int code) { uns_nc_destroy(h); return code; };
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) {
        set_last_error("uns_nc_create: cudaStreamCreate failed (no usable GPU?)");
        delete h;
        return UNS_ERR_CUDA;
    }
    Gas g;
    std::memset(&g, 0, sizeof(g));
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
    g.mref = std::max((double)0.32f, 0.5 * p->m_inf);
    g.flux = p->flux_type;
    h->qinf = make_double4(q0, q1, q2, q3);

    std::vector<double2> pxy(nop), fn(nof), wxy(m->v2v_off[nop]);
    std::vector<int2> fpt(nof);
    std::vector<int> fslot(nof, -1);
    int nbnd = 0;
    for (int i = 0; i < nop; ++i) pxy[i] = make_double2(m->px[i], m->py[i]);
    for (int f = 0; f < nof; ++f) {
        fpt[f] = make_int2(m->fp1[f], m->fp2[f]);
        fn[f] = make_double2(m->fnx[f], m->fny[f]);
        if (m->fbc[f] == 1001 || m->fbc[f] == 2001) fslot[f] = nbnd++;
    }
    for (int k = 0; k < m->v2v_off[nop]; ++k) wxy[k] = make_double2(m->wx[k], m->wy[k]);
    std::vector<int> cnt(nop + 1, 0);
    for (int f = 0; f < nof; ++f) { cnt[m->fp1[f] + 1]++; cnt[m->fp2[f] + 1]++; }
    for (int i = 0; i < nop; ++i) cnt[i + 1] += cnt[i];
    std::vector<int> vf(cnt[nop]), pos(cnt.begin(), cnt.end() - 1);
    for (int f = 0; f < nof; ++f) { vf[pos[m->fp1[f]]++] = f; vf[pos[m->fp2[f]]++] = f | P2_BIT; }

    NCView& v = h->v;
    std::memset(&v, 0, sizeof(v));
    v.nop = nop; v.nof = nof; v.nbnd = nbnd;
    v.g = g;
    v.limiter = p->limiter_type;
    v.min_res = p->min_res;
    v.eps = (double)1.1920928955078125e-07f;
    v.kappa = (double)0.01f;
    int rc;
#define UPN(field, vec) if ((rc = h->upload(*(std::remove_const<std::remove_pointer<decltype(v.field)>::type>::type**)&v.field, vec.data(), vec.size()))) return fail(rc)
#define ALN(field, n) if ((rc = h->alloc(v.field, (n)))) return fail(rc)
    UPN(pxy, pxy);
    { std::vector<double> t(m->cv, m->cv + nop); UPN(cv, t); }
    UPN(fpt, fpt);
    { std::vector<int> t(m->fbc, m->fbc + nof); UPN(fbc, t); }
    UPN(fslot, fslot);
    UPN(fn, fn);
    { std::vector<double> t(m->farea, m->farea + nof); UPN(farea, t); }
    { std::vector<int> t(m->v2v_off, m->v2v_off + nop + 1); UPN(v2v_off, t); }
    { std::vector<int> t(m->v2v, m->v2v + m->v2v_off[nop]); UPN(v2v, t); }
    UPN(wxy, wxy);
    UPN(v2f_off, cnt); UPN(v2f, vf);
    { std::vector<int> t(m->v2f_off, m->v2f_off + nop + 1); UPN(rv2f_off, t); }
    { std::vector<int> t(m->v2f, m->v2f + m->v2f_off[nop]); UPN(rv2f, t); }
    ALN(qc, nop); ALN(qp, nop); ALN(qold, nop); ALN(res, nop); ALN(gx, nop); ALN(gy, nop); ALN(phi, nop);
    ALN(dt, nop); ALN(la, nop); ALN(fla, nof); ALN(fF, nof); ALN(bres1, nbnd); ALN(bres2, nbnd); ALN(bla, nbnd);
    ALN(fold1, nof); ALN(fold2, nof); ALN(dqc, nop); ALN(diag, nop); ALN(pw, nop); ALN(pe, nop); ALN(err, 1);
    h->nparts = nblocks(nop);
    ALN(partial, 2 * h->nparts);
    ALN(partial_i, h->nparts);
    if ((rc = h->alloc(h->d_scalar, 4))) return fail(rc);
    if ((rc = h->alloc(h->d_iter, 1))) return fail(rc);
    if ((rc = h->alloc(h->d_done, 1))) return fail(rc);
    if ((rc = h->alloc(h->d_fres1, 1))) return fail(rc);
    {
        // Dataflow order of the two sweeps; a warp per node handles up to 32 edges.
        int maxdeg = 0;
        for (int i = 0; i < nop; ++i) maxdeg = std::max(maxdeg, m->v2f_off[i + 1] - m->v2f_off[i]);
        if (maxdeg > 32) { set_last_error("uns_nc_create: a node has more than 32 edges"); return fail(UNS_ERR_MESH); }
        std::vector<int> off, fwd, bwd;
        build_levels_nc(nop, m->v2f_off, m->v2f, m->fp1, m->fp2, true, off, fwd);
        build_levels_nc(nop, m->v2f_off, m->v2f, m->fp1, m->fp2, false, off, bwd);
        fwd.insert(fwd.end(), bwd.begin(), bwd.end());
        if ((rc = h->upload(h->order, fwd.data(), fwd.size()))) return fail(rc);
        if ((rc = h->alloc(h->flag, nop))) return fail(rc);
        int dev = 0, nsm = 0, per = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_nc_lusgs, kBlock, 0) != cudaSuccess || per < 1) {
            set_last_error("uns_nc_create: cannot size the cooperative LU-SGS launch");
            return fail(UNS_ERR_CUDA);
        }
        h->coop_blocks = nsm * std::min(per, 4);
    }
#undef UPN
#undef ALN
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) { set_last_error("uns_nc_create: upload failed"); return fail(UNS_ERR_CUDA); }
    if ((rc = uns_nc_initialize(h))) return fail(rc);
    *out = h;
    return UNS_OK;
}

int uns_nc_destroy(uns_nc_handle* h) {
    if (!h) return UNS_OK;
    if (h->stream) cudaStreamSynchronize(h->stream);
    if (h->graph) cudaGraphExecDestroy(h->graph);
    for (void* p : h->allocs) cudaFree(p);
    if (h->d_cfl) cudaFree(h->d_cfl);
    if (h->d_hist) cudaFree(h->d_hist);
    if (h->d_histi) cudaFree(h->d_histi);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return UNS_OK;
}

int uns_nc_initialize(uns_nc_handle* h) {
    if (!h) return UNS_ERR_ARG;
    k_nc_initialize<<<nblocks(h->v.nop), kBlock, 0, h->stream>>>(h->v, h->qinf, (double)1e20f);
    UNS_CUDA(cudaGetLastError());
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    return UNS_OK;
}

int uns_nc_set_state(uns_nc_handle* h, const double* qc) {
    if (!h || !qc) return UNS_ERR_ARG;
    UNS_CUDA(cudaMemcpyAsync(h->v.qc, qc, sizeof(double4) * h->v.nop, cudaMemcpyHostToDevice, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    return UNS_OK;
}

int uns_nc_get_state(uns_nc_handle* h, double* qc) {
    if (!h || !qc) return UNS_ERR_ARG;
    UNS_CUDA(cudaMemcpyAsync(qc, h->v.qc, sizeof(double4) * h->v.nop, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    return UNS_OK;
}

int uns_nc_get_field(uns_nc_handle* h, int field, double* out) {
    if (!h || !out) return UNS_ERR_ARG;
    const NCView& v = h->v;
    auto d2h = [&](const void* src, size_t bytes) { return cudaMemcpyAsync(out, src, bytes, cudaMemcpyDeviceToHost, h->stream); };
    switch (field) {
        case UNS_NC_QC: UNS_CUDA(d2h(v.qc, sizeof(double4) * v.nop)); break;
        case UNS_NC_QP: UNS_CUDA(d2h(v.qp, sizeof(double4) * v.nop)); break;
        case UNS_NC_QOLD: UNS_CUDA(d2h(v.qold, sizeof(double4) * v.nop)); break;
        case UNS_NC_RES: UNS_CUDA(d2h(v.res, sizeof(double4) * v.nop)); break;
        case UNS_NC_PHI: UNS_CUDA(d2h(v.phi, sizeof(double4) * v.nop)); break;
        case UNS_NC_DT: UNS_CUDA(d2h(v.dt, sizeof(double) * v.nop)); break;
        case UNS_NC_LA: UNS_CUDA(d2h(v.la, sizeof(double) * v.nop)); break;
        case UNS_NC_FLA: UNS_CUDA(d2h(v.fla, sizeof(double) * v.nof)); break;
        case UNS_NC_GRAD: {
            std::vector<double4> X(v.nop), Y(v.nop);
            UNS_CUDA(cudaMemcpyAsync(X.data(), v.gx, sizeof(double4) * v.nop, cudaMemcpyDeviceToHost, h->stream));
            UNS_CUDA(cudaMemcpyAsync(Y.data(), v.gy, sizeof(double4) * v.nop, cudaMemcpyDeviceToHost, h->stream));
            UNS_CUDA(cudaStreamSynchronize(h->stream));
            for (int i = 0; i < v.nop; ++i) {
                double a[4] = {X[i].x, X[i].y, X[i].z, X[i].w}, b[4] = {Y[i].x, Y[i].y, Y[i].z, Y[i].w};
                for (int j = 0; j < 4; ++j) { out[(size_t)i * 8 + 2 * j] = a[j]; out[(size_t)i * 8 + 2 * j + 1] = b[j]; }
            }
            return UNS_OK;
        }
        default: set_last_error("uns_nc_get_field: unknown field"); return UNS_ERR_ARG;
    }
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    return UNS_OK;
}

int uns_nc_save_old(uns_nc_handle* h) {
    if (!h) return UNS_ERR_ARG;
    NCView v = h->v;
    NLAUNCH(k_nc_save_old, v.nop, v);
    return UNS_OK;
}

int uns_nc_fvresidual(uns_nc_handle* h, double cfl) {
    if (!h) return UNS_ERR_ARG;
    NCView v = h->v;
    return enqueue_fvres_nc(h, v, cfl, 0, 0);
}

int uns_nc_rk_stage(uns_nc_handle* h, int irk) {
    if (!h || irk < 1 || irk > 3) return UNS_ERR_ARG;
    NCView v = h->v;
    NLAUNCH(k_nc_rk, v.nop, v, irk);
    return UNS_OK;
}

int uns_nc_lusgs(uns_nc_handle* h, double cfl) {
    if (!h) return UNS_ERR_ARG;
    NCView v = h->v;
    int rc = enqueue_fvres_nc(h, v, cfl, 0, 0);
    if (rc) return rc;
    return enqueue_lusgs_nc(h, v);
}

int uns_nc_residue(uns_nc_handle* h, double* fres, double* fresi, int* iresi) {
    if (!h) return UNS_ERR_ARG;
    NCView v = h->v;
    NLAUNCH(k_nc_res_partial, v.nop, v);
    k_nc_res_final<<<1, kBlock, 0, h->stream>>>(v, h->nparts, h->d_scalar);
    UNS_CUDA(cudaGetLastError());
    double r[3];
    UNS_CUDA(cudaMemcpyAsync(r, h->d_scalar, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    if (fres) *fres = r[0];
    if (fresi) *fresi = r[1];
    if (iresi) *iresi = (int)r[2];
    return check_err_nc(h);
}

int uns_nc_iterate(uns_nc_handle* h, int niter, const double* cfl, int first_iter, double* fres_raw, double* fresi,
                   int* done_iters) {
    if (!h || niter < 0 || (niter > 0 && (!cfl || !fres_raw))) return UNS_ERR_ARG;
    if (done_iters) *done_iters = 0;
    if (niter == 0) return UNS_OK;
    if (niter > h->cfl_cap) {
        if (h->d_cfl) cudaFree(h->d_cfl);
        if (h->d_hist) cudaFree(h->d_hist);
        if (h->d_histi) cudaFree(h->d_histi);
        h->d_cfl = h->d_hist = h->d_histi = nullptr;
        UNS_CUDA(cudaMalloc(&h->d_cfl, sizeof(double) * niter));
        UNS_CUDA(cudaMalloc(&h->d_hist, sizeof(double) * niter));
        UNS_CUDA(cudaMalloc(&h->d_histi, sizeof(double) * niter));
        h->cfl_cap = niter;
        if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    }
    UNS_CUDA(cudaMemcpyAsync(h->d_cfl, cfl, sizeof(double) * niter, cudaMemcpyHostToDevice, h->stream));
    UNS_CUDA(cudaMemsetAsync(h->d_iter, 0, sizeof(int), h->stream));
    UNS_CUDA(cudaMemsetAsync(h->d_done, 0, sizeof(int), h->stream));
    UNS_CUDA(cudaMemsetAsync(h->d_hist, 0, sizeof(double) * niter, h->stream));
    if (!h->graph || h->graph_first != (first_iter ? 1 : 0)) {
        if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
        NCView v = h->v;
        v.cfl_sched = h->d_cfl;
        v.iter = h->d_iter;
        v.done = h->d_done;
        v.fres_hist = h->d_hist;
        v.fresi_hist = h->d_histi;
        v.fres1 = h->d_fres1;
        v.first_iter = first_iter ? 1 : 0;
        cudaGraph_t graph;
        UNS_CUDA(cudaStreamSynchronize(h->stream));
        UNS_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        int rc = enqueue_iteration_nc(h, v);
        cudaError_t ce = cudaStreamEndCapture(h->stream, &graph);
        if (rc) return rc;
        if (ce != cudaSuccess) { set_last_error(std::string("graph capture: ") + cudaGetErrorString(ce)); return UNS_ERR_CUDA; }
        ce = cudaGraphInstantiate(&h->graph, graph, 0);
        cudaGraphDestroy(graph);
        if (ce != cudaSuccess) { set_last_error(std::string("graph instantiate: ") + cudaGetErrorString(ce)); return UNS_ERR_CUDA; }
        h->graph_first = first_iter ? 1 : 0;
    }
    for (int k = 0; k < niter; ++k) UNS_CUDA(cudaGraphLaunch(h->graph, h->stream));
    UNS_CUDA(cudaMemcpyAsync(fres_raw, h->d_hist, sizeof(double) * niter, cudaMemcpyDeviceToHost, h->stream));
    if (fresi) UNS_CUDA(cudaMemcpyAsync(fresi, h->d_histi, sizeof(double) * niter, cudaMemcpyDeviceToHost, h->stream));
    int it = 0;
    UNS_CUDA(cudaMemcpyAsync(&it, h->d_iter, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    if (done_iters) *done_iters = it;
    return check_err_nc(h);
}

void* uns_nc_stream(uns_nc_handle* h) { return h ? (void*)h->stream : nullptr; }

int uns_nc_profile(uns_nc_handle* h, double cfl, int reps, double* ms, const char** names, int nphase) {
    static const char* kNames[] = {"save_old", "grad_lim", "edge", "node_res", "fold", "lusgs_sweeps", "residue"};
    const int NP = 7;
    if (!h || reps < 1 || !ms) return UNS_ERR_ARG;
    std::vector<double> acc(NP, 0.0);
    cudaEvent_t e0, e1;
    UNS_CUDA(cudaEventCreate(&e0));
    UNS_CUDA(cudaEventCreate(&e1));
    NCView v = h->v;
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
    for (int r = 0; r < reps && !rc; ++r) {
        rc = timed(0, [&]() -> int { NLAUNCH(k_nc_save_old, v.nop, v); return UNS_OK; });
        for (int irk = 1; irk <= (rk3 ? 3 : 1) && !rc; ++irk) {
            if (!rc) rc = timed(1, [&]() -> int { NLAUNCH(k_nc_grad_lim, v.nop, v); return UNS_OK; });
            if (!rc) rc = timed(2, [&]() -> int {
                if (h->P.precision == UNS_PREC_MIXED) NLAUNCH(k_nc_edge<float>, v.nof, v);
                else NLAUNCH(k_nc_edge<double>, v.nof, v);
                return UNS_OK;
            });
            if (!rc) rc = timed(3, [&]() -> int { NLAUNCH(k_nc_node_res, v.nop, v, cfl, rk3 ? irk : 0, rk3 ? (irk == 3) : 1); return UNS_OK; });
        }
        if (!rk3) {
            if (!rc) rc = timed(4, [&]() -> int { NLAUNCH(k_nc_fold, v.nof, v); return UNS_OK; });
            if (!rc) rc = timed(5, [&]() -> int { return launch_sweeps_nc(h, v); });
        }
        if (!rc) rc = timed(6, [&]() -> int {
            k_nc_res_final<<<1, kBlock, 0, h->stream>>>(v, h->nparts, h->d_scalar);
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
    return check_err_nc(h);
}

}  // extern "C"
