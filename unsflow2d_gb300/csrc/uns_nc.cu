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
// LU-SGS (lusgs.f90:4-157) runs as a list-scheduled dataflow sweep in one cooperative launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "uns_common.cuh"
#include "uns_phys.cuh"
#include "uns_sched.hpp"
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
    float4* qpf;          // FP32 copy of qp (k_nc_save_old), read by the mixed form's gradient pass
    float4* packn;        // mixed form, per node: FP32 gx, gy, phi (k_nc_grad_lim_mixed) for the edge pass
    const float2* wxyf;   // FP32 LSQ weights per v2v entry
    const float2* edf;    // FP32 edge vector X(fp2) - X(fp1) per edge
    double4* qold;
    double4* qoldp;  // (u, v, p, e*rho) of qold per node, for the FP64 sweep records
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
    // LU-SGS sweep schedule (host-built): per position of the warp lists
    // (it, pass, first record, records); per record, in the reference v2f
    // order of the taken edges: edge, neighbour, orientation sign.
    const int4* sched;
    const int* rec_edge;
    const int* rec_nb;
    const int* rec_sign;
    int nrec;
    double4* rec;    // per record, per LU-SGS call: 3 x double4 (k_nc_sweep_prep) or 4 x float4 (k_nc_sweep_prep_mixed)
    double* diag;    // LU-SGS diagonal cv/dt + 0.5*omega*la (lusgs.f90:36)
    double* diaginv; // its FP64 reciprocal, read by the FP32 sweeps (a multiply on their critical path)
    double4* rec_a;  // sweep records [pass * nop + node]: (u, v, p, e*rho) of qc
    double4* rec_b;  //   and dqc
    double* rec_r;   //   and rho (FP64 sweep)
    double* partial;   // [2*nblk]: sum, max
    int* partial_i;    // argmax
    DevErr* err;
    long long wait_cycles;  // bound of the sweeps' waits (kWaitCycles unless a caller set one)
    int skip_code;          // test hook: the sweep item (node << 1 | pass) that publishes nothing, or -1
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
    v.qpf[i] = make_float4((float)P.rho, (float)P.u, (float)P.v, (float)P.p);
    v.qold[i] = q;
}

// k_nc_grad_lim in the mixed form: the LSQ gradient and the limiter in FP32
// on the FP32 primitives, weights and edge vectors (the same gathers,
// orders and formulas); gradient and phi stored in FP64 for the edge pass
// (phi stays the FP64 running minimum).
__global__ void __launch_bounds__(kBlock) k_nc_grad_lim_mixed(NCView v) {
    if (stopped(v)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.nop) return;
    const float4 q4 = v.qpf[i];
    const float qi[4] = {q4.x, q4.y, q4.z, q4.w};
    float gx[4] = {0.f, 0.f, 0.f, 0.f}, gy[4] = {0.f, 0.f, 0.f, 0.f};
    for (int j = v.v2v_off[i]; j < v.v2v_off[i + 1]; ++j) {
        const float4 c = v.qpf[v.v2v[j]];
        const float2 w = v.wxyf[j];
        const float qc[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            gx[k] = gx[k] + (qc[k] - qi[k]) * w.x;
            gy[k] = gy[k] + (qc[k] - qi[k]) * w.y;
        }
    }
    v.gx[i] = make_double4(gx[0], gx[1], gx[2], gx[3]);
    v.gy[i] = make_double4(gy[0], gy[1], gy[2], gy[3]);
    const float eps = (float)v.eps;
    float dmx[4], dmn[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) { dmn[k] = eps; dmx[k] = -eps; }
    const int k0 = v.v2f_off[i], k1 = v.v2f_off[i + 1];
    for (int k = k0; k < k1; ++k) {
        const int e = v.v2f[k], f = e & EDGE_MASK;
        const int2 p = v.fpt[f];
        const float4 a = v.qpf[p.x], b = v.qpf[p.y];
        const float du4[4] = {b.x - a.x, b.y - a.y, b.z - a.z, b.w - a.w};
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float du = (e & P2_BIT) ? -du4[j] : du4[j];
            dmx[j] = rmax(dmx[j], du);
            dmn[j] = rmin(dmn[j], du);
        }
    }
    double ph[4];
    g4(v.phi[i], ph);
    const float sq = sqrtf((float)v.cv[i]);
    const bool vkn = v.limiter == UNS_LIM_VKN, corrected = v.limiter == UNS_LIM_BARTH_CORRECTED;
    for (int k = k0; k < k1; ++k) {
        const int e = v.v2f[k], f = e & EDGE_MASK;
        const float2 d = v.edf[f];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const float s = gx[j] * d.x + gy[j] * d.y;
            float phj;
            if (vkn) {
                const float D_L = (e & P2_BIT) ? -(0.5f * s) : 0.5f * s;
                const float kk = (float)v.kappa * sq;
                const float TOL = kk * kk * kk;
                float alfa = D_L > 0.f ? dmx[j] : dmn[j];
                if (fabsf(alfa) < eps) alfa = 0.f;
                const float nr = alfa * alfa + 2.f * D_L * alfa + TOL;
                const float dr = alfa * alfa + 2.f * D_L * D_L + D_L * alfa + TOL;
                phj = rmin(1.f, nr / dr);
            } else {  // Barth-Jespersen: reference form projects fp2 with +1/2
                float D_L = 0.5f * s;
                if (corrected && (e & P2_BIT)) D_L = -D_L;
                if (D_L > 0.f) phj = rmin(1.f, dmx[j] / D_L);
                else if (D_L < 0.f) phj = rmin(1.f, dmn[j] / D_L);
                else phj = 1.f;
                if (corrected) phj = rmax(0.f, phj);
            }
            ph[j] = rmin(ph[j], (double)phj);
        }
    }
    v.phi[i] = m4(ph);
    float4* pk = v.packn + 3 * (size_t)i;
    pk[0] = make_float4(gx[0], gx[1], gx[2], gx[3]);
    pk[1] = make_float4(gy[0], gy[1], gy[2], gy[3]);
    pk[2] = make_float4((float)ph[0], (float)ph[1], (float)ph[2], (float)ph[3]);
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
    double sq = sqrt(v.cv[i]);
    // phi = min(phi, phj of every edge).  Each phj is min(1, n/d) (Barth:
    // clamped to [0, 1] in the corrected form) and the clamps are monotonic,
    // so only the smallest ratio needs a division: the edges' ratios are
    // compared exactly (double-double cross products, denominators made
    // positive) and the minimum of correctly rounded quotients is the
    // rounded minimum.  One IEEE division per variable instead of one per
    // edge and variable; the values are those of the per-edge form.
    const bool vkn = v.limiter == UNS_LIM_VKN, corrected = v.limiter == UNS_LIM_BARTH_CORRECTED;
    double bn[4], bd[4];
    bool have[4] = {false, false, false, false};
    auto clamp = [&](double q) {
        double phj = rmin(1.0, q);
        return (!vkn && corrected) ? rmax(0.0, phj) : phj;
    };
    for (int k = k0; k < k1; ++k) {
        int e = v.v2f[k], f = e & EDGE_MASK;
        int2 p = v.fpt[f];
        double2 a = v.pxy[p.x], b = v.pxy[p.y];
        double d0 = b.x - a.x, d1 = b.y - a.y;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            double s = gx[j] * d0 + gy[j] * d1;
            double n, d;  // phj = clamp(n / d), or 1 where there is no ratio
            bool ratio = true;
            if (vkn) {
                double D_L = (e & P2_BIT) ? -(0.5 * s) : 0.5 * s;
                double kk = v.kappa * sq;
                double TOL = kk * kk * kk;
                double alfa = D_L > 0.0 ? dmx[j] : dmn[j];
                if (fabs(alfa) < v.eps) alfa = 0.0;
                n = alfa * alfa + 2.0 * D_L * alfa + TOL;
                d = alfa * alfa + 2.0 * D_L * D_L + D_L * alfa + TOL;
            } else {  // Barth-Jespersen: reference form projects fp2 with +1/2
                double D_L = 0.5 * s;
                if (corrected && (e & P2_BIT)) D_L = -D_L;
                if (D_L > 0.0) { n = dmx[j]; d = D_L; }
                else if (D_L < 0.0) { n = -dmn[j]; d = -D_L; }  // dmn / D_L with a positive denominator
                else ratio = false;
            }
            if (!ratio) {
                ph[j] = rmin(ph[j], clamp(1.0));
            } else if (!ratio_ok(n, d)) {
                ph[j] = rmin(ph[j], clamp(n / d));
            } else if (!have[j] || ratio_less(n, d, bn[j], bd[j])) {
                bn[j] = n; bd[j] = d; have[j] = true;
            }
        }
    }
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (have[j]) ph[j] = rmin(ph[j], clamp(bn[j] / bd[j]));
    v.phi[i] = m4(ph);
}

template <class R>
__global__ void __launch_bounds__(kBlock) k_nc_edge(NCView v) {
    if (stopped(v)) return;
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= v.nof) return;
    if constexpr (std::is_same<R, float>::value) {
        // mixed form, an interior edge: FP32 copies only (primitives, the node
        // pack of gradient and limiter, edge vector), the same formulas
        const int bc = v.fbc[f];
        if (bc != 1001 && bc != 2001) {
            const int2 p = v.fpt[f];
            const float4 qa = v.qpf[p.x], qb = v.qpf[p.y];
            const float4* A = v.packn + 3 * (size_t)p.x;
            const float4* B = v.packn + 3 * (size_t)p.y;
            const float4 ga = A[0], ha = A[1], pa = A[2], gb = B[0], hb = B[1], pb = B[2];
            const float2 d = v.edf[f];
            const float q1[4] = {qa.x, qa.y, qa.z, qa.w}, q2[4] = {qb.x, qb.y, qb.z, qb.w};
            const float a[4] = {ga.x, ga.y, ga.z, ga.w}, b[4] = {ha.x, ha.y, ha.z, ha.w};
            const float c[4] = {gb.x, gb.y, gb.z, gb.w}, e[4] = {hb.x, hb.y, hb.z, hb.w};
            const float f1[4] = {pa.x, pa.y, pa.z, pa.w}, f2[4] = {pb.x, pb.y, pb.z, pb.w};
            V4<float> L, Rt, F;
#pragma unroll
            for (int k = 0; k < 4; ++k) {  // fvresidual.f90:41-54
                float g = a[k] * d.x + b[k] * d.y;
                L[k] = q1[k] + 0.5f * g * f1[k];
                g = c[k] * d.x + e[k] * d.y;
                Rt[k] = q2[k] - 0.5f * g * f2[k];
            }
            const double2 n = v.fn[f];
            const float area = (float)v.farea[f];
            const float G = (float)v.g.gamma, G1 = (float)v.g.gamma1;
            float hl, hr;
            if (v.g.flux == UNS_FLUX_AUSM) ausm_core<float>(G, G1, (float)n.x, (float)n.y, (float)v.g.mref, L, Rt, F, hl, hr);
            else vanleer_core<float>(G, G1, (float)n.x, (float)n.y, L, Rt, F, hl, hr);
            v.fF[f] = make_double4(F[0] * area, F[1] * area, F[2] * area, F[3] * area);
            // Roe-averaged spectral radius (vanleer_flux.f90:102-115)
            const float RT = sqrtf(Rt[0] / L[0]);
            const float u = (L[1] + RT * Rt[1]) / (1.f + RT);
            const float vv = (L[2] + RT * Rt[2]) / (1.f + RT);
            const float H = (hl + RT * hr) / (1.f + RT);
            const float aa = sqrtf(G1 * (H - 0.5f * (u * u + vv * vv)));
            const float un = fabsf(u * (float)n.x + vv * (float)n.y);
            v.fla[f] = (double)((un + aa) * area);
            return;
        }
    }
    int2 p = v.fpt[f];
    double2 X1 = v.pxy[p.x], X2 = v.pxy[p.y];
    double d0 = X2.x - X1.x, d1 = X2.y - X1.y;
    double q1[4], q2[4], a[4], b[4], c[4], d[4], f1[4], f2[4];
    g4(v.qp[p.x], q1); g4(v.qp[p.y], q2);
    g4(v.gx[p.x], a); g4(v.gy[p.x], b); g4(v.gx[p.y], c); g4(v.gy[p.y], d);
    g4(v.phi[p.x], f1); g4(v.phi[p.y], f2);
    V4<R> L, Rt, F;
#pragma unroll
    for (int k = 0; k < 4; ++k) {  // fvresidual.f90:41-54
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
    // Roe-averaged spectral radius (vanleer_flux.f90:102-115).
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
    if (bc == 1001) {  // solid_flux (solid_flux.f90:26-41)
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
// residual, spectral radius, time_step2 (timestep.f90:16-34), optional RK3
// stage (main.f90:63-72) and residual-norm block partials
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
        v.diaginv[i] = 1.0 / v.diag[i];
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
#pragma unroll 4
    for (int k = threadIdx.x; k < nparts; k += kBlock) {  // unrolled: loads in flight together, sums in order
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
        if (!isfinite(fres)) set_err(v.err, UNS_ERR_NAN, -1);
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

constexpr int kSweepBlock = 128;
// One sweep block per SM: one warp per SM sub-partition, so concurrently
// active items never share an FP64 unit.
constexpr int kSweepBlocksPerSM = 1;
constexpr double kOmega = 1.5;  // lusgs.f90:26

// Per LU-SGS call: everything a sweep item needs from an edge that does not
// change during the sweeps, laid out contiguously in schedule order so a
// lane fetches it with three 32-byte loads and no index chasing:
//   rec[3r]   normalflux(qold(nb)) on the edge (lusgs.f90:137-155)
//   rec[3r+1] (nx, ny, ds, omega * la)
//   rec[3r+2] (qold(nb).rho, sign, nb as integer bits, 0)
// con2prim of qold once per node (a node has about six records): the
// records' normalflux then reads (u, v, p, e*rho) instead of dividing again,
// with the same operations on the same values.
__global__ void __launch_bounds__(kBlock) k_nc_qold_prim(NCView v) {
    if (stopped(v)) return;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.nop) return;
    const double4 q = v.qold[i];
    Prim P = con2prim(v.g, q.x, q.y, q.z, q.w);
    v.qoldp[i] = make_double4(P.u, P.v, P.p, P.e * P.rho);
}

// normalflux_nc from the node's precomputed primitives (rho = qold.rho).
__device__ __forceinline__ void normalflux_nc_p(const double4& P, double rho, double nx, double ny, double ds,
                                                double o[4]) {
    const double u = P.x, vv = P.y, p = P.z, et = P.w;
    double un = u * nx + vv * ny;
    o[0] = (et + p) * un;
    o[1] = rho * un;
    o[2] = o[1] * u + p * nx;
    o[3] = o[1] * vv + p * ny;
#pragma unroll
    for (int k = 0; k < 4; ++k) o[k] = o[k] * ds;
}

__global__ void __launch_bounds__(kBlock) k_nc_sweep_prep(NCView v) {
    if (stopped(v)) return;
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= v.nrec) return;
    const int c = v.rec_edge[r], nb = v.rec_nb[r];
    const double2 n = v.fn[c];
    const double ds = v.farea[c];
    const double4 q = v.qold[nb];
    double o[4];
    normalflux_nc_p(v.qoldp[nb], q.y, n.x, n.y, ds, o);
    v.rec[3 * (size_t)r] = m4(o);
    v.rec[3 * (size_t)r + 1] = make_double4(n.x, n.y, ds, kOmega * v.fla[c]);
    v.rec[3 * (size_t)r + 2] = make_double4(q.y, (double)v.rec_sign[r], __longlong_as_double((long long)nb), 0.0);
}

// Mixed-precision sweeps (delta form): per record, in FP32, the neighbour's
// old state and primitives and the edge geometry, from which a lane forms
// normalflux(qold + dqc) - normalflux(qold) directly from dqc:
//   [rho, rho*u, rho*v, E] [u, v, p, u.n] [nx, ny, ds, omega*la] [sign, nb, 0, 0]
__global__ void __launch_bounds__(kBlock) k_nc_sweep_prep_mixed(NCView v) {
    if (stopped(v)) return;
    int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= v.nrec) return;
    const int c = v.rec_edge[r], nb = v.rec_nb[r];
    const double2 n = v.fn[c];
    const double4 q = v.qold[nb];
    Prim P = con2prim(v.g, q.x, q.y, q.z, q.w);
    float4* rf = reinterpret_cast<float4*>(v.rec) + 4 * (size_t)r;
    rf[0] = make_float4((float)q.y, (float)q.z, (float)q.w, (float)q.x);
    rf[1] = make_float4((float)P.u, (float)P.v, (float)P.p, (float)(P.u * n.x + P.v * n.y));
    rf[2] = make_float4((float)n.x, (float)n.y, (float)v.farea[c], (float)(kOmega * v.fla[c]));
    rf[3] = make_float4((float)v.rec_sign[r], __int_as_float(nb), 0.f, 0.f);
}

__device__ __forceinline__ double pick4(int k, double a, double b, double c, double d) {
    return k == 0 ? a : (k == 1 ? b : (k == 2 ? c : d));
}

// The node's own diagonal, qold and res (variable `lane`) in lanes 0..3;
// benign operands elsewhere, so the warp-wide divides meet no 0 or inf.
// (The mixed form's sweep.)
__device__ __forceinline__ void own_load(const NCView& v, const int4& S, int lane, double& D, double& o, double& r) {
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

// Lanes of a sweep item: lane = 4 * slot + k, slot = the taken edge (up to 8
// per round), k = the variable.  An FP64 instruction costs its SM
// sub-partition the same whatever the number of active lanes (about 70
// cycles on GB300), so each item's arithmetic is spread over the lanes: the
// four flux components of up to eight edges in one pass, the per-variable
// sums and divides in lanes 0..3, and the three divisions of con2prim in
// lanes 0, 2 and 3 at once.  Chosen by measurement on GB300 (sweeps at
// 1024x512, bit-identical variants): the consumer reads rho from the record
// rather than forming qold.rho + dqc.rho; the warp exchanges its per-lane
// values through shared memory rather than shuffles; the division by the
// diagonal stays an IEEE division (through a precomputed reciprocal with
// Markstein's correction it was slower, as was halving on the integer pipe);
// the next item's inputs are loaded after this item's polls.
struct SweepIn {
    double f1, nx, ny, ds, ol;  // the slot's record; f1 = component k
    double sgn;                 // orientation sign +-1 (tested where used, so no load is waited on here)
    int nb;
    double D, o, r;             // lanes 0..3: the diagonal, qold and res (pass 0) / the early-read
                                // forward dqc (pass 1), variable k
};

__device__ __forceinline__ void sweep_load_edge(const NCView& v, int rec, int k, SweepIn& x) {
    const double4* p = v.rec + 3 * (size_t)rec;
    x.f1 = reinterpret_cast<const double*>(p)[k];
    double4 b = p[1], c = p[2];
    x.nx = b.x; x.ny = b.y; x.ds = b.z; x.ol = b.w;
    x.sgn = c.y;
    x.nb = (int)__double_as_longlong(c.z);
}

__device__ __forceinline__ void sweep_load(const NCView& v, const int4& S, int lane, SweepIn& x) {
    if ((lane >> 2) < S.w) sweep_load_edge(v, S.z + (lane >> 2), lane & 3, x);
    if (lane < 4) {
        x.D = v.diag[S.x];
        x.o = reinterpret_cast<const double*>(&v.qold[S.x])[lane];
        if (S.y == 0) {
            x.r = reinterpret_cast<const double*>(&v.res[S.x])[lane];
        } else {  // the node's forward dqc: usually published long before; checked when used
            asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];"
                         : "=d"(x.r) : "l"(reinterpret_cast<const double*>(v.rec_b + S.x) + lane) : "memory");
        }
    } else {
        x.D = 1.0;
        x.o = 1.0;
        x.r = 0.0;
    }
}

// A neighbour's record: (u, v, p, e*rho) in w[0..4), dqc in w[4..8), rho.
__device__ __forceinline__ void peek_neighbour(const NCView& v, size_t rs, double w[8], double& rho) {
    const double2* pa = reinterpret_cast<const double2*>(v.rec_a + rs);
    const double2* pb = reinterpret_cast<const double2*>(v.rec_b + rs);
    double2 x0 = ld_relaxed2(pa), x1 = ld_relaxed2(pa + 1), x2 = ld_relaxed2(pb), x3 = ld_relaxed2(pb + 1);
    asm volatile("ld.relaxed.gpu.global.f64 %0, [%1];" : "=d"(rho) : "l"(v.rec_r + rs) : "memory");
    w[0] = x0.x; w[1] = x0.y; w[2] = x1.x; w[3] = x1.y;
    w[4] = x2.x; w[5] = x2.y; w[6] = x3.x; w[7] = x3.y;
}

__device__ __forceinline__ bool record_set(const double w[8], double rho) {
    bool ready = !is_unset(rho);
#pragma unroll
    for (int j = 0; j < 8; ++j) ready = ready && !is_unset(w[j]);
    return ready;
}

// A neighbour's record, waiting (bounded) until every value is published.
__device__ __forceinline__ bool poll_neighbour(const NCView& v, size_t rs, double w[8], double& rho) {
    long long t0 = 0;
    for (int spins = 0;; ++spins) {
        peek_neighbour(v, rs, w, rho);
        if (record_set(w, rho)) return true;
        if (!poll_continue(spins, t0, v.err, v.wait_cycles)) return false;
    }
}

// lusgs sweeps (lusgs.f90:48-124) as one cooperative launch.  Each warp runs
// its own list of items (node, pass) from the host-side list schedule, in
// order, loading the next item's inputs while it works on the current one.
// Per item, for each edge whose neighbour precedes the node in this pass
// (reference v2f order): the neighbour's values come from registers when the
// warp itself computed that neighbour last, else from its record (read
// during the previous item, or polled); the edge term
// 0.5*(sign*(F(qc) - F(qold)) - omega*la*dqc) is formed per component; lanes
// 0..3 add the terms in edge order (the reference's summation order) and
// divide by the diagonal; the new state is spread to all lanes, which keep
// its primitives for the next item while lanes 0..2 publish the record.
// Every rounded operation and its operand order is the reference's.
__global__ void __launch_bounds__(kSweepBlock, 1) k_nc_lusgs(NCView v, const int* __restrict__ woff) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    __shared__ __align__(16) double wxs[kSweepBlock / 32][32];  // per-warp exchange of lane values
    double* wx = wxs[wib];
    const int gw = blockIdx.x * (kSweepBlock / 32) + wib;
    const int slot = lane >> 2, k = lane & 3;
    if (stopped(v)) return;
    const int n = v.nop;
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
    double Sw[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0}, Srho = 0.0;
    bool spec = false;
    for (int kk = kbeg; kk < kend; ++kk) {
        const int4 Snn = kk + 2 < kend ? v.sched[kk + 2] : none;
        const int it = S.x, pass = S.y, ntake = S.w;
        double cres = 0.0;  // lanes 0..3: sum over edges of component k
        for (int base = 0; base < ntake; base += 8) {
            SweepIn E = X;
            if (base > 0 && base + slot < ntake) sweep_load_edge(v, S.z + base + slot, k, E);
            bool ok = true;
            double t = 0.0;
            if (base + slot < ntake) {
                double w[8], rho;
                if (((E.nb << 1) | pass) == last) {
                    w[0] = Lu; w[1] = Lv; w[2] = Lp; w[3] = Le; w[4] = L0; w[5] = L1; w[6] = L2; w[7] = L3;
                    rho = Lrho;
                } else if (base == 0 && spec && record_set(Sw, Srho)) {
#pragma unroll
                    for (int j = 0; j < 8; ++j) w[j] = Sw[j];
                    rho = Srho;
                } else {
                    ok = poll_neighbour(v, (size_t)pass * n + E.nb, w, rho);
                }
                // normalflux (lusgs.f90:144-150) component k, then the edge term
                const double u = w[0], vv = w[1], p = w[2], et = w[3];
                const double un = u * E.nx + vv * E.ny;
                const double o1 = rho * un;
                const double prod = (k == 0 ? et + p : o1) * (k == 0 ? un : (k == 2 ? u : vv));
                const double pn = p * (k == 2 ? E.nx : E.ny);
                double o = k == 1 ? o1 : (k == 0 ? prod : prod + pn);
                o = o * E.ds;
                const double diff = o - E.f1;
                const double dqk = pick4(k, w[4], w[5], w[6], w[7]);
                t = 0.5 * ((__double_as_longlong(E.sgn) < 0 ? -diff : diff) - E.ol * dqk);
            }
            if (__ballot_sync(full, !ok)) return;  // a wait gave up; the error is recorded
            // the terms in edge order, from 0.0 (the first addition is exact)
            const int nr = min(8, ntake - base);
            wx[lane] = t;
            __syncwarp();
            int e = 0;
            if (base == 0) { cres = zero_plus(wx[k]); e = 1; }
            for (; e < nr; ++e) cres = cres + wx[4 * e + k];
            __syncwarp();
        }
        // next item's inputs (independent of the sweep), issued once this
        // item's polls are done so they do not queue ahead of them
        if (kk + 1 < kend) sweep_load(v, Sn, lane, Xn);
        double r = X.r;
        bool ok = true;
        if (pass == 1 && lane < 4) {  // own forward dqc
            if ((it << 1) == last) r = pick4(lane, L0, L1, L2, L3);
            else if (is_unset(r)) ok = poll_value(reinterpret_cast<const double*>(v.rec_b + it) + lane, r, v.err, v.wait_cycles);
        }
        if (__ballot_sync(full, !ok)) return;
        // dqc and qc = qold + dqc (lusgs.f90:78-81 / 117-120), component k in lane k
        const double d = pass == 0 ? (-r - cres) / X.D : r - cres / X.D;
        const double q = X.o + d;
        // the next item's first-round neighbour records, while this item finishes
        spec = false;
        if (kk + 1 < kend && slot < Sn.w && ((Xn.nb << 1) | Sn.y) != ((it << 1) | pass)) {
            peek_neighbour(v, (size_t)Sn.y * n + Xn.nb, Sw, Srho);
            spec = true;
        }
        // con2prim (All_modules.f90:146-169): rho = q1, then E/rho, rhou/rho,
        // rhov/rho in lanes 0, 2, 3
        if (lane < 4) { wx[lane] = q; wx[4 + lane] = d; }
        __syncwarp();
        const double2 qa = reinterpret_cast<const double2*>(wx)[0], qb = reinterpret_cast<const double2*>(wx)[1];
        const double E0 = qa.x, rho = qa.y, Q2 = qb.x, Q3 = qb.y;
        const double quo = q / rho;
        // the four products of the pressure and the record as one
        // multiplication: lane 0 e*rho, lane 1 0.5*rho, lane 2 u*u, lane 3 v*v
        // (an FP64 instruction costs the warp the same for one lane or four)
        const double ma = lane == 1 ? 0.5 : quo, mb = lane < 2 ? rho : quo;
        const double pr = ma * mb;
        if (lane < 4) { wx[8 + lane] = quo; wx[12 + lane] = pr; }
        __syncwarp();
        const double2 da = reinterpret_cast<const double2*>(wx)[2], db = reinterpret_cast<const double2*>(wx)[3];
        const double2 pa = reinterpret_cast<const double2*>(wx)[6], pb = reinterpret_cast<const double2*>(wx)[7];
        const double u = wx[10], vv = wx[11];
        L0 = da.x; L1 = da.y; L2 = db.x; L3 = db.y;
        __syncwarp();
        const double qq = pb.x + pb.y;                // u*u + v*v
        const double p = gm1 * (E0 - pa.y * qq);      // gm1*(E - 0.5*rho*qq)
        Lrho = rho; Lu = u; Lv = vv; Lp = p; Le = pa.x;
        last = (it << 1) | pass;
        const size_t slotr = (size_t)pass * n + it;
        if (last == v.skip_code) {  // test hook: this item publishes nothing and hands nothing on
            last = -1;
        } else {
            // Lane 0 stores (u, v, p, e*rho), lane 1 dqc, lane 2 rho, as
            // predicated stores of one instruction sequence: lane-divergent
            // branches here cost the critical path more than the stores
            // (sweeps 11.07 -> 10.39 ms at 1024x512, measured).
            double2* dst = reinterpret_cast<double2*>(lane == 0 ? v.rec_a + slotr : v.rec_b + slotr);
            const double x0 = lane == 0 ? Lu : L0, x1 = lane == 0 ? Lv : L1;
            const double x2 = lane == 0 ? Lp : L2, x3 = lane == 0 ? Le : L3;
            const int st_ab = lane < 2, st_r = lane == 2;
            asm volatile(
                "{\n\t.reg .pred pa, pr;\n\t"
                "setp.ne.s32 pa, %0, 0;\n\t"
                "setp.ne.s32 pr, %1, 0;\n\t"
                "@pa st.relaxed.gpu.global.v2.f64 [%2], {%3, %4};\n\t"
                "@pa st.relaxed.gpu.global.v2.f64 [%5], {%6, %7};\n\t"
                "@pr st.relaxed.gpu.global.f64 [%8], %9;\n\t}"
                :
                : "r"(st_ab), "r"(st_r), "l"(dst), "d"(x0), "d"(x1), "l"(dst + 1), "d"(x2), "d"(x3), "l"(v.rec_r + slotr),
                  "d"(rho)
                : "memory");
            if (pass == 1 && lane == 2) v.qc[it] = make_double4(E0, rho, Q2, Q3);
        }
        S = Sn;
        Sn = Snn;
        X = Xn;
    }
}

// ------------------------------------------------------------ mixed (delta form)
// The FP32 sweep cannot form F(qold + dqc) - F(qold) as a difference of two
// O(1) fluxes: near convergence that difference drowns in FP32 rounding and
// the solve stalls.  It forms the change directly from dqc (dflux_k), so its
// FP32 error is relative to the change itself; items publish dqc only (FP32
// for the edge terms, FP64 for the node's own backward step) and form no
// primitives.
struct SweepInM {
    float rho, ru, rv, E, u, v, p, un, nx, ny, ds, ol, sign;  // the slot's record
    int nb;
    double D, o, r;  // lanes 0..3: the reciprocal of the node's diagonal, qold and res, variable k
};

__device__ __forceinline__ void sweep_load_edge_m(const NCView& v, int rec, SweepInM& x) {
    const float4* p = reinterpret_cast<const float4*>(v.rec) + 4 * (size_t)rec;
    float4 a = p[0], b = p[1], c = p[2], d = p[3];
    x.rho = a.x; x.ru = a.y; x.rv = a.z; x.E = a.w;
    x.u = b.x; x.v = b.y; x.p = b.z; x.un = b.w;
    x.nx = c.x; x.ny = c.y; x.ds = c.z; x.ol = c.w;
    x.sign = d.x; x.nb = __float_as_int(d.y);
}

__device__ __forceinline__ void sweep_load_m(const NCView& v, const int4& S, int lane, SweepInM& x) {
    if ((lane >> 2) < S.w) sweep_load_edge_m(v, S.z + (lane >> 2), x);
    own_load(v, S, lane, x.D, x.o, x.r);
    if (lane < 4) x.D = v.diaginv[S.x];  // the FP32 sweep multiplies by the FP64 reciprocal
}

// lusgs sweeps in the mixed form: the schedule, lanes, hand-offs and FP64
// sums / diagonal division of k_nc_lusgs; FP32 delta-form edge terms.
__global__ void __launch_bounds__(kSweepBlock, 1) k_nc_lusgs_mixed(NCView v, const int* __restrict__ woff) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const int gw = blockIdx.x * (kSweepBlock / 32) + wib;
    const int slot = lane >> 2, k = lane & 3;
    if (stopped(v)) return;
    const int n = v.nop;
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
    float LF[4] = {0.f, 0.f, 0.f, 0.f};             // previous item's dqc (FP32)
    double L0 = 0.0, L1 = 0.0, L2 = 0.0, L3 = 0.0;  // and in FP64
    float Sf[4] = {0.f, 0.f, 0.f, 0.f};
    bool spec = false;
    for (int kk = kbeg; kk < kend; ++kk) {
        const int4 Snn = kk + 2 < kend ? v.sched[kk + 2] : none;
        const int it = S.x, pass = S.y, ntake = S.w;
        double cres = 0.0;
        for (int base = 0; base < ntake; base += 8) {
            SweepInM E = X;
            if (base > 0 && base + slot < ntake) sweep_load_edge_m(v, S.z + base + slot, E);
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
                t = (double)(0.5f * ((E.sign < 0.f ? -df : df) * E.ds - E.ol * dqk));
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
        if (pass == 1 && lane < 4) {  // own forward dqc
            if ((it << 1) == last) r = pick4(lane, L0, L1, L2, L3);
            else ok = poll_value(reinterpret_cast<const double*>(v.rec_b + it) + lane, r, v.err, v.wait_cycles);
        }
        if (__ballot_sync(full, !ok)) return;
        const double d = pass == 0 ? (-r - cres) * X.D : r - cres * X.D;
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

// tecplt's vertex table (NCFVM/main.f90:190-233): per node x, y and the
// primitives of the last save_old (rho, u, v, p) with the Mach number.
__global__ void __launch_bounds__(kBlock) k_nc_tecplt(NCView v, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.nop) return;
    const double4 q = v.qp[i];
    const double2 x = v.pxy[i];
    const double q2 = q.y * q.y + q.z * q.z;
    const double mach = sqrt(q2 * q.x / (v.g.gamma * q.w));
    double* o = out + (size_t)i * 7;
    o[0] = x.x; o[1] = x.y; o[2] = q.x; o[3] = q.y; o[4] = q.z; o[5] = q.w; o[6] = mach;
}

// screen's min/max (NCFVM/main.f90:115-187) over the nodes from the current
// conserved state: density, u, v, pressure, Mach number, entropy; exact and
// order-free (warp reduction, then encoded atomics).
__global__ void __launch_bounds__(kBlock) k_nc_screen(NCView v, double ent_inf, unsigned long long* mm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long lo[6], hi[6];
    for (int k = 0; k < 6; ++k) { lo[k] = ~0ULL; hi[k] = 0ULL; }
    if (i < v.nop) {
        const double4 q = v.qc[i];
        const Prim r = con2prim(v.g, q.x, q.y, q.z, q.w);
        const double q2 = r.u * r.u + r.v * r.v;
        const double mach = sqrt(q2 * r.rho / (v.g.gamma * r.p));
        const double ent = log10(r.p / pow(r.rho, v.g.gamma) / ent_inf);
        const double x[6] = {r.rho, r.u, r.v, r.p, mach, ent};
        for (int k = 0; k < 6; ++k) { lo[k] = enc_ord(x[k]); hi[k] = lo[k]; }
    }
    for (int k = 0; k < 6; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long a = __shfl_xor_sync(0xffffffffu, lo[k], o), c = __shfl_xor_sync(0xffffffffu, hi[k], o);
            lo[k] = a < lo[k] ? a : lo[k];
            hi[k] = c > hi[k] ? c : hi[k];
        }
    }
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 6; ++k) { atomicMin(&mm[2 * k], lo[k]); atomicMax(&mm[2 * k + 1], hi[k]); }
}

__global__ void k_nc_screen_init(unsigned long long* mm) {
    if (threadIdx.x < 6) { mm[2 * threadIdx.x] = ~0ULL; mm[2 * threadIdx.x + 1] = 0ULL; }
}

__global__ void k_nc_initialize(NCView v, double4 qinf, double phi0) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.nop) return;
    v.qc[i] = qinf;
    v.phi[i] = make_double4(phi0, phi0, phi0, phi0);
}


}  // namespace

struct uns_nc_handle {
    uns_params P;
    NCView v;
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;
    int nparts = 0;
    int* woff = nullptr;    // LU-SGS warp schedule: per-warp ranges of v.sched
    int coop_blocks = 0;
    int lev_fwd = 0, lev_bwd = 0;  // dependency levels of the two sweeps (their critical path)
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
    double* d_tec = nullptr;              // tecplt vertex table, created on first use
    unsigned long long* d_mm = nullptr;   // screen min/max slots, created on first use

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
    if (h->P.precision == UNS_PREC_MIXED) NLAUNCH(k_nc_grad_lim_mixed, v.nop, v);
    else NLAUNCH(k_nc_grad_lim, v.nop, v);
    if (h->P.precision == UNS_PREC_MIXED) NLAUNCH(k_nc_edge<float>, v.nof, v);
    else NLAUNCH(k_nc_edge<double>, v.nof, v);
    NLAUNCH(k_nc_node_res, v.nop, v, cfl, irk, partial);
    return UNS_OK;
}

int launch_sweeps_nc(uns_nc_handle* h, NCView& v) {
    const bool mixed = h->P.precision != UNS_PREC_FP64;  // FP32 sweep arithmetic
    const long long n2 = 2LL * v.nop * 2;  // double2 per record array
    if (mixed)
        k_fill_unset_f<<<std::min<long long>(nblocks(2LL * v.nop), 4096), kBlock, 0, h->stream>>>((float4*)v.rec_a,
                                                                                                   2LL * v.nop);
    else {
        k_fill_unset<<<std::min<long long>(nblocks(n2), 4096), kBlock, 0, h->stream>>>((double2*)v.rec_a, n2);
        k_fill_unset<<<std::min<long long>(nblocks(v.nop), 4096), kBlock, 0, h->stream>>>((double2*)v.rec_r,
                                                                                           (long long)v.nop);
    }
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
    if (mixed) UNS_CUDA(cudaLaunchKernelEx(&cfg, k_nc_lusgs_mixed, v, (const int*)h->woff));
    else UNS_CUDA(cudaLaunchKernelEx(&cfg, k_nc_lusgs, v, (const int*)h->woff));
    return UNS_OK;
}

int enqueue_sweep_prep_nc(uns_nc_handle* h, NCView& v) {
    if (v.nrec <= 0) return UNS_OK;
    if (h->P.precision != UNS_PREC_FP64) {
        NLAUNCH(k_nc_sweep_prep_mixed, v.nrec, v);
    } else {
        NLAUNCH(k_nc_qold_prim, v.nop, v);
        NLAUNCH(k_nc_sweep_prep, v.nrec, v);
    }
    return UNS_OK;
}

int enqueue_lusgs_nc(uns_nc_handle* h, NCView& v) {
    int rc = enqueue_sweep_prep_nc(h, v);
    if (rc) return rc;
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
        p->precision < UNS_PREC_FP64 || p->precision > UNS_PREC_MIXED_SWEEP ||
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
    {  // FP32 copies for the mixed form's gradient pass
        std::vector<float2> wf(wxy.size()), ef(nof);
        for (size_t k = 0; k < wxy.size(); ++k) wf[k] = make_float2((float)wxy[k].x, (float)wxy[k].y);
        for (int f = 0; f < nof; ++f)
            ef[f] = make_float2((float)(pxy[fpt[f].y].x - pxy[fpt[f].x].x), (float)(pxy[fpt[f].y].y - pxy[fpt[f].x].y));
        UPN(wxyf, wf); UPN(edf, ef);
    }
    UPN(v2f_off, cnt); UPN(v2f, vf);
    { std::vector<int> t(m->v2f_off, m->v2f_off + nop + 1); UPN(rv2f_off, t); }
    { std::vector<int> t(m->v2f, m->v2f + m->v2f_off[nop]); UPN(rv2f, t); }
    ALN(qc, nop); ALN(qp, nop); ALN(qpf, nop); ALN(packn, 3 * (size_t)nop); ALN(qold, nop); ALN(qoldp, nop); ALN(res, nop); ALN(gx, nop); ALN(gy, nop); ALN(phi, nop);
    ALN(dt, nop); ALN(la, nop); ALN(fla, nof); ALN(fF, nof); ALN(bres1, nbnd); ALN(bres2, nbnd); ALN(bla, nbnd);
    ALN(diag, nop); ALN(diaginv, nop); ALN(rec_a, 2 * (size_t)nop); ALN(rec_b, 2 * (size_t)nop); ALN(rec_r, 2 * (size_t)nop);
    ALN(err, 1);
    h->v.wait_cycles = kWaitCycles;
    h->v.skip_code = -1;
    h->nparts = nblocks(nop);
    ALN(partial, 2 * h->nparts);
    ALN(partial_i, h->nparts);
    if ((rc = h->alloc(h->d_scalar, 4))) return fail(rc);
    if ((rc = h->alloc(h->d_iter, 1))) return fail(rc);
    if ((rc = h->alloc(h->d_done, 1))) return fail(rc);
    if ((rc = h->alloc(h->d_fres1, 1))) return fail(rc);
    {
        // LU-SGS warp schedule; a warp per item handles up to 32 edges.
        int maxdeg = 0;
        for (int i = 0; i < nop; ++i) maxdeg = std::max(maxdeg, m->v2f_off[i + 1] - m->v2f_off[i]);
        if (maxdeg > 32) { set_last_error("uns_nc_create: a node has more than 32 edges"); return fail(UNS_ERR_MESH); }
        if (nop >= (1 << 30)) { set_last_error("uns_nc_create: too many nodes"); return fail(UNS_ERR_MESH); }
        int dev = 0, nsm = 0, per = 0;
        if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_nc_lusgs, kSweepBlock, 0) != cudaSuccess || per < 1) {
            set_last_error("uns_nc_create: cannot size the cooperative LU-SGS launch");
            return fail(UNS_ERR_CUDA);
        }
        h->coop_blocks = nsm * std::min(per, kSweepBlocksPerSM);
        // other end of each v2f edge, and the reference's orientation sign
        auto other = [&](int i, int e, int* sign) {
            if (m->fp2[e] == i) { *sign = -1; return m->fp1[e]; }
            *sign = 1;
            return m->fp2[e];
        };
        std::vector<int> nbr(m->v2f_off[nop]);
        for (int i = 0; i < nop; ++i)
            for (int k = m->v2f_off[i]; k < m->v2f_off[i + 1]; ++k) {
                int sg;
                nbr[k] = other(i, m->v2f[k], &sg);
            }
        WarpSchedule ws = list_schedule(nop, m->v2f_off, nbr.data(), h->coop_blocks * (kSweepBlock / 32));
        h->lev_fwd = ws.nlev_fwd;
        h->lev_bwd = ws.nlev_bwd;
        std::vector<int4> sched(ws.items.size());
        std::vector<int> re, rn, rs;
        for (size_t pos = 0; pos < ws.items.size(); ++pos) {
            const int it = ws.items[pos] >> 1, pass = ws.items[pos] & 1;
            const int first = (int)re.size();
            for (int k = m->v2f_off[it]; k < m->v2f_off[it + 1]; ++k) {
                int sg, nb = other(it, m->v2f[k], &sg);
                bool take = nb >= 0 && nb < nop && (pass == 0 ? nb < it : nb > it);
                if (take) { re.push_back(m->v2f[k]); rn.push_back(nb); rs.push_back(sg); }
            }
            sched[pos] = make_int4(it, pass, first, (int)re.size() - first);
        }
        h->v.nrec = (int)re.size();
        if ((rc = h->upload(h->woff, ws.off.data(), ws.off.size()))) return fail(rc);
        UPN(sched, sched); UPN(rec_edge, re); UPN(rec_nb, rn); UPN(rec_sign, rs);
        ALN(rec, 3 * re.size());
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

int uns_nc_tecplt(uns_nc_handle* h, double* out) {
    if (!h || !out) { set_last_error("uns_nc_tecplt: null argument"); return UNS_ERR_ARG; }
    if (!h->d_tec) { int rc = h->alloc(h->d_tec, 7 * (size_t)h->v.nop); if (rc) return rc; }
    k_nc_tecplt<<<nblocks(h->v.nop), kBlock, 0, h->stream>>>(h->v, h->d_tec);
    UNS_CUDA(cudaGetLastError());
    UNS_CUDA(cudaMemcpyAsync(out, h->d_tec, sizeof(double) * 7 * (size_t)h->v.nop, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    return check_err_nc(h);
}

int uns_nc_screen_minmax(uns_nc_handle* h, double* out) {
    if (!h || !out) { set_last_error("uns_nc_screen_minmax: null argument"); return UNS_ERR_ARG; }
    if (!h->d_mm) { int rc = h->alloc(h->d_mm, 12); if (rc) return rc; }
    const double ent_inf = h->v.g.p_inf / std::pow(h->v.g.r_inf, h->v.g.gamma);
    k_nc_screen_init<<<1, 32, 0, h->stream>>>(h->d_mm);
    UNS_CUDA(cudaGetLastError());
    k_nc_screen<<<nblocks(h->v.nop), kBlock, 0, h->stream>>>(h->v, ent_inf, h->d_mm);
    UNS_CUDA(cudaGetLastError());
    unsigned long long e[12];
    UNS_CUDA(cudaMemcpyAsync(e, h->d_mm, sizeof(e), cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    for (int k = 0; k < 12; ++k) out[k] = dec_ord(e[k]);
    return check_err_nc(h);
}

int uns_nc_sweep_levels(uns_nc_handle* h, int* forward, int* backward) {
    if (!h || !forward || !backward) return UNS_ERR_ARG;
    *forward = h->lev_fwd;
    *backward = h->lev_bwd;
    return UNS_OK;
}

int uns_nc_set_wait_limit(uns_nc_handle* h, long long cycles) {
    if (!h || cycles <= 0) return UNS_ERR_ARG;
    h->v.wait_cycles = cycles;
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    return UNS_OK;
}

int uns_nc_debug_unpublish(uns_nc_handle* h, int node, int pass) {
    if (!h || node < -1 || node >= h->v.nop || pass < 0 || pass > 1) return UNS_ERR_ARG;
    h->v.skip_code = node < 0 ? -1 : (node << 1) | pass;
    if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    return UNS_OK;
}

int uns_nc_set_precision(uns_nc_handle* h, int precision) {
    if (!h || precision < UNS_PREC_FP64 || precision > UNS_PREC_MIXED_SWEEP) return UNS_ERR_ARG;
    if (h->P.precision != precision) {
        UNS_CUDA(cudaStreamSynchronize(h->stream));
        h->P.precision = precision;
        if (h->graph) { cudaGraphExecDestroy(h->graph); h->graph = nullptr; }
    }
    return UNS_OK;
}

void* uns_nc_stream(uns_nc_handle* h) { return h ? (void*)h->stream : nullptr; }

int uns_nc_profile(uns_nc_handle* h, double cfl, int reps, double* ms, const char** names, int nphase) {
    static const char* kNames[] = {"save_old", "grad_lim", "edge", "node_res", "sweep_prep", "lusgs_sweeps", "residue"};
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
            if (!rc) rc = timed(1, [&]() -> int {
                if (h->P.precision == UNS_PREC_MIXED) NLAUNCH(k_nc_grad_lim_mixed, v.nop, v);
                else NLAUNCH(k_nc_grad_lim, v.nop, v);
                return UNS_OK;
            });
            if (!rc) rc = timed(2, [&]() -> int {
                if (h->P.precision == UNS_PREC_MIXED) NLAUNCH(k_nc_edge<float>, v.nof, v);
                else NLAUNCH(k_nc_edge<double>, v.nof, v);
                return UNS_OK;
            });
            if (!rc) rc = timed(3, [&]() -> int { NLAUNCH(k_nc_node_res, v.nop, v, cfl, rk3 ? irk : 0, rk3 ? (irk == 3) : 1); return UNS_OK; });
        }
        if (!rk3) {
            if (!rc) rc = timed(4, [&]() -> int { return enqueue_sweep_prep_nc(h, v); });
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
