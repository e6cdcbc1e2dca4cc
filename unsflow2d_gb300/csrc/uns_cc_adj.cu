// uns_cc_adj.cu -- discrete adjoint of the CCFVM RK3 main-loop iteration.
//
// The forward iteration G maps the solver state s = (conserved state of the
// interior cells, primitives + T of the ghost cells) to the next one; C_L or
// C_D (flux-based wall forces, CCFVM/main.F90:348-353) is computed inside it.
// At a converged state s* = G(s*, alpha), reverse accumulation gives
//     lambda = G_s^T lambda + J_s^T,      dJ/dalpha = J_alpha + G_alpha^T lambda,
// iterated like the primal (same convergence rate).  G_s^T w is the iteration
// run backwards kernel by kernel: every forward kernel of the captured
// iteration (con2prim, vertex average, face average, gradient, the three RK
// stages of face flux, viscosity, diamond-path gradient, viscous flux,
// residual gather and update) has its transpose here, applied in reverse
// order, with the reference's stale-primitive stage structure (wall ghosts
// and viscosity read the current stage state, everything else the state at
// the start of the iteration).
//
// Linearisation: one forward iteration from s* is recorded (uns_cc_adjoint_
// prepare).  Nonlinear local maps -- face fluxes, boundary states, Sutherland
// viscosity, con2prim -- get exact local Jacobians from forward-mode tangents
// (uns_tan.cuh) on the same templated physics code, one input direction per
// pass, per RK stage.  The linear maps (reconstruction, gradients, averages,
// residual gather, RK update) are transposed directly from geometry.  The
// limiter is frozen: phi keeps its recorded values (its running minimum takes
// no derivative).  The local time step multiplies the residual, which is zero
// at s*, so it is held fixed.
//
// Accumulation is atomic-free: face kernels write per-face contributions and
// cell / vertex kernels gather them over index lists, as in the forward path.
#include <cuda_runtime.h>

#include <cmath>
#include <string>
#include <vector>

#include "uns_cc_impl.cuh"
#include "uns_tan.cuh"

using namespace uns;

namespace uns {

// Device arrays of the adjoint (one set per handle).
struct AdjView {
    int nstage;
    // recorded linearisation, per RK stage s = 0..2
    const double4* JF;   // [3][8][nfi]: dF/d(ql[j]) (j < 4), dF/d(qr[j-4]) of interior faces
    const double* BJ;    // [3][nbf][9 in][9 out]: d(F[4], ghost prim[4], ghost T)/d(qcl[4], qc_in[4], alpha)
    const double4* DM;   // [3][noc]: d mul / d qc
    const double* VI;    // [3][nof][9]: mu_f, u, v, ux, uy, vx, vy, Tx, Ty at the viscous flux
    const double* Dv;    // [noc]: dt / cv
    const double4* q0;   // [noc]: conserved state at the start of the recorded iteration
    // transposed connectivity
    const int* v2f_off;  // [nop+1]
    const int* v2f;      // face | (1<<30 when the vertex is the face's p2)
    const int* c2v_off;  // [ntot+1]
    const int* c2v;      // vertex whose average includes the cell
    const double* c2v_w; // its weight w / sum(w)
    // adjoint arrays
    double4 *qc, *qold, *qp, *pp, *fq, *fgx, *fgy, *sgx, *sgy, *gx, *gy, *res, *fl, *fr, *lsq;
    double *qT, *ppT, *fmu, *falpha;
    double2 *fgT, *sgT;
    double4 *cp1, *cp2, *cpi, *cpo;  // diamond-path gradient transpose, per face and point
    double *cp1T, *cp2T, *cpiT, *cpoT;
    // the adjoint vector (input and output of one transposed iteration)
    double4* lq;   // [noc]
    double4* lg;   // [nbf] ghost primitives
    double* lgT;   // [nbf] ghost T
    double* part;  // [nblocks(ntot)] partial sums of the change
    double* out;   // [2]: d/dalpha, |change|^2
    double jx, jy;      // seed * dJ/dFx1, dJ/dFy1
    double jalpha;      // seed * explicit dJ/dalpha
    double dua, dva;    // d u_inf / d alpha, d v_inf / d alpha
    // Geometry (uns_cc_adjoint_prepare_geometry): the convective closure's
    // Jacobians with respect to the face normal and length, the values of the
    // start of the iteration that the geometric partials read, and the
    // adjoints of the view's geometric arrays that one transposed iteration
    // accumulates.  Allocated only when geo is set.
    int geo;             // 1 while the transposed iteration accumulates them
    const double4* JG;   // [3][3][nfi]: dF/d(nx, ny, area) of interior faces
    const double* BG;    // [3][nbf][3 in][9 out]: d(F, ghost prim, ghost T)/d(nx, ny, area)
    const double4 *s_qp, *s_gx, *s_gy, *s_pp, *s_fq, *s_fgx, *s_fgy;
    const double *s_qT, *s_ppT, *s_fas;
    const double2* s_fgT;
    double4 *fls, *frs;  // reconstruction adjoints summed over the stages (ql, qr; boundary qcl)
    double2 *gfn, *gfcen, *gci, *gco, *gp1, *gp2;  // per face: normal, centre, parts for its cells and end points
    double* garea;
    double4* glsw;       // LSQ weights
    double2 *gpxy, *gcen;
    double *gcv, *gcov, *gv2c;
};

struct CCAdj {
    AdjView a;
    std::vector<void*> allocs;
    double cfl = 0.0, fx = 0.0, fy = 0.0;
    bool recorded = false;
    bool geo_alloc = false, geo_recorded = false;
    int nparts = 0;
    int nv2c = 0;
};

void cc_adj_free(uns_cc_handle* h) {
    if (!h || !h->adj) return;
    for (void* p : h->adj->allocs) cudaFree(p);
    delete h->adj;
    h->adj = nullptr;
}

}  // namespace uns

namespace {

constexpr int V2F_P2 = 1 << 30;

__device__ __forceinline__ double4 z4() { return make_double4(0.0, 0.0, 0.0, 0.0); }
__device__ __forceinline__ double4 add(double4 a, double4 b) { return make_double4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w); }
__device__ __forceinline__ double4 sub(double4 a, double4 b) { return make_double4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w); }
__device__ __forceinline__ double4 scl(double s, double4 a) { return make_double4(s * a.x, s * a.y, s * a.z, s * a.w); }
__device__ __forceinline__ double dot(double4 a, double4 b) { return a.x * b.x + a.y * b.y + a.z * b.z + a.w * b.w; }
__device__ __forceinline__ double at(const double4& a, int j) { return j == 0 ? a.x : j == 1 ? a.y : j == 2 ? a.z : a.w; }
__device__ __forceinline__ void put(double4& a, int j, double x) {
    if (j == 0) a.x = x; else if (j == 1) a.y = x; else if (j == 2) a.z = x; else a.w = x;
}
__device__ __forceinline__ double rk_a(int irk) { return irk == 2 ? 3.0 / 4.0 : (irk == 3 ? 1.0 / 3.0 : 0.0); }
__device__ __forceinline__ double rk_b(int irk) { return irk == 2 ? 1.0 / 4.0 : (irk == 3 ? 2.0 / 3.0 : 1.0); }

// ------------------------------------------------------------ recording
__global__ void k_rec_start(CCView v, AdjView a) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.noc) return;
    ((double*)a.Dv)[i] = v.dt[i] / v.cv[i];
    ((double4*)a.q0)[i] = v.qold[i];
}

// Local Jacobians of the face flux (interior) and of the boundary closure
// (ghost state + flux) at this stage's inputs, which are exactly the ones
// k_face_conv<double> reads next.
__global__ void k_rec_conv(CCView v, AdjView a, int s) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= v.nof) return;
    const int2 nb = v.fnb[f];
    const int in = nb.x, out = nb.y;
    const double2 n = v.fn[f];
    const double area = v.farea[f];
    const double2 fc = v.fcen[f], ci = v.cen[in];
    const double4 qi = v.qp[in], gxi = v.gx[in], gyi = v.gy[in], pi = v.phi[in];
    if (f < v.nfi) {
        const double2 co = v.cen[out];
        const double4 qo = v.qp[out], gxo = v.gx[out], gyo = v.gy[out], po = v.phi[out];
        const double zhi = 1.0 / 3.0;
        double dl0 = fc.x - ci.x, dl1 = fc.y - ci.y, dr0 = fc.x - co.x, dr1 = fc.y - co.y;
        double ql[4], qr[4];
        for (int j = 0; j < 4; ++j) {
            double alfa = at(gxi, j) * dl0 + at(gyi, j) * dl1;
            double beta = at(qo, j) - at(qi, j);
            ql[j] = at(qi, j) + 0.5 * at(pi, j) * (zhi * beta + (1.0 - zhi) * alfa);
            alfa = at(gxo, j) * dr0 + at(gyo, j) * dr1;
            beta = at(qi, j) - at(qo, j);
            qr[j] = at(qo, j) + 0.5 * at(po, j) * (zhi * beta + (1.0 - zhi) * alfa);
        }
        for (int dir = 0; dir < 8; ++dir) {
            V4<Tan> L, R, F;
            for (int j = 0; j < 4; ++j) {
                L[j] = Tan(ql[j], dir == j ? 1.0 : 0.0);
                R[j] = Tan(qr[j], dir == 4 + j ? 1.0 : 0.0);
            }
            face_flux<Tan>(v.g, Tan(n.x), Tan(n.y), Tan(area), L, R, F);
            ((double4*)a.JF)[((size_t)s * 8 + dir) * v.nfi + f] = make_double4(F[0].d, F[1].d, F[2].d, F[3].d);
        }
        if (a.geo) {
            for (int dir = 0; dir < 3; ++dir) {
                V4<Tan> L, R, F;
                for (int j = 0; j < 4; ++j) { L[j] = Tan(ql[j]); R[j] = Tan(qr[j]); }
                face_flux<Tan>(v.g, Tan(n.x, dir == 0), Tan(n.y, dir == 1), Tan(area, dir == 2), L, R, F);
                ((double4*)a.JG)[((size_t)s * 3 + dir) * v.nfi + f] = make_double4(F[0].d, F[1].d, F[2].d, F[3].d);
            }
        }
        return;
    }
    const int b = f - v.nfi, bc = v.fbc[f];
    double* J = (double*)a.BJ + ((size_t)s * v.nbf + b) * 81;
    double d0 = fc.x - ci.x, d1 = fc.y - ci.y;
    double qcl[4];
    for (int j = 0; j < 4; ++j) qcl[j] = at(qi, j) + at(pi, j) * (at(gxi, j) * d0 + at(gyi, j) * d1);
    const double4 c = v.qc[in];
    for (int dir = 0; dir < 9; ++dir) {
        V4<Tan> L, C;
        for (int j = 0; j < 4; ++j) {
            L[j] = Tan(qcl[j], dir == j ? 1.0 : 0.0);
            C[j] = Tan(at(c, j), dir == 4 + j ? 1.0 : 0.0);
        }
        Tan ui(v.g.u_inf, dir == 8 ? a.dua : 0.0), vi(v.g.v_inf, dir == 8 ? a.dva : 0.0);
        CCBnd<Tan> o = cc_boundary<Tan, Tan>(v.g, bc, n.x, n.y, area, L, C, ui, vi);
        double* row = J + dir * 9;
        for (int k = 0; k < 4; ++k) { row[k] = o.F[k].d; row[4 + k] = o.gp[k].d; }
        row[8] = o.gT.d;
    }
    if (a.geo) {
        double* G = (double*)a.BG + ((size_t)s * v.nbf + b) * 27;
        for (int dir = 0; dir < 3; ++dir) {
            V4<Tan> L, C;
            for (int j = 0; j < 4; ++j) { L[j] = Tan(qcl[j]); C[j] = Tan(at(c, j)); }
            CCBnd<Tan> o = cc_boundary<Tan, Tan, Tan>(v.g, bc, Tan(n.x, dir == 0), Tan(n.y, dir == 1),
                                                      Tan(area, dir == 2), L, C, Tan(v.g.u_inf), Tan(v.g.v_inf));
            double* row = G + dir * 9;
            for (int k = 0; k < 4; ++k) { row[k] = o.F[k].d; row[4 + k] = o.gp[k].d; }
            row[8] = o.gT.d;
        }
    }
}

// Values of the start of the iteration that the geometric partials read
// (after the gradient; the stages leave them unchanged for the flows whose
// geometry is differentiated: inviscid, and laminar with Gradient_GG_FC).
__global__ void k_rec_geo(CCView v, AdjView a) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < v.ntot) { ((double4*)a.s_qp)[i] = v.qp[i]; ((double*)a.s_qT)[i] = v.qT[i]; }
    if (i < v.noc) { ((double4*)a.s_gx)[i] = v.gx[i]; ((double4*)a.s_gy)[i] = v.gy[i]; }
    if (i < v.nop) { ((double4*)a.s_pp)[i] = v.pp[i]; ((double*)a.s_ppT)[i] = v.ppT[i]; }
    if (i < v.nof) {
        ((double4*)a.s_fq)[i] = v.fq[i];
        ((double4*)a.s_fgx)[i] = v.fgx[i];
        ((double4*)a.s_fgy)[i] = v.fgy[i];
        ((double2*)a.s_fgT)[i] = v.fgT[i];
        ((double*)a.s_fas)[i] = v.fasum[i];
    }
}

// d mul / d qc of the Sutherland viscosity at the current stage state
// (viscous_flux.F90:20-22, 127-141), as k_cell_mul evaluates it.
__global__ void k_rec_mul(CCView v, AdjView a, int s) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.noc) return;
    const double4 c = v.qc[i];
    double d[4];
    for (int dir = 0; dir < 4; ++dir) {
        Tan E(c.x, dir == 0), r(c.y, dir == 1), ru(c.z, dir == 2), rv(c.w, dir == 3);
        PrimT<Tan> P = con2prim_t<Tan>(v.g, E, r, ru, rv);
        double num = 1.0 + v.g.T_infd / v.g.SCONST;
        Tan den = P.t + v.g.T_infd / v.g.SCONST;
        Tan mu = (num / den) * pow(P.t, 1.5);
        d[dir] = mu.d;
    }
    ((double4*)a.DM)[(size_t)s * v.noc + i] = make_double4(d[0], d[1], d[2], d[3]);
}

// Inputs of the viscous face flux (viscous_flux.F90:30-76) after k_face_visc.
__global__ void k_rec_visc(CCView v, AdjView a, int s) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= v.nof) return;
    const double4 q = v.fq[f], gx = v.fgx[f], gy = v.fgy[f];
    const double2 t = v.fgT[f];
    double* o = (double*)a.VI + ((size_t)s * v.nof + f) * 9;
    o[0] = v.fmu[f]; o[1] = q.y; o[2] = q.z;
    o[3] = gx.y; o[4] = gy.y; o[5] = gx.z; o[6] = gy.z; o[7] = t.x; o[8] = t.y;
}

// ------------------------------------------------------- transposed pass
__global__ void k_adj_init(CCView v, AdjView a) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < v.noc) {
        a.qc[i] = a.lq[i];
        a.qold[i] = z4(); a.qp[i] = z4(); a.qT[i] = 0.0; a.gx[i] = z4(); a.gy[i] = z4();
    } else if (i < v.ntot) {
        a.qp[i] = a.lg[i - v.noc];
        a.qT[i] = a.lgT[i - v.noc];
    }
    if (i < v.nof) {
        a.fq[i] = z4(); a.fgx[i] = z4(); a.fgy[i] = z4(); a.fgT[i] = make_double2(0.0, 0.0);
        a.sgx[i] = z4(); a.sgy[i] = z4(); a.sgT[i] = make_double2(0.0, 0.0);
    }
    if (i < v.nbf) a.falpha[i] = 0.0;
    if (a.geo && i < v.nof) {
        const double2 z = make_double2(0.0, 0.0);
        a.fls[i] = z4(); a.frs[i] = z4(); a.glsw[i] = z4();
        a.gfn[i] = z; a.gfcen[i] = z; a.gci[i] = z; a.gco[i] = z; a.gp1[i] = z; a.gp2[i] = z;
        a.garea[i] = 0.0;
    }
}

// RK update q = a*qold + b*(q - dt/cv * res) of stage irk, transposed.
__global__ void k_adj_stage(CCView v, AdjView a, int irk) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.noc) return;
    const double4 l = a.qc[i];
    const double ak = rk_a(irk), bk = rk_b(irk);
    a.res[i] = scl(-bk * a.Dv[i], l);
    a.qold[i] = add(a.qold[i], scl(ak, l));
    a.qc[i] = scl(bk, l);
}

// Viscous face flux transposed: the face-viscosity adjoint per face, the
// face-velocity adjoint into fq, the face-gradient adjoint into fg (the
// gradients of the start of the iteration) or sg (this stage's).
__global__ void k_adj_visc(CCView v, AdjView a, int s, int last, int stage_grad) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= v.nof) return;
    const int2 nb = v.fnb[f];
    double4 b = f < v.nfi ? sub(a.res[nb.y], a.res[nb.x]) : scl(-1.0, a.res[nb.x]);
    if (last && f >= v.nfi && v.fbc[f] == 1001) { b.z = b.z - a.jx; b.w = b.w - a.jy; }
    const double* o = a.VI + ((size_t)s * v.nof + f) * 9;
    const double mu = o[0], u = o[1], vv = o[2], ux = o[3], uy = o[4], vx = o[5], vy = o[6];
    const double2 n = v.fn[f];
    const double area = v.farea[f];
    const double two_third = 2.0 / 3.0;
    const double txx = two_third * (2.0 * ux - vy), txy = uy + vx, tyy = two_third * (2.0 * vy - ux);
    const double factor = (v.g.gamma - 1.0) * v.g.m_inf * v.g.m_inf * v.g.prandtl;
    const double qx = -(o[7] / factor), qy = -(o[8] / factor);
    const double mr = mu / v.g.rey;
    const double S1 = (u * txx + vv * txy - qx) * n.x + (u * txy + vv * tyy - qy) * n.y;
    const double f1b = b.x * area, f3b = b.z * area, f4b = b.w * area;
    const double mrb = f1b * S1 + f3b * (txx * n.x + txy * n.y) + f4b * (txy * n.x + tyy * n.y);
    a.fmu[f] = mrb / v.g.rey;
    const double S1b = mr * f1b;
    const double ub = S1b * (txx * n.x + txy * n.y), vb = S1b * (txy * n.x + tyy * n.y);
    const double qxb = -S1b * n.x, qyb = -S1b * n.y;
    const double txxb = S1b * u * n.x + mr * f3b * n.x;
    const double txyb = S1b * (vv * n.x + u * n.y) + mr * f3b * n.y + mr * f4b * n.x;
    const double tyyb = S1b * vv * n.y + mr * f4b * n.y;
    const double uxb = two_third * 2.0 * txxb - two_third * tyyb;
    const double vyb = -two_third * txxb + two_third * 2.0 * tyyb;
    const double uyb = txyb, vxb = txyb;
    const double txb = -qxb / factor, tyb = -qyb / factor;
    double4 q = a.fq[f];
    q.y = q.y + ub; q.z = q.z + vb;
    a.fq[f] = q;
    double4* GX = stage_grad ? a.sgx : a.fgx;
    double4* GY = stage_grad ? a.sgy : a.fgy;
    double2* GT = stage_grad ? a.sgT : a.fgT;
    double4 gx = GX[f], gy = GY[f];
    gx.y = gx.y + uxb; gx.z = gx.z + vxb;
    gy.y = gy.y + uyb; gy.z = gy.z + vyb;
    GX[f] = gx; GY[f] = gy;
    double2 t = GT[f];
    GT[f] = make_double2(t.x + txb, t.y + tyb);
    if (a.geo) {  // flux*area = area*mr*(S1, 0, txx nx + txy ny, txy nx + tyy ny): its normal and length
        const double A = u * txx + vv * txy - qx, B = u * txy + vv * tyy - qy;
        const double t1 = txx * n.x + txy * n.y, t2 = txy * n.x + tyy * n.y;
        a.garea[f] = a.garea[f] + mr * (b.x * S1 + b.z * t1 + b.w * t2);
        const double2 gn = a.gfn[f];
        a.gfn[f] = make_double2(gn.x + area * mr * (b.x * A + b.z * txx + b.w * txy),
                                gn.y + area * mr * (b.x * B + b.z * txy + b.w * tyy));
    }
}

// Sutherland viscosity transposed onto this stage's state.
__global__ void k_adj_mul(CCView v, AdjView a, int s) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.noc) return;
    double m = 0.0;
    for (int k = v.cf_off[i]; k < v.cf_off[i + 1]; ++k) {
        int f = v.cf[k] & FACE_MASK;
        m = m + (v.fnb[f].y < v.noc ? 0.5 * a.fmu[f] : a.fmu[f]);
    }
    a.qc[i] = add(a.qc[i], scl(m, a.DM[(size_t)s * v.noc + i]));
}

// Weights of the diamond-path face gradient (gradient.F90:183-261): the
// derivative of (gx, gy) of the face with respect to the value at each of its
// four points, per unit gradient adjoint (gb_x, gb_y), as
// w = 0.5 (edge terms of the two edges at the point) / (a1 + a2).
struct GgfcW { double p1x, p1y, p2x, p2y, ix, iy, ox, oy; };
__device__ __forceinline__ GgfcW ggfc_weights(const CCView& v, int f) {
    const int2 nb = v.fnb[f], p = v.fpt[f];
    const double2 X1 = v.pxy[p.x], X2 = v.pxy[p.y], Ci = v.cen[nb.x], Co = v.cen[nb.y];
    const double s = v.fasum[f];
    // triangle 1: (P1, QO, P2) at (X1, Co, X2); triangle 2: (P1, P2, QI) at (X1, X2, Ci)
    auto tri = [&](double2 A, double2 B, double2 C, double wx[3], double wy[3]) {
        const double xs[3] = {A.x, B.x, C.x}, ys[3] = {A.y, B.y, C.y};
        double ex[3], ey[3];
        for (int i = 0; i < 3; ++i) {
            int ip1 = (i == 2) ? 0 : i + 1;
            ex[i] = ys[ip1] - ys[i];
            ey[i] = -(xs[ip1] - xs[i]);
        }
        for (int m = 0; m < 3; ++m) {
            int mm1 = (m == 0) ? 2 : m - 1;
            wx[m] = 0.5 * (ex[m] + ex[mm1]) / s;
            wy[m] = 0.5 * (ey[m] + ey[mm1]) / s;
        }
    };
    double w1x[3], w1y[3], w2x[3], w2y[3];
    tri(X1, Co, X2, w1x, w1y);
    tri(X1, X2, Ci, w2x, w2y);
    GgfcW w;
    w.p1x = w1x[0] + w2x[0]; w.p1y = w1y[0] + w2y[0];
    w.ox = w1x[1]; w.oy = w1y[1];
    w.p2x = w1x[2] + w2x[1]; w.p2y = w1y[2] + w2y[1];
    w.ix = w2x[2]; w.iy = w2y[2];
    return w;
}

// Gradient recomputed inside a viscous stage (Gradient_GG_FC over the stage's
// ghosts, then the cell gradient that the next stage reconstructs with),
// transposed: cell-gradient adjoint -> this stage's face-gradient adjoint;
// its ghost-point part goes to this stage's ghost adjoint; the rest joins
// the face-gradient adjoint of the iteration (a linear map of geometry, so
// it is transposed once at the end).
__global__ void k_adj_stage_ggfc(CCView v, AdjView a) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= v.nof) return;
    const int2 nb = v.fnb[f];
    const double s = v.fasum[f];
    double4 gx = add(a.sgx[f], scl(s / v.cov[nb.x], a.gx[nb.x]));
    double4 gy = add(a.sgy[f], scl(s / v.cov[nb.x], a.gy[nb.x]));
    if (f < v.nfi) {
        gx = add(gx, scl(s / v.cov[nb.y], a.gx[nb.y]));
        gy = add(gy, scl(s / v.cov[nb.y], a.gy[nb.y]));
    }
    const double2 gt = a.sgT[f];
    if (f >= v.nfi) {
        GgfcW w = ggfc_weights(v, f);
        a.qp[nb.y] = add(a.qp[nb.y], add(scl(w.ox, gx), scl(w.oy, gy)));
        a.qT[nb.y] = a.qT[nb.y] + w.ox * gt.x + w.oy * gt.y;
    }
    a.fgx[f] = add(a.fgx[f], gx);
    a.fgy[f] = add(a.fgy[f], gy);
    double2 t = a.fgT[f];
    a.fgT[f] = make_double2(t.x + gt.x, t.y + gt.y);
    a.sgx[f] = z4(); a.sgy[f] = z4(); a.sgT[f] = make_double2(0.0, 0.0);
}

// Convective face flux of stage s transposed through the recorded Jacobians:
// interior faces -> (ql, qr) adjoints; boundary faces -> (qcl, qc_in)
// adjoints and the angle-of-attack part; consumes this stage's ghost adjoint.
__global__ void k_adj_conv(CCView v, AdjView a, int s, int last) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= v.nof) return;
    const int2 nb = v.fnb[f];
    if (f < v.nfi) {
        const double4 Fb = sub(a.res[nb.x], a.res[nb.y]);
        double l[8];
        for (int dir = 0; dir < 8; ++dir) l[dir] = dot(a.JF[((size_t)s * 8 + dir) * v.nfi + f], Fb);
        a.fl[f] = make_double4(l[0], l[1], l[2], l[3]);
        a.fr[f] = make_double4(l[4], l[5], l[6], l[7]);
        if (a.geo) {
            const double2 gn = a.gfn[f];
            a.gfn[f] = make_double2(gn.x + dot(a.JG[((size_t)s * 3 + 0) * v.nfi + f], Fb),
                                    gn.y + dot(a.JG[((size_t)s * 3 + 1) * v.nfi + f], Fb));
            a.garea[f] = a.garea[f] + dot(a.JG[((size_t)s * 3 + 2) * v.nfi + f], Fb);
            a.fls[f] = add(a.fls[f], a.fl[f]);
            a.frs[f] = add(a.frs[f], a.fr[f]);
        }
        return;
    }
    const int b = f - v.nfi, g = nb.y;
    double4 Fb = a.res[nb.x];
    if (last && v.fbc[f] == 1001) { Fb.z = Fb.z + a.jx; Fb.w = Fb.w + a.jy; }
    const double4 gp = a.qp[g];
    const double y[9] = {Fb.x, Fb.y, Fb.z, Fb.w, gp.x, gp.y, gp.z, gp.w, a.qT[g]};
    const double* J = a.BJ + ((size_t)s * v.nbf + b) * 81;
    double x[9];
    for (int dir = 0; dir < 9; ++dir) {
        double t = 0.0;
        for (int k = 0; k < 9; ++k) t = t + J[dir * 9 + k] * y[k];
        x[dir] = t;
    }
    a.fl[f] = make_double4(x[0], x[1], x[2], x[3]);
    a.fr[f] = make_double4(x[4], x[5], x[6], x[7]);
    a.falpha[b] = a.falpha[b] + x[8];
    if (a.geo) {
        const double* G = a.BG + ((size_t)s * v.nbf + b) * 27;
        double gx = 0.0, gy = 0.0, ga = 0.0;
        for (int k = 0; k < 9; ++k) { gx = gx + G[k] * y[k]; gy = gy + G[9 + k] * y[k]; ga = ga + G[18 + k] * y[k]; }
        const double2 gn = a.gfn[f];
        a.gfn[f] = make_double2(gn.x + gx, gn.y + gy);
        a.garea[f] = a.garea[f] + ga;
        a.fls[f] = add(a.fls[f], make_double4(x[0], x[1], x[2], x[3]));
    }
    a.qp[g] = z4();
    a.qT[g] = 0.0;
}

// Reconstruction (fvresidual.F90:235-247, boundary :38-43) transposed, per
// cell over its faces: primitive adjoint (start of the iteration), gradient
// adjoint (the gradient this stage read; reset first when a viscous stage
// had recomputed it), and the wall closure's current-state adjoint.
__global__ void k_adj_recon(CCView v, AdjView a, int reset_g) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.noc) return;
    const double zhi = 1.0 / 3.0;
    const double4 ph = v.phi[i];
    const double2 c = v.cen[i];
    double4 aq = z4(), ac = z4();
    double4 gx = reset_g ? z4() : a.gx[i], gy = reset_g ? z4() : a.gy[i];
    for (int k = v.cf_off[i]; k < v.cf_off[i + 1]; ++k) {
        const int e = v.cf[k], f = e & FACE_MASK;
        const double2 fc = v.fcen[f];
        const double d0 = fc.x - c.x, d1 = fc.y - c.y;
        if (f < v.nfi) {
            const bool is_out = (e & SIDE_BIT) != 0;
            const int2 nb = v.fnb[f];
            const double4 po = v.phi[is_out ? nb.x : nb.y];
            const double4 own = is_out ? a.fr[f] : a.fl[f], oth = is_out ? a.fl[f] : a.fr[f];
            for (int j = 0; j < 4; ++j) {
                const double pj = at(ph, j), oj = at(po, j);
                put(aq, j, at(aq, j) + (1.0 - 0.5 * pj * zhi) * at(own, j) + 0.5 * oj * zhi * at(oth, j));
                const double ej = 0.5 * pj * (1.0 - zhi) * at(own, j);
                put(gx, j, at(gx, j) + ej * d0);
                put(gy, j, at(gy, j) + ej * d1);
            }
        } else {
            const double4 l = a.fl[f];
            aq = add(aq, l);
            for (int j = 0; j < 4; ++j) {
                const double ej = at(ph, j) * at(l, j);
                put(gx, j, at(gx, j) + ej * d0);
                put(gy, j, at(gy, j) + ej * d1);
            }
            ac = add(ac, a.fr[f]);
        }
    }
    a.qp[i] = add(a.qp[i], aq);
    a.gx[i] = gx;
    a.gy[i] = gy;
    a.qc[i] = add(a.qc[i], ac);
}

// The gradient of the start of the iteration transposed (Gradient_GG with
// its boundary sign, Gradient_GG_FC, Gradient_LSQR), per face.
__global__ void k_adj_start_grad(CCView v, AdjView a) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= v.nof) return;
    const int2 nb = v.fnb[f];
    const bool interior = f < v.nfi;
    if (v.grad_type == UNS_GRAD_GG) {
        const double2 n = v.fn[f];
        const double area = v.farea[f];
        const double dx = n.x * area, dy = n.y * area;
        const double si = interior ? 1.0 : -1.0;
        double4 t = add(scl(si * dx / v.cv[nb.x], a.gx[nb.x]), scl(si * dy / v.cv[nb.x], a.gy[nb.x]));
        if (interior) t = sub(t, add(scl(dx / v.cv[nb.y], a.gx[nb.y]), scl(dy / v.cv[nb.y], a.gy[nb.y])));
        a.fq[f] = add(a.fq[f], t);
    } else if (v.grad_type == UNS_GRAD_GGFC) {
        const double s = v.fasum[f];
        double4 gx = scl(s / v.cov[nb.x], a.gx[nb.x]), gy = scl(s / v.cov[nb.x], a.gy[nb.x]);
        if (interior) {
            gx = add(gx, scl(s / v.cov[nb.y], a.gx[nb.y]));
            gy = add(gy, scl(s / v.cov[nb.y], a.gy[nb.y]));
        }
        a.fgx[f] = add(a.fgx[f], gx);
        a.fgy[f] = add(a.fgy[f], gy);
    } else {
        const double4 w = v.lsw[f];
        double4 d = add(scl(w.x, a.gx[nb.x]), scl(w.y, a.gy[nb.x]));
        if (interior) d = sub(d, add(scl(w.z, a.gx[nb.y]), scl(w.w, a.gy[nb.y])));
        a.lsq[f] = d;
    }
}

// Diamond-path face gradient transposed onto its four points.
__global__ void k_adj_ggfc(CCView v, AdjView a) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= v.nof) return;
    GgfcW w = ggfc_weights(v, f);
    const double4 gx = a.fgx[f], gy = a.fgy[f];
    const double2 gt = a.fgT[f];
    a.cp1[f] = add(scl(w.p1x, gx), scl(w.p1y, gy)); a.cp1T[f] = w.p1x * gt.x + w.p1y * gt.y;
    a.cp2[f] = add(scl(w.p2x, gx), scl(w.p2y, gy)); a.cp2T[f] = w.p2x * gt.x + w.p2y * gt.y;
    a.cpi[f] = add(scl(w.ix, gx), scl(w.iy, gy)); a.cpiT[f] = w.ix * gt.x + w.iy * gt.y;
    a.cpo[f] = add(scl(w.ox, gx), scl(w.oy, gy)); a.cpoT[f] = w.ox * gt.x + w.oy * gt.y;
}

// avg_c2v face part (face value = mean of its two vertices) and the
// diamond-path vertex terms, gathered per vertex.
__global__ void k_adj_vertex(CCView v, AdjView a, int use_ggfc) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= v.nop) return;
    double4 p = z4();
    double pT = 0.0;
    for (int e = a.v2f_off[k]; e < a.v2f_off[k + 1]; ++e) {
        const int x = a.v2f[e], f = x & ~V2F_P2;
        p = add(p, scl(0.5, a.fq[f]));
        if (use_ggfc) {
            if (x & V2F_P2) { p = add(p, a.cp2[f]); pT = pT + a.cp2T[f]; }
            else { p = add(p, a.cp1[f]); pT = pT + a.cp1T[f]; }
        }
    }
    a.pp[k] = p;
    a.ppT[k] = pT;
}

// Per cell (ghosts included): vertex average transposed, diamond-path and
// LSQ cell terms, then con2prim transposed onto the state at the start of the
// iteration.  Writes the new adjoint vector in place and the squared change.
__global__ void k_adj_final(CCView v, AdjView a, int use_ggfc, int use_lsq) {
    // Ghost values of the start of the iteration reach a diamond-path
    // gradient only through Gradient_GG_FC of the start (grad_type GGFC); the
    // in-stage recomputation read each stage's own ghosts (already applied).
    const bool ghost_ggfc = use_ggfc && v.grad_type == UNS_GRAD_GGFC;
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    double dd = 0.0;
    if (i < v.ntot) {
        double4 q = a.qp[i];
        double T = a.qT[i];
        for (int e = a.c2v_off[i]; e < a.c2v_off[i + 1]; ++e) {
            const int k = a.c2v[e];
            const double w = a.c2v_w[e];
            q = add(q, scl(w, a.pp[k]));
            T = T + w * a.ppT[k];
        }
        if (use_ggfc || use_lsq) {
            auto face_terms = [&](int f, bool is_out) {
                if (use_ggfc) {
                    if (is_out) { q = add(q, a.cpo[f]); T = T + a.cpoT[f]; }
                    else { q = add(q, a.cpi[f]); T = T + a.cpiT[f]; }
                }
                if (use_lsq) q = is_out ? add(q, a.lsq[f]) : sub(q, a.lsq[f]);
            };
            if (i < v.noc) {
                for (int k = v.cf_off[i]; k < v.cf_off[i + 1]; ++k) {
                    const int e = v.cf[k];
                    face_terms(e & FACE_MASK, (e & SIDE_BIT) != 0);
                }
            } else {
                const int f = v.nfi + (i - v.noc);
                if (ghost_ggfc) { q = add(q, a.cpo[f]); T = T + a.cpoT[f]; }
                if (use_lsq) q = add(q, a.lsq[f]);
            }
        }
        if (i < v.noc) {
            const double4 c = a.q0[i];
            double r[4];
            for (int dir = 0; dir < 4; ++dir) {
                Tan E(c.x, dir == 0), rr(c.y, dir == 1), ru(c.z, dir == 2), rv(c.w, dir == 3);
                PrimT<Tan> P = con2prim_t<Tan>(v.g, E, rr, ru, rv);
                r[dir] = q.x * P.rho.d + q.y * P.u.d + q.z * P.v.d + q.w * P.p.d + T * P.t.d;
            }
            const double4 n = add(add(a.qc[i], a.qold[i]), make_double4(r[0], r[1], r[2], r[3]));
            const double4 o = a.lq[i];
            const double4 dl = sub(n, o);
            dd = dot(dl, dl);
            a.lq[i] = n;
        } else {
            const int b = i - v.noc;
            const double4 dl = sub(q, a.lg[b]);
            const double dT = T - a.lgT[b];
            dd = dot(dl, dl) + dT * dT;
            a.lg[b] = q;
            a.lgT[b] = T;
        }
    }
    dd = warp_sum(dd);
    __shared__ double sh[kBlock / 32];
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = dd;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < kBlock / 32; ++k) t = t + sh[k];
        a.part[blockIdx.x] = t;
    }
}

// d/dalpha (boundary terms in face order + the explicit term) and the norm of
// the change, in a fixed order; hist (may be null) receives sqrt(change).
__global__ void k_adj_reduce(CCView v, AdjView a, int nparts, double* hist, int k) {
    __shared__ double sa[kBlock], sd[kBlock];
    double ta = 0.0, td = 0.0;
    for (int b = threadIdx.x; b < v.nbf; b += kBlock) ta = ta + a.falpha[b];
    for (int b = threadIdx.x; b < nparts; b += kBlock) td = td + a.part[b];
    sa[threadIdx.x] = ta;
    sd[threadIdx.x] = td;
    __syncthreads();
    if (threadIdx.x == 0) {
        double x = 0.0, y = 0.0;
        for (int t = 0; t < kBlock; ++t) { x = x + sa[t]; y = y + sd[t]; }
        a.out[0] = x + a.jalpha;
        a.out[1] = y;
        if (hist) hist[k] = sqrt(y);
    }
}

// ------------------------------------------------ geometric partials
// After the transposed stages and the start gradient's transpose (a.gx, a.gy:
// the adjoint of the gradient of the start of the iteration; a.fgx, a.fgy,
// a.fgT: of the diamond-path face gradient), per face:
//  * reconstruction (fvresidual.F90:235-247, boundary :38-43): ql depends on
//    the face centre minus the cell centroid through the limited gradient;
//  * Gradient_GG (gradient.F90:95-156): g_i = sum sigma q_f n_f area_f / cv_i
//    (sigma -1 on the out side and on boundary faces);
//  * Gradient_LSQR (gradient.F90:2-93): the adjoints of the face's weights;
//  * Gradient_GG_FC (gradient.F90:159-323): the face gradient is T_f / s_f,
//    T_f the contour sum over the diamond (p1, cell out, p2, cell in) of the
//    edge means times the edge normals (the shared edge p1-p2 of the two
//    triangles cancels) and s_f the diamond's area; the cell gradient is
//    sum_f T_f / cov_i.  Contributions to the diamond's four points go to
//    gp1, gco, gp2, gci (gathered per node and cell afterwards).
__device__ __forceinline__ double dot5x(double4 a, double aT, double4 b, double bT) { return dot(a, b) + aT * bT; }

__global__ void k_geo_face(CCView v, AdjView a, int use_ggfc) {
    int f = blockIdx.x * blockDim.x + threadIdx.x;
    if (f >= v.nof) return;
    const int2 nb = v.fnb[f];
    const bool interior = f < v.nfi;
    const double zhi = 1.0 / 3.0;
    double2 gfc = make_double2(0.0, 0.0), gci = make_double2(0.0, 0.0), gco = make_double2(0.0, 0.0);
    {  // reconstruction
        const double4 ph = v.phi[nb.x], gx = a.s_gx[nb.x], gy = a.s_gy[nb.x], L = a.fls[f];
        const double c = interior ? 0.5 * (1.0 - zhi) : 1.0;
        double d0 = 0.0, d1 = 0.0;
        for (int j = 0; j < 4; ++j) {
            d0 = d0 + at(L, j) * c * at(ph, j) * at(gx, j);
            d1 = d1 + at(L, j) * c * at(ph, j) * at(gy, j);
        }
        gfc = make_double2(d0, d1);
        gci = make_double2(-d0, -d1);
        if (interior) {
            const double4 po = v.phi[nb.y], hx = a.s_gx[nb.y], hy = a.s_gy[nb.y], Rr = a.frs[f];
            double e0 = 0.0, e1 = 0.0;
            for (int j = 0; j < 4; ++j) {
                e0 = e0 + at(Rr, j) * c * at(po, j) * at(hx, j);
                e1 = e1 + at(Rr, j) * c * at(po, j) * at(hy, j);
            }
            gfc = make_double2(gfc.x + e0, gfc.y + e1);
            gco = make_double2(-e0, -e1);
        }
    }
    a.gfcen[f] = gfc;
    if (v.grad_type == UNS_GRAD_GG) {
        const double4 q = a.s_fq[f];
        const double2 n = v.fn[f];
        const double area = v.farea[f];
        const double si = interior ? 1.0 : -1.0;
        double ddx = si * dot(q, a.gx[nb.x]) / v.cv[nb.x], ddy = si * dot(q, a.gy[nb.x]) / v.cv[nb.x];
        if (interior) {
            ddx = ddx - dot(q, a.gx[nb.y]) / v.cv[nb.y];
            ddy = ddy - dot(q, a.gy[nb.y]) / v.cv[nb.y];
        }
        const double2 gn = a.gfn[f];
        a.gfn[f] = make_double2(gn.x + ddx * area, gn.y + ddy * area);
        a.garea[f] = a.garea[f] + ddx * n.x + ddy * n.y;
    } else if (v.grad_type == UNS_GRAD_LSQR) {
        const double4 var = sub(a.s_qp[nb.y], a.s_qp[nb.x]);
        a.glsw[f] = make_double4(dot(var, a.gx[nb.x]), dot(var, a.gy[nb.x]),
                                 interior ? -dot(var, a.gx[nb.y]) : 0.0, interior ? -dot(var, a.gy[nb.y]) : 0.0);
    }
    double2 g1 = make_double2(0.0, 0.0), g2 = make_double2(0.0, 0.0);
    if (use_ggfc) {
        const double s = a.s_fas[f];
        const double4 bx = a.fgx[f], by = a.fgy[f], fx = a.s_fgx[f], fy = a.s_fgy[f];
        const double2 bT = a.fgT[f], fT = a.s_fgT[f];
        // fg = T / s: the adjoint of T, and of s through fg
        double sb = -(dot5x(bx, bT.x, fx, fT.x) + dot5x(by, bT.y, fy, fT.y)) / s;
        if (v.grad_type == UNS_GRAD_GGFC) {  // the cell gradient's explicit s: sum fg s / cov
            sb = sb + (dot(fx, a.gx[nb.x]) + dot(fy, a.gy[nb.x])) / v.cov[nb.x];
            if (interior) sb = sb + (dot(fx, a.gx[nb.y]) + dot(fy, a.gy[nb.y])) / v.cov[nb.y];
        }
        const double4 tx = scl(1.0 / s, bx), ty = scl(1.0 / s, by);
        const double tTx = bT.x / s, tTy = bT.y / s;
        const int2 p = v.fpt[f];
        const double2 X[4] = {v.pxy[p.x], v.cen[nb.y], v.pxy[p.y], v.cen[nb.x]};
        const double4 Q[4] = {a.s_pp[p.x], a.s_qp[nb.y], a.s_pp[p.y], a.s_qp[nb.x]};
        const double QT[4] = {a.s_ppT[p.x], a.s_qT[nb.y], a.s_ppT[p.y], a.s_qT[nb.x]};
        double2 g[4];
        for (int k = 0; k < 4; ++k) {
            const int km = (k + 3) & 3, kp = (k + 1) & 3;
            // d T_x / d y_k = 0.5 (v_{k-1} - v_{k+1}),  d T_y / d x_k = -0.5 (v_{k-1} - v_{k+1})
            const double4 dv = sub(Q[km], Q[kp]);
            const double dT = QT[km] - QT[kp];
            const double gxk = -0.5 * dot5x(ty, tTy, dv, dT) + sb * 0.5 * (X[kp].y - X[km].y);
            const double gyk = 0.5 * dot5x(tx, tTx, dv, dT) + sb * 0.5 * (X[km].x - X[kp].x);
            g[k] = make_double2(gxk, gyk);
        }
        g1 = g[0];
        g2 = g[2];
        gco = make_double2(gco.x + g[1].x, gco.y + g[1].y);
        gci = make_double2(gci.x + g[3].x, gci.y + g[3].y);
    }
    a.gci[f] = gci;
    a.gco[f] = gco;
    a.gp1[f] = g1;
    a.gp2[f] = g2;
}

// avg_c2v vertex part transposed onto its weights: pp_k = sum w q_c / sum w.
__global__ void k_geo_vertex(CCView v, AdjView a) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= v.nop) return;
    double W = 0.0;
    for (int e = v.v2c_off[k]; e < v.v2c_off[k + 1]; ++e) W = W + v.v2c_wt[e];
    const double4 pk = a.s_pp[k], pb = a.pp[k];
    const double pkT = a.s_ppT[k], pbT = a.ppT[k];
    for (int e = v.v2c_off[k]; e < v.v2c_off[k + 1]; ++e) {
        const int c = v.v2c[e];
        a.gv2c[e] = dot5x(pb, pbT, sub(a.s_qp[c], pk), a.s_qT[c] - pkT) / W;
    }
}

// Node coordinates: the diamond-path parts of the faces at each node.
__global__ void k_geo_nodes(CCView v, AdjView a) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= v.nop) return;
    double2 g = make_double2(0.0, 0.0);
    for (int e = a.v2f_off[k]; e < a.v2f_off[k + 1]; ++e) {
        const int x = a.v2f[e], f = x & ~V2F_P2;
        const double2 t = (x & V2F_P2) ? a.gp2[f] : a.gp1[f];
        g = make_double2(g.x + t.x, g.y + t.y);
    }
    a.gpxy[k] = g;
}

// Cell centroids (ghosts included) from their faces' parts; cv (Gradient_GG)
// and cov (Gradient_GG_FC) from the start gradient g = S / cv.
__global__ void k_geo_cells(CCView v, AdjView a) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.ntot) return;
    double2 g = make_double2(0.0, 0.0);
    if (i < v.noc) {
        for (int k = v.cf_off[i]; k < v.cf_off[i + 1]; ++k) {
            const int e = v.cf[k], f = e & FACE_MASK;
            const double2 t = (e & SIDE_BIT) ? a.gco[f] : a.gci[f];
            g = make_double2(g.x + t.x, g.y + t.y);
        }
        const double d = -(dot(a.gx[i], a.s_gx[i]) + dot(a.gy[i], a.s_gy[i]));
        a.gcv[i] = v.grad_type == UNS_GRAD_GG ? d / v.cv[i] : 0.0;
        a.gcov[i] = v.grad_type == UNS_GRAD_GGFC ? d / v.cov[i] : 0.0;
    } else {
        g = a.gco[v.nfi + (i - v.noc)];
    }
    a.gcen[i] = g;
}

#define LAUNCH(kern, n, ...)                                                         \
    do {                                                                             \
        kern<<<std::max(1, nblocks(n)), kBlock, 0, h->stream>>>(__VA_ARGS__);        \
        UNS_CUDA(cudaGetLastError());                                                \
    } while (0)

// One transposed iteration: lq, lg, lgT <- G^T (lq, lg, lgT) + seed * J^T.
int enqueue_vjp(uns_cc_handle* h, double* hist, int k) {
    const CCView& v = h->v;
    const AdjView& a = h->adj->a;
    const bool lam = v.laminar != 0;
    const bool stage_grad = lam && v.grad_type != UNS_GRAD_GGFC;
    LAUNCH(k_adj_init, std::max(v.ntot, v.nof), v, a);
    for (int s = 2; s >= 0; --s) {
        const int last = s == 2;
        LAUNCH(k_adj_stage, v.noc, v, a, s + 1);
        if (lam) {
            LAUNCH(k_adj_visc, v.nof, v, a, s, last, stage_grad ? 1 : 0);
            LAUNCH(k_adj_mul, v.noc, v, a, s);
            if (stage_grad) LAUNCH(k_adj_stage_ggfc, v.nof, v, a);
        }
        LAUNCH(k_adj_conv, v.nof, v, a, s, last);
        LAUNCH(k_adj_recon, v.noc, v, a, stage_grad ? 1 : 0);
    }
    LAUNCH(k_adj_start_grad, v.nof, v, a);
    const bool use_ggfc = lam || v.grad_type == UNS_GRAD_GGFC;
    const bool use_lsq = v.grad_type == UNS_GRAD_LSQR;
    if (a.geo) LAUNCH(k_geo_face, v.nof, v, a, use_ggfc ? 1 : 0);
    if (use_ggfc) LAUNCH(k_adj_ggfc, v.nof, v, a);
    LAUNCH(k_adj_vertex, v.nop, v, a, use_ggfc ? 1 : 0);
    if (a.geo) {
        LAUNCH(k_geo_vertex, v.nop, v, a);
        LAUNCH(k_geo_nodes, v.nop, v, a);
        LAUNCH(k_geo_cells, v.ntot, v, a);
    }
    LAUNCH(k_adj_final, v.ntot, v, a, use_ggfc ? 1 : 0, use_lsq ? 1 : 0);
    k_adj_reduce<<<1, kBlock, 0, h->stream>>>(v, a, h->adj->nparts, hist, k);
    UNS_CUDA(cudaGetLastError());
    return UNS_OK;
}

int rec_hook(uns_cc_handle* h, int point, int stage, void*) {
    const CCView& v = h->v;
    const AdjView& a = h->adj->a;
    const int s = stage - 1;
    switch (point) {
        case REC_AFTER_START:
            LAUNCH(k_rec_start, v.noc, v, a);
            if (a.geo) LAUNCH(k_rec_geo, std::max(std::max(v.ntot, v.nof), v.nop), v, a);
            break;
        case REC_BEFORE_FACE_CONV: LAUNCH(k_rec_conv, v.nof, v, a, s); break;
        case REC_BEFORE_CELL_MUL: LAUNCH(k_rec_mul, v.noc, v, a, s); break;
        case REC_AFTER_FACE_VISC: LAUNCH(k_rec_visc, v.nof, v, a, s); break;
        default: break;
    }
    return UNS_OK;
}

template <class T>
int adj_alloc(uns_cc_handle* h, T*& p, size_t n) {
    void* q = nullptr;
    UNS_CUDA(cudaMalloc(&q, std::max<size_t>(n, 1) * sizeof(T)));
    UNS_CUDA(cudaMemsetAsync(q, 0, std::max<size_t>(n, 1) * sizeof(T), h->stream));
    h->adj->allocs.push_back(q);
    p = (T*)q;
    return UNS_OK;
}
template <class T>
int adj_alloc(uns_cc_handle* h, const T*& p, size_t n) {
    T* q = nullptr;
    int rc = adj_alloc(h, q, n);
    p = q;
    return rc;
}

// Arrays, transposed connectivity (from the device copies of the mesh
// lists), created once per handle.
int adj_setup(uns_cc_handle* h) {
    if (h->adj) return UNS_OK;
    h->adj = new CCAdj();
    const CCView& v = h->v;
    AdjView& a = h->adj->a;
    a.nstage = 3;
    const size_t noc = v.noc, nof = v.nof, nfi = v.nfi, nbf = v.nbf, nop = v.nop, ntot = v.ntot;
    int rc;
#define AA(field, n) if ((rc = adj_alloc(h, a.field, (n)))) return rc
    AA(JF, 3 * 8 * nfi); AA(BJ, 3 * nbf * 81); AA(DM, 3 * noc); AA(VI, 3 * nof * 9); AA(Dv, noc); AA(q0, noc);
    AA(qc, noc); AA(qold, noc); AA(qp, ntot); AA(qT, ntot); AA(pp, nop); AA(ppT, nop);
    AA(fq, nof); AA(fgx, nof); AA(fgy, nof); AA(fgT, nof); AA(sgx, nof); AA(sgy, nof); AA(sgT, nof);
    AA(gx, noc); AA(gy, noc); AA(res, noc); AA(fl, nof); AA(fr, nof); AA(lsq, nof); AA(fmu, nof); AA(falpha, nbf);
    AA(cp1, nof); AA(cp2, nof); AA(cpi, nof); AA(cpo, nof); AA(cp1T, nof); AA(cp2T, nof); AA(cpiT, nof); AA(cpoT, nof);
    AA(lq, noc); AA(lg, nbf); AA(lgT, nbf);
    h->adj->nparts = nblocks(ntot);
    AA(part, h->adj->nparts); AA(out, 2);
    // vertex -> faces and cell -> (vertex, weight) from the device lists
    std::vector<int2> fpt(nof);
    std::vector<int> v2c_off(nop + 1);
    UNS_CUDA(cudaMemcpyAsync(fpt.data(), v.fpt, nof * sizeof(int2), cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaMemcpyAsync(v2c_off.data(), v.v2c_off, (nop + 1) * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    const size_t nnz = v2c_off[nop];
    std::vector<int> v2c(nnz);
    std::vector<double> wt(nnz);
    UNS_CUDA(cudaMemcpyAsync(v2c.data(), v.v2c, nnz * sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaMemcpyAsync(wt.data(), v.v2c_wt, nnz * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    std::vector<int> vf_off(nop + 1, 0);
    for (size_t f = 0; f < nof; ++f) { vf_off[fpt[f].x + 1]++; vf_off[fpt[f].y + 1]++; }
    for (size_t k = 0; k < nop; ++k) vf_off[k + 1] += vf_off[k];
    std::vector<int> vf(vf_off[nop]), pos(vf_off.begin(), vf_off.end() - 1);
    for (size_t f = 0; f < nof; ++f) {
        vf[pos[fpt[f].x]++] = (int)f;
        vf[pos[fpt[f].y]++] = (int)f | V2F_P2;
    }
    std::vector<int> cv_off(ntot + 1, 0);
    for (size_t e = 0; e < nnz; ++e) cv_off[v2c[e] + 1]++;
    for (size_t c = 0; c < ntot; ++c) cv_off[c + 1] += cv_off[c];
    std::vector<int> cvk(nnz), cpos(cv_off.begin(), cv_off.end() - 1);
    std::vector<double> cvw(nnz);
    for (size_t k = 0; k < nop; ++k) {
        double W = 0.0;  // the forward sum, in its order
        for (int e = v2c_off[k]; e < v2c_off[k + 1]; ++e) W = W + wt[e];
        for (int e = v2c_off[k]; e < v2c_off[k + 1]; ++e) {
            int p = cpos[v2c[e]]++;
            cvk[p] = (int)k;
            cvw[p] = wt[e] / W;
        }
    }
    auto up = [&](auto& dst, const auto& vec) -> int {
        using T = typename std::decay<decltype(vec)>::type::value_type;
        T* d = nullptr;
        int r = adj_alloc(h, d, vec.size());
        if (r) return r;
        if (!vec.empty()) UNS_CUDA(cudaMemcpyAsync(d, vec.data(), vec.size() * sizeof(T), cudaMemcpyHostToDevice, h->stream));
        dst = d;
        return UNS_OK;
    };
    if ((rc = up(a.v2f_off, vf_off)) || (rc = up(a.v2f, vf)) || (rc = up(a.c2v_off, cv_off)) || (rc = up(a.c2v, cvk)) ||
        (rc = up(a.c2v_w, cvw)))
        return rc;
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    return UNS_OK;
#undef AA
}

// Arrays of the geometric linearisation, created on the first
// uns_cc_adjoint_prepare_geometry.
int geo_setup(uns_cc_handle* h) {
    CCAdj& A = *h->adj;
    if (A.geo_alloc) return UNS_OK;
    const CCView& v = h->v;
    AdjView& a = A.a;
    const size_t noc = v.noc, nof = v.nof, nfi = v.nfi, nbf = v.nbf, nop = v.nop, ntot = v.ntot;
    int nnz = 0;
    UNS_CUDA(cudaMemcpyAsync(&nnz, v.v2c_off + nop, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    A.nv2c = nnz;
    int rc;
#define AA(field, n) if ((rc = adj_alloc(h, a.field, (n)))) return rc
    AA(JG, 3 * 3 * nfi); AA(BG, 3 * nbf * 27);
    AA(s_qp, ntot); AA(s_qT, ntot); AA(s_gx, noc); AA(s_gy, noc); AA(s_pp, nop); AA(s_ppT, nop);
    AA(s_fq, nof); AA(s_fgx, nof); AA(s_fgy, nof); AA(s_fgT, nof); AA(s_fas, nof);
    AA(fls, nof); AA(frs, nof); AA(gfn, nof); AA(gfcen, nof); AA(gci, nof); AA(gco, nof); AA(gp1, nof); AA(gp2, nof);
    AA(garea, nof); AA(glsw, nof); AA(gpxy, nop); AA(gcen, ntot); AA(gcv, noc); AA(gcov, noc); AA(gv2c, (size_t)nnz);
#undef AA
    A.geo_alloc = true;
    return UNS_OK;
}

// Host part of the LSQ weights' transpose (the weights are formed on the
// host from the centroids and r11, r12, r22 at create, gradient.F90:27-44,
// 72-78): one side's (wx, wy) = (a1 - a2 r12 / r11, a2) with
// a1 = dx / r11^2, a2 = (dy - dx r12 / r11) / r22^2.
void lsw_side_vjp(double dx, double dy, double r11, double r12, double r22, double wxb, double wyb, double& dxb,
                  double& dyb, double& r11b, double& r12b, double& r22b) {
    const double num = dy - dx * r12 / r11, a2 = num / (r22 * r22);
    const double a1b = wxb, a2b = wyb - wxb * r12 / r11;
    r12b = -wxb * a2 / r11;
    r11b = wxb * a2 * r12 / (r11 * r11);
    dxb = a1b / (r11 * r11);
    r11b = r11b - 2.0 * a1b * dx / (r11 * r11 * r11);
    const double numb = a2b / (r22 * r22);
    r22b = -2.0 * a2b * num / (r22 * r22 * r22);
    dyb = numb;
    dxb = dxb - numb * r12 / r11;
    r12b = r12b - numb * dx / r11;
    r11b = r11b + numb * dx * r12 / (r11 * r11);
}

int fail_adj(const char* msg, int code) {
    set_last_error(msg);
    return code;
}

// Seeds of objective J per unit seed: dJ/dFx1, dJ/dFy1 and the explicit dJ/dalpha.
void objective_seeds(uns_cc_handle* h, int obj, double seed, AdjView& a) {
    const double al = h->P.aoa_deg * (4.0 * std::atan(1.0)) / 180.0;
    const double c = std::cos(al), s = std::sin(al), fx = h->adj->fx, fy = h->adj->fy;
    if (obj == UNS_OBJ_CL) {  // C_L = 2 (Fy cos a - Fx sin a)
        a.jx = seed * (-2.0 * s);
        a.jy = seed * (2.0 * c);
        a.jalpha = seed * (-2.0 * (fy * s + fx * c));
    } else {  // C_D = 2 (Fx cos a + Fy sin a)
        a.jx = seed * (2.0 * c);
        a.jy = seed * (2.0 * s);
        a.jalpha = seed * (2.0 * (fy * c - fx * s));
    }
}

}  // namespace

// ====================================================================== C-ABI
extern "C" {

static int adjoint_prepare_impl(uns_cc_handle* h, double cfl, double* cl, double* cd, bool geo);

int uns_cc_adjoint_prepare(uns_cc_handle* h, double cfl, double* cl, double* cd) {
    return adjoint_prepare_impl(h, cfl, cl, cd, false);
}

int uns_cc_adjoint_prepare_geometry(uns_cc_handle* h, double cfl, double* cl, double* cd) {
    return adjoint_prepare_impl(h, cfl, cl, cd, true);
}

static int adjoint_prepare_impl(uns_cc_handle* h, double cfl, double* cl, double* cd, bool geo) {
    if (!h || !(cfl > 0.0)) return fail_adj("uns_cc_adjoint_prepare: bad argument", UNS_ERR_ARG);
    if (geo && h->v.ninst > 0)
        return fail_adj("uns_cc_adjoint_prepare_geometry: one case per handle (not a packed handle)", UNS_ERR_ARG);
    if (geo && h->P.flow_type != UNS_FLOW_INVISCID && h->P.grad_type != UNS_GRAD_GGFC)
        return fail_adj("uns_cc_adjoint_prepare_geometry: a laminar flow's geometry is differentiated with the GG-FC "
                        "gradient only (the others recompute the gradient inside each stage)", UNS_ERR_ARG);
    ++h->flux_gen;  // the recorded iterations overwrite the step's arrays
    if (h->P.time_mode != UNS_TIME_RK3)
        return fail_adj("uns_cc_adjoint_prepare: the adjoint follows the RK3 iteration (time_mode = RK3)", UNS_ERR_ARG);
    if (h->P.precision != UNS_PREC_FP64)
        return fail_adj("uns_cc_adjoint_prepare: the adjoint linearises the FP64 form", UNS_ERR_ARG);
    if (h->P.irs && cfl > h->P.cfl_max)
        return fail_adj("uns_cc_adjoint_prepare: residual smoothing (cfl > cfl_max) is not differentiated", UNS_ERR_ARG);
    int rc = adj_setup(h);
    if (rc) return rc;
    CCAdj& A = *h->adj;
    if (geo && (rc = geo_setup(h))) return rc;
    const double al = h->P.aoa_deg * (4.0 * std::atan(1.0)) / 180.0;
    A.a.dua = -std::sin(al);
    A.a.dva = std::cos(al);
    A.recorded = false;
    A.geo_recorded = false;
    // The local time step of a viscous flow reads the face viscosity of the
    // previous iteration (spectral02's viscous term), which is not part of
    // the state vector: one plain iteration first makes it the converged
    // state's own, so the recorded dt is the one of the converged iteration.
    if (h->P.flow_type != UNS_FLOW_INVISCID &&
        (rc = cc_record_iteration(h, cfl, [](uns_cc_handle*, int, int, void*) { return (int)UNS_OK; }, nullptr)))
        return rc;
    A.a.geo = geo ? 1 : 0;
    rc = cc_record_iteration(h, cfl, rec_hook, nullptr);
    A.a.geo = 0;
    if (rc) return rc;
    double fx = 0.0, fy = 0.0;
    if ((rc = uns_cc_forces(h, &fx, &fy))) return rc;
    A.fx = fx;
    A.fy = fy;
    A.cfl = cfl;
    A.recorded = true;
    A.geo_recorded = geo;
    if (cl) *cl = 2.0 * (fy * std::cos(al) - fx * std::sin(al));
    if (cd) *cd = 2.0 * (fx * std::cos(al) + fy * std::sin(al));
    return cc_check_dev_err(h);
}

int uns_cc_adjoint_vjp(uns_cc_handle* h, int objective, double seed, const double* wq, const double* wg, double* oq,
                       double* og, double* oalpha) {
    if (!h || !wq || !wg || !oq || !og || (objective != UNS_OBJ_CL && objective != UNS_OBJ_CD))
        return fail_adj("uns_cc_adjoint_vjp: bad argument", UNS_ERR_ARG);
    ++h->flux_gen;  // the recorded iterations overwrite the step's arrays
    if (!h->adj || !h->adj->recorded) return fail_adj("uns_cc_adjoint_vjp: call uns_cc_adjoint_prepare first", UNS_ERR_ARG);
    const CCView& v = h->v;
    AdjView& a = h->adj->a;
    objective_seeds(h, objective, seed, a);
    std::vector<double4> g(v.nbf);
    std::vector<double> gT(v.nbf);
    for (int b = 0; b < v.nbf; ++b) {
        g[b] = make_double4(wg[5 * b], wg[5 * b + 1], wg[5 * b + 2], wg[5 * b + 3]);
        gT[b] = wg[5 * b + 4];
    }
    UNS_CUDA(cudaMemcpyAsync(a.lq, wq, sizeof(double4) * v.noc, cudaMemcpyHostToDevice, h->stream));
    UNS_CUDA(cudaMemcpyAsync(a.lg, g.data(), sizeof(double4) * v.nbf, cudaMemcpyHostToDevice, h->stream));
    UNS_CUDA(cudaMemcpyAsync(a.lgT, gT.data(), sizeof(double) * v.nbf, cudaMemcpyHostToDevice, h->stream));
    int rc = enqueue_vjp(h, nullptr, 0);
    if (rc) return rc;
    double out[2];
    UNS_CUDA(cudaMemcpyAsync(oq, a.lq, sizeof(double4) * v.noc, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaMemcpyAsync(g.data(), a.lg, sizeof(double4) * v.nbf, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaMemcpyAsync(gT.data(), a.lgT, sizeof(double) * v.nbf, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaMemcpyAsync(out, a.out, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    for (int b = 0; b < v.nbf; ++b) {
        og[5 * b] = g[b].x; og[5 * b + 1] = g[b].y; og[5 * b + 2] = g[b].z; og[5 * b + 3] = g[b].w; og[5 * b + 4] = gT[b];
    }
    if (oalpha) *oalpha = out[0];
    return cc_check_dev_err(h);
}

int uns_cc_adjoint_geometry(uns_cc_handle* h, int objective, double seed, const double* wq, const double* wg,
                            uns_cc_mesh_adj* out) {
    if (!h || !wq || !wg || !out || (objective != UNS_OBJ_CL && objective != UNS_OBJ_CD))
        return fail_adj("uns_cc_adjoint_geometry: bad argument", UNS_ERR_ARG);
    if (!h->adj || !h->adj->geo_recorded)
        return fail_adj("uns_cc_adjoint_geometry: call uns_cc_adjoint_prepare_geometry first", UNS_ERR_ARG);
    const uns_cc_mesh_adj& o = *out;
    if (!o.px || !o.py || !o.cx || !o.cy || !o.cv || !o.cov || !o.fnx || !o.fny || !o.farea || !o.fcx || !o.fcy ||
        !o.r11 || !o.r12 || !o.r22 || !o.v2c_wt)
        return fail_adj("uns_cc_adjoint_geometry: every output array is required", UNS_ERR_ARG);
    ++h->flux_gen;
    CCAdj& A = *h->adj;
    const CCView& v = h->v;
    AdjView& a = A.a;
    const int noc = v.noc, nof = v.nof, nbf = v.nbf, nop = v.nop, ntot = v.ntot;
    objective_seeds(h, objective, seed, a);
    std::vector<double4> g(nbf);
    std::vector<double> gT(nbf);
    for (int b = 0; b < nbf; ++b) {
        g[b] = make_double4(wg[5 * b], wg[5 * b + 1], wg[5 * b + 2], wg[5 * b + 3]);
        gT[b] = wg[5 * b + 4];
    }
    UNS_CUDA(cudaMemcpyAsync(a.lq, wq, sizeof(double4) * noc, cudaMemcpyHostToDevice, h->stream));
    UNS_CUDA(cudaMemcpyAsync(a.lg, g.data(), sizeof(double4) * nbf, cudaMemcpyHostToDevice, h->stream));
    UNS_CUDA(cudaMemcpyAsync(a.lgT, gT.data(), sizeof(double) * nbf, cudaMemcpyHostToDevice, h->stream));
    a.geo = 1;
    int rc = enqueue_vjp(h, nullptr, 0);
    a.geo = 0;
    if (rc) return rc;
    std::vector<double2> pxy(nop), cen(ntot), fn(nof), fc(nof), cen_val(ntot);
    std::vector<double4> lsw(nof);
    std::vector<double> cv(noc), cov(noc), area(nof), wv(A.nv2c);
    UNS_CUDA(cudaMemcpyAsync(pxy.data(), a.gpxy, sizeof(double2) * nop, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaMemcpyAsync(cen.data(), a.gcen, sizeof(double2) * ntot, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaMemcpyAsync(fn.data(), a.gfn, sizeof(double2) * nof, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaMemcpyAsync(fc.data(), a.gfcen, sizeof(double2) * nof, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaMemcpyAsync(lsw.data(), a.glsw, sizeof(double4) * nof, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaMemcpyAsync(cv.data(), a.gcv, sizeof(double) * noc, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaMemcpyAsync(cov.data(), a.gcov, sizeof(double) * noc, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaMemcpyAsync(area.data(), a.garea, sizeof(double) * nof, cudaMemcpyDeviceToHost, h->stream));
    if (A.nv2c) UNS_CUDA(cudaMemcpyAsync(wv.data(), a.gv2c, sizeof(double) * A.nv2c, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaMemcpyAsync(cen_val.data(), v.cen, sizeof(double2) * ntot, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    if ((rc = cc_check_dev_err(h))) return rc;
    for (int k = 0; k < nop; ++k) { o.px[k] = pxy[k].x; o.py[k] = pxy[k].y; }
    for (int i = 0; i < ntot; ++i) { o.cx[i] = cen[i].x; o.cy[i] = cen[i].y; }
    for (int i = 0; i < noc; ++i) { o.cv[i] = cv[i]; o.cov[i] = cov[i]; o.r11[i] = 0.0; o.r12[i] = 0.0; o.r22[i] = 0.0; }
    for (int f = 0; f < nof; ++f) {
        o.fnx[f] = fn[f].x; o.fny[f] = fn[f].y; o.farea[f] = area[f]; o.fcx[f] = fc[f].x; o.fcy[f] = fc[f].y;
    }
    for (int e = 0; e < A.nv2c; ++e) o.v2c_wt[e] = wv[e];
    if (v.grad_type == UNS_GRAD_LSQR) {  // the weights' adjoints onto the centroids and r11, r12, r22
        const std::vector<double>& r = h->lsq_r;
        for (int f = 0; f < nof; ++f) {
            const int in = h->fnb_host[f].x, ot = h->fnb_host[f].y;
            const double dx = cen_val[ot].x - cen_val[in].x, dy = cen_val[ot].y - cen_val[in].y;
            double dxb, dyb, r11b, r12b, r22b;
            lsw_side_vjp(dx, dy, r[3 * in], r[3 * in + 1], r[3 * in + 2], lsw[f].x, lsw[f].y, dxb, dyb, r11b, r12b, r22b);
            o.cx[ot] += dxb; o.cx[in] -= dxb; o.cy[ot] += dyb; o.cy[in] -= dyb;
            o.r11[in] += r11b; o.r12[in] += r12b; o.r22[in] += r22b;
            if (f < v.nfi) {
                lsw_side_vjp(-dx, -dy, r[3 * ot], r[3 * ot + 1], r[3 * ot + 2], lsw[f].z, lsw[f].w, dxb, dyb, r11b, r12b,
                             r22b);
                o.cx[in] += dxb; o.cx[ot] -= dxb; o.cy[in] += dyb; o.cy[ot] -= dyb;
                o.r11[ot] += r11b; o.r12[ot] += r12b; o.r22[ot] += r22b;
            }
        }
    }
    return UNS_OK;
}

int uns_cc_adjoint_solve(uns_cc_handle* h, int objective, int max_iter, double tol, double* dj_dalpha, double* hist,
                         int* iters) {
    if (!h || max_iter < 1 || !(tol >= 0.0) || (objective != UNS_OBJ_CL && objective != UNS_OBJ_CD))
        return fail_adj("uns_cc_adjoint_solve: bad argument", UNS_ERR_ARG);
    ++h->flux_gen;  // the recorded iterations overwrite the step's arrays
    if (!h->adj || !h->adj->recorded) return fail_adj("uns_cc_adjoint_solve: call uns_cc_adjoint_prepare first", UNS_ERR_ARG);
    CCAdj& A = *h->adj;
    const CCView& v = h->v;
    if (iters) *iters = 0;
    objective_seeds(h, objective, 1.0, A.a);
    UNS_CUDA(cudaMemsetAsync(A.a.lq, 0, sizeof(double4) * v.noc, h->stream));
    UNS_CUDA(cudaMemsetAsync(A.a.lg, 0, sizeof(double4) * v.nbf, h->stream));
    UNS_CUDA(cudaMemsetAsync(A.a.lgT, 0, sizeof(double) * v.nbf, h->stream));
    // One graph of `chunk` transposed iterations, replayed until the change
    // of the adjoint vector drops below tol relative to its first change.
    const int chunk = std::min(max_iter, 50);
    double* d_hist = nullptr;
    UNS_CUDA(cudaMalloc(&d_hist, sizeof(double) * chunk));
    int rc = UNS_OK;
    cudaGraphExec_t exec = nullptr;
    {
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess) rc = UNS_ERR_CUDA;
        for (int k = 0; k < chunk && !rc; ++k) rc = enqueue_vjp(h, d_hist, k);
        cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
        if (!rc && ce == cudaSuccess) ce = cudaGraphInstantiate(&exec, g, 0);
        if (g) cudaGraphDestroy(g);
        if (!rc && ce != cudaSuccess) { set_last_error(std::string("adjoint graph: ") + cudaGetErrorString(ce)); rc = UNS_ERR_CUDA; }
    }
    std::vector<double> hh(chunk);
    double first = -1.0;
    int done = 0;
    double out[2] = {0.0, 0.0};
    while (!rc && done < max_iter) {
        if (cudaGraphLaunch(exec, h->stream) != cudaSuccess) { rc = UNS_ERR_CUDA; break; }
        if (cudaMemcpyAsync(hh.data(), d_hist, sizeof(double) * chunk, cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
            cudaMemcpyAsync(out, A.a.out, 2 * sizeof(double), cudaMemcpyDeviceToHost, h->stream) != cudaSuccess ||
            cudaStreamSynchronize(h->stream) != cudaSuccess) { rc = UNS_ERR_CUDA; break; }
        bool conv = false;
        int k = 0;
        for (; k < chunk && done + k < max_iter; ++k) {
            if (hist) hist[done + k] = hh[k];
            if (first < 0.0) first = hh[k];
            if (!std::isfinite(hh[k])) { rc = UNS_ERR_NAN; break; }
            if (first > 0.0 && hh[k] <= tol * first) { conv = true; ++k; break; }
        }
        done += k;
        if (conv) break;
    }
    cudaStreamSynchronize(h->stream);
    if (exec) cudaGraphExecDestroy(exec);
    cudaFree(d_hist);
    if (rc) {
        if (rc == UNS_ERR_CUDA) set_last_error("uns_cc_adjoint_solve: CUDA error");
        if (rc == UNS_ERR_NAN) set_last_error("uns_cc_adjoint_solve: the adjoint iteration diverged");
        return rc;
    }
    if (iters) *iters = done;
    if (dj_dalpha) *dj_dalpha = out[0];
    return cc_check_dev_err(h);
}

int uns_cc_adjoint_get(uns_cc_handle* h, double* lambda_q, double* lambda_g) {
    if (!h || !h->adj) return fail_adj("uns_cc_adjoint_get: no adjoint", UNS_ERR_ARG);
    const CCView& v = h->v;
    const AdjView& a = h->adj->a;
    if (lambda_q) UNS_CUDA(cudaMemcpyAsync(lambda_q, a.lq, sizeof(double4) * v.noc, cudaMemcpyDeviceToHost, h->stream));
    std::vector<double4> g(v.nbf);
    std::vector<double> gT(v.nbf);
    UNS_CUDA(cudaMemcpyAsync(g.data(), a.lg, sizeof(double4) * v.nbf, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaMemcpyAsync(gT.data(), a.lgT, sizeof(double) * v.nbf, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    if (lambda_g)
        for (int b = 0; b < v.nbf; ++b) {
            double* o = lambda_g + 5 * b;
            o[0] = g[b].x; o[1] = g[b].y; o[2] = g[b].z; o[3] = g[b].w; o[4] = gT[b];
        }
    return UNS_OK;
}

}  // extern "C"
