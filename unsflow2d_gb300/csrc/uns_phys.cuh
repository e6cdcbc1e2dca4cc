// uns_phys.cuh -- per-face / per-cell physics of the UNSFlow2D hot path as
// device functions.  Templated on the arithmetic type R: double for the FP64
// form, float for the FP32 face arithmetic of the mixed form.  Expression
// order follows the reference Fortran statement by statement so the FP64 form
// rounds like it (up to fused multiply-adds).
#pragma once
#include <cuda_runtime.h>

#include "unsflow_types.h"

namespace uns {

template <class R>
struct V4 {
    R a, b, c, d;
    __host__ __device__ R& operator[](int i) { return (&a)[i]; }
    __host__ __device__ const R& operator[](int i) const { return (&a)[i]; }
};

// Gas constants shared by every kernel of one solver instance.
struct Gas {
    double gamma, gamma1;
    double m_inf, znd;                 // znd = 1/(gamma*m_inf*m_inf)
    double r_inf, u_inf, v_inf, p_inf, a_inf;
    double t_wall, T_infd, SCONST;
    double rey, prandtl, vll;
    double mref;                       // AUSM reference Mach
    int flux, flow, iwall;
};

template <class R> __device__ __forceinline__ R rmax(R a, R b) { return (a < b) ? b : a; }
template <class R> __device__ __forceinline__ R rmin(R a, R b) { return (b < a) ? b : a; }

// con2prim (CCFVM/types/pri.F90:13-37)
struct Prim {
    double rho, u, v, e, p, t;
};
__device__ __forceinline__ Prim con2prim(const Gas& g, double E, double r, double ru, double rv) {
    Prim o;
    o.rho = r;
    o.u = ru / r;
    o.v = rv / r;
    o.e = E / o.rho;
    double q = o.u * o.u + o.v * o.v;
    o.p = (g.gamma - 1.0) * (E - 0.5 * o.rho * q);
    o.t = o.p / (o.rho * g.znd);
    return o;
}

// prim2con (CCFVM/types/pri.F90:39-57)
template <class R>
__device__ __forceinline__ V4<R> prim2con(R gamma, const V4<R>& pr) {
    V4<R> c;
    R rho = pr[0], u = pr[1], v = pr[2], p = pr[3];
    c[0] = p / (gamma - R(1)) + R(0.5) * rho * (u * u + v * v);
    c[1] = rho;
    c[2] = rho * u;
    c[3] = rho * v;
    return c;
}

// Mach-number polynomials (CCFVM/solution.F90:265-359)
template <class R> __device__ __forceinline__ R m1p(R m) { return R(0.5) * (m + fabs(m)); }
template <class R> __device__ __forceinline__ R m1m(R m) { return R(0.5) * (m - fabs(m)); }
template <class R> __device__ __forceinline__ R m2p(R m) { return R(0.25) * (m + R(1)) * (m + R(1)); }
template <class R> __device__ __forceinline__ R m2m(R m) { return R(-0.25) * (m - R(1)) * (m - R(1)); }
template <class R> __device__ __forceinline__ R m4p(R m, R beta) {
    return fabs(m) >= R(1) ? R(0.5) * (m + fabs(m)) : m2p(m) * (R(1) - R(16) * beta * m2m(m));
}
template <class R> __device__ __forceinline__ R m4m(R m, R beta) {
    return fabs(m) >= R(1) ? R(0.5) * (m - fabs(m)) : m2m(m) * (R(1) + R(16) * beta * m2p(m));
}
template <class R> __device__ __forceinline__ R p5p(R m, R al) {
    return fabs(m) >= R(1) ? R(0.5) * (m + fabs(m)) / m : m2p(m) * ((R(2) - m) - R(16) * al * m * m2m(m));
}
template <class R> __device__ __forceinline__ R p5m(R m, R al) {
    return fabs(m) >= R(1) ? R(0.5) * (m - fabs(m)) / m : m2m(m) * ((R(-2) - m) + R(16) * al * m * m2p(m));
}

// Roe flux with Harten entropy fix (CCFVM/roe_flux.F90:1-155).  Returns
// false where the Roe-averaged a^2 <= 0 (the reference stops there).
template <class R>
__device__ __forceinline__ bool roe_flux(R G, R G1, R nx, R ny, R area, const V4<R>& ql, const V4<R>& qr, V4<R>& flux) {
    R rl = ql[0], ul = ql[1], vl = ql[2], pl = ql[3];
    R rr = qr[0], ur = qr[1], vr = qr[2], pr = qr[3];
    R ql2 = ul * ul + vl * vl;
    R al2 = G * pl / rl;
    R hl = al2 / G1 + R(0.5) * ql2;
    R qr2 = ur * ur + vr * vr;
    R ar2 = G * pr / rr;
    R hr = ar2 / G1 + R(0.5) * qr2;
    R unl = ul * nx + vl * ny;
    R unr = ur * nx + vr * ny;
    R fc0 = rl * hl * unl + rr * hr * unr;
    R fc1 = rl * unl + rr * unr;
    R fc2 = pl * nx + rl * ul * unl + pr * nx + rr * ur * unr;
    R fc3 = pl * ny + rl * vl * unl + pr * ny + rr * vr * unr;
    R rl12 = sqrt(rl), rr12 = sqrt(rr);
    R rd = R(1) / (rl12 + rr12);
    R ua = (ul * rl12 + ur * rr12) * rd;
    R va = (vl * rl12 + vr * rr12) * rd;
    R ha = (hl * rl12 + hr * rr12) * rd;
    R qa2 = ua * ua + va * va;
    R aa2 = G1 * (ha - R(0.5) * qa2);
    bool ok = !(aa2 <= R(0));  // roe_flux.F90:73: `if (aa2 .le. 0)` -- a NaN goes on, as there
    R aa = sqrt(aa2);
    R una = ua * nx + va * ny;
    R vna = -ua * ny + va * nx;
    R e1 = fabs(una - aa), e2 = fabs(una), e4 = fabs(una + aa);
    R del = R(0.1) * aa;
    R l1 = (e1 < del) ? R(0.5) * (del + e1 * e1 / del) : e1;
    R l2 = (e2 < del) ? R(0.5) * (del + e2 * e2 / del) : e2;
    R l3 = l2;
    R l4 = (e4 < del) ? R(0.5) * (del + e4 * e4 / del) : e4;
    R du1 = rr - rl;
    R du2 = rr * ur - rl * ul;
    R du3 = rr * vr - rl * vl;
    R du4 = (rr * hr - pr) - (rl * hl - pl);
    R m1 = (nx * du2 + ny * du3 - una * du1) / aa;
    R m2 = G1 * (du4 - ua * du2 - va * du3 + qa2 * du1) / (aa * aa);
    R a1 = R(0.5) * (m2 - m1);
    R a2 = (ny * du2 - nx * du3 + vna * du1) / aa;
    R a4 = R(0.5) * (m1 + m2);
    R a3 = du1 - a1 - a4;
    R a1l1 = a1 * l1, a2l2 = a2 * l2, a3l3 = a3 * l3, a4l4 = a4 * l4;
    R aact = aa * nx, aast = aa * ny;
    R Fd0 = a1l1 * (ha - una * aa) + a2l2 * aa * vna + a3l3 * R(0.5) * qa2 + a4l4 * (ha + una * aa);
    R Fd1 = a1l1 + a3l3 + a4l4;
    R Fd2 = a1l1 * (ua - aact) + a2l2 * aa * ny + a3l3 * ua + a4l4 * (ua + aact);
    R Fd3 = a1l1 * (va - aast) - a2l2 * aa * nx + a3l3 * va + a4l4 * (va + aast);
    R h = R(0.5) * area;
    flux[0] = h * (fc0 - Fd0);
    flux[1] = h * (fc1 - Fd1);
    flux[2] = h * (fc2 - Fd2);
    flux[3] = h * (fc3 - Fd3);
    return ok;
}

// Rusanov flux (CCFVM/rusanov_flux.F90:1-77).  Overwrites ql/qr with their
// conserved form, as the reference does.
template <class R>
__device__ __forceinline__ void rusanov_flux(R G, R G1, R nx, R ny, R area, V4<R>& ql, V4<R>& qr, V4<R>& flux) {
    R rol = ql[0], ul = ql[1], vl = ql[2], pl = ql[3];
    R ql2 = ul * ul + vl * vl;
    R al2 = G * pl / rol;
    R hl = al2 / G1 + R(0.5) * ql2;
    R cl = sqrt(G * pl / rol);
    R ror = qr[0], ur = qr[1], vr = qr[2], pr = qr[3];
    R qr2 = ur * ur + vr * vr;
    R ar2 = G * pr / ror;
    R hr = ar2 / G1 + R(0.5) * qr2;
    R cr = sqrt(G * pr / ror);
    R unl = ul * nx + vl * ny;
    R unr = ur * nx + vr * ny;
    V4<R> fl, fr;
    fl[0] = rol * hl * unl; fl[1] = rol * unl; fl[2] = rol * unl * ul + nx * pl; fl[3] = rol * unl * vl + ny * pl;
    fr[0] = ror * hr * unr; fr[1] = ror * unr; fr[2] = ror * unr * ur + nx * pr; fr[3] = ror * unr * vr + ny * pr;
    ql = prim2con(G, ql);
    qr = prim2con(G, qr);
    R eigen = rmax(fabs(unl) + cl, fabs(unr) + cr);
    for (int i = 0; i < 4; ++i) {
        R f = fl[i] + fr[i];
        f = f + eigen * (ql[i] - qr[i]);
        flux[i] = R(0.5) * area * f;
    }
}

// van Leer flux-vector splitting per unit face length
// (CCFVM/vanleer_flux.F90:1-101, NCFVM/vanleer_flux.f90:2-118).
template <class R>
__device__ __forceinline__ void vanleer_core(R G, R G1, R nx, R ny, const V4<R>& ql, const V4<R>& qr, V4<R>& flux,
                                             R& hl_o, R& hr_o) {
    R rl = ql[0], ul = ql[1], vl = ql[2], pl = ql[3];
    R unl = ul * nx + vl * ny;
    R ql2 = ul * ul + vl * vl;
    R al2 = G * pl / rl;
    R hl = al2 / G1 + R(0.5) * ql2;
    R cl = sqrt(al2);
    R ml = unl / cl;
    R rr = qr[0], ur = qr[1], vr = qr[2], pr = qr[3];
    R unr = ur * nx + vr * ny;
    R qr2 = ur * ur + vr * vr;
    R ar2 = G * pr / rr;
    R hr = ar2 / G1 + R(0.5) * qr2;
    R cr = sqrt(ar2);
    R mr = unr / cr;
    const R zero = R(0);
    R plp = p5p(ml, zero), prm = p5m(mr, zero);
    R mlp = m4p(ml, zero), mlm = m4m(ml, zero), mrp = m4p(mr, zero), mrm = m4m(mr, zero);
    R p12 = plp * pl + prm * pr;
    R fmass_p = rl * cl * mlp;
    R fmass_m = rr * cr * mrm;
    R fmass12 = fmass_p + fmass_m;
    R delta = -(G * (cr * mrp * mrm * pr - cl * mlp * mlm * pl) / (G - R(1)));
    R dissi = fmass_p - fmass_m;
    R fL[4] = {hl, R(1), ul, vl}, fR[4] = {hr, R(1), ur, vr};
    R fP[4] = {delta, R(0), nx * p12, ny * p12};
    for (int i = 0; i < 4; ++i)
        flux[i] = R(0.5) * fmass12 * (fL[i] + fR[i]) - R(0.5) * dissi * (fR[i] - fL[i]) + fP[i];
    hl_o = hl;
    hr_o = hr;
}

// AUSM+-up per |n| of the given normal (CCFVM/ausm_up_flux.F90:2-162); the
// caller multiplies by the face length where the formulation needs it.
template <class R>
__device__ __forceinline__ void ausm_core(R G, R G1, R nx, R ny, R mref, const V4<R>& ql, const V4<R>& qr, V4<R>& flux,
                                          R& hl_o, R& hr_o) {
    const R sigma = R(1), ku = R(0.75), kp = R(0.25);
    R rl = ql[0], ul = ql[1], vl = ql[2], pl = ql[3];
    R unl = ul * nx + vl * ny;
    R ql2 = ul * ul + vl * vl;
    R al2 = G * pl / rl;
    R hl = al2 / G1 + R(0.5) * ql2;
    R rr = qr[0], ur = qr[1], vr = qr[2], pr = qr[3];
    R unr = ur * nx + vr * ny;
    R qr2 = ur * ur + vr * vr;
    R ar2 = G * pr / rr;
    R hr = ar2 / G1 + R(0.5) * qr2;
    R aL_star = sqrt(R(2) * (G - R(1)) * hl / (G + R(1)));
    R aR_star = sqrt(R(2) * (G - R(1)) * hr / (G + R(1)));
    R aL_hat = aL_star * aL_star / rmax(aL_star, fabs(unl));
    R aR_hat = aR_star * aR_star / rmax(aR_star, R(-1) * fabs(unr));
    R c12 = rmin(aL_hat, aR_hat);
    R ml = unl / c12, mr = unr / c12;
    R mbar2 = R(0.5) * (unl * unl + unr * unr) / (c12 * c12);
    R fa;
    if (mbar2 >= R(1)) {
        fa = R(1);
    } else {
        R mstar2 = rmin(R(1), rmax(mbar2, mref * mref));
        R Mo = mstar2;
        fa = Mo * (R(2) - Mo);
    }
    R beta = R(1) / R(8);
    R alpha = R(3) / R(16) * (R(-4) + R(5) * fa * fa);
    R plp = p5p(ml, alpha), prm = p5m(mr, alpha);
    R mlp = m4p(ml, beta), mrm = m4m(mr, beta);
    R ro12 = R(0.5) * (rl + rr);
    R mp = -((kp / fa) * rmax((R(1) - sigma * mbar2), R(0)) * (pr - pl) / (ro12 * c12 * c12));
    R m12 = mlp + mrm + mp;
    R pu = -(ku * plp * prm * R(2) * ro12 * fa * c12 * (unr - unl));
    R p12 = plp * pl + prm * pr + pu;
    R fl[4] = {hl, R(1), ul, vl}, fr[4] = {hr, R(1), ur, vr};
    R a = m1p(m12) * rl, b = m1m(m12) * rr;
    for (int i = 0; i < 4; ++i) flux[i] = c12 * (a * fl[i] + b * fr[i]);
    flux[2] = flux[2] + nx * p12;
    flux[3] = flux[3] + ny * p12;
    hl_o = hl;
    hr_o = hr;
}

// Riemann-invariant farfield state (CCFVM/boundCond.F90:112-209).
template <class R>
__device__ __forceinline__ V4<R> farfield_state(R G, R G1, R nx, R ny, R rinf, R uinf, R vinf, R pinf, const V4<R>& ql) {
    R tx = -ny, ty = nx;
    R ainf = sqrt(G * pinf / rinf);
    R rho = ql[0], u = ql[1], v = ql[2], p = ql[3];
    R a = sqrt(G * p / rho);
    R un = u * nx + v * ny;
    R tn = u * tx + v * ty;
    V4<R> qb = {rinf, uinf, vinf, pinf};
    R mach = un / a;
    if (mach >= R(1)) {
        qb[0] = rho; qb[1] = un * nx + tn * tx; qb[2] = un * ny + tn * ty; qb[3] = p;
    } else if (R(0) <= mach && mach < R(1)) {
        R Vninf = uinf * nx + vinf * ny;
        R Rp = un + R(2) * a / G1;
        R Rm = Vninf - R(2) * ainf / G1;
        R Sb = p / pow(rho, G);
        R Vnrm = R(0.5) * (Rp + Rm);
        qb[1] = Vnrm * nx + tn * tx; qb[2] = Vnrm * ny + tn * ty;
        R ab = R(0.25) * (Rp - Rm) * G1;
        qb[0] = pow(ab * ab / G / Sb, R(1) / G1);
        qb[3] = qb[0] * ab * ab / G;
    } else if (R(-1) < mach && mach < R(0)) {
        R Vninf = uinf * nx + vinf * ny;
        R Vtinf = uinf * tx + vinf * ty;
        R Rp = un + R(2) * a / G1;
        R Rm = Vninf - R(2) * ainf / G1;
        R Sb = pinf / pow(rinf, G);
        R Vnrm = R(0.5) * (Rp + Rm);
        qb[1] = Vnrm * nx + Vtinf * tx; qb[2] = Vnrm * ny + Vtinf * ty;
        R ab = R(0.25) * (Rp - Rm) * G1;
        qb[0] = pow(ab * ab / G / Sb, R(1) / G1);
        qb[3] = qb[0] * ab * ab / G;
    }
    return qb;
}

// con2prim on any arithmetic type: the operations of con2prim above, so the
// double instantiation rounds identically.
template <class S>
struct PrimT {
    S rho, u, v, e, p, t;
};
template <class S>
__device__ __forceinline__ PrimT<S> con2prim_t(const Gas& g, S E, S r, S ru, S rv) {
    PrimT<S> o;
    o.rho = r;
    o.u = ru / r;
    o.v = rv / r;
    o.e = E / o.rho;
    S q = o.u * o.u + o.v * o.v;
    o.p = (g.gamma - 1.0) * (E - 0.5 * o.rho * q);
    o.t = o.p / (o.rho * g.znd);
    return o;
}

// Conversion between the boundary-state and flux arithmetic types (identity
// when they agree, a rounding cast between double and float).
template <class To, class From>
struct Cvt {
    __device__ __forceinline__ static To f(From x) { return (To)x; }
};
template <class T>
struct Cvt<T, T> {
    __device__ __forceinline__ static T f(T x) { return x; }
};

// Convective flux of the selected scheme (fvresidual.F90 flux selection).
template <class R>
__device__ __forceinline__ bool face_flux(const Gas& g, R nx, R ny, R area, V4<R>& ql, V4<R>& qr, V4<R>& F) {
    const R G = (R)g.gamma, G1 = (R)g.gamma1;
    bool ok = true;
    R hl, hr;
    switch (g.flux) {
        case UNS_FLUX_ROE: ok = roe_flux<R>(G, G1, nx, ny, area, ql, qr, F); break;
        case UNS_FLUX_RUSANOV: rusanov_flux<R>(G, G1, nx, ny, area, ql, qr, F); break;
        case UNS_FLUX_VANLEER:
            vanleer_core<R>(G, G1, nx, ny, ql, qr, F, hl, hr);
            for (int k = 0; k < 4; ++k) F[k] = F[k] * area;
            break;
        default: {  // AUSM+-up: the reference scales by |n| of the unit normal
            ausm_core<R>(G, G1, nx, ny, (R)g.mref, ql, qr, F, hl, hr);
            R an = sqrt(nx * nx + ny * ny);
            for (int k = 0; k < 4; ++k) F[k] = F[k] * an;
        }
    }
    return ok;
}

// One CCFVM boundary face (fvresidual.F90:27-100): the ghost state of the
// farfield (farfield_flux, boundCond.F90:112-209) or wall (slip_wall
// :46-81, NoSlip_wall :2-37) and the face flux between the reconstructed
// interior state qcl and that ghost.  S is the arithmetic of the states, R of
// the flux.  The wall ghost reads the current conserved state cin of the
// interior cell; the farfield ghost depends on uinf, vinf (the angle of
// attack).  Other bc values carry no flux (F = 0) and no ghost update (upd).
template <class S>
struct CCBnd {
    V4<S> F, gq, gp;
    S gT;
    bool ok, upd;
};
// N is the type of the face geometry: double, or a tangent type when the
// adjoint differentiates the closure with respect to the normal and length.
template <class S, class R, class N = double>
__device__ __forceinline__ CCBnd<S> cc_boundary(const Gas& g, int bc, N nx, N ny, N area,
                                                const V4<S>& qcl, const V4<S>& cin, S uinf, S vinf) {
    CCBnd<S> o;
    o.ok = true;
    o.upd = false;
    o.F = V4<S>{S(0.0), S(0.0), S(0.0), S(0.0)};
    o.gq = o.F;
    o.gp = o.F;
    o.gT = S(0.0);
    V4<R> ql, qr, F;
    if (bc == 2001) {
        V4<S> B = farfield_state<S>(S(g.gamma), S(g.gamma1), S(nx), S(ny), S(g.r_inf), uinf, vinf, S(g.p_inf), qcl);
        for (int j = 0; j < 4; ++j) { ql[j] = Cvt<R, S>::f(qcl[j]); qr[j] = Cvt<R, S>::f(B[j]); }
        o.ok = face_flux<R>(g, (R)nx, (R)ny, (R)area, ql, qr, F);
        for (int j = 0; j < 4; ++j) o.F[j] = Cvt<S, R>::f(F[j]);
        // Ghost state = prim2con of the right state the flux routine left
        // behind (Rusanov leaves it in conserved form, as in the reference).
        V4<S> R4 = B;
        if (g.flux == UNS_FLUX_RUSANOV)
            for (int j = 0; j < 4; ++j) R4[j] = Cvt<S, R>::f(qr[j]);
        o.gq = prim2con<S>(S(g.gamma), R4);
        PrimT<S> P = con2prim_t<S>(g, o.gq[0], o.gq[1], o.gq[2], o.gq[3]);
        o.gp = V4<S>{P.rho, P.u, P.v, P.p};
        o.gT = P.t;
        o.upd = true;
    } else if (bc == 1001) {
        PrimT<S> P = con2prim_t<S>(g, cin[0], cin[1], cin[2], cin[3]);
        if (g.flow == UNS_FLOW_INVISCID) {  // slip_wall (boundCond.F90:46-81)
            S un = P.u * nx + P.v * ny;
            o.gq = V4<S>{cin[0], cin[1], P.rho * P.u - 2.0 * un * nx, P.rho * P.v - 2.0 * un * ny};
            PrimT<S> Q = con2prim_t<S>(g, o.gq[0], o.gq[1], o.gq[2], o.gq[3]);
            o.gp = V4<S>{Q.rho, Q.u, Q.v, Q.p};
            o.gT = Q.t;
        } else if (g.iwall == 0) {  // isothermal NoSlip_wall (boundCond.F90:19-30)
            S tg = 2.0 * g.t_wall - P.t;
            if (tg <= S(0.0)) tg = S(0.01 * g.t_wall);
            S rhog = P.p / (P.rho * g.znd);
            o.gp = V4<S>{rhog, -P.u, -P.v, P.p};
            o.gT = tg;
            o.gq = prim2con<S>(S(g.gamma), o.gp);
        } else {  // adiabatic NoSlip_wall (boundCond.F90:31-37)
            o.gq = V4<S>{cin[0], cin[1], -cin[2], -cin[3]};
            PrimT<S> Q = con2prim_t<S>(g, o.gq[0], o.gq[1], o.gq[2], o.gq[3]);
            o.gp = V4<S>{Q.rho, Q.u, Q.v, Q.p};
            o.gT = Q.t;
        }
        for (int j = 0; j < 4; ++j) { ql[j] = Cvt<R, S>::f(qcl[j]); qr[j] = Cvt<R, S>::f(o.gp[j]); }
        o.ok = face_flux<R>(g, (R)nx, (R)ny, (R)area, ql, qr, F);
        for (int j = 0; j < 4; ++j) o.F[j] = Cvt<S, R>::f(F[j]);
        o.upd = true;
    }
    return o;
}

// Venkatakrishnan limiter function (CCFVM/limiter.F90:286-294): its
// numerator and denominator, and their quotient.
__device__ __forceinline__ void vk_terms(double a, double b, double tol, double& nr, double& dr) {
    nr = a * a + 2.0 * a * b + tol * tol;
    dr = a * a + 2.0 * b * b + a * b + tol * tol;
}
__device__ __forceinline__ double vk_limit(double a, double b, double tol) {
    double nr, dr;
    vk_terms(a, b, tol, nr, dr);
    return nr / dr;
}

// Exponent field of a double (integer pipe).
__device__ __forceinline__ int dexp_field(double x) { return (int)((__double_as_longlong(x) >> 52) & 0x7ff); }

// RN(a / b) given y = RN(1 / b), by Markstein's correction (P. Markstein,
// "Computation of elementary functions on the IBM RISC System/6000
// processor", IBM J. Res. Develop. 34(1), 1990): with q0 = RN(a y) (within
// one ulp of a/b) the remainder r = a - b q0 is exact in one FMA, and
// RN(q0 + r y) is the correctly rounded quotient.  The theorem assumes no
// overflow or underflow, so operands and results outside a margin of the
// normal range (and subnormals) take the IEEE division instead; for a zero
// numerator the quotient is q0 itself (the corrected sum would turn -0 into
// +0).  One IEEE division per distinct divisor, then three FP64 operations
// per quotient.
__device__ __forceinline__ double div_rn_recip(double a, double b, double y) {
    const double q0 = a * y;
    const bool zero = (__double_as_longlong(a) & 0x7fffffffffffffffLL) == 0;
    if (zero) return q0;
    const double r = __fma_rn(-q0, b, a);
    const double q1 = __fma_rn(r, y, q0);
    const int ea = dexp_field(a), eq = dexp_field(q1);
    if (ea < 128 || ea > 1920 || eq < 128 || eq > 1920) return a / b;
    return q1;
}

// Whether n1/d1 < n2/d2 exactly (d1, d2 > 0, all finite and normal, the
// cross products inside the normal range): n1 d2 and n2 d1 as exact
// double-double values (product and its FMA error term) compared.  The
// minimum of correctly rounded quotients is the correctly rounded quotient
// of the exact minimum (rounding is monotonic), so one division of the
// selected pair gives min_k RN(n_k / d_k).
__device__ __forceinline__ bool ratio_less(double n1, double d1, double n2, double d2) {
    const double p1 = n1 * d2, p2 = n2 * d1;
    if (p1 != p2) return p1 < p2;
    return __fma_rn(n1, d2, -p1) < __fma_rn(n2, d1, -p2);
}

// Whether the ratio test above is exact for these operands: d positive,
// both with binary exponents within [-463, 457] (n may be zero), so that
// every cross product and its error term stay normal.
__device__ __forceinline__ bool ratio_ok(double n, double d) {
    const int en = dexp_field(n), ed = dexp_field(d);
    const bool nz = (__double_as_longlong(n) & 0x7fffffffffffffffLL) == 0;
    return (nz || (en >= 560 && en <= 1480)) && ed >= 560 && ed <= 1480 && d > 0.0;
}

// Order-preserving 64-bit encoding of a double for atomicMax/atomicMin.
__device__ __forceinline__ unsigned long long enc_ord(double x) {
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    return (b & 0x8000000000000000ULL) ? ~b : (b | 0x8000000000000000ULL);
}
__host__ __device__ __forceinline__ double dec_ord(unsigned long long e) {
    unsigned long long b = (e & 0x8000000000000000ULL) ? (e & 0x7FFFFFFFFFFFFFFFULL) : ~e;
    double d;
    memcpy(&d, &b, 8);
    return d;
}

}  // namespace uns
