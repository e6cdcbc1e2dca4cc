// oracle_cc.cpp -- TEST INFRASTRUCTURE ONLY.  CPU oracle, cell-centred solver.
//
// Serial restatement of the CCFVM residual-and-update path.  Every routine
// keeps the reference's loop structure (face loops scattering into cells) and
// its expression order, and cites the Fortran it follows.  Compiled with
// -ffp-contract=off so no fused multiply-add changes the rounding.
//
// PARITY UNPINNED: no golden vectors exist for the reference and it cannot be
// built here; see oracle.h.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "oracle.h"

namespace {

struct Prim {  // the `pri` module globals set by con2prim (types/pri.F90:13-37)
    double rho, u, v, e, q, p, h, a, t, znd;
};

struct CC {
    // mesh
    int nop, noc, nfi, nbf, nof, ntot;
    std::vector<double> px, py, cx, cy, cv, cov;
    std::vector<int> fp1, fp2, fin, fout, fbc;
    std::vector<double> fnx, fny, farea, fcx, fcy;
    std::vector<double> r11, r12, r22;
    std::vector<int> nc2c, c2f_off, c2f, v2c_off, v2c;
    std::vector<double> v2c_wt;
    uns_params P;
    // constants (math, initialize)
    double gamma, gamma1, pi;
    double q_inf, aoa, p_inf, r_inf, ent_inf, a_inf, u_inf, v_inf, T_inf, T_infd, SCONST, t_wall;
    double qinf[4], fs_inf[4];
    const double prandtl = 0.72;
    // state
    std::vector<double> qc, qp, qold, res, grad, phi, dt, la, mul;
    std::vector<double> ptprim, ptmu;
    std::vector<double> fqp, fla, fmu, fgrad;
    double Fx1 = 0.0, Fy1 = 0.0, cfl = 0.0;
    int err = 0;

    void con2prim(const double* qt, Prim& r) const {
        r.rho = qt[1];
        r.u = qt[2] / qt[1];
        r.v = qt[3] / qt[1];
        double Et = qt[0];
        r.e = Et / r.rho;
        r.q = r.u * r.u + r.v * r.v;
        r.p = (gamma - 1.0) * (Et - 0.5 * r.rho * r.q);
        r.h = (Et + r.p) / r.rho;
        r.a = std::sqrt(gamma * r.p / r.rho);
        r.znd = 1.0 / (gamma * P.m_inf * P.m_inf);
        r.t = r.p / (r.rho * r.znd);
    }
    // prim2con (types/pri.F90:39-57)
    void prim2con(const double* pr, double* conv) const {
        double rho = pr[0], u = pr[1], v = pr[2], p = pr[3];
        conv[0] = p / (gamma - 1.0) + 0.5 * rho * (u * u + v * v);
        conv[1] = rho;
        conv[2] = rho * u;
        conv[3] = rho * v;
    }
    double* QC(int i) { return &qc[(size_t)i * 4]; }
    double* QP(int i) { return &qp[(size_t)i * 5]; }
    double* G(int i, int var) { return &grad[(size_t)i * 10 + var * 2]; }
    double* FG(int f, int var) { return &fgrad[(size_t)f * 10 + var * 2]; }
};

// ------------------------------------------------------------- Mach polynomials
// CCFVM/solution.F90:478-572
double m1p(double m) { return 0.50 * (m + std::fabs(m)); }
double m1m(double m) { return 0.5 * (m - std::fabs(m)); }
double m2p(double m) { return 0.25 * (m + 1.0) * (m + 1.0); }
double m2m(double m) { return -0.25 * (m - 1.0) * (m - 1.0); }
double m4p(double m, double beta) {
    if (std::fabs(m) >= 1.0) return 0.5 * (m + std::fabs(m));
    return m2p(m) * (1.0 - 16.0 * beta * m2m(m));
}
double m4m(double m, double beta) {
    if (std::fabs(m) >= 1.0) return 0.5 * (m - std::fabs(m));
    return m2m(m) * (1.0 + 16.0 * beta * m2p(m));
}
double p5p(double m, double alpha) {
    if (std::fabs(m) >= 1.0) return 0.5 * (m + std::fabs(m)) / m;
    return m2p(m) * ((2.0 - m) - 16.0 * alpha * m * m2m(m));
}
double p5m(double m, double alpha) {
    if (std::fabs(m) >= 1.0) return 0.5 * (m - std::fabs(m)) / m;
    return m2m(m) * ((-2.0 - m) + 16.0 * alpha * m * m2p(m));
}

// ------------------------------------------------------------- fluxes
// roe_flux (CCFVM/roe_flux.F90:1-155)
int roe_flux(const CC& s, int ie, const double* ql, const double* qr, double* flux) {
    const double G = s.gamma, G1 = s.gamma1;
    double nx = s.fnx[ie], ny = s.fny[ie], area = s.farea[ie];
    double rl = ql[0], ul = ql[1], vl = ql[2], pl = ql[3];
    double rr = qr[0], ur = qr[1], vr = qr[2], pr = qr[3];
    double ql2 = ul * ul + vl * vl;
    double al2 = G * pl / rl;
    double hl = al2 / G1 + 0.5 * ql2;
    double qr2 = ur * ur + vr * vr;
    double ar2 = G * pr / rr;
    double hr = ar2 / G1 + 0.5 * qr2;
    double unl = ul * nx + vl * ny;
    double unr = ur * nx + vr * ny;
    double fc[4];
    fc[0] = rl * hl * unl + rr * hr * unr;
    fc[1] = rl * unl + rr * unr;
    fc[2] = pl * nx + rl * ul * unl + pr * nx + rr * ur * unr;
    fc[3] = pl * ny + rl * vl * unl + pr * ny + rr * vr * unr;
    double rl12 = std::sqrt(rl), rr12 = std::sqrt(rr);
    double rd = 1.0 / (rl12 + rr12);
    double ua = (ul * rl12 + ur * rr12) * rd;
    double va = (vl * rl12 + vr * rr12) * rd;
    double ha = (hl * rl12 + hr * rr12) * rd;
    double qa2 = ua * ua + va * va;
    double aa2 = G1 * (ha - 0.5 * qa2);
    if (aa2 <= 0.0) return UNS_ERR_NEG_SOUND_SPEED;
    double aa = std::sqrt(aa2);
    double una = ua * nx + va * ny;
    double vna = -ua * ny + va * nx;
    double e1 = std::fabs(una - aa), e2 = std::fabs(una), e4 = std::fabs(una + aa);
    const double ETOL = 0.1;
    double del = ETOL * aa;
    double l1, l2, l3, l4;
    if (e1 < del) l1 = 0.5 * (del + e1 * e1 / del); else l1 = e1;
    if (e2 < del) { l2 = 0.5 * (del + e2 * e2 / del); l3 = l2; } else { l2 = e2; l3 = l2; }
    if (e4 < del) l4 = 0.5 * (del + e4 * e4 / del); else l4 = e4;
    double du1 = rr - rl;
    double du2 = rr * ur - rl * ul;
    double du3 = rr * vr - rl * vl;
    double du4 = (rr * hr - pr) - (rl * hl - pl);
    double m1 = (nx * du2 + ny * du3 - una * du1) / aa;
    double m2 = G1 * (du4 - ua * du2 - va * du3 + qa2 * du1) / (aa * aa);
    double a1 = 0.5 * (m2 - m1);
    double a2 = (ny * du2 - nx * du3 + vna * du1) / aa;
    double a4 = 0.5 * (m1 + m2);
    double a3 = du1 - a1 - a4;
    double a1l1 = a1 * l1, a2l2 = a2 * l2, a3l3 = a3 * l3, a4l4 = a4 * l4;
    double aact = aa * nx, aast = aa * ny;
    double Fd[4];
    Fd[0] = a1l1 * (ha - una * aa) + a2l2 * aa * vna + a3l3 * 0.5 * qa2 + a4l4 * (ha + una * aa);
    Fd[1] = a1l1 + a3l3 + a4l4;
    Fd[2] = a1l1 * (ua - aact) + a2l2 * aa * ny + a3l3 * ua + a4l4 * (ua + aact);
    Fd[3] = a1l1 * (va - aast) - a2l2 * aa * nx + a3l3 * va + a4l4 * (va + aast);
    for (int i = 0; i < 4; ++i) flux[i] = 0.5 * area * (fc[i] - Fd[i]);
    return UNS_OK;
}

// rusanov_flux (CCFVM/rusanov_flux.F90:1-77).  Like the reference it
// overwrites its two state arguments with their conserved form.
int rusanov_flux(const CC& s, int ie, double* qcl, double* qcr, double* flux) {
    const double G = s.gamma, G1 = s.gamma1;
    double nx = s.fnx[ie], ny = s.fny[ie], area = s.farea[ie];
    double rol = qcl[0], ul = qcl[1], vl = qcl[2], pl = qcl[3];
    double ql2 = ul * ul + vl * vl;
    double al2 = G * pl / rol;
    double hl = al2 / G1 + 0.5 * ql2;
    double cl = std::sqrt(G * pl / rol);
    double ror = qcr[0], ur = qcr[1], vr = qcr[2], pr = qcr[3];
    double qr2 = ur * ur + vr * vr;
    double ar2 = G * pr / ror;
    double hr = ar2 / G1 + 0.5 * qr2;
    double cr = std::sqrt(G * pr / ror);
    double unl = ul * nx + vl * ny;
    double unr = ur * nx + vr * ny;
    double fl[4], fr[4];
    fl[0] = rol * hl * unl; fl[1] = rol * unl; fl[2] = rol * unl * ul + nx * pl; fl[3] = rol * unl * vl + ny * pl;
    fr[0] = ror * hr * unr; fr[1] = ror * unr; fr[2] = ror * unr * ur + nx * pr; fr[3] = ror * unr * vr + ny * pr;
    double conv[4];
    s.prim2con(qcl, conv); for (int i = 0; i < 4; ++i) qcl[i] = conv[i];
    s.prim2con(qcr, conv); for (int i = 0; i < 4; ++i) qcr[i] = conv[i];
    double eigen = std::max(std::fabs(unl) + cl, std::fabs(unr) + cr);
    for (int i = 0; i < 4; ++i) {
        double f = fl[i] + fr[i];
        f = f + eigen * (qcl[i] - qcr[i]);
        flux[i] = 0.5 * area * f;
    }
    return UNS_OK;
}

// vanleer_flux (CCFVM/vanleer_flux.F90:1-101)
void vanleer_core(double G, double G1, double nx, double ny, const double* ql, const double* qr, double* flux) {
    double rl = ql[0], ul = ql[1], vl = ql[2], pl = ql[3];
    double unl = ul * nx + vl * ny;
    double ql2 = ul * ul + vl * vl;
    double al2 = G * pl / rl;
    double hl = al2 / G1 + 0.5 * ql2;
    double cl = std::sqrt(al2);
    double ml = unl / cl;
    double rr = qr[0], ur = qr[1], vr = qr[2], pr = qr[3];
    double unr = ur * nx + vr * ny;
    double qr2 = ur * ur + vr * vr;
    double ar2 = G * pr / rr;
    double hr = ar2 / G1 + 0.5 * qr2;
    double cr = std::sqrt(ar2);
    double mr = unr / cr;
    double beta = 0.0, alpha = 0.0;
    double plp = p5p(ml, alpha), prm = p5m(mr, alpha);
    double mlp = m4p(ml, beta), mlm = m4m(ml, beta), mrp = m4p(mr, beta), mrm = m4m(mr, beta);
    double p12 = plp * pl + prm * pr;
    double fmass_p = rl * cl * mlp;
    double fmass_m = rr * cr * mrm;
    double fmass12 = fmass_p + fmass_m;
    double delta = -(G * (cr * mrp * mrm * pr - cl * mlp * mlm * pl) / (G - 1.0));
    double dissi = fmass_p - fmass_m;
    double fL[4] = {hl, 1.0, ul, vl}, fR[4] = {hr, 1.0, ur, vr};
    double fP[4] = {delta, 0.0, nx * p12, ny * p12};
    for (int i = 0; i < 4; ++i)
        flux[i] = 0.5 * fmass12 * (fL[i] + fR[i]) - 0.5 * dissi * (fR[i] - fL[i]) + fP[i];
}

int vanleer_flux(const CC& s, int ie, const double* ql, const double* qr, double* flux) {
    vanleer_core(s.gamma, s.gamma1, s.fnx[ie], s.fny[ie], ql, qr, flux);
    double area = s.farea[ie];
    for (int i = 0; i < 4; ++i) flux[i] = flux[i] * area;
    return UNS_OK;
}

// ausmPlus_flux (CCFVM/ausm_up_flux.F90:2-162).  `area` is |n| of the unit
// normal, as in the reference.  0.32 is a default-real literal there.
int ausm_flux(const CC& s, int ie, const double* ql, const double* qr, double* flux) {
    const double G = s.gamma, G1 = s.gamma1;
    double sigma = 1.0, ku = 0.75, kp = 0.25;
    double nx = s.fnx[ie], ny = s.fny[ie];
    double area = std::sqrt(nx * nx + ny * ny);
    double rl = ql[0], ul = ql[1], vl = ql[2], pl = ql[3];
    double unl = ul * nx + vl * ny;
    double ql2 = ul * ul + vl * vl;
    double al2 = G * pl / rl;
    double hl = al2 / G1 + 0.5 * ql2;
    double rr = qr[0], ur = qr[1], vr = qr[2], pr = qr[3];
    double unr = ur * nx + vr * ny;
    double qr2 = ur * ur + vr * vr;
    double ar2 = G * pr / rr;
    double hr = ar2 / G1 + 0.5 * qr2;
    double aL_star = std::sqrt(2.0 * (G - 1.0) * hl / (G + 1.0));
    double aR_star = std::sqrt(2.0 * (G - 1.0) * hr / (G + 1.0));
    double aL_hat = aL_star * aL_star / std::max(aL_star, std::fabs(unl));
    double aR_hat = aR_star * aR_star / std::max(aR_star, -1.0 * std::fabs(unr));
    double c12 = std::min(aL_hat, aR_hat);
    double ml = unl / c12, mr = unr / c12;
    double mbar2 = 0.5 * (unl * unl + unr * unr) / (c12 * c12);
    double mref = std::max((double)0.32f, 0.5 * s.P.m_inf);
    double fa;
    if (mbar2 >= 1.0) fa = 1.0;
    else {
        double mstar2 = std::min(1.0, std::max(mbar2, mref * mref));
        double Mo = mstar2;  // reference overwrites sqrt(mstar2) with mstar2
        fa = Mo * (2.0 - Mo);
    }
    double beta = 1.0 / 8.0;
    double alpha = 3.0 / 16.0 * (-4.0 + 5.0 * fa * fa);
    double plp = p5p(ml, alpha), prm = p5m(mr, alpha);
    double mlp = m4p(ml, beta), mrm = m4m(mr, beta);
    double ro12 = 0.5 * (rl + rr);
    double mp = -((kp / fa) * std::max((1.0 - sigma * mbar2), 0.0) * (pr - pl) / (ro12 * c12 * c12));
    double m12 = mlp + mrm + mp;
    double pu = -(ku * plp * prm * 2.0 * ro12 * fa * c12 * (unr - unl));
    double p12 = plp * pl + prm * pr + pu;
    double fl[4] = {hl, 1.0, ul, vl}, fr[4] = {hr, 1.0, ur, vr};
    double a = m1p(m12) * rl, b = m1m(m12) * rr;
    for (int i = 0; i < 4; ++i) flux[i] = c12 * (a * fl[i] + b * fr[i]);
    flux[2] = flux[2] + nx * p12;
    flux[3] = flux[3] + ny * p12;
    for (int i = 0; i < 4; ++i) flux[i] = flux[i] * area;
    return UNS_OK;
}

int face_flux(const CC& s, int ie, double* ql, double* qr, double* flux) {
    switch (s.P.flux_type) {
        case UNS_FLUX_ROE: return roe_flux(s, ie, ql, qr, flux);
        case UNS_FLUX_AUSM: return ausm_flux(s, ie, ql, qr, flux);
        case UNS_FLUX_VANLEER: return vanleer_flux(s, ie, ql, qr, flux);
        case UNS_FLUX_RUSANOV: return rusanov_flux(s, ie, ql, qr, flux);
    }
    return UNS_ERR_ARG;
}

// ------------------------------------------------------------- boundary states
// farfield_flux (CCFVM/boundCond.F90:112-209): Riemann-invariant boundary state.
void farfield_state(CC& s, int ie, const double* qcl, double* qcr) {
    const double G = s.gamma, G1 = s.gamma1;
    double nx = s.fnx[ie], ny = s.fny[ie];
    double tx = -ny, ty = nx;
    double rinf = s.r_inf, uinf = s.u_inf, vinf = s.v_inf, pinf = s.p_inf;
    double ainf = std::sqrt(G * pinf / rinf);
    double rho = qcl[0], u = qcl[1], v = qcl[2], p = qcl[3];
    double a = std::sqrt(G * p / rho);
    double un = u * nx + v * ny;
    double tn = u * tx + v * ty;
    double rhob = rinf, ub = uinf, vb = vinf, pb = pinf;
    double mach = un / a;
    if (mach >= 1.0) {
        double Vnrm = un, Vtan = tn;
        rhob = rho; ub = Vnrm * nx + Vtan * tx; vb = Vnrm * ny + Vtan * ty; pb = p;
    } else if (0.0 <= mach && mach < 1.0) {
        double Vninf = uinf * nx + vinf * ny;
        double Rp = un + 2.0 * a / G1;
        double Rm = Vninf - 2.0 * ainf / G1;
        double Sb = p / std::pow(rho, G);
        double Vnrm = 0.5 * (Rp + Rm), Vtan = tn;
        ub = Vnrm * nx + Vtan * tx; vb = Vnrm * ny + Vtan * ty;
        double ab = 0.25 * (Rp - Rm) * G1;
        rhob = std::pow(ab * ab / G / Sb, 1.0 / G1);
        pb = rhob * ab * ab / G;
    } else if (-1.0 < mach && mach < 0.0) {
        double Vninf = uinf * nx + vinf * ny;
        double Vtinf = uinf * tx + vinf * ty;
        double Rp = un + 2.0 * a / G1;
        double Rm = Vninf - 2.0 * ainf / G1;
        double Sb = pinf / std::pow(rinf, G);
        double Vnrm = 0.5 * (Rp + Rm), Vtan = Vtinf;
        ub = Vnrm * nx + Vtan * tx; vb = Vnrm * ny + Vtan * ty;
        double ab = 0.25 * (Rp - Rm) * G1;
        rhob = std::pow(ab * ab / G / Sb, 1.0 / G1);
        pb = rhob * ab * ab / G;
    } else if (-1.0 <= mach) {
        rhob = rinf; ub = uinf; vb = vinf; pb = pinf;
    }
    qcr[0] = rhob; qcr[1] = ub; qcr[2] = vb; qcr[3] = pb;
}

// slip_wall (CCFVM/boundCond.F90:46-81): ghost from the cell's current qc.
void slip_wall(CC& s, int ie) {
    int in = s.fin[ie], out = s.fout[ie];
    double nx = s.fnx[ie], ny = s.fny[ie];
    Prim r;
    s.con2prim(s.QC(in), r);
    double un = r.u * nx + r.v * ny;
    double* g = s.QC(out);
    const double* c = s.QC(in);
    g[0] = c[0]; g[1] = c[1];
    g[2] = r.rho * r.u - 2.0 * un * nx;
    g[3] = r.rho * r.v - 2.0 * un * ny;
    Prim gp;
    s.con2prim(g, gp);
    double* q = s.QP(out);
    q[0] = gp.rho; q[1] = gp.u; q[2] = gp.v; q[3] = gp.p; q[4] = gp.t;
}

// NoSlip_wall (CCFVM/boundCond.F90:2-43).
void noslip_wall(CC& s, int ie) {
    int in = s.fin[ie], out = s.fout[ie];
    Prim r;
    s.con2prim(s.QC(in), r);
    if (s.P.iwall == 0) {
        double tg = 2.0 * s.t_wall - r.t;
        if (tg <= 0.0) tg = 0.01 * s.t_wall;
        double rhog = r.p / (r.rho * r.znd);  // reference sets the ghost density to T
        double* q = s.QP(out);
        q[0] = rhog; q[1] = -r.u; q[2] = -r.v; q[3] = r.p; q[4] = tg;
        s.prim2con(q, s.QC(out));
    } else {
        double* g = s.QC(out);
        const double* c = s.QC(in);
        g[0] = c[0]; g[1] = c[1]; g[2] = -c[2]; g[3] = -c[3];
        Prim gp;
        s.con2prim(g, gp);
        double* q = s.QP(out);
        q[0] = gp.rho; q[1] = gp.u; q[2] = gp.v; q[3] = gp.p; q[4] = gp.t;
    }
}

// ------------------------------------------------------------- routines
void avg_c2v(CC& s) {  // average.F90:1-39 (no ghost-viscosity term read: mul=0 there)
    for (int i = 0; i < s.nop; ++i) {
        double wt = 0.0, con[6] = {0, 0, 0, 0, 0, 0};
        for (int k = s.v2c_off[i]; k < s.v2c_off[i + 1]; ++k) {
            int c = s.v2c[k];
            double cwt = s.v2c_wt[k];
            wt = wt + cwt;
            for (int j = 0; j < 5; ++j) con[j] = con[j] + s.qp[(size_t)c * 5 + j] * cwt;
            con[5] = con[5] + s.mul[c] * cwt;
        }
        for (int j = 0; j < 5; ++j) s.ptprim[(size_t)i * 5 + j] = con[j] / wt;
        s.ptmu[i] = con[5] / wt;
    }
    for (int f = 0; f < s.nof; ++f) {
        int p1 = s.fp1[f], p2 = s.fp2[f];
        for (int j = 0; j < 5; ++j)
            s.fqp[(size_t)f * 5 + j] = 0.5 * (s.ptprim[(size_t)p1 * 5 + j] + s.ptprim[(size_t)p2 * 5 + j]);
    }
}

double time_step02(CC& s, double cfl) {  // timestep.F90:28-107
    for (int i = 0; i < s.noc; ++i) s.la[i] = 0.0;
    double Kv = 0.25, vll = 0.0;
    if (s.P.flow_type != UNS_FLOW_INVISCID) vll = 2.0 * s.gamma / (s.prandtl * s.P.rey * Kv);
    for (int ie = 0; ie < s.nof; ++ie) {
        int in = s.fin[ie], out = s.fout[ie];
        double nx = s.fnx[ie], ny = s.fny[ie], area = s.farea[ie], mu = s.fmu[ie];
        const double* c = &s.fqp[(size_t)ie * 5];
        double r0 = c[0], u0 = c[1], v0 = c[2], p0 = c[3];
        double a0 = std::sqrt(s.gamma * p0 / r0);
        double un = u0 * nx + v0 * ny;
        double ll = area * (std::fabs(un) + a0);
        ll = ll + vll * mu / r0;
        s.fla[ie] = ll;
        s.la[in] = s.la[in] + ll;
        if (out < s.noc) s.la[out] = s.la[out] + ll;
    }
    double dtglobal = 1.0e20;
    for (int i = 0; i < s.noc; ++i) {
        double ll = s.la[i];
        s.dt[i] = cfl * s.cv[i] / ll;
        dtglobal = std::min(dtglobal, s.dt[i]);
    }
    return dtglobal;
}

double vk_limit(double a, double b, double tol) {  // limiter.F90:286-294
    double nr = a * a + 2.0 * a * b + tol * tol;
    double dr = a * a + 2.0 * b * b + a * b + tol * tol;
    return nr / dr;
}

void limiter_vkn1(CC& s) {  // limiter.F90:123-296
    const double kappa = 0.05;
    double qmax[4], qmin[4];
    for (int j = 0; j < 4; ++j) {
        qmax[j] = s.qp[j]; qmin[j] = s.qp[j];
        for (int c = 1; c < s.ntot; ++c) {
            qmax[j] = std::max(qmax[j], s.qp[(size_t)c * 5 + j]);
            qmin[j] = std::min(qmin[j], s.qp[(size_t)c * 5 + j]);
        }
    }
    std::vector<double> umax((size_t)s.noc * 4), umin((size_t)s.noc * 4), phi((size_t)s.noc * 4);
    for (int i = 0; i < s.noc; ++i)
        for (int j = 0; j < 4; ++j) {
            phi[i * 4 + j] = s.phi[i * 4 + j];
            umax[i * 4 + j] = s.qp[(size_t)i * 5 + j];
            umin[i * 4 + j] = s.qp[(size_t)i * 5 + j];
        }
    for (int f = 0; f < s.nfi; ++f) {
        int in = s.fin[f], out = s.fout[f];
        for (int j = 0; j < 4; ++j) {
            umax[in * 4 + j] = std::max(umax[in * 4 + j], s.qp[(size_t)out * 5 + j]);
            umin[in * 4 + j] = std::min(umin[in * 4 + j], s.qp[(size_t)out * 5 + j]);
            umax[out * 4 + j] = std::max(umax[out * 4 + j], s.qp[(size_t)in * 5 + j]);
            umin[out * 4 + j] = std::min(umin[out * 4 + j], s.qp[(size_t)in * 5 + j]);
        }
    }
    for (int f = s.nfi; f < s.nof; ++f) {
        int in = s.fin[f], p1 = s.fp1[f], p2 = s.fp2[f];
        for (int j = 0; j < 4; ++j) {
            double var = 0.5 * (s.ptprim[(size_t)p1 * 5 + j] + s.ptprim[(size_t)p2 * 5 + j]);
            umax[in * 4 + j] = std::max(umax[in * 4 + j], var);
            umin[in * 4 + j] = std::min(umin[in * 4 + j], var);
        }
    }
    auto side = [&](int c, int f, int j, double tol) {
        double d0 = s.fcx[f] - s.cx[c], d1 = s.fcy[f] - s.cy[c];
        double D_L = s.G(c, j)[0] * d0 + s.G(c, j)[1] * d1;
        double phi0 = 1.0;
        if (D_L > 0.0) phi0 = vk_limit(umax[c * 4 + j] - s.qp[(size_t)c * 5 + j], D_L, tol);
        else if (D_L < 0.0) phi0 = vk_limit(umin[c * 4 + j] - s.qp[(size_t)c * 5 + j], D_L, tol);
        phi[c * 4 + j] = std::min(phi[c * 4 + j], phi0);
    };
    for (int f = 0; f < s.nfi; ++f)
        for (int j = 0; j < 4; ++j) {
            double tol = kappa * (qmax[j] - qmin[j]);
            side(s.fin[f], f, j, tol);
            side(s.fout[f], f, j, tol);
        }
    for (int f = s.nfi; f < s.nof; ++f)
        for (int j = 0; j < 4; ++j) side(s.fin[f], f, j, kappa * (qmax[j] - qmin[j]));
    for (int i = 0; i < s.noc * 4; ++i) s.phi[i] = phi[i];
}

void gradient_gg(CC& s) {  // gradient.F90:386-447
    std::fill(s.grad.begin(), s.grad.end(), 0.0);
    for (int f = 0; f < s.nfi; ++f) {
        int in = s.fin[f], out = s.fout[f];
        double area = s.farea[f], dx = s.fnx[f] * area, dy = s.fny[f] * area;
        for (int j = 0; j < 5; ++j) {
            double var = s.fqp[(size_t)f * 5 + j];
            s.G(in, j)[0] = s.G(in, j)[0] + var * dx;
            s.G(in, j)[1] = s.G(in, j)[1] + var * dy;
            s.G(out, j)[0] = s.G(out, j)[0] - var * dx;
            s.G(out, j)[1] = s.G(out, j)[1] - var * dy;
        }
    }
    for (int f = s.nfi; f < s.nof; ++f) {
        int in = s.fin[f];
        double area = s.farea[f], dx = -s.fnx[f] * area, dy = -s.fny[f] * area;
        for (int j = 0; j < 5; ++j) {
            double var = s.fqp[(size_t)f * 5 + j];
            s.G(in, j)[0] = s.G(in, j)[0] + var * dx;
            s.G(in, j)[1] = s.G(in, j)[1] + var * dy;
        }
    }
    for (int i = 0; i < s.noc; ++i) {
        double var = s.cv[i];
        for (int j = 0; j < 5; ++j) { s.G(i, j)[0] = s.G(i, j)[0] / var; s.G(i, j)[1] = s.G(i, j)[1] / var; }
    }
}

// gradtrixy (gradient.F90:572-612)
bool gradtrixy(const double prim[3][5], const double xy[2][3], double g[5][2], double& tarea) {
    tarea = 0.0;
    for (int i = 0; i < 3; ++i) {
        int ip1 = (i == 2) ? 0 : i + 1;
        double dx = 0.5 * (xy[0][ip1] + xy[0][i]);
        double dy = xy[1][ip1] - xy[1][i];
        tarea = tarea + dx * dy;
    }
    if (tarea <= 0.0) return false;
    for (int v = 0; v < 5; ++v) g[v][0] = g[v][1] = 0.0;
    for (int i = 0; i < 3; ++i) {
        int ip1 = (i == 2) ? 0 : i + 1;
        double dx = xy[1][ip1] - xy[1][i];
        double dy = -(xy[0][ip1] - xy[0][i]);
        for (int v = 0; v < 5; ++v) {
            double var = 0.5 * (prim[i][v] + prim[ip1][v]);
            g[v][0] = g[v][0] + var * dx;
            g[v][1] = g[v][1] + var * dy;
        }
    }
    for (int v = 0; v < 5; ++v) { g[v][0] = g[v][0] / tarea; g[v][1] = g[v][1] / tarea; }
    return true;
}

int gradient_ggfc(CC& s) {  // gradient.F90:450-614
    std::fill(s.grad.begin(), s.grad.end(), 0.0);
    std::fill(s.fgrad.begin(), s.fgrad.end(), 0.0);
    for (int f = 0; f < s.nof; ++f) {
        bool interior = f < s.nfi;
        int in = s.fin[f], out = s.fout[f], p1 = s.fp1[f], p2 = s.fp2[f];
        double prim[3][5], xy[2][3], g1[5][2], g2[5][2], a1, a2;
        xy[0][0] = s.px[p1]; xy[1][0] = s.py[p1];
        xy[0][1] = s.cx[out]; xy[1][1] = s.cy[out];
        xy[0][2] = s.px[p2]; xy[1][2] = s.py[p2];
        for (int v = 0; v < 5; ++v) {
            prim[0][v] = s.ptprim[(size_t)p1 * 5 + v];
            prim[1][v] = s.qp[(size_t)out * 5 + v];
            prim[2][v] = s.ptprim[(size_t)p2 * 5 + v];
        }
        if (!gradtrixy(prim, xy, g1, a1)) return UNS_ERR_MESH;
        xy[0][0] = s.px[p1]; xy[1][0] = s.py[p1];
        xy[0][1] = s.px[p2]; xy[1][1] = s.py[p2];
        xy[0][2] = s.cx[in]; xy[1][2] = s.cy[in];
        for (int v = 0; v < 5; ++v) {
            prim[0][v] = s.ptprim[(size_t)p1 * 5 + v];
            prim[1][v] = s.ptprim[(size_t)p2 * 5 + v];
            prim[2][v] = s.qp[(size_t)in * 5 + v];
        }
        if (!gradtrixy(prim, xy, g2, a2)) return UNS_ERR_MESH;
        for (int v = 0; v < 5; ++v) {
            s.FG(f, v)[0] = (a1 * g1[v][0] + a2 * g2[v][0]) / (a1 + a2);
            s.FG(f, v)[1] = (a1 * g1[v][1] + a2 * g2[v][1]) / (a1 + a2);
        }
        for (int v = 0; v < 5; ++v)
            for (int d = 0; d < 2; ++d) {
                s.G(in, v)[d] = s.G(in, v)[d] + s.FG(f, v)[d] * (a1 + a2);
                if (interior) s.G(out, v)[d] = s.G(out, v)[d] + s.FG(f, v)[d] * (a1 + a2);
            }
    }
    for (int i = 0; i < s.noc; ++i)
        for (int v = 0; v < 5; ++v) { s.G(i, v)[0] = s.G(i, v)[0] / s.cov[i]; s.G(i, v)[1] = s.G(i, v)[1] / s.cov[i]; }
    return UNS_OK;
}

void gradient_lsqr(CC& s) {  // gradient.F90:293-384
    std::fill(s.grad.begin(), s.grad.end(), 0.0);
    for (int f = 0; f < s.nfi; ++f) {
        int in = s.fin[f], out = s.fout[f];
        double xc = s.cx[in], yc = s.cy[in], xn = s.cx[out], yn = s.cy[out];
        double dx = xn - xc, dy = yn - yc;
        double r11 = s.r11[in], r12 = s.r12[in], r22 = s.r22[in];
        double alfa1 = dx / r11 / r11;
        double alfa2 = (dy - dx * r12 / r11) / (r22 * r22);
        double wx0 = alfa1 - alfa2 * r12 / r11, wy0 = alfa2;
        dx = xc - xn; dy = yc - yn;
        r11 = s.r11[out]; r12 = s.r12[out]; r22 = s.r22[out];
        alfa1 = dx / r11 / r11;
        alfa2 = (dy - dx * r12 / r11) / (r22 * r22);
        double wx1 = alfa1 - alfa2 * r12 / r11, wy1 = alfa2;
        for (int k = 0; k < 5; ++k) {
            double var = s.qp[(size_t)out * 5 + k] - s.qp[(size_t)in * 5 + k];
            s.G(in, k)[0] = s.G(in, k)[0] + var * wx0;
            s.G(in, k)[1] = s.G(in, k)[1] + var * wy0;
            s.G(out, k)[0] = s.G(out, k)[0] - var * wx1;
            s.G(out, k)[1] = s.G(out, k)[1] - var * wy1;
        }
    }
    for (int f = s.nfi; f < s.nof; ++f) {
        int in = s.fin[f], out = s.fout[f];
        double dx = s.cx[out] - s.cx[in], dy = s.cy[out] - s.cy[in];
        double r11 = s.r11[in], r12 = s.r12[in], r22 = s.r22[in];
        double alfa1 = dx / r11 / r11;
        double alfa2 = (dy - dx * r12 / r11) / r22 / r22;
        double wx0 = alfa1 - alfa2 * r12 / r11, wy0 = alfa2;
        for (int k = 0; k < 5; ++k) {
            double var = s.qp[(size_t)out * 5 + k] - s.qp[(size_t)in * 5 + k];
            s.G(in, k)[0] = s.G(in, k)[0] + var * wx0;
            s.G(in, k)[1] = s.G(in, k)[1] + var * wy0;
        }
    }
}

int gradient(CC& s) {
    int rc = UNS_OK;
    if (s.P.grad_type == UNS_GRAD_GG) gradient_gg(s);
    else if (s.P.grad_type == UNS_GRAD_GGFC) rc = gradient_ggfc(s);
    else if (s.P.grad_type == UNS_GRAD_LSQR) gradient_lsqr(s);
    else return UNS_ERR_ARG;
    if (rc) return rc;
    if (s.P.ilimit == 1) limiter_vkn1(s);
    return UNS_OK;
}

int viscous_flux(CC& s) {  // viscous_flux.F90:1-141
    if (s.P.grad_type != UNS_GRAD_GGFC) {
        int rc = gradient_ggfc(s);
        if (rc) return rc;
        if (s.P.ilimit == 1) limiter_vkn1(s);
    }
    for (int i = 0; i < s.noc; ++i) {
        Prim r;
        s.con2prim(s.QC(i), r);
        double num = 1.0 + s.T_infd / s.SCONST;
        double den = r.t + s.T_infd / s.SCONST;
        s.mul[i] = (num / den) * std::pow(r.t, 1.5);
    }
    const double two = 2.0, two_third = two / 3.0;
    for (int ie = 0; ie < s.nof; ++ie) {
        double flux[4] = {0, 0, 0, 0};
        double nx = s.fnx[ie], ny = s.fny[ie], area = s.farea[ie];
        int in = s.fin[ie], out = s.fout[ie], bc = s.fbc[ie];
        double mu = (out < s.noc) ? 0.5 * (s.mul[in] + s.mul[out]) : s.mul[in];
        s.fmu[ie] = mu;
        double uvel = s.fqp[(size_t)ie * 5 + 1], vvel = s.fqp[(size_t)ie * 5 + 2];
        double ux = s.FG(ie, 1)[0], uy = s.FG(ie, 1)[1], vx = s.FG(ie, 2)[0], vy = s.FG(ie, 2)[1];
        double tx = s.FG(ie, 4)[0], ty = s.FG(ie, 4)[1];
        double tauxx = two_third * (two * ux - vy);
        double tauxy = (uy + vx);
        double tauyy = two_third * (two * vy - ux);
        double factor = (s.gamma - 1.0) * s.P.m_inf * s.P.m_inf * s.prandtl;
        double qx = -(tx / factor), qy = -(ty / factor);
        double MubyRey = mu / s.P.rey;
        flux[0] = MubyRey * ((uvel * tauxx + vvel * tauxy - qx) * nx + (uvel * tauxy + vvel * tauyy - qy) * ny);
        flux[2] = MubyRey * (tauxx * nx + tauxy * ny);
        flux[3] = MubyRey * (tauxy * nx + tauyy * ny);
        for (int k = 0; k < 4; ++k) s.res[(size_t)in * 4 + k] = s.res[(size_t)in * 4 + k] - flux[k] * area;
        if (out < s.noc)
            for (int k = 0; k < 4; ++k) s.res[(size_t)out * 4 + k] = s.res[(size_t)out * 4 + k] + flux[k] * area;
        if (bc == 1001) { s.Fx1 = s.Fx1 - flux[2] * area; s.Fy1 = s.Fy1 - flux[3] * area; }
    }
    return UNS_OK;
}

void cirs(CC& s) {  // ImpResiSmoothening.F90:1-47
    double r = s.cfl / s.P.cfl_max;
    double epsirs = std::max(0.25 * (r * r - 1.0), 0.0);
    std::vector<double> old(s.res), itr((size_t)s.noc * 4);
    for (int it = 0; it < 2; ++it) {
        std::fill(itr.begin(), itr.end(), 0.0);
        for (int f = 0; f < s.nfi; ++f) {
            int in = s.fin[f], out = s.fout[f];
            for (int k = 0; k < 4; ++k) {
                itr[(size_t)in * 4 + k] = itr[(size_t)in * 4 + k] + s.res[(size_t)out * 4 + k];
                itr[(size_t)out * 4 + k] = itr[(size_t)out * 4 + k] + s.res[(size_t)in * 4 + k];
            }
        }
        for (int i = 0; i < s.noc; ++i) {
            double den = 1.0 / (1.0 + epsirs * (double)s.nc2c[i]);
            for (int k = 0; k < 4; ++k)
                s.res[(size_t)i * 4 + k] = (itr[(size_t)i * 4 + k] * epsirs + old[(size_t)i * 4 + k]) * den;
        }
    }
}

int fvresidual(CC& s) {  // fvresidual.F90:4-187
    std::fill(s.res.begin(), s.res.end(), 0.0);
    s.Fx1 = 0.0; s.Fy1 = 0.0;
    int rc;
    for (int ie = s.nfi; ie < s.nof; ++ie) {
        int in = s.fin[ie], out = s.fout[ie];
        double qcl[4] = {0, 0, 0, 0}, qcr[4] = {0, 0, 0, 0}, flux[4];
        double d0 = s.fcx[ie] - s.cx[in], d1 = s.fcy[ie] - s.cy[in];
        if (s.fbc[ie] == 2001) {
            for (int i = 0; i < 4; ++i) {
                double ph = s.phi[(size_t)in * 4 + i];
                qcl[i] = s.qp[(size_t)in * 5 + i] + ph * (s.G(in, i)[0] * d0 + s.G(in, i)[1] * d1);
            }
            farfield_state(s, ie, qcl, qcr);
            if ((rc = face_flux(s, ie, qcl, qcr, flux))) return rc;
            for (int k = 0; k < 4; ++k) s.res[(size_t)in * 4 + k] = s.res[(size_t)in * 4 + k] + flux[k];
            double conv[4];
            s.prim2con(qcr, conv);
            for (int k = 0; k < 4; ++k) s.QC(out)[k] = conv[k];
            Prim gp;
            s.con2prim(conv, gp);
            double* q = s.QP(out);
            q[0] = gp.rho; q[1] = gp.u; q[2] = gp.v; q[3] = gp.p; q[4] = gp.t;
        }
        if (s.fbc[ie] == 1001) {
            for (int i = 0; i < 4; ++i) {
                double ph = s.phi[(size_t)in * 4 + i];
                qcl[i] = s.qp[(size_t)in * 5 + i] + ph * (s.G(in, i)[0] * d0 + s.G(in, i)[1] * d1);
            }
            if (s.P.flow_type != UNS_FLOW_INVISCID) noslip_wall(s, ie); else slip_wall(s, ie);
            for (int k = 0; k < 4; ++k) qcr[k] = s.QP(out)[k];
            if ((rc = face_flux(s, ie, qcl, qcr, flux))) return rc;
            for (int k = 0; k < 4; ++k) s.res[(size_t)in * 4 + k] = s.res[(size_t)in * 4 + k] + flux[k];
            s.Fx1 = s.Fx1 + flux[2];
            s.Fy1 = s.Fy1 + flux[3];
        }
    }
    const double zhi = 1.0 / 3.0;
    for (int ie = 0; ie < s.nfi; ++ie) {
        int in = s.fin[ie], out = s.fout[ie];
        double qcl[4], qcr[4], flux[4];
        double dl0 = s.fcx[ie] - s.cx[in], dl1 = s.fcy[ie] - s.cy[in];
        double dr0 = s.fcx[ie] - s.cx[out], dr1 = s.fcy[ie] - s.cy[out];
        for (int i = 0; i < 4; ++i) {  // recon (fvresidual.F90:190-252)
            double ph = s.phi[(size_t)in * 4 + i];
            double alfa = s.G(in, i)[0] * dl0 + s.G(in, i)[1] * dl1;
            double beta = s.qp[(size_t)out * 5 + i] - s.qp[(size_t)in * 5 + i];
            qcl[i] = s.qp[(size_t)in * 5 + i] + 0.5 * ph * (zhi * beta + (1.0 - zhi) * alfa);
            ph = s.phi[(size_t)out * 4 + i];
            alfa = s.G(out, i)[0] * dr0 + s.G(out, i)[1] * dr1;
            beta = s.qp[(size_t)in * 5 + i] - s.qp[(size_t)out * 5 + i];
            qcr[i] = s.qp[(size_t)out * 5 + i] + 0.5 * ph * (zhi * beta + (1.0 - zhi) * alfa);
        }
        if ((rc = face_flux(s, ie, qcl, qcr, flux))) return rc;
        for (int k = 0; k < 4; ++k) {
            s.res[(size_t)in * 4 + k] = s.res[(size_t)in * 4 + k] + flux[k];
            s.res[(size_t)out * 4 + k] = s.res[(size_t)out * 4 + k] - flux[k];
        }
    }
    if (s.P.flow_type == UNS_FLOW_LAMINAR)
        if ((rc = viscous_flux(s))) return rc;
    if (s.P.irs == 1) cirs(s);
    return UNS_OK;
}

// lusgs2 (lusgs.F90:207-379)
int lusgs2(CC& s) {
    const double omega = 1.5;
    int rc = fvresidual(s);
    if (rc) return rc;
    std::vector<double> diag(s.noc), lower((size_t)s.noc * 4, 0.0), upper((size_t)s.noc * 4, 0.0);
    for (int it = 0; it < s.noc; ++it) diag[it] = s.cv[it] / s.dt[it] + 0.5 * omega * s.la[it];
    auto normal_flux = [&](int out, const double* dq, double nx, double ny, double area, double* flux) {
        double q[4];
        Prim r;
        double f1[4], f2[4];
        for (int k = 0; k < 4; ++k) q[k] = s.qold[(size_t)out * 4 + k];
        s.con2prim(q, r);
        double et = r.e * r.rho;
        double un = r.u * nx + r.v * ny;
        f1[0] = (et + r.p) * un; f1[1] = r.rho * un; f1[2] = f1[1] * r.u + r.p * nx; f1[3] = f1[1] * r.v + r.p * ny;
        for (int k = 0; k < 4; ++k) q[k] = s.qold[(size_t)out * 4 + k] + dq[k];
        s.con2prim(q, r);
        et = r.e * r.rho;
        un = r.u * nx + r.v * ny;
        f2[0] = (et + r.p) * un; f2[1] = r.rho * un; f2[2] = f2[1] * r.u + r.p * nx; f2[3] = f2[1] * r.v + r.p * ny;
        for (int k = 0; k < 4; ++k) flux[k] = area * (f2[k] - f1[k]);
    };
    for (int it = 0; it < s.noc; ++it) {
        double cres[4] = {0, 0, 0, 0};
        for (int k = s.c2f_off[it]; k < s.c2f_off[it + 1]; ++k) {
            int c = s.c2f[k];
            double nx = s.fnx[c], ny = s.fny[c], area = s.farea[c];
            int in = s.fin[c], out = s.fout[c];
            if (out == it) { out = in; nx = -s.fnx[c]; ny = -s.fny[c]; }
            if (out < it && out >= 0 && out < s.noc) {
                double dflux[4];
                normal_flux(out, &lower[(size_t)out * 4], nx, ny, area, dflux);
                double lam = s.fla[c];
                for (int iv = 0; iv < 4; ++iv) cres[iv] = cres[iv] + (dflux[iv] - omega * lam * lower[(size_t)out * 4 + iv]);
            }
        }
        for (int iv = 0; iv < 4; ++iv) lower[(size_t)it * 4 + iv] = (-s.res[(size_t)it * 4 + iv] - 0.5 * cres[iv]) / diag[it];
    }
    for (int it = s.noc - 1; it >= 0; --it) {
        double cres[4] = {0, 0, 0, 0};
        for (int k = s.c2f_off[it]; k < s.c2f_off[it + 1]; ++k) {
            int c = s.c2f[k];
            double nx = s.fnx[c], ny = s.fny[c], area = s.farea[c];
            int in = s.fin[c], out = s.fout[c];
            if (out == it) { out = in; nx = -s.fnx[c]; ny = -s.fny[c]; }
            if (out > it && out >= 0 && out < s.noc) {
                double dflux[4];
                normal_flux(out, &upper[(size_t)out * 4], nx, ny, area, dflux);
                double lam = s.fla[c];
                for (int iv = 0; iv < 4; ++iv) cres[iv] = cres[iv] + (dflux[iv] - omega * lam * upper[(size_t)out * 4 + iv]);
            }
        }
        for (int iv = 0; iv < 4; ++iv) upper[(size_t)it * 4 + iv] = lower[(size_t)it * 4 + iv] - 0.5 * cres[iv] / diag[it];
    }
    for (int it = 0; it < s.noc; ++it)
        for (int iv = 0; iv < 4; ++iv) s.qc[(size_t)it * 4 + iv] = s.qold[(size_t)it * 4 + iv] + upper[(size_t)it * 4 + iv];
    return UNS_OK;
}

}  // namespace

struct oracle_cc { CC s; };

extern "C" {

oracle_cc* oracle_cc_create(const uns_cc_mesh* m, const uns_params* p) {
    if (!m || !p) return nullptr;
    oracle_cc* o = new oracle_cc();
    CC& s = o->s;
    s.P = *p;
    s.nop = m->nop; s.noc = m->noc; s.nfi = m->nfi; s.nbf = m->nbf;
    s.nof = s.nfi + s.nbf; s.ntot = s.noc + s.nbf;
    s.px.assign(m->px, m->px + s.nop); s.py.assign(m->py, m->py + s.nop);
    s.cx.assign(m->cx, m->cx + s.ntot); s.cy.assign(m->cy, m->cy + s.ntot);
    s.cv.assign(m->cv, m->cv + s.noc); s.cov.assign(m->cov, m->cov + s.noc);
    s.fp1.assign(m->fp1, m->fp1 + s.nof); s.fp2.assign(m->fp2, m->fp2 + s.nof);
    s.fin.assign(m->fin, m->fin + s.nof); s.fout.assign(m->fout, m->fout + s.nof); s.fbc.assign(m->fbc, m->fbc + s.nof);
    s.fnx.assign(m->fnx, m->fnx + s.nof); s.fny.assign(m->fny, m->fny + s.nof); s.farea.assign(m->farea, m->farea + s.nof);
    s.fcx.assign(m->fcx, m->fcx + s.nof); s.fcy.assign(m->fcy, m->fcy + s.nof);
    s.r11.assign(m->r11, m->r11 + s.noc); s.r12.assign(m->r12, m->r12 + s.noc); s.r22.assign(m->r22, m->r22 + s.noc);
    s.nc2c.assign(m->nc2c, m->nc2c + s.noc);
    s.c2f_off.assign(m->c2f_off, m->c2f_off + s.noc + 1);
    s.c2f.assign(m->c2f, m->c2f + s.c2f_off.back());
    s.v2c_off.assign(m->v2c_off, m->v2c_off + s.nop + 1);
    s.v2c.assign(m->v2c, m->v2c + s.v2c_off.back());
    s.v2c_wt.assign(m->v2c_wt, m->v2c_wt + s.v2c_off.back());
    // math (read_input.F90:217-226) and initialize (read_input.F90:231-297)
    s.gamma = 1.4; s.gamma1 = s.gamma - 1.0; s.pi = 4.0 * std::atan(1.0);
    s.q_inf = 1.0;
    s.aoa = s.P.aoa_deg * s.pi / 180.0;
    s.qinf[1] = 1.0;
    s.qinf[2] = std::cos(s.aoa) * s.q_inf;
    s.qinf[3] = std::sin(s.aoa) * s.q_inf;
    s.p_inf = 1.0 / (s.gamma * s.P.m_inf * s.P.m_inf);
    s.qinf[0] = s.p_inf / (s.gamma - 1.0) + 0.5;
    s.r_inf = s.qinf[1];
    s.ent_inf = s.p_inf / std::pow(s.r_inf, s.gamma);
    s.a_inf = std::sqrt(s.gamma * s.p_inf / s.r_inf);
    s.u_inf = s.qinf[2] / s.qinf[1];
    s.v_inf = s.qinf[3] / s.qinf[1];
    s.T_inf = s.gamma * s.P.m_inf * s.P.m_inf * s.p_inf / s.r_inf;
    s.T_infd = 300.0; s.SCONST = 110.4;
    s.t_wall = s.P.t_wall / s.T_infd;
    s.fs_inf[0] = s.r_inf; s.fs_inf[1] = s.u_inf; s.fs_inf[2] = s.v_inf; s.fs_inf[3] = s.p_inf;
    s.qc.assign((size_t)s.ntot * 4, 0.0);
    s.qp.assign((size_t)s.ntot * 5, 0.0);
    s.qold.assign((size_t)s.noc * 4, 0.0);
    s.res.assign((size_t)s.noc * 4, 0.0);
    s.grad.assign((size_t)s.noc * 10, 0.0);
    s.phi.assign((size_t)s.noc * 4, 1.0);
    s.dt.assign(s.noc, 0.0); s.la.assign(s.noc, 0.0);
    s.mul.assign(s.ntot, 0.0);
    s.ptprim.assign((size_t)s.nop * 5, 0.0); s.ptmu.assign(s.nop, 0.0);
    s.fqp.assign((size_t)s.nof * 5, 0.0);
    s.fla.assign(s.nof, 0.0); s.fmu.assign(s.nof, 0.0);
    s.fgrad.assign((size_t)s.nof * 10, 0.0);
    return o;
}

void oracle_cc_free(oracle_cc* o) { delete o; }

int oracle_cc_initialize(oracle_cc* o) {
    CC& s = o->s;
    for (int j = 0; j < s.ntot; ++j)
        for (int k = 0; k < 4; ++k) s.qc[(size_t)j * 4 + k] = s.qinf[k];
    std::fill(s.phi.begin(), s.phi.end(), 1.0);
    std::fill(s.qp.begin(), s.qp.end(), 0.0);
    return UNS_OK;
}

int oracle_cc_set_state(oracle_cc* o, const double* qc) {
    std::copy(qc, qc + o->s.qc.size(), o->s.qc.begin());
    return UNS_OK;
}

int oracle_cc_con2prim(oracle_cc* o) {
    CC& s = o->s;
    for (int i = 0; i < s.noc; ++i) {
        Prim r;
        s.con2prim(s.QC(i), r);
        double* q = s.QP(i);
        q[0] = r.rho; q[1] = r.u; q[2] = r.v; q[3] = r.p; q[4] = r.t;
    }
    return UNS_OK;
}
int oracle_cc_avg_c2v(oracle_cc* o) { avg_c2v(o->s); return UNS_OK; }
int oracle_cc_time_step(oracle_cc* o, double cfl, double* dtg) {
    o->s.cfl = cfl;
    double d = time_step02(o->s, cfl);
    if (dtg) *dtg = d;
    return UNS_OK;
}
int oracle_cc_save_old(oracle_cc* o) {
    CC& s = o->s;
    for (int i = 0; i < s.noc * 4; ++i) s.qold[i] = s.qc[i];
    return UNS_OK;
}
int oracle_cc_gradient(oracle_cc* o) { return gradient(o->s); }
int oracle_cc_limit(oracle_cc* o) { limiter_vkn1(o->s); return UNS_OK; }
int oracle_cc_fvresidual(oracle_cc* o) { return fvresidual(o->s); }
int oracle_cc_rk_stage(oracle_cc* o, int irk) {
    static const double airk[3] = {0.0, 3.0 / 4.0, 1.0 / 3.0};
    static const double birk[3] = {1.0, 1.0 / 4.0, 2.0 / 3.0};
    if (irk < 1 || irk > 3) return UNS_ERR_ARG;
    CC& s = o->s;
    double a = airk[irk - 1], b = birk[irk - 1];
    for (int i = 0; i < s.noc; ++i) {
        double dtbyarea = s.dt[i] / s.cv[i];
        for (int j = 0; j < 4; ++j) {
            size_t k = (size_t)i * 4 + j;
            s.qc[k] = a * s.qold[k] + b * (s.qc[k] - dtbyarea * s.res[k]);
        }
    }
    return UNS_OK;
}
int oracle_cc_lusgs(oracle_cc* o) { return lusgs2(o->s); }
int oracle_cc_check_positivity(oracle_cc* o, int* bad) {
    CC& s = o->s;
    *bad = -1;
    for (int i = 0; i < s.noc; ++i)
        if (s.qp[(size_t)i * 5] <= 0.0 || s.qp[(size_t)i * 5 + 3] <= 0.0) { *bad = i; return UNS_ERR_NONPOSITIVE; }
    return UNS_OK;
}
int oracle_cc_residue(oracle_cc* o, double* fres) {
    CC& s = o->s;
    double f = 0.0;
    for (int i = 0; i < s.noc; ++i)
        for (int j = 0; j < 4; ++j) { double r = s.res[(size_t)i * 4 + j]; f = f + r * r; }
    *fres = std::sqrt(f / (double)s.noc / 4.0);
    return UNS_OK;
}
int oracle_cc_forces(oracle_cc* o, double* fx, double* fy) { *fx = o->s.Fx1; *fy = o->s.Fy1; return UNS_OK; }

int oracle_cc_iteration(oracle_cc* o, double cfl, double* fres) {
    int rc;
    oracle_cc_con2prim(o);
    avg_c2v(o->s);
    oracle_cc_time_step(o, cfl, nullptr);
    oracle_cc_save_old(o);
    if ((rc = gradient(o->s))) return rc;
    if (o->s.P.time_mode == UNS_TIME_RK3) {
        for (int irk = 1; irk <= 3; ++irk) {
            if ((rc = fvresidual(o->s))) return rc;
            oracle_cc_rk_stage(o, irk);
        }
    } else {
        if ((rc = lusgs2(o->s))) return rc;
    }
    int bad;
    if ((rc = oracle_cc_check_positivity(o, &bad))) return rc;
    return oracle_cc_residue(o, fres);
}

int oracle_cc_get(oracle_cc* o, int field, double* out) {
    CC& s = o->s;
    switch (field) {
        case UNS_CC_QC: std::copy(s.qc.begin(), s.qc.end(), out); break;
        case UNS_CC_QP: std::copy(s.qp.begin(), s.qp.end(), out); break;
        case UNS_CC_QOLD: std::copy(s.qold.begin(), s.qold.end(), out); break;
        case UNS_CC_RES: std::copy(s.res.begin(), s.res.end(), out); break;
        case UNS_CC_GRAD:
            for (int i = 0; i < s.noc; ++i)
                for (int v = 0; v < 4; ++v) { out[(size_t)i * 8 + v * 2] = s.G(i, v)[0]; out[(size_t)i * 8 + v * 2 + 1] = s.G(i, v)[1]; }
            break;
        case UNS_CC_PHI: std::copy(s.phi.begin(), s.phi.end(), out); break;
        case UNS_CC_DT: std::copy(s.dt.begin(), s.dt.end(), out); break;
        case UNS_CC_LA: std::copy(s.la.begin(), s.la.end(), out); break;
        case UNS_CC_PTPRIM: std::copy(s.ptprim.begin(), s.ptprim.end(), out); break;
        case UNS_CC_FQP: std::copy(s.fqp.begin(), s.fqp.end(), out); break;
        case UNS_CC_FLA: std::copy(s.fla.begin(), s.fla.end(), out); break;
        case UNS_CC_FMU: std::copy(s.fmu.begin(), s.fmu.end(), out); break;
        case UNS_CC_FGRAD: std::copy(s.fgrad.begin(), s.fgrad.end(), out); break;
        case UNS_CC_MUL: std::copy(s.mul.begin(), s.mul.begin() + s.noc, out); break;
        default: return UNS_ERR_ARG;
    }
    return UNS_OK;
}

int oracle_cc_set(oracle_cc* o, int field, const double* in) {
    CC& s = o->s;
    switch (field) {
        case UNS_CC_QC: std::copy(in, in + s.qc.size(), s.qc.begin()); break;
        case UNS_CC_QP: std::copy(in, in + s.qp.size(), s.qp.begin()); break;
        case UNS_CC_PHI: std::copy(in, in + s.phi.size(), s.phi.begin()); break;
        case UNS_CC_GRAD:
            for (int i = 0; i < s.noc; ++i)
                for (int v = 0; v < 4; ++v) { s.G(i, v)[0] = in[(size_t)i * 8 + v * 2]; s.G(i, v)[1] = in[(size_t)i * 8 + v * 2 + 1]; }
            break;
        default: return UNS_ERR_ARG;
    }
    return UNS_OK;
}

}  // extern "C"
