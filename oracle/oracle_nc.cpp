// oracle_nc.cpp -- TEST INFRASTRUCTURE ONLY.  CPU oracle, vertex-centred
// median-dual solver (NCFVM).  Serial restatement of the reference loops in
// their own order (edge loops scattering into nodes), cited per routine.
// Compiled with -ffp-contract=off.  PARITY UNPINNED: see oracle.h.
//
// The HEAD side of the merge conflict in NCFVM/fvresidual.f90:11-17 is taken
// (Gradient_LSQR).  AUSM+-up has no compiled NCFVM reference
// (NCFVM/ausm_up_flux.f90 is not in NCFVM/makefile:30-31 and references fields
// that do not exist); it is restated from the CCFVM formulation
// (CCFVM/ausm_up_flux.F90:2-162) on the dual face, scaled by the dual-face
// length, with the Roe-averaged spectral radius of NCFVM/vanleer_flux.f90.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "oracle.h"

namespace {

struct NC {
    int nop, noc, nof;
    std::vector<double> px, py, cv;
    std::vector<int> fp1, fp2, fbc;
    std::vector<double> fnx, fny, farea;
    std::vector<int> v2v_off, v2v, v2f_off, v2f;
    std::vector<double> wx, wy;
    uns_params P;
    double gamma, gamma1, pi, q_inf, aoa, p_inf, r_inf, ent_inf, a_inf, u_inf, v_inf;
    double qinf[4];
    const double eps = (double)1.1920928955078125e-07f;  // epsilon(1.0), All_modules.f90:15
    std::vector<double> qc, qp, qold, res, grad, phi, dt, la, fla, dumax, dumin;
    double cfl = 0.0;
};

struct Prim { double rho, u, v, e, q, p, h, a; };
void con2prim(const NC& s, const double* qt, Prim& r) {  // All_modules.f90:146-169
    r.rho = qt[1];
    r.u = qt[2] / qt[1];
    r.v = qt[3] / qt[1];
    double Et = qt[0];
    r.e = Et / r.rho;
    r.q = r.u * r.u + r.v * r.v;
    r.p = (s.gamma - 1.0) * (Et - 0.5 * r.rho * r.q);
    r.h = (Et + r.p) / r.rho;
    r.a = std::sqrt(s.gamma * r.p / r.rho);
}

double m1p(double m) { return 0.50 * (m + std::fabs(m)); }
double m1m(double m) { return 0.5 * (m - std::fabs(m)); }
double m2p(double m) { return 0.25 * (m + 1.0) * (m + 1.0); }
double m2m(double m) { return -0.25 * (m - 1.0) * (m - 1.0); }
double m4p(double m, double beta) { return std::fabs(m) >= 1.0 ? 0.5 * (m + std::fabs(m)) : m2p(m) * (1.0 - 16.0 * beta * m2m(m)); }
double m4m(double m, double beta) { return std::fabs(m) >= 1.0 ? 0.5 * (m - std::fabs(m)) : m2m(m) * (1.0 + 16.0 * beta * m2p(m)); }
double p5p(double m, double a) { return std::fabs(m) >= 1.0 ? 0.5 * (m + std::fabs(m)) / m : m2p(m) * ((2.0 - m) - 16.0 * a * m * m2m(m)); }
double p5m(double m, double a) { return std::fabs(m) >= 1.0 ? 0.5 * (m - std::fabs(m)) / m : m2m(m) * ((-2.0 - m) + 16.0 * a * m * m2p(m)); }

// Gradient_LSQR (NCFVM/gradient.f90:2-30)
void gradient_lsqr(NC& s) {
    std::fill(s.grad.begin(), s.grad.end(), 0.0);
    for (int i = 0; i < s.nop; ++i)
        for (int k = 0; k < 4; ++k)
            for (int j = s.v2v_off[i]; j < s.v2v_off[i + 1]; ++j) {
                int c = s.v2v[j];
                double d = s.qp[(size_t)c * 4 + k] - s.qp[(size_t)i * 4 + k];
                s.grad[(size_t)i * 8 + k * 2] = s.grad[(size_t)i * 8 + k * 2] + d * s.wx[j];
                d = s.qp[(size_t)c * 4 + k] - s.qp[(size_t)i * 4 + k];
                s.grad[(size_t)i * 8 + k * 2 + 1] = s.grad[(size_t)i * 8 + k * 2 + 1] + d * s.wy[j];
            }
}

void du_minmax(NC& s) {  // limiter.f90:24-39
    for (int i = 0; i < s.nop * 4; ++i) { s.dumin[i] = s.eps; s.dumax[i] = -s.eps; }
    for (int f = 0; f < s.nof; ++f) {
        int p1 = s.fp1[f], p2 = s.fp2[f];
        for (int j = 0; j < 4; ++j) {
            double du = s.qp[(size_t)p2 * 4 + j] - s.qp[(size_t)p1 * 4 + j];
            s.dumax[p1 * 4 + j] = std::max(s.dumax[p1 * 4 + j], du);
            s.dumin[p1 * 4 + j] = std::min(s.dumin[p1 * 4 + j], du);
            s.dumax[p2 * 4 + j] = std::max(s.dumax[p2 * 4 + j], -du);
            s.dumin[p2 * 4 + j] = std::min(s.dumin[p2 * 4 + j], -du);
        }
    }
}

// limiter_VKN (NCFVM/limiter.f90:15-98); kappa=0.01 is a default-real literal.
void limiter_vkn(NC& s) {
    du_minmax(s);
    const double kappa = (double)0.01f;
    for (int f = 0; f < s.nof; ++f) {
        int p1 = s.fp1[f], p2 = s.fp2[f];
        double d0 = s.px[p2] - s.px[p1], d1 = s.py[p2] - s.py[p1];
        for (int j = 0; j < 4; ++j) {
            for (int side = 0; side < 2; ++side) {
                int p = side == 0 ? p1 : p2;
                double sum = s.grad[(size_t)p * 8 + j * 2] * d0 + s.grad[(size_t)p * 8 + j * 2 + 1] * d1;
                double D_L = side == 0 ? 0.5 * sum : -(0.5 * sum);
                double k = kappa * std::sqrt(s.cv[p]);
                double TOL = k * k * k;
                double alfa = D_L > 0.0 ? s.dumax[p * 4 + j] : s.dumin[p * 4 + j];
                if (std::fabs(alfa) < s.eps) alfa = 0.0;
                double nr = alfa * alfa + 2.0 * D_L * alfa + TOL;
                double dr = alfa * alfa + 2.0 * D_L * D_L + D_L * alfa + TOL;
                double ph = std::min(1.0, nr / dr);
                s.phi[p * 4 + j] = std::min(s.phi[p * 4 + j], ph);
            }
        }
    }
}

// limiter_min_max (Barth-Jespersen, NCFVM/limiter.f90:192-260), including
// the reference's +1/2 projection on the p2 side.
void limiter_barth(NC& s) {
    du_minmax(s);
    for (int f = 0; f < s.nof; ++f) {
        int p1 = s.fp1[f], p2 = s.fp2[f];
        double d0 = s.px[p2] - s.px[p1], d1 = s.py[p2] - s.py[p1];
        for (int j = 0; j < 4; ++j)
            for (int side = 0; side < 2; ++side) {
                int p = side == 0 ? p1 : p2;
                double D_L = 0.5 * (s.grad[(size_t)p * 8 + j * 2] * d0 + s.grad[(size_t)p * 8 + j * 2 + 1] * d1);
                if (side == 1 && s.P.limiter_type == UNS_LIM_BARTH_CORRECTED) D_L = -D_L;
                double ph;
                if (D_L > 0.0) ph = std::min(1.0, s.dumax[p * 4 + j] / D_L);
                else if (D_L < 0.0) ph = std::min(1.0, s.dumin[p * 4 + j] / D_L);
                else ph = 1.0;
                if (s.P.limiter_type == UNS_LIM_BARTH_CORRECTED) ph = std::max(0.0, ph);
                s.phi[p * 4 + j] = std::min(s.phi[p * 4 + j], ph);
            }
    }
}

// Roe-averaged spectral radius accumulation (vanleer_flux.f90:102-115).
void edge_lambda(NC& s, int ie, int c1, int c2, double rL, double uL, double vL, double HL,
                 double rR, double uR, double vR, double HR) {
    double nx = s.fnx[ie], ny = s.fny[ie], area = s.farea[ie];
    double RT = std::sqrt(rR / rL);
    double u = (uL + RT * uR) / (1.0 + RT);
    double v = (vL + RT * vR) / (1.0 + RT);
    double H = (HL + RT * HR) / (1.0 + RT);
    double a = std::sqrt((s.gamma1) * (H - 0.5 * (u * u + v * v)));
    double un = std::fabs(u * nx + v * ny);
    double ll = (un + a) * area;
    s.la[c1] = s.la[c1] + ll;
    s.la[c2] = s.la[c2] + ll;
    s.fla[ie] = ll;
    (void)rL;
}

// vanleer_flux (NCFVM/vanleer_flux.f90:2-118)
void vanleer_flux(NC& s, int ie, int c1, int c2, const double* qcl, const double* qcr) {
    const double G = s.gamma, G1 = s.gamma1;
    double nx = s.fnx[ie], ny = s.fny[ie], area = s.farea[ie];
    double rl = qcl[0], ul = qcl[1], vl = qcl[2], pl = qcl[3];
    double unl = ul * nx + vl * ny, ql2 = ul * ul + vl * vl, al2 = G * pl / rl;
    double hl = al2 / G1 + 0.5 * ql2, cl = std::sqrt(al2), ml = unl / cl;
    double rr = qcr[0], ur = qcr[1], vr = qcr[2], pr = qcr[3];
    double unr = ur * nx + vr * ny, qr2 = ur * ur + vr * vr, ar2 = G * pr / rr;
    double hr = ar2 / G1 + 0.5 * qr2, cr = std::sqrt(ar2), mr = unr / cr;
    double beta = 0.0, alpha = 0.0;
    double plp = p5p(ml, alpha), prm = p5m(mr, alpha);
    double mlp = m4p(ml, beta), mlm = m4m(ml, beta), mrp = m4p(mr, beta), mrm = m4m(mr, beta);
    double p12 = plp * pl + prm * pr;
    double fmass_p = rl * cl * mlp, fmass_m = rr * cr * mrm;
    double fmass12 = fmass_p + fmass_m;
    double delta = -(G * (cr * mrp * mrm * pr - cl * mlp * mlm * pl) / (G - 1.0));
    double dissi = fmass_p - fmass_m;
    double fL[4] = {hl, 1.0, ul, vl}, fR[4] = {hr, 1.0, ur, vr};
    double fP[4] = {delta, 0.0, nx * p12, ny * p12};
    for (int i = 0; i < 4; ++i) {
        double flux = 0.5 * fmass12 * (fL[i] + fR[i]) - 0.5 * dissi * (fR[i] - fL[i]) + fP[i];
        s.res[(size_t)c1 * 4 + i] = s.res[(size_t)c1 * 4 + i] + flux * area;
        s.res[(size_t)c2 * 4 + i] = s.res[(size_t)c2 * 4 + i] - flux * area;
    }
    edge_lambda(s, ie, c1, c2, rl, ul, vl, hl, rr, ur, vr, hr);
}

// AUSM+-up on the dual face (restated; see file header).
void ausm_flux(NC& s, int ie, int c1, int c2, const double* ql, const double* qr) {
    const double G = s.gamma, G1 = s.gamma1;
    double sigma = 1.0, ku = 0.75, kp = 0.25;
    double nx = s.fnx[ie], ny = s.fny[ie], area = s.farea[ie];
    double rl = ql[0], ul = ql[1], vl = ql[2], pl = ql[3];
    double unl = ul * nx + vl * ny, ql2 = ul * ul + vl * vl, al2 = G * pl / rl;
    double hl = al2 / G1 + 0.5 * ql2;
    double rr = qr[0], ur = qr[1], vr = qr[2], pr = qr[3];
    double unr = ur * nx + vr * ny, qr2 = ur * ur + vr * vr, ar2 = G * pr / rr;
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
    else { double mstar2 = std::min(1.0, std::max(mbar2, mref * mref)); double Mo = mstar2; fa = Mo * (2.0 - Mo); }
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
    double flux[4];
    for (int i = 0; i < 4; ++i) flux[i] = c12 * (a * fl[i] + b * fr[i]);
    flux[2] = flux[2] + nx * p12;
    flux[3] = flux[3] + ny * p12;
    for (int i = 0; i < 4; ++i) {
        s.res[(size_t)c1 * 4 + i] = s.res[(size_t)c1 * 4 + i] + flux[i] * area;
        s.res[(size_t)c2 * 4 + i] = s.res[(size_t)c2 * 4 + i] - flux[i] * area;
    }
    edge_lambda(s, ie, c1, c2, rl, ul, vl, hl, rr, ur, vr, hr);
}

// solid_flux (NCFVM/solid_flux.f90:1-43)
void solid_flux(NC& s, int c1, int c2) {
    double p1 = 0.75 * s.qp[(size_t)c1 * 4 + 3] + 0.25 * s.qp[(size_t)c2 * 4 + 3];
    double p2 = 0.25 * s.qp[(size_t)c1 * 4 + 3] + 0.75 * s.qp[(size_t)c2 * 4 + 3];
    double nx = 0.5 * (s.py[c2] - s.py[c1]);
    double ny = -0.5 * (s.px[c2] - s.px[c1]);
    double area = std::sqrt(nx * nx + ny * ny);
    s.la[c1] = s.la[c1] + std::sqrt(s.gamma * s.qp[(size_t)c1 * 4 + 3] / s.qp[(size_t)c1 * 4]) * area;
    s.la[c2] = s.la[c2] + std::sqrt(s.gamma * s.qp[(size_t)c2 * 4 + 3] / s.qp[(size_t)c2 * 4]) * area;
    s.res[(size_t)c1 * 4 + 2] = s.res[(size_t)c1 * 4 + 2] + p1 * nx;
    s.res[(size_t)c1 * 4 + 3] = s.res[(size_t)c1 * 4 + 3] + p1 * ny;
    s.res[(size_t)c2 * 4 + 2] = s.res[(size_t)c2 * 4 + 2] + p2 * nx;
    s.res[(size_t)c2 * 4 + 3] = s.res[(size_t)c2 * 4 + 3] + p2 * ny;
}

// farfield_flux1 (NCFVM/farfield_flux.f90:1-95)
void farfield_flux1(NC& s, int c1, int c2) {
    const double G = s.gamma, G1 = s.gamma1;
    double nx = -(0.5 * (s.py[c2] - s.py[c1]));
    double ny = 0.5 * (s.px[c2] - s.px[c1]);
    double dr = std::sqrt(nx * nx + ny * ny);
    nx = nx / dr; ny = ny / dr;
    double uinf = s.u_inf, vinf = s.v_inf, pinf = s.p_inf, rinf = s.r_inf, ainf = s.a_inf;
    double un_inf = uinf * nx + vinf * ny;
    double con[4];
    for (int k = 0; k < 4; ++k) con[k] = 0.5 * (s.qp[(size_t)c1 * 4 + k] + s.qp[(size_t)c2 * 4 + k]);
    double rho = con[0], u = con[1], v = con[2], p = con[3];
    double a = std::sqrt(G * p / rho);
    double un = u * nx + v * ny;
    double Rp = un + 2.0 * a / G1;
    double Rm = un_inf - 2.0 * ainf / G1;
    double Unf = 0.5 * (Rp + Rm);
    double af = 0.25 * (Rp - Rm) * G1;
    double uf, vf, Sf;
    if (Unf > 0.0) { uf = u + nx * (Unf - un); vf = v + ny * (Unf - un); Sf = p / std::pow(rho, G); }
    else { uf = uinf + nx * (Unf - un_inf); vf = vinf + ny * (Unf - un_inf); Sf = pinf / std::pow(rinf, G); }
    double rhof = std::pow(af * af / G / Sf, 1.0 / G1);
    double pf = rhof * af * af / G;
    double ef = pf / G1 + 0.5 * rhof * (uf * uf + vf * vf);
    double flux[4];
    flux[0] = (ef + pf) * Unf;
    flux[1] = rhof * Unf;
    flux[2] = flux[1] * uf + pf * nx;
    flux[3] = flux[1] * vf + pf * ny;
    double area = std::sqrt(nx * nx + ny * ny);
    s.la[c1] = s.la[c1] + (std::fabs(Unf) + std::sqrt(G * s.qp[(size_t)c1 * 4 + 3] / s.qp[(size_t)c1 * 4])) * area;
    s.la[c2] = s.la[c2] + (std::fabs(Unf) + std::sqrt(G * s.qp[(size_t)c2 * 4 + 3] / s.qp[(size_t)c2 * 4])) * area;
    for (int i = 0; i < 4; ++i) {
        s.res[(size_t)c1 * 4 + i] = s.res[(size_t)c1 * 4 + i] + dr * flux[i];
        s.res[(size_t)c2 * 4 + i] = s.res[(size_t)c2 * 4 + i] + dr * flux[i];
    }
}

// fvresidual (NCFVM/fvresidual.f90:4-85) + time_step2 (timestep.f90:5-37)
void fvresidual(NC& s, double cfl) {
    gradient_lsqr(s);
    std::fill(s.res.begin(), s.res.end(), 0.0);
    std::fill(s.la.begin(), s.la.end(), 0.0);
    std::fill(s.fla.begin(), s.fla.end(), 0.0);
    if (s.P.limiter_type == UNS_LIM_VKN) limiter_vkn(s); else limiter_barth(s);
    for (int ie = 0; ie < s.nof; ++ie) {
        int p1 = s.fp1[ie], p2 = s.fp2[ie];
        double d0 = s.px[p2] - s.px[p1], d1 = s.py[p2] - s.py[p1];
        double left[4], right[4];
        for (int k = 0; k < 4; ++k) {
            double g = s.grad[(size_t)p1 * 8 + k * 2] * d0 + s.grad[(size_t)p1 * 8 + k * 2 + 1] * d1;
            left[k] = s.qp[(size_t)p1 * 4 + k] + 0.5 * g * s.phi[p1 * 4 + k];
            g = s.grad[(size_t)p2 * 8 + k * 2] * d0 + s.grad[(size_t)p2 * 8 + k * 2 + 1] * d1;
            right[k] = s.qp[(size_t)p2 * 4 + k] - 0.5 * g * s.phi[p2 * 4 + k];
        }
        if (s.P.flux_type == UNS_FLUX_AUSM) ausm_flux(s, ie, p1, p2, left, right);
        else vanleer_flux(s, ie, p1, p2, left, right);
        if (s.fbc[ie] == 1001) solid_flux(s, p1, p2);
        if (s.fbc[ie] == 2001) farfield_flux1(s, p1, p2);
    }
    for (int i = 0; i < s.nop; ++i) s.dt[i] = cfl * s.cv[i] / s.la[i];
}

// lusgs (NCFVM/lusgs.f90:4-157)
void lusgs(NC& s, double cfl) {
    const double omega = 1.5;
    fvresidual(s, cfl);
    std::vector<double> D(s.nop), dqc((size_t)s.nop * 4, 0.0);
    for (int it = 0; it < s.nop; ++it) D[it] = s.cv[it] / s.dt[it] + 0.5 * omega * s.la[it];
    auto normalflux = [&](const double* q, double nx, double ny, double ds, double* f) {
        Prim r;
        con2prim(s, q, r);
        double et = r.e * r.rho;
        double un = r.u * nx + r.v * ny;
        f[0] = (et + r.p) * un; f[1] = r.rho * un; f[2] = f[1] * r.u + r.p * nx; f[3] = f[1] * r.v + r.p * ny;
        for (int k = 0; k < 4; ++k) f[k] = f[k] * ds;
    };
    for (int pass = 0; pass < 2; ++pass) {
        for (int step = 0; step < s.nop; ++step) {
            int it = pass == 0 ? step : s.nop - 1 - step;
            double cres[4] = {0, 0, 0, 0};
            for (int j = s.v2f_off[it]; j < s.v2f_off[it + 1]; ++j) {
                int c = s.v2f[j];
                double nx = s.fnx[c], ny = s.fny[c], ds = s.farea[c];
                int p1 = s.fp1[c], p2 = s.fp2[c];
                double sign = 1.0;
                if (p2 == it) { p2 = p1; sign = -1.0; }
                bool take = pass == 0 ? (p2 < it && p2 >= 0) : (p2 > it && p2 >= 0);
                if (!take) continue;
                double f1[4], f2[4];
                normalflux(&s.qold[(size_t)p2 * 4], nx, ny, ds, f1);
                normalflux(&s.qc[(size_t)p2 * 4], nx, ny, ds, f2);
                for (int iv = 0; iv < 4; ++iv)
                    cres[iv] = cres[iv] + 0.5 * (sign * (f2[iv] - f1[iv]) - omega * s.fla[c] * dqc[(size_t)p2 * 4 + iv]);
            }
            for (int iv = 0; iv < 4; ++iv) {
                size_t k = (size_t)it * 4 + iv;
                if (pass == 0) dqc[k] = (-s.res[k] - cres[iv]) / D[it];
                else dqc[k] = dqc[k] - cres[iv] / D[it];
                s.qc[k] = s.qold[k] + dqc[k];
            }
        }
    }
}

}  // namespace

struct oracle_nc { NC s; };

extern "C" {

oracle_nc* oracle_nc_create(const uns_nc_mesh* m, const uns_params* p) {
    if (!m || !p) return nullptr;
    oracle_nc* o = new oracle_nc();
    NC& s = o->s;
    s.P = *p;
    s.nop = m->nop; s.noc = m->noc; s.nof = m->nof;
    s.px.assign(m->px, m->px + s.nop); s.py.assign(m->py, m->py + s.nop); s.cv.assign(m->cv, m->cv + s.nop);
    s.fp1.assign(m->fp1, m->fp1 + s.nof); s.fp2.assign(m->fp2, m->fp2 + s.nof); s.fbc.assign(m->fbc, m->fbc + s.nof);
    s.fnx.assign(m->fnx, m->fnx + s.nof); s.fny.assign(m->fny, m->fny + s.nof); s.farea.assign(m->farea, m->farea + s.nof);
    s.v2v_off.assign(m->v2v_off, m->v2v_off + s.nop + 1);
    s.v2v.assign(m->v2v, m->v2v + s.v2v_off.back());
    s.wx.assign(m->wx, m->wx + s.v2v_off.back()); s.wy.assign(m->wy, m->wy + s.v2v_off.back());
    s.v2f_off.assign(m->v2f_off, m->v2f_off + s.nop + 1);
    s.v2f.assign(m->v2f, m->v2f + s.v2f_off.back());
    // math / initialize (NCFVM/common.f90:4-54)
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
    size_t n4 = (size_t)s.nop * 4;
    s.qc.assign(n4, 0.0); s.qp.assign(n4, 0.0); s.qold.assign(n4, 0.0); s.res.assign(n4, 0.0);
    s.grad.assign((size_t)s.nop * 8, 0.0);
    s.phi.assign(n4, (double)1e20f);  // phi=1e20 default-real initialiser, All_modules.f90:190
    s.dt.assign(s.nop, 0.0); s.la.assign(s.nop, 0.0); s.fla.assign(s.nof, 0.0);
    s.dumax.assign(n4, 0.0); s.dumin.assign(n4, 0.0);
    return o;
}

void oracle_nc_free(oracle_nc* o) { delete o; }

int oracle_nc_initialize(oracle_nc* o) {
    NC& s = o->s;
    for (int j = 0; j < s.nop; ++j)
        for (int k = 0; k < 4; ++k) s.qc[(size_t)j * 4 + k] = s.qinf[k];
    std::fill(s.phi.begin(), s.phi.end(), (double)1e20f);
    return UNS_OK;
}

int oracle_nc_set_state(oracle_nc* o, const double* qc) {
    std::copy(qc, qc + o->s.qc.size(), o->s.qc.begin());
    return UNS_OK;
}

int oracle_nc_save_old(oracle_nc* o) {
    NC& s = o->s;
    for (int i = 0; i < s.nop; ++i) {
        Prim r;
        con2prim(s, &s.qc[(size_t)i * 4], r);
        s.qp[(size_t)i * 4] = r.rho; s.qp[(size_t)i * 4 + 1] = r.u; s.qp[(size_t)i * 4 + 2] = r.v; s.qp[(size_t)i * 4 + 3] = r.p;
        for (int j = 0; j < 4; ++j) s.qold[(size_t)i * 4 + j] = s.qc[(size_t)i * 4 + j];
    }
    return UNS_OK;
}

int oracle_nc_fvresidual(oracle_nc* o, double cfl) { o->s.cfl = cfl; fvresidual(o->s, cfl); return UNS_OK; }

int oracle_nc_rk_stage(oracle_nc* o, int irk) {
    static const double airk[3] = {0.0, 3.0 / 4.0, 1.0 / 3.0};
    static const double birk[3] = {1.0, 1.0 / 4.0, 2.0 / 3.0};
    if (irk < 1 || irk > 3) return UNS_ERR_ARG;
    NC& s = o->s;
    double a = airk[irk - 1], b = birk[irk - 1];
    for (int i = 0; i < s.nop; ++i) {
        double dtbyarea = s.dt[i] / s.cv[i];
        for (int j = 0; j < 4; ++j) {
            size_t k = (size_t)i * 4 + j;
            s.qc[k] = a * s.qold[k] + b * (s.qc[k] - dtbyarea * s.res[k]);
        }
    }
    return UNS_OK;
}

int oracle_nc_lusgs(oracle_nc* o, double cfl) { o->s.cfl = cfl; lusgs(o->s, cfl); return UNS_OK; }

int oracle_nc_residue(oracle_nc* o, double* fres, double* fresi, int* iresi) {
    NC& s = o->s;
    double f = 0.0, fi = 0.0;
    int ii = -1;
    for (int i = 0; i < s.nop; ++i) {
        double fr = 0.0;
        for (int j = 0; j < 4; ++j) { double r = s.res[(size_t)i * 4 + j]; fr = fr + r * r; }
        f = f + fr;
        fr = std::sqrt(fr);
        if (fr > fi) { fi = fr; ii = i; }
    }
    *fres = std::sqrt(f / (double)s.nop);
    if (fresi) *fresi = fi;
    if (iresi) *iresi = ii;
    return UNS_OK;
}

int oracle_nc_iteration(oracle_nc* o, double cfl, double* fres, double* fresi) {
    oracle_nc_save_old(o);
    if (o->s.P.time_mode == UNS_TIME_RK3) {
        for (int irk = 1; irk <= 3; ++irk) { fvresidual(o->s, cfl); oracle_nc_rk_stage(o, irk); }
    } else {
        lusgs(o->s, cfl);
    }
    return oracle_nc_residue(o, fres, fresi, nullptr);
}

// tecplt's vertex table (NCFVM/main.f90:190-233): per node x, y and the
// primitives of the last save_old, rho, u, v, p, Mach.
int oracle_nc_tecplt(oracle_nc* o, double* out) {
    NC& s = o->s;
    for (int i = 0; i < s.nop; ++i) {
        const double* q = &s.qp[(size_t)i * 4];
        double ro = q[0], uo = q[1], vo = q[2], po = q[3];
        double q2 = uo * uo + vo * vo;
        double mach = std::sqrt(q2 * ro / (s.gamma * po));
        double* r = out + (size_t)i * 7;
        r[0] = s.px[i]; r[1] = s.py[i]; r[2] = ro; r[3] = uo; r[4] = vo; r[5] = po; r[6] = mach;
    }
    return UNS_OK;
}

// screen's min/max diagnostics (NCFVM/main.f90:115-187) over the nodes from
// the current conserved state: out = min, max of density, u, v, pressure,
// Mach number, entropy.
int oracle_nc_screen_minmax(oracle_nc* o, double* out) {
    NC& s = o->s;
    double lo[6], hi[6];
    for (int k = 0; k < 6; ++k) { lo[k] = 1.0e10; hi[k] = -1.0e10; }
    for (int is = 0; is < s.nop; ++is) {
        Prim r;
        con2prim(s, &s.qc[(size_t)is * 4], r);
        double q2 = r.u * r.u + r.v * r.v;
        double mach = std::sqrt(q2 * r.rho / (s.gamma * r.p));
        double ent = std::log10(r.p / std::pow(r.rho, s.gamma) / s.ent_inf);
        const double x[6] = {r.rho, r.u, r.v, r.p, mach, ent};
        for (int k = 0; k < 6; ++k) { lo[k] = std::min(lo[k], x[k]); hi[k] = std::max(hi[k], x[k]); }
    }
    for (int k = 0; k < 6; ++k) { out[2 * k] = lo[k]; out[2 * k + 1] = hi[k]; }
    return UNS_OK;
}

int oracle_nc_get(oracle_nc* o, int field, double* out) {
    NC& s = o->s;
    switch (field) {
        case UNS_NC_QC: std::copy(s.qc.begin(), s.qc.end(), out); break;
        case UNS_NC_QP: std::copy(s.qp.begin(), s.qp.end(), out); break;
        case UNS_NC_QOLD: std::copy(s.qold.begin(), s.qold.end(), out); break;
        case UNS_NC_RES: std::copy(s.res.begin(), s.res.end(), out); break;
        case UNS_NC_GRAD: std::copy(s.grad.begin(), s.grad.end(), out); break;
        case UNS_NC_PHI: std::copy(s.phi.begin(), s.phi.end(), out); break;
        case UNS_NC_DT: std::copy(s.dt.begin(), s.dt.end(), out); break;
        case UNS_NC_LA: std::copy(s.la.begin(), s.la.end(), out); break;
        case UNS_NC_FLA: std::copy(s.fla.begin(), s.fla.end(), out); break;
        default: return UNS_ERR_ARG;
    }
    return UNS_OK;
}

int oracle_nc_set(oracle_nc* o, int field, const double* in) {
    NC& s = o->s;
    switch (field) {
        case UNS_NC_QC: std::copy(in, in + s.qc.size(), s.qc.begin()); break;
        case UNS_NC_QP: std::copy(in, in + s.qp.size(), s.qp.begin()); break;
        case UNS_NC_GRAD: std::copy(in, in + s.grad.size(), s.grad.begin()); break;
        case UNS_NC_PHI: std::copy(in, in + s.phi.size(), s.phi.begin()); break;
        default: return UNS_ERR_ARG;
    }
    return UNS_OK;
}

}  // extern "C"
