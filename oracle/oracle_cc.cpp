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
using R = double;
using std::atan;
using std::cos;
using std::fabs;
using std::log10;
using std::max;
using std::min;
using std::pow;
using std::sin;
using std::sqrt;
inline double add_imag(double x, double) { return x; }

#include "oracle_cc_body.inc"

}  // namespace

struct oracle_cc { CC s; };

extern "C" {

oracle_cc* oracle_cc_create(const uns_cc_mesh* m, const uns_params* p) {
    if (!m || !p) return nullptr;
    oracle_cc* o = new oracle_cc();
    cc_init(o->s, m, p, 0.0);
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
    cc_con2prim(o->s);
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
    cc_save_old(o->s);
    return UNS_OK;
}
int oracle_cc_gradient(oracle_cc* o) { return gradient(o->s); }
int oracle_cc_limit(oracle_cc* o) { limiter_vkn1(o->s); return UNS_OK; }
int oracle_cc_fvresidual(oracle_cc* o) { return fvresidual(o->s); }
int oracle_cc_rk_stage(oracle_cc* o, int irk) { return cc_rk_stage(o->s, irk); }
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

int oracle_cc_find_cl_cd(oracle_cc* o, double xref, double yref, double* coef, double* wall, int* nwall) {
    std::vector<double> w((size_t)o->s.nbf * 4);
    int n = cc_find_cl_cd(o->s, xref, yref, coef, w.data());
    if (wall) std::copy(w.begin(), w.begin() + (size_t)n * 4, wall);
    if (nwall) *nwall = n;
    return UNS_OK;
}

int oracle_cc_screen_minmax(oracle_cc* o, double* out) {
    cc_screen_minmax(o->s, out);
    return UNS_OK;
}

int oracle_cc_tecplt(oracle_cc* o, double* out) {
    cc_tecplt(o->s, out);
    return UNS_OK;
}

}  // extern "C"
