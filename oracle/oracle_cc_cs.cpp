// oracle_cc_cs.cpp -- TEST INFRASTRUCTURE ONLY.  The CCFVM oracle on
// complex-step numbers: the same routines (oracle_cc_body.inc) on a complex
// scalar whose comparisons, fabs, max and min act on the real part (the
// branch of the real computation), so that for an input x + i h with h tiny
// Im(f)/h is df/dx to round-off, with no subtractive cancellation.  It is the
// complex-step reference of the discrete adjoint's tests.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "oracle.h"

namespace {

struct cs {
    std::complex<double> z;
    cs(double r = 0.0) : z(r, 0.0) {}
    cs(double r, double i) : z(r, i) {}
    explicit cs(std::complex<double> w) : z(w) {}
};
inline cs operator+(cs a, cs b) { return cs(a.z + b.z); }
inline cs operator-(cs a, cs b) { return cs(a.z - b.z); }
inline cs operator*(cs a, cs b) { return cs(a.z * b.z); }
inline cs operator/(cs a, cs b) { return cs(a.z / b.z); }
inline cs operator-(cs a) { return cs(-a.z); }
inline cs& operator+=(cs& a, cs b) { a.z += b.z; return a; }
inline cs& operator-=(cs& a, cs b) { a.z -= b.z; return a; }
inline cs& operator*=(cs& a, cs b) { a.z *= b.z; return a; }
inline cs& operator/=(cs& a, cs b) { a.z /= b.z; return a; }
inline bool operator<(cs a, cs b) { return a.z.real() < b.z.real(); }
inline bool operator>(cs a, cs b) { return a.z.real() > b.z.real(); }
inline bool operator<=(cs a, cs b) { return a.z.real() <= b.z.real(); }
inline bool operator>=(cs a, cs b) { return a.z.real() >= b.z.real(); }
inline bool operator==(cs a, cs b) { return a.z.real() == b.z.real(); }
inline bool operator!=(cs a, cs b) { return a.z.real() != b.z.real(); }
using std::atan;
using std::cos;
using std::fabs;
using std::log10;
using std::max;
using std::min;
using std::pow;
using std::sin;
using std::sqrt;
inline cs fabs(cs a) { return a.z.real() < 0.0 ? cs(-a.z) : a; }
inline cs sqrt(cs a) { return cs(std::sqrt(a.z)); }
inline cs pow(cs a, cs b) { return cs(std::pow(a.z, b.z)); }
inline cs max(cs a, cs b) { return (a < b) ? b : a; }
inline cs min(cs a, cs b) { return (b < a) ? b : a; }
inline cs cos(cs a) { return cs(std::cos(a.z)); }
inline cs sin(cs a) { return cs(std::sin(a.z)); }
inline cs atan(cs a) { return cs(std::atan(a.z)); }
inline cs log10(cs a) { return cs(std::log10(a.z)); }
inline cs add_imag(cs x, double im) { return cs(x.z + std::complex<double>(0.0, im)); }

using R = cs;
#include "oracle_cc_body.inc"

}  // namespace

struct oracle_cc_cs {
    CC s;
    bool freeze_dt = false;
};

extern "C" {

oracle_cc_cs* oracle_cc_cs_create(const uns_cc_mesh* m, const uns_params* p, double aoa_im) {
    if (!m || !p) return nullptr;
    oracle_cc_cs* o = new oracle_cc_cs();
    cc_init(o->s, m, p, aoa_im);
    return o;
}

void oracle_cc_cs_free(oracle_cc_cs* o) { delete o; }

int oracle_cc_cs_set(oracle_cc_cs* o, int field, const double* re, const double* im) {
    CC& s = o->s;
    std::vector<cs>* v = field == UNS_CC_QC ? &s.qc : field == UNS_CC_QP ? &s.qp : field == UNS_CC_PHI ? &s.phi : nullptr;
    if (!v || !re) return UNS_ERR_ARG;
    for (size_t k = 0; k < v->size(); ++k) (*v)[k] = cs(re[k], im ? im[k] : 0.0);
    return UNS_OK;
}

int oracle_cc_cs_get(oracle_cc_cs* o, int field, double* re, double* im) {
    CC& s = o->s;
    const std::vector<cs>* v = field == UNS_CC_QC ? &s.qc : field == UNS_CC_QP ? &s.qp : nullptr;
    if (!v || !re || !im) return UNS_ERR_ARG;
    for (size_t k = 0; k < v->size(); ++k) { re[k] = (*v)[k].z.real(); im[k] = (*v)[k].z.imag(); }
    return UNS_OK;
}

// One main-loop iteration (CCFVM/main.F90:57-117), as oracle_cc_iteration.
int oracle_cc_cs_iteration(oracle_cc_cs* o, double cfl) {
    CC& s = o->s;
    int rc;
    cc_con2prim(s);
    avg_c2v(s);
    s.cfl = cfl;
    time_step02(s, cfl);
    // The adjoint holds the RK update's dt / cv at its recorded value (it
    // multiplies the residual, which vanishes at a converged state); with
    // freeze_dt the complex step does the same -- dt is replaced by
    // real(dt / cv) * cv -- so that the two agree at any state.
    if (o->freeze_dt)
        for (int i = 0; i < s.noc; ++i) s.dt[i] = cs((s.dt[i].z / s.cv[i].z).real()) * s.cv[i];
    cc_save_old(s);
    if ((rc = gradient(s))) return rc;
    if (s.P.time_mode != UNS_TIME_RK3) return UNS_ERR_ARG;
    for (int irk = 1; irk <= 3; ++irk) {
        if ((rc = fvresidual(s))) return rc;
        cc_rk_stage(s, irk);
    }
    return UNS_OK;
}

// Geometric arrays in uns_cc_mesh_adj order.
int oracle_cc_cs_set_geometry_im(oracle_cc_cs* o, int field, const double* im) {
    if (!o || !im) return UNS_ERR_ARG;
    CC& s = o->s;
    std::vector<cs>* tab[15] = {&s.px, &s.py, &s.cx, &s.cy, &s.cv, &s.cov, &s.fnx, &s.fny, &s.farea,
                                &s.fcx, &s.fcy, &s.r11, &s.r12, &s.r22, &s.v2c_wt};
    if (field < 0 || field >= 15) return UNS_ERR_ARG;
    std::vector<cs>& v = *tab[field];
    for (size_t k = 0; k < v.size(); ++k) v[k] = cs(v[k].z.real(), im[k]);
    return UNS_OK;
}

int oracle_cc_cs_freeze_dt(oracle_cc_cs* o, int on) {
    if (!o) return UNS_ERR_ARG;
    o->freeze_dt = on != 0;
    return UNS_OK;
}

int oracle_cc_cs_forces(oracle_cc_cs* o, double* fx, double* fy) {
    fx[0] = o->s.Fx1.z.real(); fx[1] = o->s.Fx1.z.imag();
    fy[0] = o->s.Fy1.z.real(); fy[1] = o->s.Fy1.z.imag();
    return UNS_OK;
}

}  // extern "C"
