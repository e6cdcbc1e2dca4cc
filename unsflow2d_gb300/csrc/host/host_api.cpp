// host_api.cpp -- C-ABI of libunsflow_host.so (declared in unsflow_host.h):
// mesh handles, flo.inp, CFL schedules and FLO.DAT I/O.  It needs no GPU
// library; the main programs that drive libunsflow_gpu.so are host_main.cpp
// (libunsflow_driver.so).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../uns_sched.hpp"
#include "host_mesh.hpp"
#include "unsflow_host.h"

using namespace unshost;

struct uns_host_cc { RawCC raw; MeshCC mesh; };
struct uns_host_nc { RawNC raw; MeshNC mesh; };

namespace {
thread_local std::string g_err;
}  // namespace

namespace unshost {
int fail(int code, const std::string& msg) { g_err = msg; return code; }

// Fortran Ew.d edit descriptor (e16.6): 0.dddddd mantissa, 2-digit exponent.
std::string fort_e(double x, int w, int d) {
    char buf[80];
    if (std::isnan(x)) { std::snprintf(buf, sizeof buf, "%*s", w, "NaN"); return buf; }
    if (std::isinf(x)) { std::snprintf(buf, sizeof buf, "%*s", w, x > 0 ? "Infinity" : "-Infinity"); return buf; }
    std::string digits(d, '0');
    int e = 0;
    if (x != 0.0) {
        char tmp[64];
        std::snprintf(tmp, sizeof tmp, "%.*e", d - 1, std::fabs(x));  // d.ddddde+XX
        digits.clear();
        for (const char* c = tmp; *c && *c != 'e'; ++c)
            if (*c >= '0' && *c <= '9') digits.push_back(*c);
        e = std::atoi(std::strchr(tmp, 'e') + 1) + 1;
    }
    char body[64];
    std::snprintf(body, sizeof body, "%s0.%sE%c%02d", x < 0 ? "-" : "", digits.c_str(), e < 0 ? '-' : '+', std::abs(e));
    std::snprintf(buf, sizeof buf, "%*s", w, body);
    return buf;
}

std::string dir_of(const std::string& p) {
    size_t k = p.find_last_of('/');
    return k == std::string::npos ? std::string(".") : p.substr(0, k);
}
std::string join(const std::string& d, const std::string& f) {
    if (!f.empty() && f[0] == '/') return f;
    return d + "/" + f;
}
}  // namespace unshost

extern "C" {

const char* uns_host_last_error(void) { return g_err.c_str(); }

int uns_host_cc_airfoil(int ni, int nj, double t, double rfar, double dwall, uns_host_cc** out) {
    if (!out) return fail(UNS_ERR_ARG, "null out");
    AirfoilSpec s{ni, nj, t, rfar, dwall};
    auto* m = new uns_host_cc();
    std::string err;
    int rc = gen_airfoil_cc(s, m->raw, err);
    if (!rc) rc = geometric_cc(m->raw, m->mesh, err);
    if (rc) { delete m; return fail(rc, err); }
    *out = m;
    return UNS_OK;
}

int uns_host_cc_airfoil_dy(int ni, int nj, double t, double rfar, double dwall, const double* dy, uns_host_cc** out) {
    if (!out) return fail(UNS_ERR_ARG, "null out");
    AirfoilSpec s{ni, nj, t, rfar, dwall, dy};
    auto* m = new uns_host_cc();
    std::string err;
    int rc = gen_airfoil_cc(s, m->raw, err);
    if (!rc) rc = geometric_cc(m->raw, m->mesh, err);
    if (rc) { delete m; return fail(rc, err); }
    *out = m;
    return UNS_OK;
}

int uns_host_cc_moved(const uns_host_cc* m, const double* px, const double* py, uns_host_cc** out) {
    if (!m || !px || !py || !out) return fail(UNS_ERR_ARG, "uns_host_cc_moved: null argument");
    auto* o = new uns_host_cc();
    std::string err;
    int rc = moved_cc(m->raw, px, py, o->raw, err);
    if (!rc) rc = geometric_cc(o->raw, o->mesh, err);
    if (rc) { delete o; return fail(rc, err); }
    *out = o;
    return UNS_OK;
}

int uns_host_cc_mesh_vjp(const uns_host_cc* m, const uns_cc_mesh_adj* a, double* gpx, double* gpy) {
    if (!m || !a || !gpx || !gpy || !a->px || !a->py || !a->cx || !a->cy || !a->cv || !a->cov || !a->fnx || !a->fny ||
        !a->farea || !a->fcx || !a->fcy || !a->r11 || !a->r12 || !a->r22 || !a->v2c_wt)
        return fail(UNS_ERR_ARG, "uns_host_cc_mesh_vjp: null argument");
    std::string err;
    int rc = mesh_vjp_cc(m->mesh, *a, gpx, gpy, err);
    return rc ? fail(rc, err) : UNS_OK;
}

int uns_host_nc_airfoil(int ni, int nj, double t, double rfar, double dwall, uns_host_nc** out) {
    if (!out) return fail(UNS_ERR_ARG, "null out");
    AirfoilSpec s{ni, nj, t, rfar, dwall};
    auto* m = new uns_host_nc();
    std::string err;
    int rc = gen_airfoil_nc(s, m->raw, err);
    if (!rc) rc = geometric_nc(m->raw, m->mesh, err);
    if (rc) { delete m; return fail(rc, err); }
    *out = m;
    return UNS_OK;
}

int uns_host_cc_plot3d(const char* path, uns_host_cc** out) {
    if (!path || !out) return fail(UNS_ERR_ARG, "null argument");
    auto* m = new uns_host_cc();
    std::string err;
    int rc = read_plot3d_cc(path, m->raw, err);
    if (!rc) rc = geometric_cc(m->raw, m->mesh, err);
    if (rc) { delete m; return fail(rc, err); }
    *out = m;
    return UNS_OK;
}

int uns_host_nc_plot3d(const char* path, uns_host_nc** out) {
    if (!path || !out) return fail(UNS_ERR_ARG, "null argument");
    auto* m = new uns_host_nc();
    std::string err;
    int rc = read_plot3d_nc(path, m->raw, err);
    if (!rc) rc = geometric_nc(m->raw, m->mesh, err);
    if (rc) { delete m; return fail(rc, err); }
    *out = m;
    return UNS_OK;
}

int uns_host_airfoil_plot3d(int ni, int nj, double t, double rfar, double dwall, const char* path) {
    if (!path) return fail(UNS_ERR_ARG, "null path");
    AirfoilSpec s{ni, nj, t, rfar, dwall};
    std::string err;
    int rc = write_plot3d_airfoil(s, path, err);
    return rc ? fail(rc, err) : UNS_OK;
}

int uns_host_cc_read(const char* path, uns_host_cc** out) {
    if (!path || !out) return fail(UNS_ERR_ARG, "null argument");
    auto* m = new uns_host_cc();
    std::string err;
    int rc = read_geometry_cc(path, m->raw, err);
    if (!rc) rc = geometric_cc(m->raw, m->mesh, err);
    if (rc) { delete m; return fail(rc, err); }
    *out = m;
    return UNS_OK;
}

int uns_host_nc_read(const char* path, uns_host_nc** out) {
    if (!path || !out) return fail(UNS_ERR_ARG, "null argument");
    auto* m = new uns_host_nc();
    std::string err;
    int rc = read_geometry_nc(path, m->raw, err);
    if (!rc) rc = geometric_nc(m->raw, m->mesh, err);
    if (rc) { delete m; return fail(rc, err); }
    *out = m;
    return UNS_OK;
}

int uns_host_cc_write(const uns_host_cc* m, const char* path) {
    if (!m || !path) return fail(UNS_ERR_ARG, "null argument");
    std::string err;
    int rc = write_geometry_cc(path, m->raw, err);
    return rc ? fail(rc, err) : UNS_OK;
}

int uns_host_nc_write(const uns_host_nc* m, const char* path) {
    if (!m || !path) return fail(UNS_ERR_ARG, "null argument");
    std::string err;
    int rc = write_geometry_nc(path, m->raw, err);
    return rc ? fail(rc, err) : UNS_OK;
}

int uns_host_cc_view(const uns_host_cc* m, uns_cc_mesh* v) {
    if (!m || !v) return fail(UNS_ERR_ARG, "null argument");
    *v = m->mesh.view();
    return UNS_OK;
}

int uns_host_nc_view(const uns_host_nc* m, uns_nc_mesh* v) {
    if (!m || !v) return fail(UNS_ERR_ARG, "null argument");
    *v = m->mesh.view();
    return UNS_OK;
}

int uns_host_cc_newnum(const uns_host_cc* m, int32_t* out) {
    if (!m || !out) return fail(UNS_ERR_ARG, "null argument");
    std::copy(m->mesh.newnum.begin(), m->mesh.newnum.end(), out);
    return UNS_OK;
}

int uns_host_nc_newnum(const uns_host_nc* m, int32_t* out) {
    if (!m || !out) return fail(UNS_ERR_ARG, "null argument");
    std::copy(m->mesh.newnum.begin(), m->mesh.newnum.end(), out);
    return UNS_OK;
}

void uns_host_cc_free(uns_host_cc* m) { delete m; }
void uns_host_nc_free(uns_host_nc* m) { delete m; }

int uns_host_read_flo_cc(const char* path, uns_params* p, char* grid, int gridlen) {
    if (!path || !p) return fail(UNS_ERR_ARG, "null argument");
    std::string g, err;
    int rc = read_flo_inp_cc(path, *p, g, err);
    if (rc) return fail(rc, err);
    if (grid && gridlen > 0) { std::strncpy(grid, g.c_str(), gridlen - 1); grid[gridlen - 1] = 0; }
    return UNS_OK;
}

int uns_host_read_flo_nc(const char* path, uns_params* p, char* grid, int gridlen) {
    if (!path || !p) return fail(UNS_ERR_ARG, "null argument");
    std::string g, err;
    int rc = read_flo_inp_nc(path, *p, g, err);
    if (rc) return fail(rc, err);
    if (grid && gridlen > 0) { std::strncpy(grid, g.c_str(), gridlen - 1); grid[gridlen - 1] = 0; }
    return UNS_OK;
}

double uns_host_cfl_cc(const uns_params* p, int iter, double prev) {
    if (p->cfl_type == UNS_CFL_TANH) {
        double s = (double)iter / (double)(p->cfl_ramp_steps - 1);
        return 0.5 * p->cfl_max * (1.0 + std::tanh(s * 7.0 - 3.5));
    }
    if (iter <= p->cfl_ramp_steps) {
        double ef = 0.5;
        double s = (double)iter / (double)p->cfl_ramp_steps;
        return p->cfl_min + (p->cfl_max - p->cfl_min) * (1.0 - std::exp(-(s * ef))) / (1.0 - std::exp(-ef));
    }
    return prev;
}

double uns_host_cfl_nc(const uns_params* p, int iter) {
    return 0.5 * p->cfl_max * (1.0 + std::tanh((double)iter * 7.0 / 500.0 - 3.5));
}

int uns_host_save_flow(const char* path, const double* qc, int n) {
    if (!path || !qc || n < 0) return fail(UNS_ERR_ARG, "uns_host_save_flow: bad argument");
    FILE* f = std::fopen(path, "w");
    if (!f) return fail(UNS_ERR_IO, std::string("cannot write ") + path);
    for (int i = 0; i < n; ++i)  // write(50,'(4e20.10)') qc(1:nvar)
        std::fprintf(f, "%s%s%s%s\n", fort_e(qc[4 * i], 20, 10).c_str(), fort_e(qc[4 * i + 1], 20, 10).c_str(),
                     fort_e(qc[4 * i + 2], 20, 10).c_str(), fort_e(qc[4 * i + 3], 20, 10).c_str());
    return std::fclose(f) == 0 ? UNS_OK : fail(UNS_ERR_IO, std::string("cannot write ") + path);
}

int uns_host_read_flow(const char* path, double* qc, int n) {
    if (!path || !qc || n < 0) return fail(UNS_ERR_ARG, "uns_host_read_flow: bad argument");
    FILE* f = std::fopen(path, "r");
    if (!f) return fail(UNS_ERR_IO, std::string("cannot open ") + path);
    for (int i = 0; i < 4 * n; ++i) {  // list-directed read(50,*): Fortran E or D exponents
        char tok[64];
        if (std::fscanf(f, "%63s", tok) != 1) {
            std::fclose(f);
            return fail(UNS_ERR_IO, std::string(path) + ": fewer than " + std::to_string(n) + " states");
        }
        for (char* c = tok; *c; ++c)
            if (*c == 'D' || *c == 'd') *c = 'e';
        char* end = nullptr;
        qc[i] = std::strtod(tok, &end);
        if (end == tok || *end) {
            std::fclose(f);
            return fail(UNS_ERR_IO, std::string(path) + ": bad number '" + tok + "'");
        }
    }
    std::fclose(f);
    return UNS_OK;
}

int uns_host_sweep_schedule(int n, const int32_t* nbr_off, const int32_t* nbr, int nwarps, int32_t* off, int32_t* items,
                            int32_t* levels) {
    if (n < 0 || nwarps < 1 || !nbr_off || (n > 0 && !nbr) || !off || (n > 0 && !items) || !levels)
        return fail(UNS_ERR_ARG, "uns_host_sweep_schedule: bad argument");
    if (nbr_off[0] != 0) return fail(UNS_ERR_ARG, "uns_host_sweep_schedule: nbr_off[0] != 0");
    for (int i = 0; i < n; ++i)
        if (nbr_off[i + 1] < nbr_off[i]) return fail(UNS_ERR_ARG, "uns_host_sweep_schedule: nbr_off decreases");
    const uns::WarpSchedule ws = uns::list_schedule(n, nbr_off, nbr, nwarps);
    std::copy(ws.off.begin(), ws.off.end(), off);
    std::copy(ws.items.begin(), ws.items.end(), items);
    levels[0] = ws.nlev_fwd;
    levels[1] = ws.nlev_bwd;
    return UNS_OK;
}

}  // extern "C"
