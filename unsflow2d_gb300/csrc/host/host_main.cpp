// host_main.cpp -- the C++ mirror of the reference main programs
// (uns_host_cc_main, uns_host_nc_main in unsflow_host.h), built into
// libunsflow_driver.so: they read flo.inp and the geometry through
// libunsflow_host.so and drive the hot path through libunsflow_gpu.so.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "host_mesh.hpp"
#include "unsflow_gpu.h"
#include "unsflow_host.h"

using namespace unshost;

extern "C" {

int uns_host_cc_main(const char* flo_inp, const char* outdir, int mode, int* iters_out, double* fres_out) {
    if (!flo_inp || !outdir) return fail(UNS_ERR_ARG, "null argument");
    uns_params P;
    std::string grid, err;
    int rc = read_flo_inp_cc(flo_inp, P, grid, err);
    if (rc) return fail(rc, err);
    RawCC raw;
    MeshCC mesh;
    if ((rc = read_geometry_cc(join(dir_of(flo_inp), grid), raw, err)) || (rc = geometric_cc(raw, mesh, err))) return fail(rc, err);
    uns_cc_mesh view = mesh.view();
    uns_cc_handle* h = nullptr;
    if ((rc = uns_cc_create(&view, &P, &h))) return fail(rc, uns_last_error());
    const int nst = view.noc + view.nbf;
    std::vector<double> state(4 * (size_t)nst);
    if (P.istart == 2) {  // read_flow (CCFVM/solution.F90:103-114): interior cells
        fail(UNS_OK, "");
        if ((rc = uns_cc_get_state(h, state.data())) ||
            (rc = uns_host_read_flow(join(dir_of(flo_inp), "FLO.DAT").c_str(), state.data(), view.noc)) ||
            (rc = uns_cc_set_state(h, state.data()))) {
            std::string e = std::string(uns_host_last_error()).empty() ? std::string(uns_last_error()) : std::string(uns_host_last_error());
            uns_cc_destroy(h);
            return fail(rc, e);
        }
    }
    std::string res_path = std::string(outdir) + "/FLO.RES";
    FILE* fo = std::fopen(res_path.c_str(), "w");
    if (!fo) { uns_cc_destroy(h); return fail(UNS_ERR_IO, "cannot write " + res_path); }
    int iter = 0;
    double fres = 1.0, fres1 = 0.0, cfl = 0.0;
    const double eps = 2.220446049250313e-16;
    while (iter < P.max_iter && fres > P.min_res) {
        if (mode == 0) {
            ++iter;
            cfl = uns_host_cfl_cc(&P, iter, cfl);
            double raw_f;
            int bad;
            if ((rc = uns_cc_con2prim(h)) || (rc = uns_cc_avg_c2v(h)) || (rc = uns_cc_time_step(h, cfl, nullptr)) ||
                (rc = uns_cc_save_old(h)) || (rc = uns_cc_gradient(h)))
                break;
            if (P.time_mode == UNS_TIME_RK3) {
                for (int irk = 1; irk <= 3 && !rc; ++irk)
                    if (!(rc = uns_cc_fvresidual(h))) rc = uns_cc_rk_stage(h, irk);
            } else {
                rc = uns_cc_lusgs(h);
            }
            if (rc || (rc = uns_cc_check_positivity(h, &bad)) || (rc = uns_cc_residue(h, &raw_f))) break;
            if (iter == 1) fres1 = raw_f;
            fres = (fres1 >= eps) ? raw_f / fres1 : raw_f;
            std::fprintf(fo, "%6d%s%s\n", iter, fort_e(std::log10(fres), 16, 6).c_str(), fort_e(cfl, 16, 6).c_str());
        } else {
            int chunk = std::min(200, P.max_iter - iter);
            std::vector<double> cf(chunk), fr(chunk);
            double c = cfl;
            for (int k = 0; k < chunk; ++k) { c = uns_host_cfl_cc(&P, iter + 1 + k, c); cf[k] = c; }
            int done = 0;
            rc = uns_cc_iterate(h, chunk, cf.data(), iter == 0 ? 1 : 0, fr.data(), &done);
            for (int k = 0; k < done; ++k) {
                ++iter;
                cfl = cf[k];
                if (iter == 1) fres1 = fr[k];
                fres = (fres1 >= eps) ? fr[k] / fres1 : fr[k];
                std::fprintf(fo, "%6d%s%s\n", iter, fort_e(std::log10(fres), 16, 6).c_str(), fort_e(cfl, 16, 6).c_str());
            }
            if (rc || done < chunk) break;
        }
    }
    std::fclose(fo);
    fail(UNS_OK, "");
    if (!rc && !(rc = uns_cc_get_state(h, state.data())))  // save_flow (CCFVM/solution.F90:88-99)
        rc = uns_host_save_flow((std::string(outdir) + "/FLO.DAT").c_str(), state.data(), view.noc);
    std::string e = rc ? (std::string(uns_host_last_error()).empty() ? std::string(uns_last_error()) : std::string(uns_host_last_error())) : std::string();
    uns_cc_destroy(h);
    if (iters_out) *iters_out = iter;
    if (fres_out) *fres_out = fres;
    return rc ? fail(rc, e) : UNS_OK;
}

int uns_host_nc_main(const char* flo_inp, const char* outdir, int mode, int* iters_out, double* fres_out) {
    if (!flo_inp || !outdir) return fail(UNS_ERR_ARG, "null argument");
    uns_params P;
    std::string grid, err;
    int rc = read_flo_inp_nc(flo_inp, P, grid, err);
    if (rc) return fail(rc, err);
    RawNC raw;
    MeshNC mesh;
    if ((rc = read_geometry_nc(join(dir_of(flo_inp), grid), raw, err)) || (rc = geometric_nc(raw, mesh, err))) return fail(rc, err);
    uns_nc_mesh view = mesh.view();
    uns_nc_handle* h = nullptr;
    if ((rc = uns_nc_create(&view, &P, &h))) return fail(rc, uns_last_error());
    std::vector<double> state(4 * (size_t)view.nop);
    if (P.istart == 2) {  // read_flow (NCFVM/common.f90:73-84)
        fail(UNS_OK, "");
        if ((rc = uns_host_read_flow(join(dir_of(flo_inp), "FLO.DAT").c_str(), state.data(), view.nop)) ||
            (rc = uns_nc_set_state(h, state.data()))) {
            std::string e = std::string(uns_host_last_error()).empty() ? std::string(uns_last_error()) : std::string(uns_host_last_error());
            uns_nc_destroy(h);
            return fail(rc, e);
        }
    }
    std::string res_path = std::string(outdir) + "/FLO.RES";
    FILE* fo = std::fopen(res_path.c_str(), "w");
    if (!fo) { uns_nc_destroy(h); return fail(UNS_ERR_IO, "cannot write " + res_path); }
    int iter = 0;
    double fres = 1.0, fres1 = 0.0;
    while (iter < P.max_iter && fres > P.min_res) {
        if (mode == 0) {
            ++iter;
            double cfl = uns_host_cfl_nc(&P, iter), raw_f, fresi;
            if ((rc = uns_nc_save_old(h))) break;
            if (P.time_mode == UNS_TIME_RK3) {
                for (int irk = 1; irk <= 3 && !rc; ++irk)
                    if (!(rc = uns_nc_fvresidual(h, cfl))) rc = uns_nc_rk_stage(h, irk);
            } else {
                rc = uns_nc_lusgs(h, cfl);
            }
            if (rc || (rc = uns_nc_residue(h, &raw_f, &fresi, nullptr))) break;
            if (iter == 1) fres1 = raw_f;
            fres = (fres1 != 0.0) ? raw_f / fres1 : raw_f;
            std::fprintf(fo, "%6d%s%s%s\n", iter, fort_e(std::log10(fres), 16, 6).c_str(),
                         fort_e(std::log10(fresi), 16, 6).c_str(), fort_e(cfl, 16, 6).c_str());
        } else {
            int chunk = std::min(200, P.max_iter - iter);
            std::vector<double> cf(chunk), fr(chunk), fi(chunk);
            for (int k = 0; k < chunk; ++k) cf[k] = uns_host_cfl_nc(&P, iter + 1 + k);
            int done = 0;
            rc = uns_nc_iterate(h, chunk, cf.data(), iter == 0 ? 1 : 0, fr.data(), fi.data(), &done);
            for (int k = 0; k < done; ++k) {
                ++iter;
                if (iter == 1) fres1 = fr[k];
                fres = (fres1 != 0.0) ? fr[k] / fres1 : fr[k];
                std::fprintf(fo, "%6d%s%s%s\n", iter, fort_e(std::log10(fres), 16, 6).c_str(),
                             fort_e(std::log10(fi[k]), 16, 6).c_str(), fort_e(cf[k], 16, 6).c_str());
            }
            if (rc || done < chunk) break;
        }
    }
    std::fclose(fo);
    fail(UNS_OK, "");
    if (!rc && !(rc = uns_nc_get_state(h, state.data())))  // save_flow (NCFVM/common.f90:58-69)
        rc = uns_host_save_flow((std::string(outdir) + "/FLO.DAT").c_str(), state.data(), view.nop);
    std::string e = rc ? (std::string(uns_host_last_error()).empty() ? std::string(uns_last_error()) : std::string(uns_host_last_error())) : std::string();
    uns_nc_destroy(h);
    if (iters_out) *iters_out = iter;
    if (fres_out) *fres_out = fres;
    return rc ? fail(rc, e) : UNS_OK;
}

}  // extern "C"
