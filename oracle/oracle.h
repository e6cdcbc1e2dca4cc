/*
 * oracle.h -- TEST INFRASTRUCTURE ONLY.  CPU oracle for the UNSFlow2D hot path.
 *
 * A serial C++ restatement of the reference Fortran routines on the
 * residual-and-update path (CCFVM and NCFVM), written loop for loop in the
 * reference's own order (face loops that scatter into cells/nodes).  Only the
 * test-suite, __graft_entry__.smoke() and bench.py's CPU-baseline leg use it,
 * always as the checker; the product library never links it.
 *
 * PARITY UNPINNED: the reference ships no tests, fixtures or golden vectors,
 * and it cannot be compiled here (no Fortran compiler in this image; NCFVM
 * also carries unresolved merge-conflict markers).  The oracle is checked
 * against analytic known answers instead (freestream preservation, flux
 * consistency, exact linear gradients, conservation) -- see tests/.
 */
#ifndef UNS_ORACLE_H
#define UNS_ORACLE_H
#include "unsflow_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct oracle_cc oracle_cc;
typedef struct oracle_nc oracle_nc;

/* ------------------------------------------------------------ CCFVM */
oracle_cc* oracle_cc_create(const uns_cc_mesh* m, const uns_params* p);
void oracle_cc_free(oracle_cc* o);
int oracle_cc_initialize(oracle_cc* o);                 /* solution.F90:18-84 */
int oracle_cc_set_state(oracle_cc* o, const double* qc);/* [noc+nbf][4]          */
int oracle_cc_con2prim(oracle_cc* o);                   /* main.F90:62-67        */
int oracle_cc_avg_c2v(oracle_cc* o);                    /* average.F90:1-39      */
int oracle_cc_time_step(oracle_cc* o, double cfl, double* dtglobal); /* timestep.F90:28-107 */
int oracle_cc_save_old(oracle_cc* o);                   /* solution.F90:118-132  */
int oracle_cc_gradient(oracle_cc* o);                   /* gradient.F90 (+limit) */
int oracle_cc_limit(oracle_cc* o);                      /* limiter.F90:3-17,123-296 */
int oracle_cc_fvresidual(oracle_cc* o);                 /* fvresidual.F90:4-187  */
int oracle_cc_rk_stage(oracle_cc* o, int irk);          /* main.F90:90-101       */
int oracle_cc_lusgs(oracle_cc* o);                      /* lusgs.F90:207-379     */
int oracle_cc_check_positivity(oracle_cc* o, int* bad); /* main.F90:358-414      */
int oracle_cc_residue(oracle_cc* o, double* fres_raw);  /* solution.F90:136-180  */
int oracle_cc_forces(oracle_cc* o, double* fx1, double* fy1);
/* One full iteration of main.F90:57-117 (cfl given). */
int oracle_cc_iteration(oracle_cc* o, double cfl, double* fres_raw);
int oracle_cc_get(oracle_cc* o, int field, double* out);
/* Test hook: overwrite QC, QP (all cells incl. ghosts), GRAD or PHI. */
int oracle_cc_set(oracle_cc* o, int field, const double* in);
/* find_cl_cd (main.F90:263-355): coef[5] = C_L, C_D (wall integral), C_m,
 * C_L, C_D (flux-based); wall [nwall][4] = x, y, -cp, cf (may be NULL). */
int oracle_cc_find_cl_cd(oracle_cc* o, double xref, double yref, double* coef, double* wall, int* nwall);
/* screen's min/max diagnostics (main.F90:187-221): out[14]. */
int oracle_cc_screen_minmax(oracle_cc* o, double* out);
/* tecplt's vertex table (main.F90:417-480) after avg_c2v: out[nop][11]. */
int oracle_cc_tecplt(oracle_cc* o, double* out);

/* Complex-step instance of the CCFVM oracle (oracle_cc_cs.cpp): the same
 * routines on a complex scalar whose branches follow the real part.  Inputs
 * carry re + i*im; for im = h*u with h ~ 1e-30, Im(output)/h is the exact
 * directional derivative.  aoa_im adds i*aoa_im to the angle of attack (rad). */
typedef struct oracle_cc_cs oracle_cc_cs;
oracle_cc_cs* oracle_cc_cs_create(const uns_cc_mesh* m, const uns_params* p, double aoa_im);
void oracle_cc_cs_free(oracle_cc_cs* o);
/* UNS_CC_QC [noc+nbf][4], UNS_CC_QP [noc+nbf][5], UNS_CC_PHI [noc][4]; im may be NULL. */
int oracle_cc_cs_set(oracle_cc_cs* o, int field, const double* re, const double* im);
/* UNS_CC_QC or UNS_CC_QP. */
int oracle_cc_cs_get(oracle_cc_cs* o, int field, double* re, double* im);
/* One RK3 main-loop iteration (as oracle_cc_iteration, without the norm). */
int oracle_cc_cs_iteration(oracle_cc_cs* o, double cfl);
/* Hold the RK update's dt / cv real (dt = real(dt / cv) * cv), as the
   adjoint holds it fixed; off by default. */
int oracle_cc_cs_freeze_dt(oracle_cc_cs* o, int on);
/* Imaginary parts of one geometric array (field: index in uns_cc_mesh_adj
   order px, py, cx, cy, cv, cov, fnx, fny, farea, fcx, fcy, r11, r12, r22,
   v2c_wt), real parts kept. */
int oracle_cc_cs_set_geometry_im(oracle_cc_cs* o, int field, const double* im);
/* Fx1, Fy1 of the last residual: fx[0] + i fx[1], fy[0] + i fy[1]. */
int oracle_cc_cs_forces(oracle_cc_cs* o, double* fx, double* fy);

/* ------------------------------------------------------------ NCFVM */
oracle_nc* oracle_nc_create(const uns_nc_mesh* m, const uns_params* p);
void oracle_nc_free(oracle_nc* o);
int oracle_nc_initialize(oracle_nc* o);                 /* NCFVM/common.f90:19-54 */
int oracle_nc_set_state(oracle_nc* o, const double* qc);
int oracle_nc_save_old(oracle_nc* o);                   /* common.f90:88-104      */
int oracle_nc_fvresidual(oracle_nc* o, double cfl);     /* fvresidual.f90:4-85    */
int oracle_nc_rk_stage(oracle_nc* o, int irk);          /* main.f90:59-80       */
int oracle_nc_lusgs(oracle_nc* o, double cfl);          /* lusgs.f90:4-157        */
int oracle_nc_residue(oracle_nc* o, double* fres_raw, double* fresi, int* iresi); /* common.f90:108-154 */
/* tecplt's vertex table (NCFVM/main.f90:190-233): out[nop][7]; screen's
 * min/max (NCFVM/main.f90:115-187): out[12]. */
int oracle_nc_tecplt(oracle_nc* o, double* out);
int oracle_nc_screen_minmax(oracle_nc* o, double* out);
int oracle_nc_iteration(oracle_nc* o, double cfl, double* fres_raw, double* fresi);
int oracle_nc_get(oracle_nc* o, int field, double* out);
/* Test hook: overwrite QC, QP, GRAD or PHI. */
int oracle_nc_set(oracle_nc* o, int field, const double* in);

#ifdef __cplusplus
}
#endif
#endif
