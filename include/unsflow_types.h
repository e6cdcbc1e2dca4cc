/*
 * unsflow_types.h -- plain-C types shared by the UNSFlow2D GB300 drop-in library
 * (libunsflow_gpu.so), the caller-side host library (libunsflow_host.so) and the
 * CPU oracle.  No C++ or CUDA types appear here, so a Fortran iso_c_binding
 * module can mirror every struct field for field.
 *
 * Index convention: every index in these structs is 0-based.  A Fortran caller
 * subtracts 1 from cell/face/point numbers when it fills a view.
 */
#ifndef UNSFLOW_TYPES_H
#define UNSFLOW_TYPES_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The reference prints a message and `stop`s on these
 * conditions (CCFVM/roe_flux.F90:73-87 negative Roe sound speed,
 * CCFVM/main.F90:384-411 non-positive density/pressure, CCFVM/geometric.F90
 * mesh checks); the library returns the code instead and never traps. */
enum {
    UNS_OK = 0,
    UNS_ERR_ARG = 1,             /* bad argument / option                   */
    UNS_ERR_CUDA = 2,            /* CUDA runtime error                      */
    UNS_ERR_NEG_SOUND_SPEED = 3, /* Roe-averaged a^2 <= 0                   */
    UNS_ERR_NONPOSITIVE = 4,     /* density or pressure <= 0                */
    UNS_ERR_MESH = 5,            /* inconsistent mesh / negative volume     */
    UNS_ERR_TIMEOUT = 6,         /* a bounded device wait gave up           */
    UNS_ERR_NAN = 7,             /* non-finite residual norm                */
    UNS_ERR_IO = 8,              /* file could not be read / written        */
    UNS_ERR_NOMEM = 9            /* allocation failed                       */
};

/* flo.inp option values (CCFVM/read_input.F90:31-50). */
enum { UNS_FLOW_INVISCID = 0, UNS_FLOW_LAMINAR = 1 };
enum { UNS_FLUX_ROE = 0, UNS_FLUX_AUSM = 1, UNS_FLUX_VANLEER = 2, UNS_FLUX_RUSANOV = 3 };
enum { UNS_GRAD_GG = 0, UNS_GRAD_GGFC = 1, UNS_GRAD_LSQR = 2 };
enum { UNS_TIME_RK3 = 0, UNS_TIME_LUSGS = 1 };
enum { UNS_CFL_TANH = 0, UNS_CFL_RAMP = 1 };
/* NCFVM limiter: limiter_VKN (NCFVM/limiter.f90:15-98) or limiter_min_max
 * (Barth-Jespersen, NCFVM/limiter.f90:192-260).  limiter_min_max projects
 * the fp2 gradient with +1/2 (limiter.f90:241), i.e. toward the wrong face
 * side, and the solve then diverges; UNS_LIM_BARTH_CORRECTED uses -1/2 there,
 * as limiter_VKN does (limiter.f90:71). */
enum { UNS_LIM_VKN = 0, UNS_LIM_BARTH = 1, UNS_LIM_BARTH_CORRECTED = 2 };
/* Arithmetic form.  UNS_PREC_FP64: FP64 everywhere (the reference's).
 * UNS_PREC_MIXED: FP32 face reconstruction and flux arithmetic, in the
 * residual and in the LU-SGS sweeps; FP64 residual accumulation, norm, dt and
 * LU-SGS diagonal inversion.  Its residual floors near a 1e-5 drop (FP32
 * rounding of the near-cancelling fluxes).  UNS_PREC_MIXED_SWEEP: FP64
 * residual, FP32 flux arithmetic only inside the LU-SGS sweeps (the implicit
 * operator), so the solve converges as far as the FP64 one. */
enum { UNS_PREC_FP64 = 0, UNS_PREC_MIXED = 1, UNS_PREC_MIXED_SWEEP = 2 };
/* Objectives of the discrete adjoint: the flux-based force coefficients
 * C_L = 2 (Fy1 cos a - Fx1 sin a), C_D = 2 (Fx1 cos a + Fy1 sin a)
 * (CCFVM/main.F90:348-353). */
enum { UNS_OBJ_CL = 0, UNS_OBJ_CD = 1 };

/* Field identifiers for the state accessors (uns_cc_get_field,
 * uns_nc_get_field).  Layouts are row-major with the variable index fastest,
 * i.e. the memory order of the Fortran component arrays (cell(i)%qc(1:4),
 * cell(i)%grad(1:2,1:4), ...). */
enum {
    UNS_CC_QC = 0,     /* [noc+nbf][4]  E, rho, rho*u, rho*v                 */
    UNS_CC_QP = 1,     /* [noc+nbf][5]  rho, u, v, p, T                      */
    UNS_CC_QOLD = 2,   /* [noc][4]                                           */
    UNS_CC_RES = 3,    /* [noc][4]                                           */
    UNS_CC_GRAD = 4,   /* [noc][4][2]   d/dx, d/dy of rho, u, v, p           */
    UNS_CC_PHI = 5,    /* [noc][4]                                           */
    UNS_CC_DT = 6,     /* [noc]                                              */
    UNS_CC_LA = 7,     /* [noc]         cell spectral radius                 */
    UNS_CC_PTPRIM = 8, /* [nop][5]      vertex-averaged primitives           */
    UNS_CC_FQP = 9,    /* [nfi+nbf][5]  face-averaged primitives             */
    UNS_CC_FLA = 10,   /* [nfi+nbf]     face spectral radius                 */
    UNS_CC_FMU = 11,   /* [nfi+nbf]     face viscosity                       */
    UNS_CC_FGRAD = 12, /* [nfi+nbf][5][2] diamond-path face gradients        */
    UNS_CC_MUL = 13,   /* [noc]         Sutherland viscosity                 */
    UNS_CC_FWALL = 14  /* [nbf][4]      wall force terms of the last residual:
                        *               convective (x, y), viscous (x, y);
                        *               Fx1 = sum(conv x - visc x) over walls */
};
enum {
    UNS_NC_QC = 0,     /* [nop][4] */
    UNS_NC_QP = 1,     /* [nop][4] */
    UNS_NC_QOLD = 2,   /* [nop][4] */
    UNS_NC_RES = 3,    /* [nop][4] */
    UNS_NC_GRAD = 4,   /* [nop][4][2] */
    UNS_NC_PHI = 5,    /* [nop][4] */
    UNS_NC_DT = 6,     /* [nop] */
    UNS_NC_LA = 7,     /* [nop] */
    UNS_NC_FLA = 8     /* [nof] */
};

/* Solver parameters: the fields of flo.inp that the hot path reads. */
typedef struct {
    double m_inf;        /* Mach                                           */
    double aoa_deg;      /* AOA [deg]                                       */
    double rey;          /* Reynolds                                        */
    double t_wall;       /* FlowType wall temperature [K] (divided by 300)  */
    int32_t flow_type;   /* UNS_FLOW_*                                      */
    int32_t iwall;       /* 0 isothermal, 1 adiabatic                       */
    int32_t flux_type;   /* UNS_FLUX_*                                      */
    int32_t grad_type;   /* UNS_GRAD_* (CC)                                 */
    int32_t ilimit;      /* 0/1                                             */
    int32_t irs;         /* 0/1 implicit residual smoothing (CC)            */
    int32_t time_mode;   /* UNS_TIME_*                                      */
    int32_t cfl_type;    /* UNS_CFL_* (CC)                                  */
    double cfl_min;      /* CFL line, 2nd value (CC ramp)                   */
    double cfl_max;      /* CFL line, 3rd value (NC: the only value)        */
    int32_t cfl_ramp_steps;
    int32_t limiter_type;/* UNS_LIM_* (NC)                                  */
    int32_t precision;   /* UNS_PREC_*                                      */
    int32_t max_iter;    /* MaxIter                                         */
    double min_res;      /* MinRes                                          */
    int32_t scr_interval;/* ScrInt                                          */
    int32_t istart;      /* Start: 1 scratch, 2 restart from FLO.DAT        */
} uns_params;

/* Cell-centred mesh after the caller's geometric preprocessing
 * (CCFVM/geometric.F90:1-1013).  Cells [0,noc) are interior, cells
 * [noc, noc+nbf) are the ghost cells of boundary faces [nfi, nfi+nbf).
 * Faces [0,nfi) are interior faces, faces [nfi, nfi+nbf) boundary faces;
 * the unit normal points from `in` to `out`. */
typedef struct {
    int32_t nop, noc, nfi, nbf;
    const double *px, *py;                 /* [nop]                         */
    const double *cx, *cy;                 /* [noc+nbf] centroids           */
    const double *cv;                      /* [noc] cell area               */
    const double *cov;                     /* [noc] cell co-volume          */
    const int32_t *fp1, *fp2;              /* [nfi+nbf] face end points     */
    const int32_t *fin, *fout;             /* [nfi+nbf]                     */
    const int32_t *fbc;                    /* [nfi+nbf] 0, 1001 wall, 2001 farfield */
    const double *fnx, *fny, *farea;       /* [nfi+nbf]                     */
    const double *fcx, *fcy;               /* [nfi+nbf] face midpoint       */
    const double *r11, *r12, *r22;         /* [noc] LSQ QR coefficients     */
    const int32_t *nc2c;                   /* [noc] interior neighbour count*/
    const int32_t *c2f_off, *c2f;          /* CSR [noc+1], reference order  */
    const int32_t *v2c_off, *v2c;          /* CSR [nop+1], cells incl ghosts*/
    const double *v2c_wt;                  /* pseudo-Laplacian weights      */
} uns_cc_mesh;

/* Adjoints (dJ/d array) of the geometric arrays of a uns_cc_mesh, in the same
 * layout: written by uns_cc_adjoint_geometry, read by uns_host_cc_mesh_vjp. */
typedef struct {
    double *px, *py;                       /* [nop]                         */
    double *cx, *cy;                       /* [noc+nbf]                     */
    double *cv, *cov;                      /* [noc]                         */
    double *fnx, *fny, *farea;             /* [nfi+nbf]                     */
    double *fcx, *fcy;                     /* [nfi+nbf]                     */
    double *r11, *r12, *r22;               /* [noc]                         */
    double *v2c_wt;                        /* [v2c_off[nop]]                */
} uns_cc_mesh_adj;

/* Vertex-centred median-dual mesh after the caller's geometric
 * preprocessing (NCFVM/geometric.f90:1-806).  Faces are mesh edges; the
 * dual-face unit normal points from fp1's dual cell to fp2's. */
typedef struct {
    int32_t nop, noc, nof, pad_;
    const double *px, *py;                 /* [nop]                         */
    const double *cv;                      /* [nop] median-dual volume      */
    const int32_t *fp1, *fp2, *fbc;        /* [nof]                         */
    const double *fnx, *fny, *farea;       /* [nof] dual face               */
    const int32_t *v2v_off, *v2v;          /* CSR [nop+1]                   */
    const double *wx, *wy;                 /* LSQ weights per v2v entry     */
    const int32_t *v2f_off, *v2f;          /* CSR [nop+1], reference order  */
} uns_nc_mesh;

#ifdef __cplusplus
}
#endif
#endif /* UNSFLOW_TYPES_H */
