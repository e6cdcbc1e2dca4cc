/*
 * unsflow_host.h -- C-ABI of libunsflow_host.so, the caller side of the drop-in.
 *
 * The reference keeps the Fortran driver, flo.inp and geometry.inp as they
 * are and replaces only the hot-path subroutines.  For hosts without a
 * Fortran compiler the caller side is also provided in C++:
 * the geometry.inp readers and the geometric preprocessing restated from
 * CCFVM/geometric.F90 and NCFVM/geometric.f90 (connectivity orders matter:
 * they fix summation and LU-SGS sweep order), a flo.inp reader, an analytic
 * airfoil O-mesh generator (the reference ships no meshes), and a driver that
 * runs the reference main loop through the libunsflow_gpu.so entry points.
 */
#ifndef UNSFLOW_HOST_H
#define UNSFLOW_HOST_H
#include "unsflow_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct uns_host_cc uns_host_cc; /* raw + preprocessed CC mesh */
typedef struct uns_host_nc uns_host_nc; /* raw + preprocessed NC mesh */

const char* uns_host_last_error(void);

/* Symmetric 4-digit-thickness airfoil O-mesh: ni circumferential x nj radial
 * quads, each split into two triangles; farfield circle of radius rfar chords
 * about mid-chord; geometric radial spacing from dwall at the wall. */
int uns_host_cc_airfoil(int ni, int nj, double thickness, double rfar, double dwall, uns_host_cc** out);
int uns_host_nc_airfoil(int ni, int nj, double thickness, double rfar, double dwall, uns_host_nc** out);
/* The CCFVM airfoil mesh with wall node i (the point of index i, at the
 * surface parameter 2 pi i / ni from the trailing edge over the upper
 * surface) displaced by dy[i] in y, its radial line following with weight
 * 1 - s (s = 0 at the wall, 1 at the farfield): the shape perturbations of
 * the adjoint's wall-node and Hicks-Henne derivatives. */
int uns_host_cc_airfoil_dy(int ni, int nj, double thickness, double rfar, double dwall, const double* dy,
                           uns_host_cc** out);
/* The mesh m with its nodes moved to (px, py) [nop]: same topology, cell
 * centroids and areas of the moved triangles, then geometric (triangle cells
 * only; UNS_ERR_MESH otherwise or for a degenerate cell). */
int uns_host_cc_moved(const uns_host_cc* m, const double* px, const double* py, uns_host_cc** out);
/* Transpose of geometric (cell_face_norm, face_co_volume, LSQR_Coeff,
 * pseudo_Laplacian, the ghost mirror) and of the triangles' centroids and
 * areas: given the adjoints `a` of m's mesh arrays (uns_cc_adjoint_geometry),
 * writes dJ/dpx, dJ/dpy [nop].  UNS_ERR_MESH when m's arrays are not those of
 * its triangles. */
int uns_host_cc_mesh_vjp(const uns_host_cc* m, const uns_cc_mesh_adj* a, double* gpx, double* gpy);
/* geometry.inp readers (CCFVM/read_input.F90:123-213, NCFVM/read_input.f90:
 * 479-512) followed by geometric. */
int uns_host_cc_read(const char* path, uns_host_cc** out);
int uns_host_nc_read(const char* path, uns_host_nc** out);
/* MeshGen's input (MeshGen/SolverInputMESH.f90:56-67): a single-block
 * formatted plot3d O-grid (nbk; nx ny nz; x, y, z with i fastest; the last i
 * column repeats the first; j = 1 on the wall, j = ny on the farfield), its
 * quads split into triangles as the airfoil generator splits them, preprocessed
 * for either solver (the reference's MeshGen writes NCFVM quads only). */
int uns_host_cc_plot3d(const char* path, uns_host_cc** out);
int uns_host_nc_plot3d(const char* path, uns_host_nc** out);
/* The airfoil generator's O-grid written in that plot3d layout. */
int uns_host_airfoil_plot3d(int ni, int nj, double thickness, double rfar, double dwall, const char* path);
/* Write the raw (file) form in the reference's geometry.inp layout. */
int uns_host_cc_write(const uns_host_cc* m, const char* path);
int uns_host_nc_write(const uns_host_nc* m, const char* path);
/* Views of the preprocessed mesh (pointers valid until the free call). */
int uns_host_cc_view(const uns_host_cc* m, uns_cc_mesh* view);
int uns_host_nc_view(const uns_host_nc* m, uns_nc_mesh* view);
/* Renumbering map: file index (0-based) -> index after geometric. */
int uns_host_cc_newnum(const uns_host_cc* m, int32_t* out);  /* [noc] */
int uns_host_nc_newnum(const uns_host_nc* m, int32_t* out);  /* [nop] */
void uns_host_cc_free(uns_host_cc* m);
void uns_host_nc_free(uns_host_nc* m);

/* Test hook (no reference counterpart): the LU-SGS sweeps' warp schedule as
 * uns_cc_create / uns_nc_create build it (the forward and backward sweeps of
 * CCFVM/lusgs.F90:245-318 and NCFVM/lusgs.f90:48-124 as one dependency
 * graph), for n entities with CSR neighbour lists nbr_off[n+1] / nbr
 * (entries outside [0, n) ignored) on nwarps warps: off[nwarps+1] offsets
 * into items[2n], each item (entity << 1) | pass (pass 0 forward, 1
 * backward), in each warp's execution order; levels[2] = the dependency
 * levels of the forward and backward sweeps. */
int uns_host_sweep_schedule(int n, const int32_t* nbr_off, const int32_t* nbr, int nwarps, int32_t* off, int32_t* items,
                            int32_t* levels);

/* flo.inp readers.  `grid` receives the GridFile value (up to gridlen-1
 * characters). */
int uns_host_read_flo_cc(const char* path, uns_params* p, char* grid, int gridlen);
int uns_host_read_flo_nc(const char* path, uns_params* p, char* grid, int gridlen);

/* CFL schedules: cfl_number (CCFVM/main.F90:148-168; `prev` is the value kept
 * when the ramp is over) and the fixed tanh ramp of NCFVM/main.f90:54. */
double uns_host_cfl_cc(const uns_params* p, int iter, double prev);
double uns_host_cfl_nc(const uns_params* p, int iter);

/* save_flow / read_flow (CCFVM/solution.F90:88-114, NCFVM/common.f90:58-84):
 * the conserved state of the first n cells (nodes), one '(4e20.10)' line
 * each, as [n][4] row-major.  The reference defines them but never calls
 * them; uns_host_*_main reads FLO.DAT from flo.inp's directory when flo.inp's
 * Start is 2 and writes FLO.DAT into outdir at the end of the run. */
int uns_host_save_flow(const char* path, const double* qc, int n);
int uns_host_read_flow(const char* path, double* qc, int n);

/* The reference main program (CCFVM/main.F90:4-170, NCFVM/main.f90:4-112)
 * on the GPU library; exported by libunsflow_driver.so (every other function
 * here by libunsflow_host.so, which needs no GPU library): reads flo.inp, the geometry named there (relative to
 * flo.inp's directory), runs to MaxIter / MinRes and writes FLO.RES into
 * outdir.  mode 0 calls one entry point per reference subroutine each
 * iteration; mode 1 uses the graph-replayed uns_*_iterate fast path.
 * iters_out / fres_out (may be NULL) receive the iteration count and the
 * final normalised residual. */
int uns_host_cc_main(const char* flo_inp, const char* outdir, int mode, int* iters_out, double* fres_out);
int uns_host_nc_main(const char* flo_inp, const char* outdir, int mode, int* iters_out, double* fres_out);

#ifdef __cplusplus
}
#endif
#endif /* UNSFLOW_HOST_H */
