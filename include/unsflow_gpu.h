/*
 * unsflow_gpu.h -- C-ABI of libunsflow_gpu.so, the GB300 (sm_103a) drop-in for
 * the residual-and-update hot path of UNSFlow2D.
 *
 * The reference hot-path subroutines take no arguments and work on Fortran
 * module arrays.  Here each of them becomes one entry point that works on the
 * device copy of those arrays held by an opaque handle; the caller (the
 * Fortran main program through iso_c_binding, or the C++ driver in
 * libunsflow_host.so) calls them in the same order as the reference main
 * loop.  Every call returns a UNS_* status (unsflow_types.h) instead of
 * printing and stopping.  One handle = one CUDA stream; calls on one handle
 * must come from one host thread at a time; handles are independent.
 *
 * Citations are file:line in the UNSFlow2D sources.
 */
#ifndef UNSFLOW_GPU_H
#define UNSFLOW_GPU_H
#include "unsflow_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Text of the last error raised on the calling thread ("" if none). */
const char* uns_last_error(void);
/* Library version string. */
const char* uns_version(void);
/* Test hooks (no reference counterpart), n host values each:
 * out[i] = a[i] / b[i] by the kernels' division through the reciprocal
 * (must equal IEEE division), and lt[i] = whether a[i]/b[i] < c[i]/d[i]
 * by the kernels' exact ratio comparison (-1 where it does not apply). */
int uns_selftest_div(const double* a, const double* b, double* out, int n);
int uns_selftest_ratio(const double* a, const double* b, const double* c, const double* d, int* lt, int n);

/* ============================================================ CCFVM =====*/
typedef struct uns_cc_handle uns_cc_handle;

/* Copies the preprocessed mesh (the `grid` module after geometric,
 * CCFVM/geometric.F90:1-57) and the flo.inp parameters to the device and
 * sets the freestream (CCFVM/solution.F90:24-45).  The caller may free
 * its arrays afterwards. */
int uns_cc_create(const uns_cc_mesh* mesh, const uns_params* params, uns_cc_handle** out);
int uns_cc_destroy(uns_cc_handle* h);

/* initialize (CCFVM/solution.F90:18-84): qc = freestream on every cell
 * including ghosts, phi = 1, primitives 0. */
int uns_cc_initialize(uns_cc_handle* h);
/* Conserved state of all noc+nbf cells, [noc+nbf][4] row-major. */
int uns_cc_set_state(uns_cc_handle* h, const double* qc);
int uns_cc_get_state(uns_cc_handle* h, double* qc);
/* Any UNS_CC_* field (unsflow_types.h) copied to host memory. */
int uns_cc_get_field(uns_cc_handle* h, int field, double* out);
/* Overwrites UNS_CC_QC, UNS_CC_QP (all noc+nbf cells, ghosts included, with
 * T) or UNS_CC_PHI from host memory: the rest of the state a restart or a
 * frozen-limiter continuation needs besides uns_cc_set_state (no reference
 * counterpart: the reference restarts from qc alone). */
int uns_cc_set_field(uns_cc_handle* h, int field, const double* in);

/* con2prim over the interior cells (CCFVM/main.F90:62-67). */
int uns_cc_con2prim(uns_cc_handle* h);
/* avg_c2v (CCFVM/average.F90:1-39). */
int uns_cc_avg_c2v(uns_cc_handle* h);
/* time_step02 + spectral02 (CCFVM/timestep.F90:28-107); dtglobal may be NULL. */
int uns_cc_time_step(uns_cc_handle* h, double cfl, double* dtglobal);
/* save_old (CCFVM/solution.F90:118-132). */
int uns_cc_save_old(uns_cc_handle* h);
/* Gradient_GG / Gradient_GG_FC / Gradient_LSQR per params.grad_type,
 * followed by limit when params.ilimit == 1 (CCFVM/gradient.F90:2-323). */
int uns_cc_gradient(uns_cc_handle* h);
/* limit -> limiter_VKN1 (CCFVM/limiter.F90:3-17,123-296). */
int uns_cc_limit(uns_cc_handle* h);
/* fvresidual (CCFVM/fvresidual.F90:4-187): boundary and interior convective
 * fluxes, ghost states, viscous flux, implicit residual smoothing. */
int uns_cc_fvresidual(uns_cc_handle* h);
/* One RK3 stage update, irk = 1..3 (CCFVM/main.F90:90-101). */
int uns_cc_rk_stage(uns_cc_handle* h, int irk);
/* lusgs -> lusgs2 (CCFVM/lusgs.F90:5-10,207-379): both sweeps as one
 * list-scheduled dataflow launch in the reference's cell order. */
int uns_cc_lusgs(uns_cc_handle* h);
/* check_positivity (CCFVM/main.F90:358-414): UNS_ERR_NONPOSITIVE and the
 * 0-based cell index in *bad_cell (-1 when none). */
int uns_cc_check_positivity(uns_cc_handle* h, int* bad_cell);
/* residue (CCFVM/solution.F90:136-180): sqrt(sum res^2 / noc / 4) before the
 * first-iteration normalisation, which stays with the caller. */
int uns_cc_residue(uns_cc_handle* h, double* fres_raw);
/* Flux-based wall forces Fx1, Fy1 of the last fvresidual
 * (CCFVM/fvresidual.F90:99-100, CCFVM/viscous_flux.F90:73-74). */
int uns_cc_forces(uns_cc_handle* h, double* fx1, double* fy1);
/* find_cl_cd (CCFVM/main.F90:263-355) on the device, from the last residual:
 * coef[0..4] = C_L, C_D of the pressure + viscous wall integral, C_m about
 * (xref, yref) (flo.inp's reference point), and C_L, C_D of the flux-based
 * Fx1, Fy1.  wall (may be NULL; room for nbf rows) receives per wall face, in
 * face order, the row x, y, -C_p, C_f that the reference writes to
 * XYCpCf.dat; *nwall (may be NULL) their count. */
int uns_cc_find_cl_cd(uns_cc_handle* h, double xref, double yref, double* coef, double* wall, int* nwall);
/* screen's min/max diagnostics (CCFVM/main.F90:187-221) over the interior
 * cells from the current state: out[2k], out[2k+1] = min, max of density, u,
 * v, pressure, temperature, Mach number, entropy log10(p / rho^gamma / ent_inf). */
int uns_cc_screen_minmax(uns_cc_handle* h, double* out);
/* tecplt's vertex table (CCFVM/main.F90:417-480) on the device: the avg_c2v
 * vertex average of the current cell primitives and viscosity, then per
 * vertex x, y, density, u, v, Mach, pressure, temperature, entropy, |V|, mu:
 * out[nop][11].  The solver's own vertex values are not changed. */
int uns_cc_tecplt(uns_cc_handle* h, double* out);
/* Fast path: `niter` whole iterations of the main loop body
 * (CCFVM/main.F90:59-115) replayed from one captured CUDA graph.  cfl[k] is
 * the CFL of iteration k; fres_raw[k] receives that iteration's raw residual
 * norm.  When first_iter is non-zero the first iteration is iteration 1 of
 * the run and its norm becomes the normalisation; iterations after the
 * normalised norm drops to params.min_res are skipped on the device, as the
 * reference loop stops there.  Returns the number of iterations executed in
 * *done_iters (may be NULL). */
int uns_cc_iterate(uns_cc_handle* h, int niter, const double* cfl, int first_iter, double* fres_raw,
                   int* done_iters);

/* ============================================================ NCFVM =====*/
typedef struct uns_nc_handle uns_nc_handle;

/* Mesh and parameters of the vertex-centred solver (NCFVM/geometric.f90,
 * NCFVM/common.f90:19-54). */
int uns_nc_create(const uns_nc_mesh* mesh, const uns_params* params, uns_nc_handle** out);
int uns_nc_destroy(uns_nc_handle* h);
/* initialize (NCFVM/common.f90:50-52): qc = freestream; phi = 1e20. */
int uns_nc_initialize(uns_nc_handle* h);
int uns_nc_set_state(uns_nc_handle* h, const double* qc);
int uns_nc_get_state(uns_nc_handle* h, double* qc);
int uns_nc_get_field(uns_nc_handle* h, int field, double* out);
/* save_old (NCFVM/common.f90:88-104): con2prim + qold. */
int uns_nc_save_old(uns_nc_handle* h);
/* fvresidual (NCFVM/fvresidual.f90:4-85): Gradient_LSQR, limiter, edge
 * fluxes, wall and farfield closures, then time_step2 with this CFL. */
int uns_nc_fvresidual(uns_nc_handle* h, double cfl);
/* One RK3 stage update, irk = 1..3 (NCFVM/main.f90:59-80). */
int uns_nc_rk_stage(uns_nc_handle* h, int irk);
/* lusgs (NCFVM/lusgs.f90:4-157): both sweeps as one list-scheduled
 * dataflow launch in the reference's node order; calls fvresidual. */
int uns_nc_lusgs(uns_nc_handle* h, double cfl);
/* residue (NCFVM/common.f90:108-154) before normalisation: L2 over nodes,
 * Linf and its 0-based node (any output pointer may be NULL). */
int uns_nc_residue(uns_nc_handle* h, double* fres_raw, double* fresi, int* iresi);
/* Fast path as uns_cc_iterate for the loop body NCFVM/main.f90:53-86;
 * fresi may be NULL. */
int uns_nc_iterate(uns_nc_handle* h, int niter, const double* cfl, int first_iter, double* fres_raw,
                   double* fresi, int* done_iters);

/* =========================================================== batches ====*/
/* Many independent CCFVM instances (different meshes, flow conditions,
 * fluxes) advanced together.  No reference counterpart: the reference runs
 * one case per process.  One CUDA graph holds every instance's captured
 * main-loop iteration as a parallel branch; each launch advances all of them
 * by one iteration, so small meshes fill the GPU together.  Instances keep
 * their own state, CFL schedule, residual history and stop test (an
 * instance whose residual has dropped to its min_res skips its kernels).
 * The handles stay owned by the caller, must outlive the batch and must not
 * be used on their own while a batch call runs. */
typedef struct uns_cc_batch uns_cc_batch;
int uns_cc_batch_create(uns_cc_handle* const* handles, int n, uns_cc_batch** out);
int uns_cc_batch_destroy(uns_cc_batch* b);
/* The cudaStream_t batch launches go to (for the caller's CUDA events). */
void* uns_cc_batch_stream(uns_cc_batch* b);
/* As uns_cc_iterate for every instance i: cfl[i*niter + k] is its CFL of
 * iteration k, fres_raw[i*niter + k] receives its raw residual norm and
 * done_iters[i] the iterations it executed.  Rebuilds the graph when an
 * instance's precision (uns_cc_set_precision) or first_iter changed. */
int uns_cc_batch_iterate(uns_cc_batch* b, int niter, const double* cfl, int first_iter, double* fres_raw,
                         int* done_iters);

/* =========================================================== adjoint ====*/
/* Discrete adjoint of the CCFVM RK3 iteration (no reference counterpart).
 * The state s is the conserved state of the noc interior cells plus the
 * primitives and T of the nbf ghost cells; one iteration maps s to G(s) and
 * computes the objective J (UNS_OBJ_*) from its last stage's wall fluxes.
 * At a converged state, lambda = G_s^T lambda + J_s^T gives
 * dJ/dalpha = J_alpha + G_alpha^T lambda (alpha in radians).  The limiter is
 * frozen at its current phi; RK3, FP64, no residual smoothing.
 *
 * prepare records the linearisation: one forward iteration at `cfl` from the
 * current state (two for a viscous flow, whose time step reads the previous
 * iteration's face viscosity), which advances the state by those iterations
 * (at convergence it does not change), and returns C_L, C_D of the recorded
 * iteration (either pointer may be NULL). */
int uns_cc_adjoint_prepare(uns_cc_handle* h, double cfl, double* cl, double* cd);
/* One transposed iteration: (oq, og) = G_s^T (wq, wg) + seed * J_s^T and
 * *oalpha = G_alpha^T (wq, wg) + seed * J_alpha.  wq, oq: [noc][4] conserved;
 * wg, og: [nbf][5] ghost rho, u, v, p, T. */
int uns_cc_adjoint_vjp(uns_cc_handle* h, int objective, double seed, const double* wq, const double* wg, double* oq,
                       double* og, double* oalpha);
/* Reverse accumulation from lambda = 0 until the change of lambda falls to
 * tol times its first change, or max_iter transposed iterations.  hist[k]
 * (may be NULL; max_iter entries) receives the change of iteration k. */
int uns_cc_adjoint_solve(uns_cc_handle* h, int objective, int max_iter, double tol, double* dj_dalpha, double* hist,
                         int* iters);
/* The adjoint vector of the last solve: [noc][4] and [nbf][5] (either may be NULL). */
int uns_cc_adjoint_get(uns_cc_handle* h, double* lambda_q, double* lambda_g);
/* Geometry.  prepare_geometry records what uns_cc_adjoint_prepare records
 * plus the convective closure's Jacobians with respect to the face normal and
 * length and the values of the start of the iteration (inviscid flows, and
 * laminar flows with the GG-FC gradient; not a packed handle).
 * uns_cc_adjoint_geometry then runs one transposed iteration like
 * uns_cc_adjoint_vjp and writes G_X^T (wq, wg) + seed * J_X^T for every
 * geometric array X of the handle's uns_cc_mesh into `out` (same layout;
 * every array required): the explicit dependence of one iteration on the
 * mesh at the recorded state.  With (wq, wg) the converged adjoint vector
 * and seed 1 it is the total dJ/dX of the converged flow, which
 * uns_host_cc_mesh_vjp carries to the node coordinates.  It overwrites the
 * adjoint vector as uns_cc_adjoint_vjp does. */
int uns_cc_adjoint_prepare_geometry(uns_cc_handle* h, double cfl, double* cl, double* cd);
int uns_cc_adjoint_geometry(uns_cc_handle* h, int objective, double seed, const double* wq, const double* wg,
                            uns_cc_mesh_adj* out);

/* ==================================================== packed cases ====*/
/* Many independent CCFVM cases in ONE index space (no reference
 * counterpart: the reference runs one case per process).  The n meshes are
 * concatenated -- interior cells padded per case to a multiple of 256, ghosts
 * in case order -- and every element records its case, so one launch of each
 * kernel advances all cases by one iteration (about twelve launches per
 * iteration for any number of cases).  Each case keeps its mesh, Mach number,
 * angle of attack, flux scheme, CFL schedule, residual norm, normalisation
 * and stop level (params[i].min_res) and evolves bit-identically to a handle
 * of its own; the cases share RK3 without residual smoothing, the gradient,
 * limiter, flow type and precision.  The result is a CCFVM handle: its state
 * (uns_cc_get_state: ntot rows), precision switch and destroy are the usual
 * calls; it iterates with uns_cc_packed_iterate. */
int uns_cc_create_packed(const uns_cc_mesh* meshes, const uns_params* params, int n, uns_cc_handle** out);
/* Where case i lives in the packed state: its interior cells are rows
 * cell_off[i] .. cell_off[i] + noc_i, its ghosts rows cell_off[n] +
 * ghost_off[i] .. cell_off[n] + ghost_off[i + 1]; both arrays [n + 1]. */
int uns_cc_packed_layout(uns_cc_handle* h, int* cell_off, int* ghost_off);
/* As uns_cc_iterate for every case i: cfl[i*niter + k], fres_raw[i*niter + k],
 * done_iters[i]. */
int uns_cc_packed_iterate(uns_cc_handle* h, int niter, const double* cfl, int first_iter, double* fres_raw,
                          int* done_iters);

/* ========================================================= precision ====*/
/* Switches the arithmetic form (UNS_PREC_*) between calls; waits for the
 * handle's stream, and the next uns_*_iterate captures a new graph.  No
 * reference counterpart: it lets a caller run the FP32-flux form while it
 * converges and finish in FP64 below the FP32 residual floor. */
int uns_cc_set_precision(uns_cc_handle* h, int precision);
int uns_nc_set_precision(uns_nc_handle* h, int precision);

/* ============================================================ timing ====*/
/* The cudaStream_t a handle queues its work on, so a caller can bracket
 * calls with its own CUDA events (no reference counterpart: measurement). */
void* uns_cc_stream(uns_cc_handle* h);
void* uns_nc_stream(uns_nc_handle* h);
/* Device time of each phase of one main-loop iteration, averaged over `reps`
 * iterations run with a CUDA event between phases (no reference
 * counterpart: measurement).  ms[k] for phase k < nphase; names[k] (may be
 * NULL) receives a static phase name.  The state advances by reps
 * iterations, exactly as uns_*_iterate would advance it. */
int uns_cc_profile(uns_cc_handle* h, double cfl, int reps, double* ms, const char** names, int nphase);
/* Launch-geometry autotuner (no reference counterpart): times the face,
 * vertex and cell-gradient kernels at each candidate block size on the
 * handle's mesh and state (writing scratch copies only), keeps the fastest
 * and re-captures the step.  blocks (may be NULL) receives the chosen
 * sizes: faces, vertices, cell gradient. */
int uns_cc_autotune(uns_cc_handle* h, int reps, int* blocks);
int uns_nc_profile(uns_nc_handle* h, double cfl, int reps, double* ms, const char** names, int nphase);
/* NCFVM tecplt's vertex table (NCFVM/main.f90:190-233): per node x, y and the
 * primitives of the last save_old (rho, u, v, p) with the Mach number:
 * out[nop][7]. */
int uns_nc_tecplt(uns_nc_handle* h, double* out);
/* NCFVM screen's min/max diagnostics (NCFVM/main.f90:115-187) over the nodes
 * from the current state: out[6][2] = min, max of density, u, v, pressure,
 * Mach number, entropy. */
int uns_nc_screen_minmax(uns_nc_handle* h, double* out);
/* Dependency levels of the LU-SGS forward and backward sweeps on the
 * handle's node order (NCFVM/lusgs.f90:48-124): their sum is the sweep's
 * critical path in items.  No reference counterpart (measurement). */
int uns_nc_sweep_levels(uns_nc_handle* h, int* forward, int* backward);
/* Bound of every wait in the handle's LU-SGS sweeps, in device clock cycles
 * (default 4e9, about 2 s); a sweep whose wait runs out returns
 * UNS_ERR_TIMEOUT with the context intact.  No reference counterpart (the
 * reference sweeps are sequential and never wait). */
int uns_cc_set_wait_limit(uns_cc_handle* h, long long cycles);
int uns_nc_set_wait_limit(uns_nc_handle* h, long long cycles);
/* Test hook, no reference counterpart: the sweep item of cell / node
 * `entity` in sweep `pass` (0 forward, 1 backward) publishes no record, so
 * the items that depend on it wait until the wait limit runs out; entity -1
 * clears it. */
int uns_cc_debug_unpublish(uns_cc_handle* h, int entity, int pass);
int uns_nc_debug_unpublish(uns_nc_handle* h, int entity, int pass);

/* ===================================================== no-allocation ====*/
/* Largest ncells uns_residue_rms_noalloc accepts: its scratch is a static
 * device array of UNS_RMS_NOALLOC_MAX_CELLS / 256 partial sums (128 KiB). */
#define UNS_RMS_NOALLOC_MAX_CELLS 4194304

/* The residual norm of uns_cc_residue, sqrt(sum res^2 / ncells / 4), over a
 * residual array the caller owns on the current device (ncells rows of 4
 * doubles, 32-byte aligned), queued on `stream` (NULL: the default stream)
 * and returned in *fres_raw after the stream synchronises.  No reference
 * counterpart: it exists for callers that must not allocate.  The call
 * allocates and frees nothing; its scratch is a fixed static device array,
 * whose every slot a call writes before reading it, so nothing needs to start
 * at zero.  ncells > UNS_RMS_NOALLOC_MAX_CELLS, NULL pointers or a misaligned
 * array give UNS_ERR_ARG before any device work.  The first call on each
 * device looks up the scratch address (cudaGetSymbolAddress, which allocates
 * nothing).  The address belongs to the context it was looked up in: the
 * first call in a new context of the device (after cudaDeviceReset) looks it
 * up again.
 * Every call synchronises `stream` before it returns.
 * Calls that overlap on one device (other threads or streams) share the
 * scratch and race: serialise them. */
int uns_residue_rms_noalloc(const double* res, int ncells, double* fres_raw, void* stream);

#ifdef __cplusplus
}
#endif
#endif /* UNSFLOW_GPU_H */
