// uns_cc_impl.cuh -- internal state of a CCFVM handle, shared by the
// translation units of libunsflow_gpu.so (uns_cc.cu: the forward path;
// uns_cc_adj.cu: the discrete adjoint).  Not part of the C-ABI.
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <vector>

#include "uns_common.cuh"
#include "uns_phys.cuh"
#include "unsflow_gpu.h"

namespace uns {

constexpr int SIDE_BIT = 1 << 30;  // cell is the `out` side of this face
constexpr int FACE_MASK = SIDE_BIT - 1;

struct CCView {
    int nop, noc, nfi, nbf, nof, ntot;
    // geometry (read-only)
    const double2* pxy;
    const double2* cen;
    const double* cv;
    const double* cov;
    const int2* fnb;      // (in, out)
    const int2* fpt;      // (p1, p2)
    const double2* fn;    // unit normal
    const double* farea;
    const double2* fcen;
    const int* fbc;
    const double4* lsw;   // LSQ weights (wx0, wy0, wx1, wy1) per face
    const int* nc2c;
    const int* cf_off;    // index-sorted faces per cell, SIDE_BIT for `out`
    const int* cf;
    const float4* sideg;  // per cf entry (GG, inviscid): outward-signed unit normal x, y; this side's offset x, y
    const int4* sidei;    // per cf entry: cell across (-1 on a boundary), end points p1, p2, length (float bits)
    int blk_face, blk_vert, blk_grad;  // block sizes of k_face_conv, k_vertex_avg, k_cell_grad_side
    const unsigned* bcell;  // bit i: interior cell i has a wall face
    const int* wcell;       // those cells in increasing order
    int nwcell;
    const int* rc2f_off;  // reference c2f order (LU-SGS)
    const int* rc2f;
    const int* v2c_off;
    const int* v2c;
    const double* v2c_wt;
    // state
    double4* qc;  // [ntot] E, rho, rho u, rho v
    double4* qp;  // [ntot] rho, u, v, p
    double* qT;   // [ntot] T
    double4* qold;
    double4* res;
    double4* res0;
    double4* restmp;
    double4* gx;
    double4* gy;
    double4* phi;
    double* dt;
    double* la;
    double* mul;
    double4* pp;
    double* ppT;
    double4* fq;
    double* fqT;
    double* fla;
    double* fmu;
    double4* fF;   // convective face flux (boundary: flux into `in`)
    double4* fV;   // viscous flux * area
    double4* fgx;  // diamond-path face gradient, rho,u,v,p
    double4* fgy;
    double2* fgT;  // face gradient of T
    double* fasum; // a1 + a2
    double2* fwall;   // per boundary face: wall convective (flux3, flux4)
    double2* fwallv;  // per boundary face: wall viscous (-flux3*A, -flux4*A)
    double* diag;     // lusgs2 diagonal cv/dt + 0.5*omega*la (lusgs.F90:236)
    double* diaginv;  // its FP64 reciprocal (the FP32 sweep multiplies by it)
    // LU-SGS sweep schedule (host-built): per position of the warp lists
    // (it, pass, first record, records); per record, in the reference c2f
    // order of the taken faces: face, neighbour, 1 if the face normal points
    // into the cell (the sweep then uses -n).
    const int4* sched;
    const int* rec_face;
    const int* rec_nb;
    const int* rec_flip;
    int nrec;
    double4* rec;     // per record, per LU-SGS call: 3 x double4 (k_cc_sweep_prep) or 4 x float4 (k_cc_sweep_prep_mixed)
    double4* rec_a;   // sweep records [pass * noc + cell]: (u, v, p, e*rho) of qold + dq
    double4* rec_b;   //   and dq (lower / upper); rho is rebuilt as qold.rho + dq.rho
    unsigned long long* minmax;  // encoded qmax[4], qmin[4]
    unsigned long long* dtmin;   // encoded dtglobal
    double* partial;
    DevErr* err;
    long long wait_cycles;  // bound of the sweeps' waits (kWaitCycles unless a caller set one)
    int skip_code;          // test hook: the sweep item (cell << 1 | pass) that publishes nothing, or -1
    // iteration control (graph fast path)
    const double* cfl_sched;
    int* iter;
    int* done;
    double* fres_hist;
    double* fres1;
    // FP32 copies read by the FP32-flux (mixed) form, so that its kernels do
    // their arithmetic in FP32 without per-value FP64->FP32 conversions
    // (which issue on the FP64 unit).  Geometry is rounded once from FP64.
    const float4* fgeof;  // per face: fc - cen[in] (x, y), fc - cen[out] (x, y; 0 on boundary faces)
    const float4* fnaf;   // per face: nx, ny, area, 0
    const float4* lswf;   // LSQ weights
    float4* qpf;          // [ntot] rho, u, v, p (ghost cells: always kept)
    float4* fqf;          // [nof] face primitives of avg_c2v
    float* flaf;          // [nof] face spectral radius
    float4* packf;        // [4 * noc] per cell: primitives, gx, gy, phi (the gradient and phi of record in the mixed form)
    float4* ppf;          // [nop] vertex-averaged primitives
    const float* v2c_wtf; // pseudo-Laplacian weights
    double* dcv;          // [noc] dt / cv of the current time step (both forms)
    // packed instances (uns_cc_create_packed; ninst = 0 for one case): every
    // element knows its instance; per-instance constants and loop control
    // are arrays indexed by it (iter, done, fres1, minmax [8 each], dtmin,
    // cfl_sched / fres_hist [cfl_stride each]).  Interior cells of each
    // instance are padded to a multiple of kBlock (padding: instance -1), so
    // every block of cells belongs to one instance.
    int ninst, cfl_stride;
    // 1 when `partial` holds one sum per warp of 32 cells (a small mesh's
    // spread k_cell_rk23): k_res_final adds each 8 of them in warp order,
    // which is the 256-cell block partial bit for bit.
    int wpart;
    const int* cinst;       // [ntot] instance of each cell, ghosts included
    const int* finst;       // [nof]
    const int* pinst;       // [nop]
    const Gas* gas;         // [ninst]
    const double4* qinfs;   // [ninst] freestream conserved state
    const int* boff;        // [ninst + 1] norm blocks of each instance
    const int* ncell;       // [ninst] real interior cells
    const double* minres;   // [ninst]
    Gas g;
    int grad_type, ilimit, irs, laminar, first_iter;
    int mixed;            // UNS_PREC_MIXED: keep the FP32 copies, run the FP32 kernels
    double cfl_max, min_res;
};

struct CCAdj;  // discrete-adjoint state (uns_cc_adj.cu), created on first use

}  // namespace uns

struct uns_cc_handle {
    uns_params P;
    uns::Gas g;
    uns::CCView v;
    cudaStream_t stream = nullptr;
    std::vector<void*> allocs;
    int nparts = 0;
    // LU-SGS levels
    int* woff = nullptr;   // LU-SGS warp schedule: per-warp ranges of v.sched
    int coop_blocks = 0;
    int nsm = 1;           // SMs of the device (launch widths of small meshes)
    double4 qinf;
    // graph fast path
    cudaGraphExec_t graph = nullptr;
    double* d_cfl = nullptr;
    int cfl_cap = 0;
    int* d_iter = nullptr;
    int* d_done = nullptr;
    double* d_hist = nullptr;
    double* d_fres1 = nullptr;
    double* d_scalar = nullptr;  // [4] scratch for host-visible scalars
    int graph_first = -1;
    int gen = 0;           // bumped whenever the captured iteration changes (precision, capacity)
    double cfl_cur = 0.0;  // CFL passed to the last time_step call
    // uns_cc_fvresidual's flux cache: flux_gen is bumped by every call that may
    // change the inputs of the interior and farfield face fluxes (primitives,
    // gradient, limiter, precision, the whole step); res_gen is the flux_gen
    // of the last fvresidual that computed every face.
    long long flux_gen = 0;
    long long res_gen = -1;
    uns::CCAdj* adj = nullptr;  // discrete-adjoint state, created by uns_cc_adjoint_prepare
    double* d_post = nullptr;   // post-processing scratch (uns_cc_post.cu), created on first use
    double* d_tec = nullptr;    // tecplt vertex table (uns_cc_post.cu), created on first use
    // Host copies the geometry adjoint transposes through (the LSQ weights are
    // formed on the host from them): r11, r12, r22 per cell, fin/fout per face.
    std::vector<double> lsq_r;  // [noc][3]
    std::vector<int2> fnb_host; // [nof]

    template <class T>
    int alloc(T*& p, size_t n) {
        void* q = nullptr;
        size_t bytes = std::max<size_t>(n, 1) * sizeof(T);
        UNS_CUDA(cudaMalloc(&q, bytes));
        UNS_CUDA(cudaMemsetAsync(q, 0, bytes, stream));
        allocs.push_back(q);
        p = (T*)q;
        return UNS_OK;
    }
    template <class T>
    int upload(T*& p, const T* src, size_t n) {
        int rc = alloc(p, n);
        if (rc) return rc;
        if (n) UNS_CUDA(cudaMemcpyAsync(p, src, n * sizeof(T), cudaMemcpyHostToDevice, stream));
        return UNS_OK;
    }
};

namespace uns {
// Forward-path services the adjoint translation unit uses (uns_cc.cu).
int cc_check_dev_err(uns_cc_handle* h);
// Points of one recorded main-loop iteration at which the adjoint records
// the values it linearises around (stage = 1..3 of RK3).
enum CCRecPoint { REC_AFTER_START = 0, REC_BEFORE_FACE_CONV = 1, REC_BEFORE_CELL_MUL = 2, REC_AFTER_FACE_VISC = 3 };
typedef int (*CCRecHook)(uns_cc_handle* h, int point, int stage, void* ctx);
// One RK3 main-loop iteration with the limiter frozen (phi kept), calling
// `hook` at each CCRecPoint; the state advances by that iteration.
int cc_record_iteration(uns_cc_handle* h, double cfl, CCRecHook hook, void* ctx);
void cc_adj_free(uns_cc_handle* h);
}  // namespace uns
