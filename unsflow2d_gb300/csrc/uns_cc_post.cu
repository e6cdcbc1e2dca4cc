// uns_cc_post.cu -- output-cadence post-processing of the CCFVM solver on the
// device: find_cl_cd (wall C_p / C_f rows and force coefficients,
// CCFVM/main.F90:263-355) and screen's min/max diagnostics (:187-221), so a
// driver that prints or writes them at its output cadence downloads a few
// numbers instead of the state.
#include <cuda_runtime.h>

#include <cmath>
#include <vector>

#include "uns_cc_impl.cuh"

using namespace uns;

namespace {

constexpr int kRow = 10;  // per boundary face: x, y, -cp, cf, p-term x, y, viscous term x, y, cm terms a, b

// Per wall face: the terms of find_cl_cd in its expression order.
__global__ void k_wall_terms(CCView v, double xref, double yref, double dyna, double* t) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= v.nbf) return;
    const int ie = v.nfi + b;
    double* o = t + (size_t)b * kRow;
    if (v.fbc[ie] != 1001) return;
    const double pwall = v.qp[v.fnb[ie].x].w;
    const int2 p = v.fpt[ie];
    const double2 P1 = v.pxy[p.x], P2 = v.pxy[p.y];
    const double xi = 0.5 * (P1.x + P2.x);
    const double yi = 0.5 * (P1.y + P2.y);
    const double xa = xi - xref;
    const double ya = yi - yref;
    const double area = v.farea[ie];
    const double2 n = v.fn[ie];
    const double cp = (pwall - v.g.p_inf) / dyna;
    const double dcx = cp * n.x * area;
    const double dcy = cp * n.y * area;
    double vx = 0.0, vy = 0.0, cf = 0.0;
    if (v.laminar) {
        const double two = 2.0, two_third = two / 3.0;
        const double mu = v.fmu[ie] / v.g.rey;
        const double4 gx = v.fgx[ie], gy = v.fgy[ie];
        const double ux = gx.y, uy = gy.y, wx = gx.z, wy = gy.z;
        const double tauxx = two_third * (two * ux - wy);
        const double tauxy = (uy + wx);
        const double tauyy = two_third * (two * wy - ux);
        vx = mu * (tauxx * n.x + tauxy * n.y) * area;
        vy = mu * (tauxy * n.x + tauyy * n.y) * area;
        const double tx = n.y, ty = -n.x;
        const double tw = mu * ((ux * tx + wx * ty) * n.x + (uy * tx + wy * ty) * n.y);
        cf = tw * area / dyna;
    }
    o[0] = xi; o[1] = yi; o[2] = -cp; o[3] = cf;
    o[4] = pwall * n.x * area; o[5] = pwall * n.y * area;
    o[6] = vx; o[7] = vy;
    o[8] = dcx * ya; o[9] = dcy * xa;
}

// The reference's sequential sums in face order, and the wall rows compacted
// in that order: out[0..2] = Fx, Fy, Cm, out[3] = wall face count, out[4 + 4k..] rows.
__global__ void k_wall_sum(CCView v, const double* t, double* out) {
    double fx = 0.0, fy = 0.0, cm = 0.0;
    int i = 0;
#pragma unroll 4
    for (int b = 0; b < v.nbf; ++b) {  // unrolled: loads in flight together, sums in order
        if (v.fbc[v.nfi + b] != 1001) continue;
        const double* o = t + (size_t)b * kRow;
        fx = fx + o[4];
        fy = fy + o[5];
        if (v.laminar) { fx = fx - o[6]; fy = fy - o[7]; }
        cm = cm + o[8] - o[9];
        double* r = out + 4 + 4 * (size_t)i;
        r[0] = o[0]; r[1] = o[1]; r[2] = o[2]; r[3] = o[3];
        ++i;
    }
    out[0] = fx; out[1] = fy; out[2] = cm; out[3] = (double)i;
}

// screen's min/max over the interior cells from the current conserved state
// (exact, order-free: warp reduction then encoded atomics).
__global__ void k_screen_minmax(CCView v, double ent_inf, unsigned long long* mm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    unsigned long long lo[7], hi[7];
    for (int k = 0; k < 7; ++k) { lo[k] = ~0ULL; hi[k] = 0ULL; }
    if (i < v.noc) {
        const double4 q = v.qc[i];
        const Prim r = con2prim(v.g, q.x, q.y, q.z, q.w);
        const double q2 = r.u * r.u + r.v * r.v;
        const double mach = sqrt(q2 * r.rho / (v.g.gamma * r.p));
        const double ent = log10(r.p / pow(r.rho, v.g.gamma) / ent_inf);
        const double x[7] = {r.rho, r.u, r.v, r.p, r.t, mach, ent};
        for (int k = 0; k < 7; ++k) { lo[k] = enc_ord(x[k]); hi[k] = lo[k]; }
    }
    for (int k = 0; k < 7; ++k) {
        for (int o = 16; o > 0; o >>= 1) {
            unsigned long long a = __shfl_xor_sync(0xffffffffu, lo[k], o), c = __shfl_xor_sync(0xffffffffu, hi[k], o);
            lo[k] = a < lo[k] ? a : lo[k];
            hi[k] = c > hi[k] ? c : hi[k];
        }
    }
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 7; ++k) { atomicMin(&mm[2 * k], lo[k]); atomicMax(&mm[2 * k + 1], hi[k]); }
}

// tecplt's vertex table (CCFVM/main.F90:417-480): the avg_c2v vertex average
// (the FP64 k_vertex_avg's operations and order, plus the viscosity as
// average.F90:23-28 forms it) and per vertex x, y, density, u, v, Mach,
// pressure, temperature, entropy, |V|, mu.  The solver's own vertex values
// are left untouched.
__global__ void __launch_bounds__(kBlock) k_tecplt(CCView v, double ent_inf, double* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.nop) return;
    double wt = 0.0, c0 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0, c4 = 0.0, c5 = 0.0;
    for (int k = v.v2c_off[i]; k < v.v2c_off[i + 1]; ++k) {
        const int c = v.v2c[k];
        const double w = v.v2c_wt[k];
        wt = wt + w;
        const double4 q = v.qp[c];
        c0 = c0 + q.x * w;
        c1 = c1 + q.y * w;
        c2 = c2 + q.z * w;
        c3 = c3 + q.w * w;
        c4 = c4 + v.qT[c] * w;
        c5 = c5 + v.mul[c] * w;
    }
    const double ro = c0 / wt, uo = c1 / wt, vo = c2 / wt, po = c3 / wt, to = c4 / wt, mu = c5 / wt;
    const double vmag = sqrt(uo * uo + vo * vo);
    const double q2 = uo * uo + vo * vo;
    const double mach = sqrt(q2 * ro / (v.g.gamma * po));
    const double entropy = log10(po / pow(ro, v.g.gamma) / ent_inf);
    const double2 x = v.pxy[i];
    double* o = out + (size_t)i * 11;
    o[0] = x.x; o[1] = x.y; o[2] = ro; o[3] = uo; o[4] = vo; o[5] = mach;
    o[6] = po; o[7] = to; o[8] = entropy; o[9] = vmag; o[10] = mu;
}

__global__ void k_screen_init(unsigned long long* mm) {
    const int k = threadIdx.x;
    if (k < 7) { mm[2 * k] = ~0ULL; mm[2 * k + 1] = 0ULL; }
}

int ensure_post(uns_cc_handle* h) {
    if (h->d_post) return UNS_OK;
    // terms [nbf][kRow], sums + rows [4 + 4 nbf], min/max slots [14]
    return h->alloc(h->d_post, (size_t)h->v.nbf * kRow + 4 + 4 * (size_t)h->v.nbf + 14);
}

}  // namespace

extern "C" {

int uns_cc_find_cl_cd(uns_cc_handle* h, double xref, double yref, double* coef, double* wall, int* nwall) {
    if (!h || !coef) { set_last_error("uns_cc_find_cl_cd: null argument"); return UNS_ERR_ARG; }
    int rc = ensure_post(h);
    if (rc) return rc;
    const CCView& v = h->v;
    const Gas& g = v.g;
    // dyna = 0.5 gamma p_inf M^2 (main.F90:284), in its expression order
    const double dyna = 0.5 * g.gamma * g.p_inf * g.m_inf * g.m_inf;
    double* t = h->d_post;
    double* out = t + (size_t)v.nbf * kRow;
    k_wall_terms<<<std::max(1, nblocks(v.nbf)), kBlock, 0, h->stream>>>(v, xref, yref, dyna, t);
    UNS_CUDA(cudaGetLastError());
    k_wall_sum<<<1, 1, 0, h->stream>>>(v, t, out);
    UNS_CUDA(cudaGetLastError());
    std::vector<double> r(4 + 4 * (size_t)v.nbf);
    UNS_CUDA(cudaMemcpyAsync(r.data(), out, sizeof(double) * r.size(), cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    double fx1 = 0.0, fy1 = 0.0;
    if ((rc = uns_cc_forces(h, &fx1, &fy1))) return rc;
    const double fx = r[0], fy = r[1];
    const int n = (int)r[3];
    // cos / sin of the angle of attack are u_inf, v_inf (solution.F90:35-36)
    coef[0] = (fy * g.u_inf - fx * g.v_inf) / dyna;
    coef[1] = (fy * g.v_inf + fx * g.u_inf) / dyna;
    coef[2] = r[2];
    coef[3] = (fy1 * g.u_inf - fx1 * g.v_inf) / dyna;
    coef[4] = (fy1 * g.v_inf + fx1 * g.u_inf) / dyna;
    if (wall) std::copy(r.begin() + 4, r.begin() + 4 + 4 * (size_t)n, wall);
    if (nwall) *nwall = n;
    return cc_check_dev_err(h);
}

int uns_cc_tecplt(uns_cc_handle* h, double* out) {
    if (!h || !out) { set_last_error("uns_cc_tecplt: null argument"); return UNS_ERR_ARG; }
    if (h->v.ninst) { set_last_error("uns_cc_tecplt: a packed handle has no single vertex table"); return UNS_ERR_ARG; }
    const CCView& v = h->v;
    if (!h->d_tec) { int rc = h->alloc(h->d_tec, 11 * (size_t)v.nop); if (rc) return rc; }
    const double ent_inf = v.g.p_inf / std::pow(v.g.r_inf, v.g.gamma);
    k_tecplt<<<std::max(1, nblocks(v.nop)), kBlock, 0, h->stream>>>(v, ent_inf, h->d_tec);
    UNS_CUDA(cudaGetLastError());
    UNS_CUDA(cudaMemcpyAsync(out, h->d_tec, sizeof(double) * 11 * (size_t)v.nop, cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    return cc_check_dev_err(h);
}

int uns_cc_screen_minmax(uns_cc_handle* h, double* out) {
    if (!h || !out) { set_last_error("uns_cc_screen_minmax: null argument"); return UNS_ERR_ARG; }
    int rc = ensure_post(h);
    if (rc) return rc;
    const CCView& v = h->v;
    unsigned long long* mm = reinterpret_cast<unsigned long long*>(h->d_post + (size_t)v.nbf * kRow + 4 + 4 * (size_t)v.nbf);
    const double ent_inf = v.g.p_inf / std::pow(v.g.r_inf, v.g.gamma);
    k_screen_init<<<1, 32, 0, h->stream>>>(mm);
    UNS_CUDA(cudaGetLastError());
    k_screen_minmax<<<std::max(1, nblocks(v.noc)), kBlock, 0, h->stream>>>(v, ent_inf, mm);
    UNS_CUDA(cudaGetLastError());
    unsigned long long e[14];
    UNS_CUDA(cudaMemcpyAsync(e, mm, sizeof(e), cudaMemcpyDeviceToHost, h->stream));
    UNS_CUDA(cudaStreamSynchronize(h->stream));
    for (int k = 0; k < 14; ++k) out[k] = dec_ord(e[k]);
    return cc_check_dev_err(h);
}

}  // extern "C"
