// host_shape.cpp -- shape derivatives on the host (no reference counterpart):
// a CCFVM mesh rebuilt at moved node coordinates, and the transpose of the
// geometric preprocessing (geometric_cc, CCFVM/geometric.F90:62-198,
// 619-674, 898-1013 and the ghost mirror of CCFVM/read_input.F90:179-203)
// that carries the adjoints of the mesh arrays (uns_cc_adjoint_geometry) to
// the node coordinates.  The cells are triangles whose centroid is the mean
// of their vertices and whose volume is their area (the airfoil generator's
// and the plot3d triangulation's meshes); other meshes are rejected.
#include <cmath>
#include <string>
#include <vector>

#include "host_mesh.hpp"

namespace unshost {
namespace {

// Signed doubled area of triangle (a, b, c) and its derivatives.
inline double area2(double ax, double ay, double bx, double by, double cx, double cy) {
    return (bx - ax) * (cy - ay) - (by - ay) * (cx - ax);
}

// Adjoint of the shoelace area of a closed polygon (positive for
// counter-clockwise order): dA/dx_k = (y_{k+1} - y_{k-1}) / 2,
// dA/dy_k = (x_{k-1} - x_{k+1}) / 2.
template <int N>
void polygon_area_vjp(const double (&x)[N], const double (&y)[N], double w, double (&xb)[N], double (&yb)[N]) {
    for (int k = 0; k < N; ++k) {
        const int kp = (k + 1) % N, km = (k + N - 1) % N;
        xb[k] = w * 0.5 * (y[kp] - y[km]);
        yb[k] = w * 0.5 * (x[km] - x[kp]);
    }
}

// The three distinct vertices of every raw cell, from its faces.
bool raw_triangles(const RawCC& r, std::vector<int>& tri, std::string& err) {
    tri.assign((size_t)r.noc * 3, -1);
    std::vector<int> n(r.noc, 0);
    auto add = [&](int c, int p) {
        for (int k = 0; k < n[c]; ++k)
            if (tri[3 * c + k] == p) return true;
        if (n[c] == 3) return false;
        tri[3 * c + n[c]++] = p;
        return true;
    };
    const int nof = r.nfi + r.nbf;
    for (int f = 0; f < nof; ++f) {
        const int cells[2] = {r.fin[f], r.fout[f]};
        for (int c : cells) {
            if (c < 0 || c >= r.noc) continue;
            if (!add(c, r.fp1[f]) || !add(c, r.fp2[f])) { err = "cell " + std::to_string(c) + " is not a triangle"; return false; }
        }
    }
    for (int c = 0; c < r.noc; ++c)
        if (n[c] != 3) { err = "cell " + std::to_string(c) + " is not a triangle"; return false; }
    return true;
}

}  // namespace

int moved_cc(const RawCC& raw, const double* px, const double* py, RawCC& out, std::string& err) {
    std::vector<int> tri;
    if (!raw_triangles(raw, tri, err)) return UNS_ERR_MESH;
    out = raw;
    out.px.assign(px, px + raw.nop);
    out.py.assign(py, py + raw.nop);
    for (int c = 0; c < raw.noc; ++c) {
        const int a = tri[3 * c], b = tri[3 * c + 1], d = tri[3 * c + 2];
        out.cx[c] = (out.px[a] + out.px[b] + out.px[d]) / 3.0;
        out.cy[c] = (out.py[a] + out.py[b] + out.py[d]) / 3.0;
        out.cv[c] = 0.5 * std::fabs(area2(out.px[a], out.py[a], out.px[b], out.py[b], out.px[d], out.py[d]));
        if (!(out.cv[c] > 0.0)) { err = "moved mesh: cell " + std::to_string(c) + " is degenerate"; return UNS_ERR_MESH; }
    }
    const int nof = raw.nfi + raw.nbf;
    for (int f = 0; f < nof; ++f) {  // file normals (dy, -dx) of p1 -> p2
        out.fnx[f] = out.py[raw.fp2[f]] - out.py[raw.fp1[f]];
        out.fny[f] = -(out.px[raw.fp2[f]] - out.px[raw.fp1[f]]);
    }
    return UNS_OK;
}

int mesh_vjp_cc(const MeshCC& m, const uns_cc_mesh_adj& a, double* gpx, double* gpy, std::string& err) {
    const int nop = m.nop, noc = m.noc, nfi = m.nfi, nbf = m.nbf, nof = nfi + nbf, ntot = noc + nbf;
    const auto& px = m.px;
    const auto& py = m.py;
    std::vector<double> gx(a.px, a.px + nop), gy(a.py, a.py + nop);
    std::vector<double> cxb(a.cx, a.cx + ntot), cyb(a.cy, a.cy + ntot);
    auto close = [](double u, double v, double scale) { return std::fabs(u - v) <= 1e-9 * scale; };

    // pseudo_Laplacian: w_c = 1 + gx dx_c + gy dy_c, (gx, gy) = (Nx, Ny) / det
    // with Nx = ixy ry - iyy rx, Ny = ixy rx - ixx ry, det = ixx iyy - ixy^2.
    for (int i = 0; i < nop; ++i) {
        double ixx = 0, iyy = 0, ixy = 0, rx = 0, ry = 0;
        for (int k = m.v2c_off[i]; k < m.v2c_off[i + 1]; ++k) {
            const int c = m.v2c[k];
            const double dx = m.cx[c] - px[i], dy = m.cy[c] - py[i];
            rx += dx; ry += dy; ixx += dx * dx; iyy += dy * dy; ixy += dx * dy;
        }
        const double det = ixx * iyy - ixy * ixy;
        const double gxv = (ixy * ry - iyy * rx) / det, gyv = (ixy * rx - ixx * ry) / det;
        double gxb = 0.0, gyb = 0.0;
        for (int k = m.v2c_off[i]; k < m.v2c_off[i + 1]; ++k) {
            const int c = m.v2c[k];
            gxb += a.v2c_wt[k] * (m.cx[c] - px[i]);
            gyb += a.v2c_wt[k] * (m.cy[c] - py[i]);
        }
        const double nxb = gxb / det, nyb = gyb / det, detb = -(gxb * gxv + gyb * gyv) / det;
        const double ixyb = nxb * ry + nyb * rx - 2.0 * ixy * detb;
        const double ryb = nxb * ixy - nyb * ixx, rxb = -nxb * iyy + nyb * ixy;
        const double iyyb = -nxb * rx + detb * ixx, ixxb = -nyb * ry + detb * iyy;
        for (int k = m.v2c_off[i]; k < m.v2c_off[i + 1]; ++k) {
            const int c = m.v2c[k];
            const double dx = m.cx[c] - px[i], dy = m.cy[c] - py[i];
            const double dxb = a.v2c_wt[k] * gxv + rxb + 2.0 * dx * ixxb + dy * ixyb;
            const double dyb = a.v2c_wt[k] * gyv + ryb + 2.0 * dy * iyyb + dx * ixyb;
            cxb[c] += dxb; gx[i] -= dxb;
            cyb[c] += dyb; gy[i] -= dyb;
        }
    }

    // LSQR_Coeff: r11 = sqrt(R11), r12 = R12 / r11, r22 = sqrt(R22 - r12^2),
    // R the sums of dx^2, dx dy, dy^2 over the cell's faces (ghosts across
    // boundary faces).
    {
        std::vector<double> R11(noc, 0.0), R12(noc, 0.0), R22(noc, 0.0);
        auto acc = [&](int c, double dx, double dy) {
            if (c >= noc) return;
            R11[c] += dx * dx; R12[c] += dx * dy; R22[c] += dy * dy;
        };
        for (int f = 0; f < nof; ++f) {
            const int in = m.fin[f], out = m.fout[f];
            const double dx = m.cx[out] - m.cx[in], dy = m.cy[out] - m.cy[in];
            acc(in, dx, dy);
            if (f < nfi) acc(out, -dx, -dy);
        }
        std::vector<double> B11(noc), B12(noc), B22(noc);
        for (int i = 0; i < noc; ++i) {
            const double r11 = std::sqrt(R11[i]), r12 = R12[i] / r11, r22 = std::sqrt(R22[i] - r12 * r12);
            if (!close(r11, m.r11[i], 1.0 + std::fabs(r11)) || !close(r22, m.r22[i], 1.0 + std::fabs(r22))) {
                err = "mesh_vjp: LSQ coefficients do not match the centroids";
                return UNS_ERR_MESH;
            }
            const double r22b = a.r22[i];
            B22[i] = r22b / (2.0 * r22);
            const double r12b = a.r12[i] - r22b * r12 / r22;
            B12[i] = r12b / r11;
            const double r11b = a.r11[i] - r12b * R12[i] / (r11 * r11);
            B11[i] = r11b / (2.0 * r11);
        }
        auto back = [&](int c, int o, double dx, double dy) {  // d = x_o - x_c, summed into cell c
            if (c >= noc) return;
            const double dxb = 2.0 * dx * B11[c] + dy * B12[c], dyb = 2.0 * dy * B22[c] + dx * B12[c];
            cxb[o] += dxb; cxb[c] -= dxb;
            cyb[o] += dyb; cyb[c] -= dyb;
        };
        for (int f = 0; f < nof; ++f) {
            const int in = m.fin[f], out = m.fout[f];
            const double dx = m.cx[out] - m.cx[in], dy = m.cy[out] - m.cy[in];
            back(in, out, dx, dy);
            if (f < nfi) back(out, in, -dx, -dy);
        }
    }

    // face_co_volume: cov_c = sum over the cell's faces of the areas of
    // (p1, p2, c_in) and (p1, c_out, p2).
    for (int f = 0; f < nof; ++f) {
        const int p1 = m.fp1[f], p2 = m.fp2[f], in = m.fin[f], out = m.fout[f];
        const double w = a.cov[in] + (out < noc ? a.cov[out] : 0.0);
        if (w == 0.0) continue;
        const double x1[3] = {px[p1], px[p2], m.cx[in]}, y1[3] = {py[p1], py[p2], m.cy[in]};
        const double x2[3] = {px[p1], m.cx[out], px[p2]}, y2[3] = {py[p1], m.cy[out], py[p2]};
        double xb[3], yb[3];
        polygon_area_vjp(x1, y1, w, xb, yb);
        gx[p1] += xb[0]; gy[p1] += yb[0]; gx[p2] += xb[1]; gy[p2] += yb[1]; cxb[in] += xb[2]; cyb[in] += yb[2];
        polygon_area_vjp(x2, y2, w, xb, yb);
        gx[p1] += xb[0]; gy[p1] += yb[0]; cxb[out] += xb[1]; cyb[out] += yb[1]; gx[p2] += xb[2]; gy[p2] += yb[2];
    }

    // cell_face_norm: centre = midpoint; n = N / |N|, area = |N|,
    // N = (y2 - y1, -(x2 - x1)) of the final end points.
    for (int f = 0; f < nof; ++f) {
        const int p1 = m.fp1[f], p2 = m.fp2[f];
        gx[p1] += 0.5 * a.fcx[f]; gx[p2] += 0.5 * a.fcx[f];
        gy[p1] += 0.5 * a.fcy[f]; gy[p2] += 0.5 * a.fcy[f];
        const double Nx = py[p2] - py[p1], Ny = -(px[p2] - px[p1]);
        const double ar = std::sqrt(Nx * Nx + Ny * Ny), nx = Nx / ar, ny = Ny / ar;
        if (!close(nx, m.fnx[f], 1.0) || !close(ny, m.fny[f], 1.0) || !close(ar, m.farea[f], ar)) {
            err = "mesh_vjp: face " + std::to_string(f) + " normal does not match its end points";
            return UNS_ERR_MESH;
        }
        const double dn = a.fnx[f] * nx + a.fny[f] * ny;
        const double Nxb = (a.fnx[f] - dn * nx) / ar + a.farea[f] * nx;
        const double Nyb = (a.fny[f] - dn * ny) / ar + a.farea[f] * ny;
        gy[p2] += Nxb; gy[p1] -= Nxb;
        gx[p2] -= Nyb; gx[p1] += Nyb;
    }

    // Ghost centroids: the mirror of the inside centroid q across the face
    // line through s = p1, e = p2: c_g = 2 s - q - 2 k d, d = e - s,
    // k = ((s - q) . d) / (d . d).
    for (int b = 0; b < nbf; ++b) {
        const int f = nfi + b, g = noc + b, in = m.fin[f];
        const double sx = px[m.fp1[f]], sy = py[m.fp1[f]], ex = px[m.fp2[f]], ey = py[m.fp2[f]];
        const double qx = m.cx[in], qy = m.cy[in];
        const double vx = sx - qx, vy = sy - qy, dx = ex - sx, dy = ey - sy, L = dx * dx + dy * dy;
        const double k = (vx * dx + vy * dy) / L;
        const double cgx = 2.0 * sx - qx - 2.0 * k * dx, cgy = 2.0 * sy - qy - 2.0 * k * dy;
        const double sc = 1.0 + std::fabs(qx) + std::fabs(qy);
        if (!close(cgx, m.cx[g], sc) || !close(cgy, m.cy[g], sc)) {
            err = "mesh_vjp: ghost centroid " + std::to_string(g) + " is not the mirror of its cell";
            return UNS_ERR_MESH;
        }
        const double gbx = cxb[g], gby = cyb[g];
        double sbx = 2.0 * gbx, sby = 2.0 * gby, qbx = -gbx, qby = -gby;
        double dbx = -2.0 * k * gbx, dby = -2.0 * k * gby;
        const double kb = -2.0 * (gbx * dx + gby * dy);
        const double vbx = kb * dx / L, vby = kb * dy / L;
        dbx += kb * (vx / L - 2.0 * k * dx / L);
        dby += kb * (vy / L - 2.0 * k * dy / L);
        sbx += vbx; sby += vby; qbx -= vbx; qby -= vby;
        sbx -= dbx; sby -= dby;
        gx[m.fp1[f]] += sbx; gy[m.fp1[f]] += sby;
        gx[m.fp2[f]] += dbx; gy[m.fp2[f]] += dby;
        cxb[in] += qbx; cyb[in] += qby;
    }

    // Interior cells: centroid = vertex mean, volume = |signed area| / 2.
    for (int i = 0; i < noc; ++i) {
        const int k0 = m.c2v_off[i];
        if (m.c2v_off[i + 1] - k0 != 4) { err = "mesh_vjp: cell " + std::to_string(i) + " is not a triangle"; return UNS_ERR_MESH; }
        const int v[3] = {m.c2v[k0], m.c2v[k0 + 1], m.c2v[k0 + 2]};
        const double x[3] = {px[v[0]], px[v[1]], px[v[2]]}, y[3] = {py[v[0]], py[v[1]], py[v[2]]};
        const double mx = (x[0] + x[1] + x[2]) / 3.0, my = (y[0] + y[1] + y[2]) / 3.0;
        const double A2 = area2(x[0], y[0], x[1], y[1], x[2], y[2]);
        const double sc = 1.0 + std::fabs(mx) + std::fabs(my);
        if (!close(mx, m.cx[i], sc) || !close(my, m.cy[i], sc) || !close(0.5 * std::fabs(A2), m.cv[i], std::fabs(A2))) {
            err = "mesh_vjp: cell " + std::to_string(i) + " centroid or area is not that of its triangle";
            return UNS_ERR_MESH;
        }
        double xb[3], yb[3];
        polygon_area_vjp(x, y, (A2 > 0.0 ? 1.0 : -1.0) * a.cv[i], xb, yb);
        for (int k = 0; k < 3; ++k) {
            gx[v[k]] += cxb[i] / 3.0 + xb[k];
            gy[v[k]] += cyb[i] / 3.0 + yb[k];
        }
    }
    for (int k = 0; k < nop; ++k) { gpx[k] = gx[k]; gpy[k] = gy[k]; }
    return UNS_OK;
}

}  // namespace unshost
