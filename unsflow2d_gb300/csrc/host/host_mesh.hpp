// host_mesh.hpp -- caller-side mesh data of the UNSFlow2D drop-in.
//
// These structures hold what the reference's Fortran driver keeps in its
// `grid` module after `read_grid` + `geometric` (CCFVM/types/grid.F90:11-77,
// NCFVM/All_modules.f90:177-230), in structure-of-arrays form with 0-based
// indices.  They live on the host only; the GPU library receives a flat
// `uns_cc_mesh` / `uns_nc_mesh` view of them.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

#include "unsflow_types.h"

namespace unshost {

// What a CCFVM geometry.inp holds (CCFVM/read_input.F90:139-173), 0-based,
// before any preprocessing.  Interior faces first, then boundary faces.
struct RawCC {
    int nop = 0, noc = 0, nfi = 0, nbf = 0;
    std::vector<double> px, py;
    std::vector<int> pbc;
    std::vector<double> cx, cy, cv;                 // [noc]
    std::vector<int> fp1, fp2, fin, fout, fbc;      // [nfi+nbf]; fout of bnd = -1
    std::vector<double> fnx, fny;                   // file normals (un-normalised)
};

// What an NCFVM geometry.inp holds (NCFVM/read_input.f90:102-112), 0-based;
// a missing cell on a boundary edge is -1 (0 in the 1-based file).
struct RawNC {
    int nop = 0, noc = 0, nof = 0;
    std::vector<double> px, py;
    std::vector<int> pbc;
    std::vector<double> cx, cy, cv;
    std::vector<int> fp1, fp2, fin, fout, fbc;
    std::vector<double> fsx, fsy;
};

// CC mesh after geometric (CCFVM/geometric.F90:1-1013).
struct MeshCC {
    int nop = 0, noc = 0, nfi = 0, nbf = 0;
    std::vector<double> px, py;
    std::vector<int> pbc;
    std::vector<double> cx, cy;        // [noc+nbf]
    std::vector<double> cv;            // [noc]
    std::vector<double> cov;           // [noc+nbf] (ghost entries accumulate too)
    std::vector<int> fp1, fp2, fin, fout, fbc;
    std::vector<double> fnx, fny, farea, fcx, fcy, fcov;
    std::vector<double> r11, r12, r22; // [noc]
    std::vector<int> nc2c;             // [noc]
    std::vector<int> c2c_off, c2c;     // CSR [noc+1]
    std::vector<int> c2f_off, c2f;     // CSR [noc+1] (order after cell_2_vertex)
    std::vector<int> c2v_off, c2v;     // CSR [noc+1] (closed loop: first vertex repeated)
    std::vector<int> v2c_off, v2c;     // CSR [nop+1]
    std::vector<double> v2c_wt;
    std::vector<int> newnum;           // file cell index -> renumbered index
    uns_cc_mesh view() const;
};

// NC mesh after geometric (NCFVM/geometric.f90:1-806).
struct MeshNC {
    int nop = 0, noc = 0, nof = 0;
    std::vector<double> px, py, cv;
    std::vector<int> pbc;
    std::vector<double> cx, cy, ccv;   // cell data (unchanged by renumbering)
    std::vector<int> fp1, fp2, fin, fout, fbc;
    std::vector<double> fnx, fny, farea, fcx, fcy, fcov;
    std::vector<int> v2v_off, v2v;
    std::vector<double> wx, wy;
    std::vector<int> v2f_off, v2f;
    std::vector<int> newnum;           // file node index -> renumbered index
    uns_nc_mesh view() const;
};

struct AirfoilSpec {
    int ni = 128, nj = 64;       // circumferential x radial quads
    double thickness = 0.12;     // symmetric 4-digit thickness / chord
    double rfar = 20.0;          // farfield radius [chord]
    double dwall = 1e-3;         // first radial spacing at the wall [chord]
    // Optional wall-node y displacements [ni] (shape perturbations): node i
    // of the wall moves by dy[i] and the points of its radial line follow
    // with weight 1 - s, s the line's fractional arc position (0 at the
    // wall, 1 at the farfield), so the farfield stays fixed.
    const double* dy = nullptr;
};

// Analytic airfoil O-mesh, quads split into two triangles.
int gen_airfoil_cc(const AirfoilSpec& s, RawCC& out, std::string& err);
int gen_airfoil_nc(const AirfoilSpec& s, RawNC& out, std::string& err);

// Single-block plot3d O-grid (MeshGen's input), triangulated as the generator does.
int read_plot3d_cc(const std::string& path, RawCC& out, std::string& err);
int read_plot3d_nc(const std::string& path, RawNC& out, std::string& err);
int write_plot3d_airfoil(const AirfoilSpec& s, const std::string& path, std::string& err);

int read_geometry_cc(const std::string& path, RawCC& out, std::string& err);
int write_geometry_cc(const std::string& path, const RawCC& m, std::string& err);
int read_geometry_nc(const std::string& path, RawNC& out, std::string& err);
int write_geometry_nc(const std::string& path, const RawNC& m, std::string& err);

int geometric_cc(const RawCC& raw, MeshCC& m, std::string& err);
int geometric_nc(const RawNC& raw, MeshNC& m, std::string& err);

// Shape derivatives (host_shape.cpp): raw rebuilt at moved nodes, and the
// transpose of geometric_cc onto the node coordinates.
int moved_cc(const RawCC& raw, const double* px, const double* py, RawCC& out, std::string& err);
int mesh_vjp_cc(const MeshCC& m, const uns_cc_mesh_adj& a, double* gpx, double* gpy, std::string& err);

// flo.inp readers (CCFVM/read_input.F90:4-121, NCFVM/read_input.f90:4-86).
int read_flo_inp_cc(const std::string& path, uns_params& p, std::string& gridfile, std::string& err);
int read_flo_inp_nc(const std::string& path, uns_params& p, std::string& gridfile, std::string& err);

// Shared by libunsflow_host.so and libunsflow_driver.so: the calling thread's
// message for uns_host_last_error (returns code), the Fortran Ew.d edit
// descriptor, and path helpers.
int fail(int code, const std::string& msg);
std::string fort_e(double x, int w, int d);
std::string dir_of(const std::string& p);
std::string join(const std::string& d, const std::string& f);

}  // namespace unshost
