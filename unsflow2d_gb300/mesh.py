"""Caller-side meshes: analytic airfoil O-meshes and geometry.inp files, after the
reference's geometric preprocessing (libunsflow_host.so)."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi


class _HostMesh:
    kind = ""

    def __init__(self, handle: int):
        self._lib = abi.host_lib()
        self._h = C.c_void_p(handle)
        view_t = abi.CCMeshView if self.kind == "cc" else abi.NCMeshView
        v = view_t()
        fn = getattr(self._lib, f"uns_host_{self.kind}_view")
        abi.check(fn(self._h, C.byref(v)), self._lib, "view")
        self.arrays = abi.cc_view_arrays(v) if self.kind == "cc" else abi.nc_view_arrays(v)

    @classmethod
    def airfoil(cls, ni: int, nj: int, thickness: float = 0.12, rfar: float = 20.0, dwall: float = 1e-3):
        lib = abi.host_lib()
        h = C.c_void_p()
        fn = getattr(lib, f"uns_host_{cls.kind}_airfoil")
        abi.check(fn(ni, nj, thickness, rfar, dwall, C.byref(h)), lib, f"{cls.kind} airfoil")
        return cls(h.value)

    @classmethod
    def read(cls, path: str):
        lib = abi.host_lib()
        h = C.c_void_p()
        fn = getattr(lib, f"uns_host_{cls.kind}_read")
        abi.check(fn(str(path).encode(), C.byref(h)), lib, f"read {path}")
        return cls(h.value)

    @classmethod
    def plot3d(cls, path: str):
        """A single-block plot3d O-grid (MeshGen's input), triangulated."""
        lib = abi.host_lib()
        h = C.c_void_p()
        fn = getattr(lib, f"uns_host_{cls.kind}_plot3d")
        abi.check(fn(str(path).encode(), C.byref(h)), lib, f"plot3d {path}")
        return cls(h.value)

    def write(self, path: str) -> None:
        fn = getattr(self._lib, f"uns_host_{self.kind}_write")
        abi.check(fn(self._h, str(path).encode()), self._lib, f"write {path}")

    def newnum(self) -> np.ndarray:
        n = self.arrays["noc"] if self.kind == "cc" else self.arrays["nop"]
        out = np.zeros(n, dtype=np.int32)
        fn = getattr(self._lib, f"uns_host_{self.kind}_newnum")
        abi.check(fn(self._h, out.ctypes.data_as(C.POINTER(C.c_int32))), self._lib, "newnum")
        return out

    def __getitem__(self, k):
        return self.arrays[k]

    def close(self) -> None:
        if self._h:
            getattr(self._lib, f"uns_host_{self.kind}_free")(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CCMesh(_HostMesh):
    """Cell-centred mesh (CCFVM geometry.inp + CCFVM/geometric.F90)."""
    kind = "cc"

    @classmethod
    def airfoil_dy(cls, ni: int, nj: int, dy, thickness: float = 0.12, rfar: float = 20.0, dwall: float = 1e-3):
        """The airfoil mesh with wall node i displaced by dy[i] in y (radial lines follow)."""
        lib = abi.host_lib()
        h = C.c_void_p()
        d = np.ascontiguousarray(dy, dtype=np.float64)
        assert d.shape == (ni,)
        abi.check(lib.uns_host_cc_airfoil_dy(ni, nj, thickness, rfar, dwall, d.ctypes.data_as(C.POINTER(C.c_double)),
                                             C.byref(h)), lib, "cc airfoil dy")
        return cls(h.value)

    def moved(self, px, py) -> "CCMesh":
        """This mesh with its nodes at (px, py): same topology, the moved
        triangles' centroids and areas, then the geometric preprocessing."""
        x = np.ascontiguousarray(px, dtype=np.float64)
        y = np.ascontiguousarray(py, dtype=np.float64)
        n = self.arrays["nop"]
        assert x.shape == (n,) and y.shape == (n,)
        h = C.c_void_p()
        abi.check(self._lib.uns_host_cc_moved(self._h, x.ctypes.data_as(abi._D), y.ctypes.data_as(abi._D), C.byref(h)),
                  self._lib, "cc moved")
        return CCMesh(h.value)

    def node_adjoint(self, geom: dict) -> tuple[np.ndarray, np.ndarray]:
        """dJ/d(px, py) from the adjoints of this mesh's geometric arrays
        (solver.CCSolver.adjoint_geometry): the transposed geometric
        preprocessing (uns_host_cc_mesh_vjp)."""
        st, keep = abi.cc_mesh_adj(self.arrays, geom)
        n = self.arrays["nop"]
        gx, gy = np.zeros(n), np.zeros(n)
        abi.check(self._lib.uns_host_cc_mesh_vjp(self._h, C.byref(st), gx.ctypes.data_as(abi._D),
                                                 gy.ctypes.data_as(abi._D)), self._lib, "cc mesh vjp")
        del keep
        return gx, gy

    @property
    def ncells(self) -> int:
        return self.arrays["noc"]


class NCMesh(_HostMesh):
    """Vertex-centred median-dual mesh (NCFVM geometry.inp + NCFVM/geometric.f90)."""
    kind = "nc"

    @property
    def nnodes(self) -> int:
        return self.arrays["nop"]


def write_airfoil_plot3d(path: str, ni: int, nj: int, thickness: float = 0.12, rfar: float = 20.0,
                         dwall: float = 1e-3) -> None:
    """The analytic airfoil O-grid as a single-block plot3d file."""
    lib = abi.host_lib()
    abi.check(lib.uns_host_airfoil_plot3d(ni, nj, thickness, rfar, dwall, str(path).encode()), lib, "plot3d write")


def read_flo_inp(path: str, kind: str = "cc") -> tuple[abi.Params, str]:
    lib = abi.host_lib()
    p = abi.Params()
    grid = C.create_string_buffer(256)
    fn = lib.uns_host_read_flo_cc if kind == "cc" else lib.uns_host_read_flo_nc
    abi.check(fn(str(path).encode(), C.byref(p), grid, 256), lib, f"flo.inp {path}")
    return p, grid.value.decode()


def cfl_schedule(p: abi.Params, first: int, n: int, kind: str = "cc", prev: float = 0.0) -> np.ndarray:
    """CFL of iterations first..first+n-1 (CCFVM/main.F90:148-168, NCFVM/main.f90:54)."""
    lib = abi.host_lib()
    out = np.zeros(n)
    c = prev
    for k in range(n):
        if kind == "cc":
            c = lib.uns_host_cfl_cc(C.byref(p), first + k, c)
        else:
            c = lib.uns_host_cfl_nc(C.byref(p), first + k)
        out[k] = c
    return out


def run_main(flo_inp: str, outdir: str, kind: str = "cc", mode: int = 1) -> tuple[int, float]:
    """Reference main program on the GPU library; writes outdir/FLO.RES."""
    lib = abi.driver_lib()
    it = C.c_int()
    fr = C.c_double()
    fn = lib.uns_host_cc_main if kind == "cc" else lib.uns_host_nc_main
    abi.check(fn(str(flo_inp).encode(), str(outdir).encode(), mode, C.byref(it), C.byref(fr)), lib, "main")
    return it.value, fr.value


def cc_cell_vertices(arrays: dict) -> np.ndarray:
    """Vertices of each interior cell (0-based), from its faces' end points in
    c2f order: the first face's two points, then the others' new points."""
    off, c2f, fp1, fp2 = arrays["c2f_off"], arrays["c2f"], arrays["fp1"], arrays["fp2"]
    out = []
    for i in range(int(arrays["noc"])):
        vs: list[int] = []
        for f in c2f[off[i]:off[i + 1]]:
            for p in (int(fp1[f]), int(fp2[f])):
                if p not in vs:
                    vs.append(p)
        out.append(vs)
    return np.array(out, dtype=np.int64)


def write_tecplt(path, table: np.ndarray, variables: list[str], elements: np.ndarray | None = None) -> None:
    """The reference's tecplt.dat (CCFVM/main.F90:417-480, NCFVM/main.f90:
    190-233) from a device vertex table (uns_cc_tecplt / uns_nc_tecplt): node
    rows written 7 values per line (format 1x,7(f15.6,2x), reused for longer
    rows) and, when given, the elements' 1-based vertex lists."""
    with open(path, "w") as f:
        f.write(' TITLE = "flo2d output" \n')
        f.write(" VARIABLES=" + ",".join(f'"{v}"' for v in variables) + "\n")
        ne = 0 if elements is None else len(elements)
        et = "TRIANGLE" if elements is not None and elements.shape[1] == 3 else "quadrilateral"
        f.write(f" ZONE F=FEPOINT,ET={et}\n" if ne else " ZONE F=POINT\n")
        f.write(f" N={len(table)},E={ne}\n")
        for row in table:
            for k in range(0, len(row), 7):
                f.write(" " + "".join(f"{x:15.6f}  " for x in row[k:k + 7]) + "\n")
        if elements is not None:
            for e in elements:
                f.write(" " + " ".join(str(int(x) + 1) for x in e) + "\n")
