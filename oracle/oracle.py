"""TEST INFRASTRUCTURE ONLY -- ctypes face of the CPU oracle (oracle/_build/liboracle.so).

Used by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker.  The method names match unsflow2d_gb300.solver so a parity test runs
the same call sequence on both.  PARITY UNPINNED: see oracle.h.
"""
from __future__ import annotations

import ctypes as C
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent))

from unsflow2d_gb300 import abi  # noqa: E402

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        import importlib.util
        spec = importlib.util.spec_from_file_location("oracle_build", HERE / "build.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        path = mod.build()
        L = C.CDLL(str(path))
        vp, i32, dp = C.c_void_p, C.c_int, C.POINTER(C.c_double)
        ip = C.POINTER(C.c_int)
        sig = {
            "oracle_cc_create": ([C.POINTER(abi.CCMeshView), C.POINTER(abi.Params)], vp),
            "oracle_cc_free": ([vp], None), "oracle_cc_initialize": ([vp], i32),
            "oracle_cc_set_state": ([vp, dp], i32), "oracle_cc_con2prim": ([vp], i32),
            "oracle_cc_avg_c2v": ([vp], i32), "oracle_cc_time_step": ([vp, C.c_double, dp], i32),
            "oracle_cc_save_old": ([vp], i32), "oracle_cc_gradient": ([vp], i32), "oracle_cc_limit": ([vp], i32),
            "oracle_cc_fvresidual": ([vp], i32), "oracle_cc_rk_stage": ([vp, i32], i32),
            "oracle_cc_lusgs": ([vp], i32), "oracle_cc_check_positivity": ([vp, ip], i32),
            "oracle_cc_residue": ([vp, dp], i32), "oracle_cc_forces": ([vp, dp, dp], i32),
            "oracle_cc_iteration": ([vp, C.c_double, dp], i32), "oracle_cc_get": ([vp, i32, dp], i32),
            "oracle_cc_set": ([vp, i32, dp], i32), "oracle_nc_set": ([vp, i32, dp], i32),
            "oracle_nc_create": ([C.POINTER(abi.NCMeshView), C.POINTER(abi.Params)], vp),
            "oracle_nc_free": ([vp], None), "oracle_nc_initialize": ([vp], i32),
            "oracle_nc_set_state": ([vp, dp], i32), "oracle_nc_save_old": ([vp], i32),
            "oracle_nc_fvresidual": ([vp, C.c_double], i32), "oracle_nc_rk_stage": ([vp, i32], i32),
            "oracle_nc_lusgs": ([vp, C.c_double], i32), "oracle_nc_residue": ([vp, dp, dp, ip], i32),
            "oracle_nc_iteration": ([vp, C.c_double, dp, dp], i32), "oracle_nc_get": ([vp, i32, dp], i32),
            "oracle_cc_cs_create": ([C.POINTER(abi.CCMeshView), C.POINTER(abi.Params), C.c_double], vp),
            "oracle_cc_cs_free": ([vp], None), "oracle_cc_cs_set": ([vp, i32, dp, dp], i32),
            "oracle_cc_cs_get": ([vp, i32, dp, dp], i32), "oracle_cc_cs_iteration": ([vp, C.c_double], i32),
            "oracle_cc_cs_forces": ([vp, dp, dp], i32), "oracle_cc_cs_freeze_dt": ([vp, i32], i32),
            "oracle_cc_cs_set_geometry_im": ([vp, i32, dp], i32),
            "oracle_cc_find_cl_cd": ([vp, C.c_double, C.c_double, dp, dp, ip], i32),
            "oracle_cc_screen_minmax": ([vp, dp], i32), "oracle_cc_tecplt": ([vp, dp], i32),
            "oracle_nc_tecplt": ([vp, dp], i32), "oracle_nc_screen_minmax": ([vp, dp], i32),
        }
        for fn, (args, res) in sig.items():
            f = getattr(L, fn)
            f.argtypes, f.restype = args, res
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class OracleError(RuntimeError):
    pass


class _Oracle:
    kind = ""

    def _call(self, name, *args):
        rc = getattr(self._L, f"oracle_{self.kind}_{name}")(self._h, *args)
        if rc != 0:
            raise OracleError(f"oracle_{self.kind}_{name}: {abi.STATUS.get(rc, rc)}")
        return rc

    def close(self):
        if getattr(self, "_h", None):
            getattr(self._L, f"oracle_{self.kind}_free")(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initialize(self):
        self._call("initialize")

    def set_state(self, qc):
        a = np.ascontiguousarray(qc, dtype=np.float64)
        self._call("set_state", _dp(a))

    def get(self, field):
        out = np.zeros(self._field_shape(field))
        self._call("get", self.fields[field], _dp(out))
        return out

    def get_state(self):
        return self.get("qc")

    def set(self, field, data):
        a = np.ascontiguousarray(data, dtype=np.float64)
        assert a.size == int(np.prod(self._field_shape(field))), field
        self._call("set", self.fields[field], _dp(a))


class OracleCC(_Oracle):
    kind = "cc"
    fields = abi.CC_FIELDS

    def __init__(self, mesh, params):
        self._L = lib()
        arr = mesh.arrays if hasattr(mesh, "arrays") else mesh
        self.m = arr
        view, self._keep = abi.cc_view_from_arrays(arr)
        self._h = self._L.oracle_cc_create(C.byref(view), C.byref(params))
        self.params = params
        self.noc, self.nbf = arr["noc"], arr["nbf"]
        self.nstate = self.noc + self.nbf
        self.initialize()

    def _field_shape(self, f):
        m = self.m
        nof = m["nfi"] + m["nbf"]
        return {"qc": (self.nstate, 4), "qp": (self.nstate, 5), "qold": (self.noc, 4), "res": (self.noc, 4),
                "grad": (self.noc, 4, 2), "phi": (self.noc, 4), "dt": (self.noc,), "la": (self.noc,),
                "ptprim": (m["nop"], 5), "fqp": (nof, 5), "fla": (nof,), "fmu": (nof,),
                "fgrad": (nof, 5, 2), "mul": (self.noc,)}[f]

    def find_cl_cd(self, xref=0.25, yref=0.0):
        coef, wall, n = np.zeros(5), np.zeros((self.nbf, 4)), C.c_int()
        self._call("find_cl_cd", C.c_double(xref), C.c_double(yref), _dp(coef), _dp(wall), C.byref(n))
        return coef, wall[:n.value]

    def screen_minmax(self):
        out = np.zeros(14)
        self._call("screen_minmax", _dp(out))
        return out.reshape(7, 2)

    def tecplt(self):
        out = np.zeros((self.m["nop"], 11))
        self._call("tecplt", _dp(out))
        return out

    def con2prim(self): self._call("con2prim")
    def avg_c2v(self): self._call("avg_c2v")
    def save_old(self): self._call("save_old")
    def gradient(self): self._call("gradient")
    def limit(self): self._call("limit")
    def fvresidual(self): self._call("fvresidual")
    def rk_stage(self, irk): self._call("rk_stage", irk)
    def lusgs(self): self._call("lusgs")

    def time_step(self, cfl):
        d = C.c_double()
        self._call("time_step", C.c_double(cfl), C.byref(d))
        return d.value

    def check_positivity(self):
        bad = C.c_int(-1)
        self._call("check_positivity", C.byref(bad))
        return bad.value

    def residue(self):
        d = C.c_double()
        self._call("residue", C.byref(d))
        return d.value

    def forces(self):
        fx, fy = C.c_double(), C.c_double()
        self._call("forces", C.byref(fx), C.byref(fy))
        return fx.value, fy.value

    def iteration(self, cfl):
        d = C.c_double()
        self._call("iteration", C.c_double(cfl), C.byref(d))
        return d.value


class OracleNC(_Oracle):
    kind = "nc"
    fields = abi.NC_FIELDS

    def __init__(self, mesh, params):
        self._L = lib()
        arr = mesh.arrays if hasattr(mesh, "arrays") else mesh
        self.m = arr
        view, self._keep = abi.nc_view_from_arrays(arr)
        self._h = self._L.oracle_nc_create(C.byref(view), C.byref(params))
        self.params = params
        self.nop = arr["nop"]
        self.nstate = self.nop
        self.initialize()

    def _field_shape(self, f):
        return {"qc": (self.nop, 4), "qp": (self.nop, 4), "qold": (self.nop, 4), "res": (self.nop, 4),
                "grad": (self.nop, 4, 2), "phi": (self.nop, 4), "dt": (self.nop,), "la": (self.nop,),
                "fla": (self.m["nof"],)}[f]

    def save_old(self): self._call("save_old")
    def fvresidual(self, cfl): self._call("fvresidual", C.c_double(cfl))
    def rk_stage(self, irk): self._call("rk_stage", irk)
    def lusgs(self, cfl): self._call("lusgs", C.c_double(cfl))

    def residue(self):
        f, fi, ii = C.c_double(), C.c_double(), C.c_int()
        self._call("residue", C.byref(f), C.byref(fi), C.byref(ii))
        return f.value, fi.value, ii.value

    def iteration(self, cfl):
        f, fi = C.c_double(), C.c_double()
        self._call("iteration", C.c_double(cfl), C.byref(f), C.byref(fi))
        return f.value, fi.value

    def tecplt(self):
        out = np.zeros((self.nop, 7))
        self._call("tecplt", _dp(out))
        return out

    def screen_minmax(self):
        out = np.zeros(12)
        self._call("screen_minmax", _dp(out))
        return out.reshape(6, 2)


class OracleCCComplexStep:
    """The CCFVM oracle on complex-step numbers (oracle_cc_cs.cpp): one main-loop
    iteration from a state x + i*im, returning real and imaginary parts.  With
    im = h*u (h ~ 1e-30) Im(G)/h is the exact derivative of the iteration in
    direction u; aoa_im perturbs the angle of attack (radians) the same way."""

    def __init__(self, mesh, params, aoa_im: float = 0.0):
        self._L = lib()
        arr = mesh.arrays if hasattr(mesh, "arrays") else mesh
        view, self._keep = abi.cc_view_from_arrays(arr)
        self._h = self._L.oracle_cc_cs_create(C.byref(view), C.byref(params), C.c_double(aoa_im))
        self.noc, self.nbf = arr["noc"], arr["nbf"]
        self.nstate = self.noc + self.nbf

    def set(self, field: str, re: np.ndarray, im: np.ndarray | None = None) -> None:
        re = np.ascontiguousarray(re, dtype=np.float64)
        im = np.zeros_like(re) if im is None else np.ascontiguousarray(im, dtype=np.float64)
        if self._L.oracle_cc_cs_set(self._h, abi.CC_FIELDS[field], _dp(re), _dp(im)):
            raise OracleError(f"oracle_cc_cs_set {field}")

    def get(self, field: str) -> np.ndarray:
        shape = (self.nstate, 4) if field == "qc" else (self.nstate, 5)
        re, im = np.zeros(shape), np.zeros(shape)
        if self._L.oracle_cc_cs_get(self._h, abi.CC_FIELDS[field], _dp(re), _dp(im)):
            raise OracleError(f"oracle_cc_cs_get {field}")
        return re + 1j * im

    def iteration(self, cfl: float) -> None:
        if self._L.oracle_cc_cs_iteration(self._h, C.c_double(cfl)):
            raise OracleError("oracle_cc_cs_iteration")

    def freeze_dt(self, on: bool = True) -> None:
        """Hold the RK update's dt / cv real (no derivative), as the adjoint does."""
        self._L.oracle_cc_cs_freeze_dt(self._h, int(on))

    def set_geometry_im(self, field: str, im: np.ndarray) -> None:
        """Imaginary parts of one geometric mesh array (abi.CC_GEOM_FIELDS name)."""
        a = np.ascontiguousarray(im, dtype=np.float64)
        if self._L.oracle_cc_cs_set_geometry_im(self._h, abi.CC_GEOM_FIELDS.index(field), _dp(a)):
            raise OracleError(f"oracle_cc_cs_set_geometry_im {field}")

    def forces(self) -> tuple[complex, complex]:
        fx, fy = np.zeros(2), np.zeros(2)
        self._L.oracle_cc_cs_forces(self._h, _dp(fx), _dp(fy))
        return complex(fx[0], fx[1]), complex(fy[0], fy[1])

    def close(self):
        if getattr(self, "_h", None):
            self._L.oracle_cc_cs_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
