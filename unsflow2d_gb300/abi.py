"""ctypes mirror of include/unsflow_types.h plus loaders for the in-tree libraries.

The libraries are built in-tree by unsflow2d_gb300.build (called from
__graft_entry__.build()); loading fails loudly when they are missing -- there is
no CPU fallback for the GPU library.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_DIR = PKG / "lib"

# status codes
UNS_OK, UNS_ERR_ARG, UNS_ERR_CUDA, UNS_ERR_NEG_SOUND_SPEED, UNS_ERR_NONPOSITIVE, UNS_ERR_MESH, \
    UNS_ERR_TIMEOUT, UNS_ERR_NAN, UNS_ERR_IO, UNS_ERR_NOMEM = range(10)
STATUS = {0: "UNS_OK", 1: "UNS_ERR_ARG", 2: "UNS_ERR_CUDA", 3: "UNS_ERR_NEG_SOUND_SPEED",
          4: "UNS_ERR_NONPOSITIVE", 5: "UNS_ERR_MESH", 6: "UNS_ERR_TIMEOUT", 7: "UNS_ERR_NAN",
          8: "UNS_ERR_IO", 9: "UNS_ERR_NOMEM"}

FLOW = {"inviscid": 0, "laminar": 1}
FLUX = {"roe": 0, "ausm": 1, "vanleer": 2, "rusanov": 3}
GRAD = {"gg": 0, "ggfc": 1, "lsqr": 2}
TIME = {"rk3": 0, "lusgs": 1}
CFLT = {"tanh": 0, "ramp": 1}
LIMITER = {"vkn": 0, "barth": 1, "barth_corrected": 2}
PREC = {"fp64": 0, "mixed": 1, "mixed_sweep": 2}
OBJ = {"cl": 0, "cd": 1}

CC_FIELDS = {"qc": 0, "qp": 1, "qold": 2, "res": 3, "grad": 4, "phi": 5, "dt": 6, "la": 7,
             "ptprim": 8, "fqp": 9, "fla": 10, "fmu": 11, "fgrad": 12, "mul": 13, "fwall": 14}
NC_FIELDS = {"qc": 0, "qp": 1, "qold": 2, "res": 3, "grad": 4, "phi": 5, "dt": 6, "la": 7, "fla": 8}


class UnsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class Params(C.Structure):
    _fields_ = [("m_inf", C.c_double), ("aoa_deg", C.c_double), ("rey", C.c_double), ("t_wall", C.c_double),
                ("flow_type", C.c_int32), ("iwall", C.c_int32), ("flux_type", C.c_int32),
                ("grad_type", C.c_int32), ("ilimit", C.c_int32), ("irs", C.c_int32),
                ("time_mode", C.c_int32), ("cfl_type", C.c_int32), ("cfl_min", C.c_double),
                ("cfl_max", C.c_double), ("cfl_ramp_steps", C.c_int32), ("limiter_type", C.c_int32),
                ("precision", C.c_int32), ("max_iter", C.c_int32), ("min_res", C.c_double),
                ("scr_interval", C.c_int32), ("istart", C.c_int32)]


def make_params(m_inf=0.5, aoa_deg=2.0, rey=5000.0, t_wall=300.0, flow="inviscid", iwall=1,
                flux="roe", grad="gg", ilimit=1, irs=0, time="rk3", cfl_type="tanh", cfl_min=0.1,
                cfl_max=0.9, cfl_ramp_steps=500, limiter="vkn", precision="fp64", max_iter=2000,
                min_res=1e-8, scr_interval=100, istart=1) -> Params:
    return Params(m_inf, aoa_deg, rey, t_wall, FLOW[flow], iwall, FLUX[flux], GRAD[grad], ilimit, irs,
                  TIME[time], CFLT[cfl_type], cfl_min, cfl_max, cfl_ramp_steps, LIMITER[limiter],
                  PREC[precision], max_iter, min_res, scr_interval, istart)


_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)


class CCMeshView(C.Structure):
    _fields_ = [("nop", C.c_int32), ("noc", C.c_int32), ("nfi", C.c_int32), ("nbf", C.c_int32),
                ("px", _D), ("py", _D), ("cx", _D), ("cy", _D), ("cv", _D), ("cov", _D),
                ("fp1", _I), ("fp2", _I), ("fin", _I), ("fout", _I), ("fbc", _I),
                ("fnx", _D), ("fny", _D), ("farea", _D), ("fcx", _D), ("fcy", _D),
                ("r11", _D), ("r12", _D), ("r22", _D), ("nc2c", _I),
                ("c2f_off", _I), ("c2f", _I), ("v2c_off", _I), ("v2c", _I), ("v2c_wt", _D)]


class NCMeshView(C.Structure):
    _fields_ = [("nop", C.c_int32), ("noc", C.c_int32), ("nof", C.c_int32), ("pad_", C.c_int32),
                ("px", _D), ("py", _D), ("cv", _D), ("fp1", _I), ("fp2", _I), ("fbc", _I),
                ("fnx", _D), ("fny", _D), ("farea", _D), ("v2v_off", _I), ("v2v", _I),
                ("wx", _D), ("wy", _D), ("v2f_off", _I), ("v2f", _I)]


#: Geometric arrays of a CC mesh, in uns_cc_mesh_adj order, and their lengths.
CC_GEOM_FIELDS = ("px", "py", "cx", "cy", "cv", "cov", "fnx", "fny", "farea", "fcx", "fcy", "r11", "r12", "r22",
                  "v2c_wt")


class CCMeshAdj(C.Structure):
    _fields_ = [(k, _D) for k in CC_GEOM_FIELDS]


def cc_geom_sizes(arr: dict) -> dict:
    nop, noc, nof, ntot = arr["nop"], arr["noc"], arr["nfi"] + arr["nbf"], arr["noc"] + arr["nbf"]
    n = {"px": nop, "py": nop, "cx": ntot, "cy": ntot, "cv": noc, "cov": noc, "r11": noc, "r12": noc, "r22": noc,
         "v2c_wt": int(arr["v2c_off"][-1])}
    n.update({k: nof for k in ("fnx", "fny", "farea", "fcx", "fcy")})
    return n


def cc_mesh_adj(arr: dict, values: dict | None = None) -> tuple[CCMeshAdj, dict]:
    """A uns_cc_mesh_adj over numpy arrays sized for mesh `arr` (zeros, or
    copies of `values`); returns the struct and the arrays it points into."""
    out = {}
    for k, n in cc_geom_sizes(arr).items():
        out[k] = np.zeros(n) if values is None else np.ascontiguousarray(values[k], dtype=np.float64).copy()
        assert out[k].shape == (n,), k
    st = CCMeshAdj(**{k: out[k].ctypes.data_as(_D) for k in CC_GEOM_FIELDS})
    return st, out


def _arr(ptr, n, dtype):
    if n == 0:
        return np.zeros(0, dtype=dtype)
    ct = C.c_double if dtype == np.float64 else C.c_int32
    buf = C.cast(ptr, C.POINTER(ct * n)).contents
    return np.frombuffer(buf, dtype=dtype).copy()


def cc_view_arrays(v: CCMeshView) -> dict:
    """Copy a CC mesh view into numpy arrays (host-owned, independent of the handle)."""
    nop, noc, nfi, nbf = v.nop, v.noc, v.nfi, v.nbf
    nof, ntot = nfi + nbf, noc + nbf
    d, i = np.float64, np.int32
    out = {"nop": nop, "noc": noc, "nfi": nfi, "nbf": nbf,
           "px": _arr(v.px, nop, d), "py": _arr(v.py, nop, d), "cx": _arr(v.cx, ntot, d),
           "cy": _arr(v.cy, ntot, d), "cv": _arr(v.cv, noc, d), "cov": _arr(v.cov, noc, d)}
    for k in ("fp1", "fp2", "fin", "fout", "fbc"):
        out[k] = _arr(getattr(v, k), nof, i)
    for k in ("fnx", "fny", "farea", "fcx", "fcy"):
        out[k] = _arr(getattr(v, k), nof, d)
    for k in ("r11", "r12", "r22"):
        out[k] = _arr(getattr(v, k), noc, d)
    out["nc2c"] = _arr(v.nc2c, noc, i)
    out["c2f_off"] = _arr(v.c2f_off, noc + 1, i)
    out["c2f"] = _arr(v.c2f, int(out["c2f_off"][-1]), i)
    out["v2c_off"] = _arr(v.v2c_off, nop + 1, i)
    out["v2c"] = _arr(v.v2c, int(out["v2c_off"][-1]), i)
    out["v2c_wt"] = _arr(v.v2c_wt, int(out["v2c_off"][-1]), d)
    return out


def nc_view_arrays(v: NCMeshView) -> dict:
    nop, nof = v.nop, v.nof
    d, i = np.float64, np.int32
    out = {"nop": nop, "noc": v.noc, "nof": nof, "px": _arr(v.px, nop, d), "py": _arr(v.py, nop, d),
           "cv": _arr(v.cv, nop, d)}
    for k in ("fp1", "fp2", "fbc"):
        out[k] = _arr(getattr(v, k), nof, i)
    for k in ("fnx", "fny", "farea"):
        out[k] = _arr(getattr(v, k), nof, d)
    out["v2v_off"] = _arr(v.v2v_off, nop + 1, i)
    out["v2v"] = _arr(v.v2v, int(out["v2v_off"][-1]), i)
    out["wx"] = _arr(v.wx, int(out["v2v_off"][-1]), d)
    out["wy"] = _arr(v.wy, int(out["v2v_off"][-1]), d)
    out["v2f_off"] = _arr(v.v2f_off, nop + 1, i)
    out["v2f"] = _arr(v.v2f, int(out["v2f_off"][-1]), i)
    return out


def _ptr(a: np.ndarray, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def cc_view_from_arrays(m: dict) -> tuple[CCMeshView, list]:
    """Build a CC view over numpy arrays; the returned list keeps them alive."""
    keep = []

    def D(k):
        a = np.ascontiguousarray(m[k], dtype=np.float64); keep.append(a); return _ptr(a, C.c_double)

    def I(k):
        a = np.ascontiguousarray(m[k], dtype=np.int32); keep.append(a); return _ptr(a, C.c_int32)

    v = CCMeshView(m["nop"], m["noc"], m["nfi"], m["nbf"], D("px"), D("py"), D("cx"), D("cy"), D("cv"),
                   D("cov"), I("fp1"), I("fp2"), I("fin"), I("fout"), I("fbc"), D("fnx"), D("fny"),
                   D("farea"), D("fcx"), D("fcy"), D("r11"), D("r12"), D("r22"), I("nc2c"), I("c2f_off"),
                   I("c2f"), I("v2c_off"), I("v2c"), D("v2c_wt"))
    return v, keep


def nc_view_from_arrays(m: dict) -> tuple[NCMeshView, list]:
    keep = []

    def D(k):
        a = np.ascontiguousarray(m[k], dtype=np.float64); keep.append(a); return _ptr(a, C.c_double)

    def I(k):
        a = np.ascontiguousarray(m[k], dtype=np.int32); keep.append(a); return _ptr(a, C.c_int32)

    v = NCMeshView(m["nop"], m["noc"], m["nof"], 0, D("px"), D("py"), D("cv"), I("fp1"), I("fp2"), I("fbc"),
                   D("fnx"), D("fny"), D("farea"), I("v2v_off"), I("v2v"), D("wx"), D("wy"), I("v2f_off"),
                   I("v2f"))
    return v, keep


_libs: dict[str, C.CDLL] = {}


def _load(name: str) -> C.CDLL:
    if name in _libs:
        return _libs[name]
    path = LIB_DIR / f"lib{name}.so"
    if not path.exists():
        raise ImportError(f"{path} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
                          "(there is no fallback implementation)")
    lib = C.CDLL(str(path), mode=C.RTLD_GLOBAL)
    _libs[name] = lib
    return lib


def gpu_library_name() -> str:
    """The GPU library this process uses: the bit-exact build, or with
    UNSFLOW_FP64_FMA=1 the one whose FP64 kernels contract multiply-adds."""
    return "unsflow_gpu_fma" if os.environ.get("UNSFLOW_FP64_FMA", "0") == "1" else "unsflow_gpu"


def gpu_lib() -> C.CDLL:
    lib = _load(gpu_library_name())
    if not getattr(lib, "_typed", False):
        vp, i32, dp = C.c_void_p, C.c_int, _D
        pp = C.POINTER(C.c_void_p)
        sig = {
            "uns_last_error": ([], C.c_char_p), "uns_version": ([], C.c_char_p),
            "uns_cc_create": ([C.POINTER(CCMeshView), C.POINTER(Params), pp], i32),
            "uns_cc_destroy": ([vp], i32), "uns_cc_initialize": ([vp], i32),
            "uns_cc_set_state": ([vp, dp], i32), "uns_cc_get_state": ([vp, dp], i32),
            "uns_cc_get_field": ([vp, i32, dp], i32), "uns_cc_con2prim": ([vp], i32),
            "uns_cc_avg_c2v": ([vp], i32), "uns_cc_time_step": ([vp, C.c_double, dp], i32),
            "uns_cc_save_old": ([vp], i32), "uns_cc_gradient": ([vp], i32), "uns_cc_limit": ([vp], i32),
            "uns_cc_fvresidual": ([vp], i32), "uns_cc_rk_stage": ([vp, i32], i32), "uns_cc_lusgs": ([vp], i32),
            "uns_cc_check_positivity": ([vp, C.POINTER(C.c_int)], i32), "uns_cc_residue": ([vp, dp], i32),
            "uns_cc_forces": ([vp, dp, dp], i32),
            "uns_cc_iterate": ([vp, i32, dp, i32, dp, C.POINTER(C.c_int)], i32),
            "uns_nc_create": ([C.POINTER(NCMeshView), C.POINTER(Params), pp], i32),
            "uns_nc_destroy": ([vp], i32), "uns_nc_initialize": ([vp], i32),
            "uns_nc_set_state": ([vp, dp], i32), "uns_nc_get_state": ([vp, dp], i32),
            "uns_nc_get_field": ([vp, i32, dp], i32), "uns_nc_save_old": ([vp], i32),
            "uns_nc_fvresidual": ([vp, C.c_double], i32), "uns_nc_rk_stage": ([vp, i32], i32),
            "uns_nc_lusgs": ([vp, C.c_double], i32),
            "uns_nc_residue": ([vp, dp, dp, C.POINTER(C.c_int)], i32),
            "uns_nc_iterate": ([vp, i32, dp, i32, dp, dp, C.POINTER(C.c_int)], i32),
            "uns_cc_stream": ([vp], vp), "uns_nc_stream": ([vp], vp),
            "uns_cc_profile": ([vp, C.c_double, i32, dp, C.POINTER(C.c_char_p), i32], i32),
            "uns_cc_autotune": ([vp, i32, C.POINTER(C.c_int)], i32),
            "uns_nc_profile": ([vp, C.c_double, i32, dp, C.POINTER(C.c_char_p), i32], i32),
            "uns_residue_rms_noalloc": ([vp, i32, dp, vp], i32),
            "uns_cc_set_wait_limit": ([vp, C.c_longlong], i32), "uns_nc_set_wait_limit": ([vp, C.c_longlong], i32),
            "uns_cc_debug_unpublish": ([vp, i32, i32], i32), "uns_nc_debug_unpublish": ([vp, i32, i32], i32),
            "uns_cc_batch_create": ([C.POINTER(C.c_void_p), i32, pp], i32), "uns_cc_batch_destroy": ([vp], i32),
            "uns_cc_batch_stream": ([vp], vp),
            "uns_cc_batch_iterate": ([vp, i32, dp, i32, dp, C.POINTER(C.c_int)], i32),
            "uns_cc_set_precision": ([vp, i32], i32), "uns_nc_set_precision": ([vp, i32], i32),
            "uns_cc_set_field": ([vp, i32, dp], i32),
            "uns_cc_find_cl_cd": ([vp, C.c_double, C.c_double, dp, dp, C.POINTER(C.c_int)], i32),
            "uns_cc_screen_minmax": ([vp, dp], i32), "uns_cc_tecplt": ([vp, dp], i32),
            "uns_nc_tecplt": ([vp, dp], i32), "uns_nc_screen_minmax": ([vp, dp], i32),
            "uns_nc_sweep_levels": ([vp, C.POINTER(C.c_int), C.POINTER(C.c_int)], i32),
            "uns_cc_create_packed": ([C.POINTER(CCMeshView), C.POINTER(Params), i32, pp], i32),
            "uns_cc_packed_layout": ([vp, C.POINTER(C.c_int), C.POINTER(C.c_int)], i32),
            "uns_cc_packed_iterate": ([vp, i32, dp, i32, dp, C.POINTER(C.c_int)], i32),
            "uns_cc_adjoint_prepare": ([vp, C.c_double, dp, dp], i32),
            "uns_cc_adjoint_vjp": ([vp, i32, C.c_double, dp, dp, dp, dp, dp], i32),
            "uns_cc_adjoint_solve": ([vp, i32, i32, C.c_double, dp, dp, C.POINTER(C.c_int)], i32),
            "uns_cc_adjoint_get": ([vp, dp, dp], i32),
            "uns_cc_adjoint_prepare_geometry": ([vp, C.c_double, dp, dp], i32),
            "uns_cc_adjoint_geometry": ([vp, i32, C.c_double, dp, dp, C.POINTER(CCMeshAdj)], i32),
        }
        for fn, (args, res) in sig.items():
            f = getattr(lib, fn)
            f.argtypes, f.restype = args, res
        lib._typed = True
        lib._kind = "gpu"
    return lib


def host_lib() -> C.CDLL:
    """libunsflow_host.so: meshes, flo.inp, CFL schedules, FLO.DAT (no GPU)."""
    lib = _load("unsflow_host")
    if not getattr(lib, "_typed", False):
        vp, i32, dp = C.c_void_p, C.c_int, C.c_double
        pp = C.POINTER(C.c_void_p)
        sig = {
            "uns_host_last_error": ([], C.c_char_p),
            "uns_host_cc_airfoil": ([i32, i32, dp, dp, dp, pp], i32),
            "uns_host_cc_airfoil_dy": ([i32, i32, dp, dp, dp, _D, pp], i32),
            "uns_host_cc_moved": ([vp, _D, _D, pp], i32),
            "uns_host_cc_mesh_vjp": ([vp, C.POINTER(CCMeshAdj), _D, _D], i32),
            "uns_host_cc_plot3d": ([C.c_char_p, pp], i32), "uns_host_nc_plot3d": ([C.c_char_p, pp], i32),
            "uns_host_airfoil_plot3d": ([i32, i32, dp, dp, dp, C.c_char_p], i32),
            "uns_host_nc_airfoil": ([i32, i32, dp, dp, dp, pp], i32),
            "uns_host_cc_read": ([C.c_char_p, pp], i32), "uns_host_nc_read": ([C.c_char_p, pp], i32),
            "uns_host_cc_write": ([vp, C.c_char_p], i32), "uns_host_nc_write": ([vp, C.c_char_p], i32),
            "uns_host_cc_view": ([vp, C.POINTER(CCMeshView)], i32),
            "uns_host_nc_view": ([vp, C.POINTER(NCMeshView)], i32),
            "uns_host_cc_newnum": ([vp, _I], i32), "uns_host_nc_newnum": ([vp, _I], i32),
            "uns_host_cc_free": ([vp], None), "uns_host_nc_free": ([vp], None),
            "uns_host_read_flo_cc": ([C.c_char_p, C.POINTER(Params), C.c_char_p, i32], i32),
            "uns_host_read_flo_nc": ([C.c_char_p, C.POINTER(Params), C.c_char_p, i32], i32),
            "uns_host_cfl_cc": ([C.POINTER(Params), i32, dp], dp),
            "uns_host_cfl_nc": ([C.POINTER(Params), i32], dp),
            "uns_host_save_flow": ([C.c_char_p, _D, i32], i32), "uns_host_read_flow": ([C.c_char_p, _D, i32], i32),
        }
        for fn, (args, res) in sig.items():
            f = getattr(lib, fn)
            f.argtypes, f.restype = args, res
        lib._typed = True
        lib._kind = "host"
    return lib


def driver_lib() -> C.CDLL:
    """libunsflow_driver.so: the main programs on the GPU library."""
    gpu_lib()
    host_lib()
    lib = _load("unsflow_driver")
    if not getattr(lib, "_typed", False):
        for fn in ("uns_host_cc_main", "uns_host_nc_main"):
            f = getattr(lib, fn)
            f.argtypes, f.restype = [C.c_char_p, C.c_char_p, C.c_int, C.POINTER(C.c_int), _D], C.c_int
        lib._typed = True
        lib._kind = "host"
    return lib


def check(rc: int, lib: C.CDLL, where: str) -> None:
    if rc != UNS_OK:
        getter = lib.uns_host_last_error if getattr(lib, "_kind", "") == "host" else lib.uns_last_error
        msg = getter()
        raise UnsError(rc, f"{where}: {msg.decode() if msg else ''}")
