"""Python face of the GB300 drop-in: one class per solver, one method per
reference subroutine, each a thin call into libunsflow_gpu.so.

The method names follow the Fortran routines they replace (fvresidual,
gradient, limit, time_step, lusgs, residue ...), so a test reads like the
reference main loop.  Nothing here computes: a missing library or a CUDA error
raises.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi


def _raise_with_history(rc: int, lib, where: str, history) -> None:
    if rc != abi.UNS_OK:
        msg = lib.uns_last_error()
        err = abi.UnsError(rc, f"{where}: {msg.decode() if msg else ''}")
        err.history = history
        raise err


def _dp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class _Solver:
    kind = ""
    fields: dict = {}

    def _call(self, name: str, *args):
        rc = getattr(self._lib, f"uns_{self.kind}_{name}")(self._h, *args)
        abi.check(rc, self._lib, f"uns_{self.kind}_{name}")

    def close(self) -> None:
        if getattr(self, "_h", None):
            getattr(self._lib, f"uns_{self.kind}_destroy")(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def initialize(self):
        self._call("initialize")

    def set_state(self, qc: np.ndarray):
        a = np.ascontiguousarray(qc, dtype=np.float64)
        assert a.size == self.nstate * 4
        self._call("set_state", _dp(a))

    def set_precision(self, precision: str) -> None:
        """Switch between "fp64", "mixed" and "mixed_sweep" between calls."""
        self._call("set_precision", abi.PREC[precision])

    def get_state(self) -> np.ndarray:
        out = np.zeros((self.nstate, 4))
        self._call("get_state", _dp(out))
        return out

    def stream(self) -> int:
        """cudaStream_t of this handle (for CUDA events recorded by the caller)."""
        return int(getattr(self._lib, f"uns_{self.kind}_stream")(self._h) or 0)

    def profile(self, cfl: float, reps: int = 3) -> dict:
        """Average device time [ms] of each phase of one iteration."""
        n = 16
        ms = np.zeros(n)
        names = (C.c_char_p * n)()
        self._call("profile", C.c_double(cfl), reps, _dp(ms), names, n)
        return {names[k].decode(): float(ms[k]) for k in range(n) if names[k] and names[k].decode()}

    def autotune(self, reps: int = 3) -> dict:
        """Pick the block sizes of the face, vertex and cell-gradient kernels by
        timing them on this handle (uns_cc_autotune; CCFVM only)."""
        if self.kind != "cc":
            raise NotImplementedError("the launch-geometry autotuner covers the CCFVM kernels")
        b = (C.c_int * 3)()
        self._call("autotune", reps, b)
        return {"face": b[0], "vertex": b[1], "cell_grad": b[2]}

    def set_wait_limit(self, cycles: int) -> None:
        """Bound of the LU-SGS sweeps' waits, in device clock cycles."""
        self._call("set_wait_limit", C.c_longlong(int(cycles)))

    def debug_unpublish(self, entity: int, sweep: int) -> None:
        """Test hook: sweep item (entity, sweep 0 forward / 1 backward)
        publishes nothing, so the items that need it wait until the wait
        limit and the sweep returns UNS_ERR_TIMEOUT; entity -1 clears it."""
        self._call("debug_unpublish", int(entity), int(sweep))

    def get(self, field: str) -> np.ndarray:
        shape = self._field_shape(field)
        out = np.zeros(shape)
        self._call("get_field", self.fields[field], _dp(out))
        return out


class CCSolver(_Solver):
    """Cell-centred solver (CCFVM hot path) on the GPU."""
    kind = "cc"
    fields = abi.CC_FIELDS

    def __init__(self, mesh, params: abi.Params):
        self._lib = abi.gpu_lib()
        arr = mesh.arrays if hasattr(mesh, "arrays") else mesh
        self.m = arr
        view, self._keep = abi.cc_view_from_arrays(arr)
        h = C.c_void_p()
        abi.check(self._lib.uns_cc_create(C.byref(view), C.byref(params), C.byref(h)), self._lib, "uns_cc_create")
        self._h = h
        self.params = params
        self.noc, self.nbf = arr["noc"], arr["nbf"]
        self.nstate = self.noc + self.nbf

    def _field_shape(self, f):
        m = self.m
        nof = m["nfi"] + m["nbf"]
        return {"qc": (self.nstate, 4), "qp": (self.nstate, 5), "qold": (self.noc, 4), "res": (self.noc, 4),
                "grad": (self.noc, 4, 2), "phi": (self.noc, 4), "dt": (self.noc,), "la": (self.noc,),
                "ptprim": (m["nop"], 5), "fqp": (nof, 5), "fla": (nof,), "fmu": (nof,),
                "fgrad": (nof, 5, 2), "mul": (self.noc,), "fwall": (self.nbf, 4)}[f]

    # one method per reference subroutine
    def con2prim(self): self._call("con2prim")
    def avg_c2v(self): self._call("avg_c2v")
    def save_old(self): self._call("save_old")
    def gradient(self): self._call("gradient")
    def limit(self): self._call("limit")
    def fvresidual(self): self._call("fvresidual")
    def rk_stage(self, irk: int): self._call("rk_stage", irk)
    def lusgs(self): self._call("lusgs")

    def time_step(self, cfl: float) -> float:
        d = C.c_double()
        self._call("time_step", C.c_double(cfl), C.byref(d))
        return d.value

    def check_positivity(self) -> int:
        bad = C.c_int(-1)
        self._call("check_positivity", C.byref(bad))
        return bad.value

    def residue(self) -> float:
        d = C.c_double()
        self._call("residue", C.byref(d))
        return d.value

    def forces(self) -> tuple[float, float]:
        fx, fy = C.c_double(), C.c_double()
        self._call("forces", C.byref(fx), C.byref(fy))
        return fx.value, fy.value

    def set(self, field: str, values: np.ndarray) -> None:
        """Overwrite "qc", "qp" (ghosts included, with T) or "phi"."""
        a = np.ascontiguousarray(values, dtype=np.float64)
        assert a.shape == self._field_shape(field), (field, a.shape)
        self._call("set_field", self.fields[field], _dp(a))

    def find_cl_cd(self, xref: float = 0.25, yref: float = 0.0):
        """find_cl_cd on the device: (C_L, C_D, C_m, C_L1, C_D1) and the wall rows (x, y, -C_p, C_f)."""
        coef, wall, n = np.zeros(5), np.zeros((self.nbf, 4)), C.c_int()
        self._call("find_cl_cd", C.c_double(xref), C.c_double(yref), _dp(coef), _dp(wall), C.byref(n))
        return coef, wall[:n.value]

    def screen_minmax(self) -> np.ndarray:
        """screen's [7][2] min/max of density, u, v, p, T, Mach, entropy."""
        out = np.zeros(14)
        self._call("screen_minmax", _dp(out))
        return out.reshape(7, 2)

    def tecplt(self) -> np.ndarray:
        """tecplt's [nop][11] vertex table: x, y, density, u, v, Mach, p, T, entropy, |V|, mu."""
        out = np.zeros((self.m["nop"], 11))
        self._call("tecplt", _dp(out))
        return out

    def cl_cd(self) -> tuple[float, float]:
        """Flux-based C_L, C_D of the last residual (CCFVM/main.F90:348-353)."""
        fx, fy = self.forces()
        a = np.deg2rad(self.params.aoa_deg)
        return 2.0 * (fy * np.cos(a) - fx * np.sin(a)), 2.0 * (fx * np.cos(a) + fy * np.sin(a))

    # discrete adjoint (no reference counterpart)
    def adjoint_prepare(self, cfl: float) -> tuple[float, float]:
        """Record the linearisation at the current (converged) state; returns C_L, C_D."""
        cl, cd = C.c_double(), C.c_double()
        self._call("adjoint_prepare", C.c_double(cfl), C.byref(cl), C.byref(cd))
        return cl.value, cd.value

    def adjoint_vjp(self, objective: str, seed: float, wq: np.ndarray, wg: np.ndarray):
        """One transposed iteration: returns (G_s^T w + seed J_s^T, G_alpha^T w + seed J_alpha)."""
        wq = np.ascontiguousarray(wq, dtype=np.float64).reshape(self.noc, 4)
        wg = np.ascontiguousarray(wg, dtype=np.float64).reshape(self.nbf, 5)
        oq, og, oa = np.zeros((self.noc, 4)), np.zeros((self.nbf, 5)), C.c_double()
        self._call("adjoint_vjp", abi.OBJ[objective], C.c_double(seed), _dp(wq), _dp(wg), _dp(oq), _dp(og), C.byref(oa))
        return oq, og, oa.value

    def adjoint_solve(self, objective: str, max_iter: int = 20000, tol: float = 1e-10):
        """Reverse accumulation to convergence; returns (dJ/dalpha per radian, change history)."""
        hist = np.zeros(max_iter)
        d, it = C.c_double(), C.c_int()
        self._call("adjoint_solve", abi.OBJ[objective], max_iter, C.c_double(tol), C.byref(d), _dp(hist), C.byref(it))
        return d.value, hist[:it.value]

    def adjoint_get(self) -> tuple[np.ndarray, np.ndarray]:
        lq, lg = np.zeros((self.noc, 4)), np.zeros((self.nbf, 5))
        self._call("adjoint_get", _dp(lq), _dp(lg))
        return lq, lg

    def adjoint_prepare_geometry(self, cfl: float) -> tuple[float, float]:
        """adjoint_prepare plus the geometric linearisation (uns_cc_adjoint_prepare_geometry)."""
        cl, cd = C.c_double(), C.c_double()
        self._call("adjoint_prepare_geometry", C.c_double(cfl), C.byref(cl), C.byref(cd))
        return cl.value, cd.value

    def adjoint_geometry(self, objective: str, seed: float, wq: np.ndarray, wg: np.ndarray) -> dict:
        """G_X^T w + seed J_X^T for every geometric array X of the mesh
        (uns_cc_adjoint_geometry): a dict of arrays shaped like the mesh's."""
        wq = np.ascontiguousarray(wq, dtype=np.float64).reshape(self.noc, 4)
        wg = np.ascontiguousarray(wg, dtype=np.float64).reshape(self.nbf, 5)
        st, out = abi.cc_mesh_adj(self.m)
        self._call("adjoint_geometry", abi.OBJ[objective], C.c_double(seed), _dp(wq), _dp(wg), C.byref(st))
        return out

    def iteration(self, cfl: float) -> float:
        """One main-loop iteration (CCFVM/main.F90:60-115) through the per-routine entry points."""
        self.con2prim()
        self.avg_c2v()
        self.time_step(cfl)
        self.save_old()
        self.gradient()
        if self.params.time_mode == abi.TIME["rk3"]:
            for irk in (1, 2, 3):
                self.fvresidual()
                self.rk_stage(irk)
        else:
            self.lusgs()
        self.check_positivity()
        return self.residue()

    def iterate(self, cfl: np.ndarray, first_iter: bool) -> np.ndarray:
        """Graph-replayed iterations; returns the raw residual norms of the
        iterations run.  A device error (a non-positive state, a negative Roe
        sound speed, a non-finite residual norm) raises abi.UnsError, whose
        `history` holds the norms of the iterations run until then."""
        cfl = np.ascontiguousarray(cfl, dtype=np.float64)
        out = np.zeros(len(cfl))
        done = C.c_int()
        rc = self._lib.uns_cc_iterate(self._h, len(cfl), _dp(cfl), 1 if first_iter else 0, _dp(out), C.byref(done))
        _raise_with_history(rc, self._lib, "uns_cc_iterate", out[:done.value])
        return out[:done.value]


class NCSolver(_Solver):
    """Vertex-centred median-dual solver (NCFVM hot path) on the GPU."""
    kind = "nc"
    fields = abi.NC_FIELDS

    def __init__(self, mesh, params: abi.Params):
        self._lib = abi.gpu_lib()
        arr = mesh.arrays if hasattr(mesh, "arrays") else mesh
        self.m = arr
        view, self._keep = abi.nc_view_from_arrays(arr)
        h = C.c_void_p()
        abi.check(self._lib.uns_nc_create(C.byref(view), C.byref(params), C.byref(h)), self._lib, "uns_nc_create")
        self._h = h
        self.params = params
        self.nop = arr["nop"]
        self.nstate = self.nop

    def _field_shape(self, f):
        return {"qc": (self.nop, 4), "qp": (self.nop, 4), "qold": (self.nop, 4), "res": (self.nop, 4),
                "grad": (self.nop, 4, 2), "phi": (self.nop, 4), "dt": (self.nop,), "la": (self.nop,),
                "fla": (self.m["nof"],)}[f]

    def save_old(self): self._call("save_old")
    def fvresidual(self, cfl: float): self._call("fvresidual", C.c_double(cfl))
    def rk_stage(self, irk: int): self._call("rk_stage", irk)
    def lusgs(self, cfl: float): self._call("lusgs", C.c_double(cfl))

    def residue(self) -> tuple[float, float, int]:
        f, fi, ii = C.c_double(), C.c_double(), C.c_int()
        self._call("residue", C.byref(f), C.byref(fi), C.byref(ii))
        return f.value, fi.value, ii.value

    def sweep_levels(self) -> tuple[int, int]:
        """Dependency levels of the forward and backward LU-SGS sweeps."""
        f, b = C.c_int(), C.c_int()
        self._call("sweep_levels", C.byref(f), C.byref(b))
        return f.value, b.value

    def tecplt(self) -> np.ndarray:
        """tecplt's [nop][7] vertex table: x, y, rho, u, v, p, Mach."""
        out = np.zeros((self.nop, 7))
        self._call("tecplt", _dp(out))
        return out

    def screen_minmax(self) -> np.ndarray:
        """screen's [6][2] min/max of density, u, v, p, Mach, entropy."""
        out = np.zeros(12)
        self._call("screen_minmax", _dp(out))
        return out.reshape(6, 2)

    def iteration(self, cfl: float) -> tuple[float, float, int]:
        """One main-loop iteration (NCFVM/main.f90:53-86)."""
        self.save_old()
        if self.params.time_mode == abi.TIME["rk3"]:
            for irk in (1, 2, 3):
                self.fvresidual(cfl)
                self.rk_stage(irk)
        else:
            self.lusgs(cfl)
        return self.residue()

    def iterate(self, cfl: np.ndarray, first_iter: bool) -> tuple[np.ndarray, np.ndarray]:
        cfl = np.ascontiguousarray(cfl, dtype=np.float64)
        out = np.zeros(len(cfl))
        outi = np.zeros(len(cfl))
        done = C.c_int()
        rc = self._lib.uns_nc_iterate(self._h, len(cfl), _dp(cfl), 1 if first_iter else 0, _dp(out), _dp(outi),
                                      C.byref(done))
        _raise_with_history(rc, self._lib, "uns_nc_iterate", (out[:done.value], outi[:done.value]))
        return out[:done.value], outi[:done.value]


class CCBatch:
    """Independent CCSolver instances advanced together by one graph launch
    per iteration (uns_cc_batch_*)."""

    def __init__(self, solvers):
        self.solvers = list(solvers)
        self._lib = abi.gpu_lib()
        arr = (C.c_void_p * len(self.solvers))(*[s._h.value for s in self.solvers])
        h = C.c_void_p()
        abi.check(self._lib.uns_cc_batch_create(arr, len(self.solvers), C.byref(h)), self._lib, "uns_cc_batch_create")
        self._h = h

    def iterate(self, cfl: np.ndarray, first_iter: bool) -> tuple[list[np.ndarray], np.ndarray]:
        """cfl: [instances, niter].  Returns each instance's raw residual norms
        of the iterations it ran, and those counts."""
        cfl = np.ascontiguousarray(cfl, dtype=np.float64)
        n, niter = cfl.shape
        assert n == len(self.solvers)
        out = np.zeros((n, niter))
        done = (C.c_int * n)()
        rc = self._lib.uns_cc_batch_iterate(self._h, niter, _dp(cfl), 1 if first_iter else 0, _dp(out), done)
        abi.check(rc, self._lib, "uns_cc_batch_iterate")
        d = np.array(list(done))
        return [out[i, :d[i]] for i in range(n)], d

    def stream(self) -> int:
        return self._lib.uns_cc_batch_stream(self._h)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.uns_cc_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class CCPacked:
    """Many CCFVM cases in one index space (uns_cc_create_packed): one launch
    of each kernel advances every case per iteration.  Cases share RK3, the
    gradient, limiter, flow type and precision; mesh, Mach number, angle of
    attack, flux scheme, CFL schedule and stop level are their own."""

    def __init__(self, meshes, params_list):
        self._lib = abi.gpu_lib()
        n = len(meshes)
        views, self._keep = [], []
        self.noc, self.nbf = [], []
        for m in meshes:
            arr = m.arrays if hasattr(m, "arrays") else m
            v, k = abi.cc_view_from_arrays(arr)
            views.append(v)
            self._keep.append((k, arr))
            self.noc.append(int(arr["noc"]))
            self.nbf.append(int(arr["nbf"]))
        va = (abi.CCMeshView * n)(*views)
        pa = (abi.Params * n)(*params_list)
        h = C.c_void_p()
        abi.check(self._lib.uns_cc_create_packed(va, pa, n, C.byref(h)), self._lib, "uns_cc_create_packed")
        self._h = h
        co, go = (C.c_int * (n + 1))(), (C.c_int * (n + 1))()
        abi.check(self._lib.uns_cc_packed_layout(h, co, go), self._lib, "uns_cc_packed_layout")
        self.cell_off, self.ghost_off = np.array(list(co)), np.array(list(go))
        self.n = n
        self.ntot = int(self.cell_off[-1]) + int(self.ghost_off[-1])

    def iterate(self, cfl: np.ndarray, first_iter: bool) -> tuple[list[np.ndarray], np.ndarray]:
        """cfl: [cases, niter].  Returns each case's raw residual norms of the
        iterations it ran, and those counts."""
        cfl = np.ascontiguousarray(cfl, dtype=np.float64)
        n, niter = cfl.shape
        assert n == self.n
        out = np.zeros((n, niter))
        done = (C.c_int * n)()
        rc = self._lib.uns_cc_packed_iterate(self._h, niter, _dp(cfl), 1 if first_iter else 0, _dp(out), done)
        abi.check(rc, self._lib, "uns_cc_packed_iterate")
        d = np.array(list(done))
        return [out[i, :d[i]] for i in range(n)], d

    def get_state(self, i: int) -> np.ndarray:
        """Conserved state of case i: its cells then its ghosts, [noc + nbf][4]."""
        full = np.zeros((self.ntot, 4))
        abi.check(self._lib.uns_cc_get_state(self._h, _dp(full)), self._lib, "uns_cc_get_state")
        c0, g0 = int(self.cell_off[i]), int(self.cell_off[-1]) + int(self.ghost_off[i])
        return np.concatenate([full[c0:c0 + self.noc[i]], full[g0:g0 + self.nbf[i]]])

    def set_precision(self, precision: str) -> None:
        abi.check(self._lib.uns_cc_set_precision(self._h, abi.PREC[precision]), self._lib, "uns_cc_set_precision")

    def _field(self, field: str, rows: int, cols: int) -> np.ndarray:
        out = np.zeros((rows, cols))
        abi.check(self._lib.uns_cc_get_field(self._h, abi.CC_FIELDS[field], _dp(out)), self._lib, "uns_cc_get_field")
        return out

    def forces(self, fbc: list) -> np.ndarray:
        """Flux-based wall forces (Fx1, Fy1) of every case from the last
        residual, summed in each case's boundary-face order as the single-case
        path does (CCFVM/fvresidual.F90:99-100); fbc[i] = case i's boundary
        codes.  Returns [cases, 2]."""
        fw = self._field("fwall", int(self.ghost_off[-1]), 4)
        out = np.zeros((self.n, 2))
        for i in range(self.n):
            g0, g1 = int(self.ghost_off[i]), int(self.ghost_off[i + 1])
            fx = fy = 0.0
            walls = [k for k in range(g1 - g0) if fbc[i][k] == 1001]
            for k in walls:  # convective wall fluxes, then the viscous ones (viscous_flux.F90:73-74)
                fx, fy = fx + fw[g0 + k, 0], fy + fw[g0 + k, 1]
            if np.any(fw[g0:g1, 2:] != 0.0):
                for k in walls:
                    fx, fy = fx - fw[g0 + k, 2], fy - fw[g0 + k, 3]
            out[i] = fx, fy
        return out

    def density_residual_l2(self) -> np.ndarray:
        """L2 of the density residual (component 1 of E, rho, rho u, rho v) of
        every case's interior cells."""
        res = self._field("res", int(self.cell_off[-1]), 4)
        return np.array([np.sqrt(np.mean(res[int(self.cell_off[i]):int(self.cell_off[i]) + self.noc[i], 1] ** 2))
                         for i in range(self.n)])

    def converge(self, params_list, target: float, max_iter: int, switch_drop: float | None = 1e-4,
                 chunk: int = 500) -> dict:
        """Every case from iteration 1 to a `target` drop of its normalised
        residual (each case stops on the device there, CCFVM/main.F90:57) or
        `max_iter` iterations.  With `switch_drop`, the handle's current form
        (the mixed one: FP32 fluxes) runs until every case still running has
        dropped by `switch_drop` or stopped falling over a chunk (its FP32
        rounding floor, or a stall at any level), then the whole handle
        switches to FP64.  A case that has stopped runs
        one more iteration per chunk (the stop test is re-armed per call),
        which leaves it converged.  Returns per case the normalised history,
        the iteration where it reached the target (or None) and the density
        residual of iteration 1 and of the end."""
        from . import mesh as _mesh
        n = self.n
        hist = [[] for _ in range(n)]
        norm = [None] * n
        it = np.zeros(n, dtype=np.int64)
        prev_cfl = np.zeros(n)
        reached_at = [None] * n
        best_prev = np.full(n, np.inf)
        switched = None
        total = 0
        rho1 = None
        while total < max_iter and not all(r is not None for r in reached_at):
            m = 1 if total == 0 else min(chunk, max_iter - total)
            cfl = np.stack([_mesh.cfl_schedule(params_list[i], int(it[i]) + 1, m, "cc", float(prev_cfl[i]))
                            for i in range(n)])
            h, done = self.iterate(cfl, first_iter=(total == 0))
            if total == 0:
                rho1 = self.density_residual_l2()
            best = np.full(n, np.inf)
            for i in range(n):
                if done[i] == 0:
                    continue
                if norm[i] is None:
                    norm[i] = h[i][0]
                f = h[i] / norm[i]
                if reached_at[i] is None:
                    hist[i].extend(f.tolist())
                    if done[i] < m or f[-1] <= target:
                        reached_at[i] = int(it[i] + done[i])
                it[i] += done[i]
                prev_cfl[i] = cfl[i, done[i] - 1]
                best[i] = f.min()
            total += m
            if switch_drop is not None and switched is None and total > 1:
                live = [i for i in range(n) if reached_at[i] is None]
                # a case is done with the FP32 form once it has dropped by
                # switch_drop or stopped falling, at whatever level (a case
                # held up by a limiter cycle must not keep the others in FP32)
                floor = [best[i] <= switch_drop or best[i] > 0.9 * best_prev[i] for i in live]
                if all(floor):
                    self.set_precision("fp64")
                    switched = total
                best_prev = np.minimum(best_prev, best)
        return {"history": [np.array(x) for x in hist], "reached_at": reached_at, "switched_at": switched,
                "iterations": total, "density_l2_first": rho1, "density_l2_last": self.density_residual_l2()}

    def profile(self, cfl: float, reps: int = 3) -> dict:
        """Average device time [ms] of each phase of one iteration of all the
        cases (uns_cc_profile; one CFL for every case)."""
        n = 16
        ms = np.zeros(n)
        names = (C.c_char_p * n)()
        abi.check(self._lib.uns_cc_profile(self._h, C.c_double(cfl), reps, _dp(ms), names, n), self._lib,
                  "uns_cc_profile")
        return {names[k].decode(): float(ms[k]) for k in range(n) if names[k] and names[k].decode()}

    def autotune(self, reps: int = 3) -> dict:
        """Block sizes of the face, vertex and cell-gradient kernels picked by
        timing them on the packed mesh (uns_cc_autotune)."""
        b = (C.c_int * 3)()
        abi.check(self._lib.uns_cc_autotune(self._h, reps, b), self._lib, "uns_cc_autotune")
        return {"face": b[0], "vertex": b[1], "cell_grad": b[2]}

    def stream(self) -> int:
        return int(self._lib.uns_cc_stream(self._h) or 0)

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.uns_cc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def converge(solver, target: float, max_iter: int, switch_drop: float | None = None, chunk: int = 500,
             on_chunk=None) -> dict:
    """Run the main loop from iteration 1 until the density residual has dropped
    by `target` (the device stops at params.min_res) or `max_iter` iterations.

    With `switch_drop`, the solver's current form (e.g. "mixed", FP32 fluxes)
    runs until the residual has dropped by `switch_drop` or stops falling
    (the FP32 rounding floor), and the rest runs in FP64 -- the precision
    ramp that lets the FP32-flux form reach drops below its floor.  Returns
    the residual history (normalised by iteration 1), the iteration of the
    switch (or None) and the number of iterations run."""
    from . import mesh as _mesh
    kind = solver.kind
    p = solver.params
    hist: list[float] = []
    norm = None
    prev_cfl = 0.0
    switched = None
    it = 1
    best_prev = np.inf
    while it <= max_iter:
        n = min(chunk, max_iter - it + 1)
        cfl = _mesh.cfl_schedule(p, it, n, kind, prev_cfl)
        prev_cfl = float(cfl[-1])
        r = solver.iterate(cfl, first_iter=(it == 1))
        f = r if kind == "cc" else r[0]
        if norm is None and len(f):
            norm = f[0]
        hist.extend((f / norm).tolist())
        it += len(f)
        if on_chunk is not None:
            on_chunk(it - 1, hist)
        if len(f) < n or (hist and hist[-1] <= target):
            break
        if switch_drop is not None and switched is None:
            best = min(hist[-len(f):])
            if best <= switch_drop or (best < 100 * switch_drop and best > 0.9 * best_prev):
                solver.set_precision("fp64")
                switched = it
            best_prev = best
    return {"history": np.array(hist), "switched_at": switched, "iterations": it - 1}
