"""Shape derivatives of the flux-based force coefficients (CCFVM, airfoil
O-mesh): dJ/d(wall-node y) and dJ/d(Hicks-Henne bump amplitudes).

At a converged state s* with adjoint vector lambda (uns_cc_adjoint_solve),
the total derivative with respect to the mesh coordinates X is

    dJ/dX = dJ^/dX + lambda^T dG/dX        (state s* held fixed),

where G is one main-loop iteration and J^ the objective computed inside it.

method="transposed" (default): one transposed iteration with the geometric
linearisation (uns_cc_adjoint_geometry) gives lambda^T G_A + J_A for every
geometric array A of the mesh, and the transposed geometric preprocessing
(uns_host_cc_mesh_vjp) carries them to the node coordinates; a wall node's
y moves its radial line with weight 1 - s, so dJ/d(wall y_i) is the sum of
dJ/dy over the line's nodes times those weights.  Exact to rounding.

method="differenced": the explicit geometry partials from central
differences of ONE forward iteration at s* on meshes whose wall nodes are
displaced (no re-convergence).  One iteration's output depends on the
geometry within three columns of a cell, so wall nodes eight columns apart
are displaced together (eight colours), each cell's lambda-weighted change is
credited to the nearest displaced line, and 16 forward iterations give the
derivative for every wall node; the step h is a small fraction of the first
wall spacing.

This module is the caller side of the adjoint (Python over the C-ABI); the
limiter is frozen at the state's phi, as in the adjoint.
"""
from __future__ import annotations

import numpy as np

from . import abi, mesh
from .solver import CCSolver

#: Peak chord positions of the eight bumps per surface.
PEAKS = (0.05, 0.15, 0.25, 0.35, 0.5, 0.65, 0.8, 0.9)


def hicks_henne(x: np.ndarray, peak: float, width: float = 3.0) -> np.ndarray:
    """Hicks-Henne bump sin(pi x^m)^width with m = ln 0.5 / ln peak (1 at x = peak, 0 at x = 0, 1)."""
    x = np.clip(np.asarray(x, dtype=np.float64), 0.0, 1.0)
    m = np.log(0.5) / np.log(peak)
    return np.sin(np.pi * x ** m) ** width


def wall_x(ni: int) -> np.ndarray:
    """Chordwise position of the generator's wall nodes (node i at surface parameter 2 pi i / ni)."""
    sp = 2.0 * np.pi * np.arange(ni) / ni
    return 0.5 * (1.0 + np.cos(sp))


def bump_basis(ni: int, peaks=PEAKS, width: float = 3.0) -> np.ndarray:
    """[2 len(peaks), ni] wall-node y displacement per unit amplitude: bumps on the
    upper surface first, then the same peaks on the lower surface."""
    sp = 2.0 * np.pi * np.arange(ni) / ni
    x = wall_x(ni)
    upper = (sp > 0.0) & (sp < np.pi)
    lower = sp > np.pi
    B = np.zeros((2 * len(peaks), ni))
    for k, pk in enumerate(peaks):
        b = hicks_henne(x, pk, width)
        B[k] = np.where(upper, b, 0.0)
        B[len(peaks) + k] = np.where(lower, b, 0.0)
    return B


def cell_columns(m: mesh.CCMesh, ni: int) -> np.ndarray:
    """Generator column (0..ni-1) of every cell, in the solver's cell order."""
    new = m.newnum()
    col = np.empty(len(new), dtype=np.int64)
    col[new] = (np.arange(len(new)) // 2) % ni
    return col


def _objective_weights(objective: str, aoa_deg: float) -> tuple[float, float]:
    a = np.deg2rad(aoa_deg)
    if objective == "cl":  # C_L = 2 (Fy cos a - Fx sin a)
        return -2.0 * np.sin(a), 2.0 * np.cos(a)
    return 2.0 * np.cos(a), 2.0 * np.sin(a)


class ShapeCase:
    """A converged CCFVM airfoil case whose shape derivatives are wanted.

    ni, nj, mesh_kw: the generator's arguments; params_kw: make_params
    arguments (the limiter is frozen: ilimit is forced to 0); state: (qc with
    ghosts, qp with ghosts and T, phi) of the converged solution."""

    def __init__(self, ni, nj, params_kw, state, cfl, mesh_kw=None):
        self.ni, self.nj = ni, nj
        self.mesh_kw = dict(mesh_kw or {})
        self.params_kw = dict(params_kw)
        self.params_kw["ilimit"] = 0
        self.params_kw.setdefault("min_res", 1e-30)
        self.state = state
        self.cfl = cfl

    def mesh(self, dy=None) -> mesh.CCMesh:
        if dy is None:
            return mesh.CCMesh.airfoil(self.ni, self.nj, **self.mesh_kw)
        return mesh.CCMesh.airfoil_dy(self.ni, self.nj, dy, **self.mesh_kw)

    def solver(self, dy=None, prime=True) -> CCSolver:
        """A frozen-limiter solver on the (displaced) mesh loaded with the state;
        primed by one iteration so that the time step of the next one reads the
        converged face viscosity (viscous flows)."""
        s = CCSolver(self.mesh(dy), abi.make_params(**self.params_kw))
        self.load(s)
        if prime:
            s.iterate(np.array([self.cfl]), first_iter=True)
            self.load(s)
        return s

    def load(self, s: CCSolver) -> None:
        qc, qp, phi = self.state
        s.set("qc", qc)
        s.set("qp", qp)
        s.set("phi", phi)

    def one_iteration(self, dy) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
        """G(s*, X(dy)): interior qc, ghost primitives + T, per-boundary-face wall force terms."""
        s = self.solver(dy)
        s.iterate(np.array([self.cfl]), first_iter=True)
        out = s.get_state()[:s.noc], s.get("qp")[s.noc:], s.get("fwall")
        s.close()
        return out

    def line_weights(self) -> np.ndarray:
        """[nop] weight 1 - s of every node along its radial line (the
        displacement of node (i, j) per unit displacement of wall node i)."""
        base = self.mesh().arrays["py"]
        moved = self.mesh(np.ones(self.ni)).arrays["py"]
        return moved - base

    def wall_gradient(self, objective: str, lam_q: np.ndarray, lam_g: np.ndarray, method: str = "transposed",
                      h: float = None, spacing: int = 8) -> np.ndarray:
        """dJ/dy of every wall node (ni values)."""
        if method == "transposed":
            return self._wall_gradient_transposed(objective, lam_q, lam_g)
        if method != "differenced":
            raise ValueError(method)
        ni = self.ni
        dwall = self.mesh_kw.get("dwall", 1e-3)
        h = 1e-4 * dwall if h is None else h
        m0 = self.mesh()
        col = cell_columns(m0, ni)
        nbf = m0.arrays["nbf"]
        fbc = m0.arrays["fbc"][m0.arrays["nfi"]:]
        bcol = np.where(np.arange(nbf) < ni, np.arange(nbf), np.arange(nbf) - ni) % ni
        wx, wy = _objective_weights(objective, self.params_kw.get("aoa_deg", 2.0))
        wall = (fbc == 1001).astype(np.float64)
        grad = np.zeros(ni)
        k = np.arange(ni)
        for c in range(spacing):
            lines = np.arange(c, ni, spacing)
            dy = np.zeros(ni)
            dy[lines] = h
            qa, ga, fa = self.one_iteration(dy)
            qb, gb, fb = self.one_iteration(-dy)
            phi_c = np.sum(lam_q * (qa - qb), axis=1) / (2 * h)
            phi_g = np.sum(lam_g * (ga - gb), axis=1) / (2 * h)
            df = (fa - fb) / (2 * h)
            phi_j = wall * (wx * (df[:, 0] - df[:, 2]) + wy * (df[:, 1] - df[:, 3]))
            # column k -> nearest displaced line (line i borders columns i-1 and i)
            d = np.minimum((k[:, None] - lines[None, :]) % ni, (lines[None, :] - 1 - k[:, None]) % ni)
            near = lines[np.argmin(d, axis=1)]
            grad += np.bincount(near[col], weights=phi_c, minlength=ni)
            grad += np.bincount(near[bcol], weights=phi_g + phi_j, minlength=ni)
        return grad

    def _wall_gradient_transposed(self, objective: str, lam_q: np.ndarray, lam_g: np.ndarray) -> np.ndarray:
        s = self.solver()
        s.adjoint_prepare_geometry(self.cfl)
        geom = s.adjoint_geometry(objective, 1.0, lam_q, lam_g)
        s.close()
        _, gy = self.mesh().node_adjoint(geom)
        w = self.line_weights()
        node = np.arange(len(w))
        return np.bincount(node % self.ni, weights=gy * w, minlength=self.ni)

    def bump_gradient(self, objective: str, lam_q: np.ndarray, lam_g: np.ndarray, **kw) -> np.ndarray:
        """dJ/d(amplitude) of the 16 Hicks-Henne bumps (bump_basis order)."""
        return bump_basis(self.ni) @ self.wall_gradient(objective, lam_q, lam_g, **kw)
