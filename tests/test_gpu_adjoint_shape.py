"""Shape derivatives (unsflow2d_gb300.shape): dC_L/d(Hicks-Henne amplitude)
from the adjoint vector plus the transposed geometric linearisation
(uns_cc_adjoint_geometry, then the transposed geometric preprocessing),
against the same adjoint with one-iteration differenced geometry partials
and against central differences of C_L between solutions re-converged on
meshes with the bump applied at +- 1e-5 (limiter frozen at the base phi in
both)."""
import numpy as np
import pytest

from unsflow2d_gb300 import abi, mesh, shape
from unsflow2d_gb300.solver import CCSolver

pytestmark = pytest.mark.gpu

CFL = 0.8
NI, NJ = 32, 16
CASES = {
    "euler": dict(flux="roe", grad="gg", m_inf=0.5, aoa_deg=2.0),
    "laminar": dict(flow="laminar", iwall=0, rey=5000.0, flux="roe", grad="ggfc", m_inf=0.5, aoa_deg=3.0),
}


def _converge(s, target, chunk=5000, max_iter=300000):
    last, done = np.inf, 0
    while done < max_iter and last > target:
        last = s.iterate(np.full(chunk, CFL), first_iter=(done == 0))[-1]
        done += chunk
    return last


@pytest.mark.parametrize("name", list(CASES))
def test_bump_gradient_matches_reconverged_differences(name):
    kw = CASES[name]
    p = abi.make_params(min_res=1e-30, **kw)
    s = CCSolver(mesh.CCMesh.airfoil(NI, NJ), p)
    r0 = s.iterate(mesh.cfl_schedule(p, 1, 600, "cc"), first_iter=True)[0]
    target = 1e-12 * r0
    case = shape.ShapeCase(NI, NJ, kw, (s.get_state(), s.get("qp"), s.get("phi")), CFL)
    f = case.solver(prime=False)
    assert _converge(f, target) <= target
    case.state = (f.get_state(), f.get("qp"), f.get("phi"))
    a = case.solver()
    a.adjoint_prepare(CFL)
    a.adjoint_solve("cl", max_iter=300000, tol=1e-12)
    lq, lg = a.adjoint_get()
    grad = case.bump_gradient("cl", lq, lg)
    assert grad.shape == (16,) and np.isfinite(grad).all()
    grad_fd = case.bump_gradient("cl", lq, lg, method="differenced")
    rel = np.max(np.abs(grad - grad_fd)) / np.max(np.abs(grad))
    print(f"{name}: transposed vs one-iteration differences, max rel {rel:.2e}")
    assert rel <= 1e-5, (grad, grad_fd)
    B = shape.bump_basis(NI)
    delta = 1e-5
    for k in (2, 12):  # upper-surface bump at x = 0.25, lower-surface bump at x = 0.5
        cl = {}
        for sgn in (1, -1):
            t = case.solver(sgn * delta * B[k], prime=False)
            assert _converge(t, target) <= target
            t.iterate(np.array([CFL]), first_iter=True)
            cl[sgn] = t.cl_cd()[0]
        fd = (cl[1] - cl[-1]) / (2 * delta)
        print(f"{name} bump {k}: adjoint {grad[k]:.10e} re-converged differences {fd:.10e} rel {abs(grad[k] - fd) / abs(fd):.2e}")
        assert abs(grad[k] - fd) <= 1e-4 * abs(fd), (k, grad[k], fd)
