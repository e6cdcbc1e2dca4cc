"""A torch.autograd.Function over the C-ABI adjoint, loaded through ctypes.

Forward: converge the CCFVM flow at the angle of attack held in a 0-d tensor
(limiter frozen at the converged phi of the base case) and return C_L and
C_D.  Backward: uns_cc_adjoint_solve for each objective, combined with the
incoming gradients.  torch only carries the scalar through autograd; all the
work is the library's.
"""
import numpy as np
import pytest

from unsflow2d_gb300 import abi, mesh
from unsflow2d_gb300.solver import CCSolver

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CFL = 0.8
KW = dict(flux="roe", grad="gg", m_inf=0.5)


def _converge(s, target, chunk=5000, max_iter=300000):
    last, done = np.inf, 0
    while done < max_iter and last > target:
        last = s.iterate(np.full(chunk, CFL), first_iter=(done == 0))[-1]
        done += chunk
    return last


class _Case:
    """Base state at 2 degrees: limiter active while the flow develops, then frozen."""

    def __init__(self):
        self.m = mesh.CCMesh.airfoil(32, 16)
        p = abi.make_params(aoa_deg=2.0, min_res=1e-30, **KW)
        s = CCSolver(self.m, p)
        r0 = s.iterate(mesh.cfl_schedule(p, 1, 600, "cc"), first_iter=True)[0]
        self.target = 1e-12 * r0
        self.state = (s.get_state(), s.get("qp"), s.get("phi"))

    def solver(self, aoa):
        s = CCSolver(self.m, abi.make_params(aoa_deg=aoa, ilimit=0, min_res=1e-30, **KW))
        for name, x in zip(("qc", "qp", "phi"), self.state):
            s.set(name, x)
        assert _converge(s, self.target) <= self.target
        return s


class ForceCoefficients(torch.autograd.Function):
    @staticmethod
    def forward(ctx, alpha_deg, case):
        s = case.solver(float(alpha_deg))
        cl, cd = s.adjoint_prepare(CFL)
        ctx.solver = s
        return torch.tensor([cl, cd], dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad):
        s = ctx.solver
        dcl, _ = s.adjoint_solve("cl", max_iter=300000, tol=1e-12)
        dcd, _ = s.adjoint_solve("cd", max_iter=300000, tol=1e-12)
        per_deg = np.pi / 180.0
        g = grad[0].item() * dcl * per_deg + grad[1].item() * dcd * per_deg
        return torch.tensor(g, dtype=torch.float64), None


def test_autograd_function_matches_differences():
    case = _Case()
    alpha = torch.tensor(2.0, dtype=torch.float64, requires_grad=True)
    out = ForceCoefficients.apply(alpha, case)
    # L/D-like combination exercises both objectives
    y = out[0] / out[1]
    y.backward()
    da = 5e-4
    p_, m_ = (ForceCoefficients.apply(torch.tensor(2.0 + sgn * da, dtype=torch.float64), case) for sgn in (1, -1))
    fd = ((p_[0] / p_[1]) - (m_[0] / m_[1])).item() / (2 * da)
    assert abs(alpha.grad.item() - fd) <= 2e-5 * abs(fd), (alpha.grad.item(), fd)
