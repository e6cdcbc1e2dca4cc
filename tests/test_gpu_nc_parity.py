"""NCFVM hot path on the GPU vs the CPU oracle.

Criteria (see conftest.py): states, spectral radii, dt 1e-12 of their max
magnitude; node residuals 1e-12 of the flux scale lambda_i * max|q_j| (a
node residual is a near-cancelling sum of ~6 dual-face fluxes); gradients
1e-12 with the rounding-noise floor; the limiter value phi 1e-10.
"""
import numpy as np
import pytest

from conftest import grad_err, inv_h_nc, res_err
from oracle import OracleNC
from unsflow2d_gb300 import abi, mesh
from unsflow2d_gb300.solver import NCSolver

pytestmark = pytest.mark.gpu
RTOL = 1e-12
RTOL_PHI = 1e-10

CASES = [
    dict(flux="vanleer", limiter="vkn", time="rk3", cfl_max=0.9, m_inf=0.6, aoa_deg=2.89),
    dict(flux="vanleer", limiter="vkn", time="lusgs", cfl_max=1000.0, m_inf=0.8, aoa_deg=1.25),
    dict(flux="ausm", limiter="barth", time="lusgs", cfl_max=50.0, m_inf=0.8, aoa_deg=1.25),
    dict(flux="ausm", limiter="barth_corrected", time="lusgs", cfl_max=50.0, m_inf=0.8, aoa_deg=1.25),
    dict(flux="ausm", limiter="vkn", time="rk3", cfl_max=0.9, m_inf=0.5, aoa_deg=3.0),
]


@pytest.fixture(scope="module")
def nc_mesh():
    return mesh.NCMesh.airfoil(24, 12)


@pytest.mark.parametrize("case", CASES, ids=[str(i) for i in range(len(CASES))])
def test_nc_routine_parity(nc_mesh, case, assert_close):
    p = abi.make_params(**case)
    g, o = NCSolver(nc_mesh, p), OracleNC(nc_mesh, p)
    for it in range(1, 4):
        cfl = mesh.cfl_schedule(p, it, 1, "nc")[0]
        for s in (g, o):
            s.save_old()
        assert_close("qp", g.get("qp"), o.get("qp"), RTOL)
        stages = (1, 2, 3) if p.time_mode == abi.TIME["rk3"] else (0,)
        for irk in stages:
            for s in (g, o):
                if irk:
                    s.fvresidual(cfl)
                else:
                    s.lusgs(cfl)
            assert grad_err(g.get("grad"), o.get("grad"), o.get("qp"), inv_h_nc(nc_mesh.arrays)) <= RTOL
            assert_close("phi", g.get("phi"), o.get("phi"), RTOL_PHI)
            assert_close("la", g.get("la"), o.get("la"), RTOL)
            assert_close("fla", g.get("fla"), o.get("fla"), RTOL)
            assert_close("dt", g.get("dt"), o.get("dt"), RTOL)
            assert res_err(g.get("res"), o.get("res"), o.get("la"), o.get("qc")) <= RTOL
            if irk:
                for s in (g, o):
                    s.rk_stage(irk)
            assert_close("qc", g.get("qc"), o.get("qc"), RTOL)
        fg, gi, gii = g.residue()
        fo, oi, oii = o.residue()
        assert abs(fg - fo) <= 1e-10 * fo and abs(gi - oi) <= 1e-10 * oi and gii == oii


@pytest.mark.parametrize("case", [CASES[0], CASES[1], CASES[3]], ids=["rk3", "lusgs_vkn", "lusgs_barth"])
def test_nc_history_graph_vs_oracle(nc_mesh, case):
    p = abi.make_params(**case)
    g, o = NCSolver(nc_mesh, p), OracleNC(nc_mesh, p)
    n = 60
    cfl = mesh.cfl_schedule(p, 1, n, "nc")
    fg, gi = g.iterate(cfl, first_iter=True)
    fo = np.array([o.iteration(c) for c in cfl])
    assert len(fg) == n and np.isfinite(fg).all()
    assert np.max(np.abs(np.log10(fg / fg[0]) - np.log10(fo[:, 0] / fo[0, 0]))) < 1e-8
    assert np.max(np.abs(np.log10(gi) - np.log10(fo[:, 1]))) < 1e-8
    assert np.max(np.abs(g.get_state() - o.get_state())) <= 1e-10 * np.max(np.abs(o.get_state()))


def test_nc_reference_barth_diverges_on_both(nc_mesh):
    """limiter_min_max as written (DUmax=-eps / DUmin=+eps start, +1/2 on fp2,
    no clip at 0, NCFVM/limiter.f90:192-260) blows up the LU-SGS solve; the GPU
    reproduces it iteration for iteration until the first non-finite norm."""
    p = abi.make_params(**CASES[2])
    g, o = NCSolver(nc_mesh, p), OracleNC(nc_mesh, p)
    cfl = mesh.cfl_schedule(p, 1, 40, "nc")
    try:
        fg, _ = g.iterate(cfl, first_iter=True)
    except abi.UnsError as e:  # the first non-finite norm ends the iteration
        assert e.code == abi.UNS_ERR_NAN
        fg = e.history[0]
    fo = np.array([o.iteration(c)[0] for c in cfl])
    k = int(np.argmax(~np.isfinite(fo)))
    assert not np.isfinite(fo).all() and k > 5
    assert np.allclose(fg[:k - 3], fo[:k - 3], rtol=1e-9)


@pytest.mark.parametrize("case", [
    dict(flux="vanleer", limiter="barth_corrected", time="lusgs", cfl_max=50.0, m_inf=0.8, aoa_deg=1.25),
    dict(flux="vanleer", limiter="vkn", time="lusgs", cfl_max=1000.0, m_inf=0.8, aoa_deg=1.25),
], ids=["barth_corrected", "vkn"])
def test_nc_routines_bit_exact(nc_mesh, case):
    """Without pow in the path (van Leer flux), the FP64 NCFVM routines give
    the oracle's values bit for bit -- gradient, limiter, radii, dt,
    residual and the LU-SGS update -- over 20 iterations, as the limiters
    become active."""
    p = abi.make_params(**case)
    g, o = NCSolver(nc_mesh, p), OracleNC(nc_mesh, p)
    limited = False
    for it in range(1, 21):
        cfl = mesh.cfl_schedule(p, it, 1, "nc")[0]
        for s in (g, o):
            s.save_old()
            s.lusgs(cfl)
        for name in ("grad", "phi", "la", "fla", "dt", "res", "qc"):
            a, b = g.get(name), o.get(name)
            assert np.array_equal(a, b), (it, name, float(np.max(np.abs(a - b))))
        limited = limited or bool(np.any(g.get("phi") < 1.0))
    assert limited
