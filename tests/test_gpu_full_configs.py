"""The GPU path against the oracle at the sizes of the benchmark configurations.

The routine-level parity tests run on small meshes; these run the same
comparisons on the configurations the benchmark names, on meshes from the
same seeded airfoil generator:

* CCFVM Euler, 128x64 O-mesh (16,384 cells), M 0.5, alpha 2, Roe, Green-Gauss
  + Venkatakrishnan, RK3 at CFL 0.9: the whole 2,000-iteration residual
  history (FLO.RES) through the graph-replayed iteration, then the per-cell
  residual of the final state;
* NCFVM median-dual Euler, 1024x512 O-mesh (525,312 nodes), M 0.8,
  alpha 1.25, AUSM+-up, LSQ + corrected Barth, LU-SGS at CFL 50: three
  iterations, routine by routine;
* CCFVM laminar Navier-Stokes, Re 5000, M 0.5, alpha 3, 512x256 O-mesh with
  2e-5 first wall spacing (262,144 cells), Roe, GG-FC: two iterations;
* CCFVM Euler, 2048x1024 O-mesh (4,194,304 cells), M 0.75, alpha 2, Roe,
  Green-Gauss, FP64: one iteration.

Criteria as in conftest.py: fields 1e-12 of their max magnitude, residuals
1e-12 of the flux scale, gradients 1e-12 with the rounding-noise floor, the
limiter value 1e-10.
"""
import numpy as np
import pytest

from conftest import grad_err, inv_h_cc, inv_h_nc, res_err
from oracle import OracleCC, OracleNC
from unsflow2d_gb300 import abi, mesh
from unsflow2d_gb300.solver import CCSolver, NCSolver

pytestmark = pytest.mark.gpu
RTOL = 1e-12
RTOL_PHI = 1e-10


def cc_routines_check(g, o, m, p, cfl, assert_close):
    """One main-loop iteration through the per-routine entry points on both
    sides, every intermediate compared (CCFVM/main.F90:59-115)."""
    for s in (g, o):
        s.con2prim()
    assert_close("qp", g.get("qp"), o.get("qp"), RTOL)
    for s in (g, o):
        s.avg_c2v()
    assert_close("ptprim", g.get("ptprim"), o.get("ptprim"), RTOL)
    for s in (g, o):
        s.time_step(cfl)
    assert_close("fla", g.get("fla"), o.get("fla"), RTOL)
    assert_close("dt", g.get("dt"), o.get("dt"), RTOL)
    for s in (g, o):
        s.save_old()
        s.gradient()
    assert grad_err(g.get("grad"), o.get("grad"), o.get("qp")[:o.noc], inv_h_cc(m.arrays)) <= RTOL
    assert_close("phi", g.get("phi"), o.get("phi"), RTOL_PHI)
    for irk in (1, 2, 3):
        for s in (g, o):
            s.fvresidual()
        assert res_err(g.get("res"), o.get("res"), o.get("la"), o.get("qc")[:o.noc]) <= RTOL
        if p.flow_type == abi.FLOW["laminar"]:
            assert_close("fmu", g.get("fmu"), o.get("fmu"), RTOL)
        for s in (g, o):
            s.rk_stage(irk)
        assert_close("qc", g.get("qc"), o.get("qc"), RTOL)
    assert g.check_positivity() == o.check_positivity() == -1
    fg, fo = g.residue(), o.residue()
    assert abs(fg - fo) <= RTOL * abs(fo)


def test_cc_euler_128x64_2000_iterations(assert_close):
    m = mesh.CCMesh.airfoil(128, 64, 0.12, 20.0, 1e-3)
    assert m.arrays["noc"] == 16384
    p = abi.make_params(m_inf=0.5, aoa_deg=2.0, flux="roe", grad="gg", time="rk3", cfl_max=0.9, min_res=0.0)
    g, o = CCSolver(m, p), OracleCC(m, p)
    n = 2000
    cfl = mesh.cfl_schedule(p, 1, n, "cc")
    fg = g.iterate(cfl, first_iter=True)
    fo = np.array([o.iteration(c) for c in cfl])
    assert len(fg) == n
    assert np.max(np.abs(fg - fo) / fo) <= RTOL
    # FLO.RES lines (i6,2e16.6: iteration, log10(fres), cfl), printed to the
    # same seven significant digits on both sides
    flo = lambda f: [f"{i + 1:6d}{np.log10(x):16.6E}{c:16.6E}" for i, (x, c) in enumerate(zip(f, cfl))]
    assert flo(fg) == flo(fo)
    assert fo[-1] < 0.1 * fo[0]  # well past the start-up transient
    assert_close("qc", g.get_state(), o.get_state(), RTOL)
    # the per-cell residual of the final state, one more iteration routine by routine
    cc_routines_check(g, o, m, p, float(cfl[-1]), assert_close)


def test_nc_ausm_1024x512_three_lusgs_iterations(assert_close):
    m = mesh.NCMesh.airfoil(1024, 512, 0.12, 20.0, 1e-3)
    assert m.arrays["nop"] == 525312
    p = abi.make_params(m_inf=0.8, aoa_deg=1.25, flux="ausm", limiter="barth_corrected", time="lusgs", cfl_max=50.0,
                        min_res=0.0)
    g, o = NCSolver(m, p), OracleNC(m, p)
    inv_h = inv_h_nc(m.arrays)
    for it in range(1, 4):
        cfl = mesh.cfl_schedule(p, it, 1, "nc")[0]
        for s in (g, o):
            s.save_old()
        assert_close("qp", g.get("qp"), o.get("qp"), RTOL)
        for s in (g, o):
            s.lusgs(cfl)
        assert grad_err(g.get("grad"), o.get("grad"), o.get("qp"), inv_h) <= RTOL
        assert_close("phi", g.get("phi"), o.get("phi"), RTOL_PHI)
        assert_close("la", g.get("la"), o.get("la"), RTOL)
        assert_close("dt", g.get("dt"), o.get("dt"), RTOL)
        assert res_err(g.get("res"), o.get("res"), o.get("la"), o.get("qc")) <= RTOL
        assert_close("qc", g.get("qc"), o.get("qc"), RTOL)
        (fg, fgi, ig), (fo, foi, io) = g.residue(), o.residue()
        assert abs(fg - fo) <= RTOL * fo and abs(fgi - foi) <= RTOL * foi and ig == io


def test_cc_laminar_512x256_two_iterations(assert_close):
    m = mesh.CCMesh.airfoil(512, 256, 0.12, 20.0, 2e-5)
    assert m.arrays["noc"] == 262144
    p = abi.make_params(m_inf=0.5, aoa_deg=3.0, rey=5000.0, flow="laminar", iwall=0, flux="roe", grad="ggfc",
                        time="rk3", cfl_max=0.9, min_res=0.0)
    g, o = CCSolver(m, p), OracleCC(m, p)
    c = 0.0
    for it in (1, 2):
        c = mesh.cfl_schedule(p, it, 1, "cc", c)[0]
        cc_routines_check(g, o, m, p, c, assert_close)


def test_cc_euler_2048x1024_one_iteration(assert_close):
    m = mesh.CCMesh.airfoil(2048, 1024, 0.12, 20.0, 1e-3)
    assert m.arrays["noc"] == 4194304
    p = abi.make_params(m_inf=0.75, aoa_deg=2.0, flux="roe", grad="gg", time="rk3", cfl_max=0.9, min_res=0.0)
    g, o = CCSolver(m, p), OracleCC(m, p)
    cc_routines_check(g, o, m, p, mesh.cfl_schedule(p, 1, 1, "cc")[0], assert_close)


def test_cc_lusgs_2048x1024_one_iteration(assert_close):
    """Configuration 3's mesh with the implicit scheme (lusgs2 sweeps over
    4.2 M cells): one iteration routine by routine."""
    m = mesh.CCMesh.airfoil(2048, 1024, 0.12, 20.0, 1e-3)
    p = abi.make_params(m_inf=0.75, aoa_deg=2.0, flux="roe", grad="gg", time="lusgs", cfl_max=5.0, cfl_type="ramp",
                        cfl_min=0.5, cfl_ramp_steps=50, min_res=0.0)
    g, o = CCSolver(m, p), OracleCC(m, p)
    cfl = mesh.cfl_schedule(p, 1, 1, "cc")[0]
    for s in (g, o):
        s.con2prim(); s.avg_c2v(); s.time_step(cfl); s.save_old(); s.gradient(); s.lusgs()
    assert res_err(g.get("res"), o.get("res"), o.get("la"), o.get("qc")[:o.noc]) <= RTOL
    assert_close("qc", g.get("qc"), o.get("qc"), RTOL)


def test_nc_rk3_vanleer_1024x512_two_iterations(assert_close):
    """Configuration 2's mesh with the explicit scheme the NCFVM reference
    hard-wires (van Leer + Venkatakrishnan, RK3): two iterations, stage by
    stage."""
    m = mesh.NCMesh.airfoil(1024, 512, 0.12, 20.0, 1e-3)
    p = abi.make_params(m_inf=0.8, aoa_deg=1.25, flux="vanleer", limiter="vkn", time="rk3", cfl_max=0.9, min_res=0.0)
    g, o = NCSolver(m, p), OracleNC(m, p)
    for it in (1, 2):
        cfl = mesh.cfl_schedule(p, it, 1, "nc")[0]
        for s in (g, o):
            s.save_old()
        for irk in (1, 2, 3):
            for s in (g, o):
                s.fvresidual(cfl)
            assert res_err(g.get("res"), o.get("res"), o.get("la"), o.get("qc")) <= RTOL
            for s in (g, o):
                s.rk_stage(irk)
            assert_close("qc", g.get("qc"), o.get("qc"), RTOL)
    assert_close("phi", g.get("phi"), o.get("phi"), RTOL_PHI)
