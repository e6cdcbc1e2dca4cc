"""CCFVM hot path on the GPU vs the CPU oracle, routine by routine.

Criteria (see conftest.py): fields 1e-12 of their max magnitude; residuals
1e-12 of the cell's flux scale; gradients 1e-12 with the rounding-noise floor;
the limiter value phi 1e-10 (the Venkatakrishnan ratio is evaluated on
D_L = grad.dx, a cancellation).  The GPU performs the reference's IEEE
operations in the reference's order (no multiply-add contraction), so the
remaining differences come from the math library's pow.
"""
import numpy as np
import pytest

from conftest import grad_err, inv_h_cc, res_err
from unsflow2d_gb300 import abi, mesh
from unsflow2d_gb300.solver import CCSolver
from oracle import OracleCC

pytestmark = pytest.mark.gpu
RTOL = 1e-12
RTOL_PHI = 1e-10

CASES = [
    dict(flux="roe", grad="gg"),
    dict(flux="rusanov", grad="gg"),
    dict(flux="vanleer", grad="lsqr"),
    dict(flux="ausm", grad="ggfc"),
    dict(flux="roe", grad="gg", time="lusgs", cfl_max=5.0, cfl_type="ramp", cfl_min=0.5, cfl_ramp_steps=10),
    dict(flux="roe", grad="ggfc", flow="laminar", iwall=0, rey=500.0, m_inf=0.5),
    dict(flux="vanleer", grad="gg", flow="laminar", iwall=1, rey=5000.0),
    dict(flux="roe", grad="lsqr", irs=1, ilimit=0),
]


@pytest.fixture(scope="module")
def cc_mesh():
    return mesh.CCMesh.airfoil(24, 12)


@pytest.mark.parametrize("case", CASES, ids=[str(i) for i in range(len(CASES))])
def test_cc_routine_parity(cc_mesh, case, assert_close):
    p = abi.make_params(**case)
    g, o = CCSolver(cc_mesh, p), OracleCC(cc_mesh, p)
    cfl = 0.0
    for it in range(1, 4):
        cfl = mesh.cfl_schedule(p, it, 1, "cc", cfl)[0]
        for s in (g, o):
            s.con2prim()
        assert_close("qp", g.get("qp"), o.get("qp"), RTOL)
        for s in (g, o):
            s.avg_c2v()
        assert_close("ptprim", g.get("ptprim"), o.get("ptprim"), RTOL)
        assert_close("fqp", g.get("fqp"), o.get("fqp"), RTOL)
        for s in (g, o):
            s.time_step(cfl)
        assert_close("fla", g.get("fla"), o.get("fla"), RTOL)
        assert_close("dt", g.get("dt"), o.get("dt"), RTOL)
        for s in (g, o):
            s.save_old()
            s.gradient()
        assert grad_err(g.get("grad"), o.get("grad"), o.get("qp")[:o.noc], inv_h_cc(cc_mesh.arrays)) <= RTOL
        assert_close("phi", g.get("phi"), o.get("phi"), RTOL_PHI)
        if p.time_mode == abi.TIME["rk3"]:
            for irk in (1, 2, 3):
                for s in (g, o):
                    s.fvresidual()
                assert res_err(g.get("res"), o.get("res"), o.get("la"), o.get("qc")[:o.noc]) <= RTOL
                assert_close("ghost qc", g.get("qc")[g.noc:], o.get("qc")[o.noc:], RTOL)
                for s in (g, o):
                    s.rk_stage(irk)
                assert_close("qc", g.get("qc"), o.get("qc"), RTOL)
        else:
            for s in (g, o):
                s.lusgs()
            assert res_err(g.get("res"), o.get("res"), o.get("la"), o.get("qc")[:o.noc]) <= RTOL
            assert_close("qc", g.get("qc"), o.get("qc"), RTOL)
        assert g.check_positivity() == o.check_positivity() == -1
        fg, fo = g.residue(), o.residue()
        assert abs(fg - fo) <= RTOL * abs(fo)
        if case.get("flow") == "laminar":
            assert_close("fmu", g.get("fmu"), o.get("fmu"), RTOL)
        fx, fy = g.forces()
        ox, oy = o.forces()
        assert abs(fx - ox) <= RTOL * (abs(ox) + 1e-300) and abs(fy - oy) <= RTOL * (abs(oy) + 1e-300)


@pytest.mark.parametrize("case", [CASES[0], CASES[4]], ids=["rk3", "lusgs"])
def test_cc_history_graph_vs_oracle(cc_mesh, case):
    """FLO.RES residual history: graph-replayed iterations vs the oracle loop."""
    p = abi.make_params(**case)
    g, o = CCSolver(cc_mesh, p), OracleCC(cc_mesh, p)
    n = 60
    cfl = mesh.cfl_schedule(p, 1, n, "cc")
    fg = g.iterate(cfl, first_iter=True)
    fo = np.array([o.iteration(c) for c in cfl])
    assert len(fg) == n
    lg, lo = np.log10(fg / fg[0]), np.log10(fo / fo[0])
    # the FLO.RES text (e16.6) agrees to its printed digits
    assert np.max(np.abs(lg - lo)) < 1e-9
    assert np.max(np.abs(g.get_state() - o.get_state())) <= 1e-10 * np.max(np.abs(o.get_state()))


@pytest.mark.parametrize("case", [CASES[0], CASES[2], dict(CASES[0], precision="mixed")],
                         ids=["roe_gg", "vanleer_lsqr", "roe_gg_mixed"])
def test_cc_graph_step_equals_routine_calls(cc_mesh, case):
    """Stages 2 and 3 of the graph-replayed inviscid RK3 step keep the first
    stage's interior and farfield face fluxes (their inputs are formed once
    per step) and recompute only the boundary faces and the residuals of the
    cells beside them; the per-routine calls recompute every face in every
    stage.  In FP64 both paths give the same states and norms bit for bit.
    The mixed form's graph step fuses the stage update with multiply-adds and
    the per-routine rk_stage does not; those last-bit differences of the FP64
    state move FP32 roundings of the face arithmetic, so there the two paths
    agree to 1e-8 after 30 steps (a stage reusing a wrong flux or residual
    would differ by the size of a stage increment, ~1e-3)."""
    p = abi.make_params(**case)
    g, r = CCSolver(cc_mesh, p), CCSolver(cc_mesh, p)
    cfl = mesh.cfl_schedule(p, 1, 30, "cc")
    fg = g.iterate(cfl, first_iter=True)
    fr = np.array([r.iteration(c) for c in cfl])
    qg, qr = g.get_state(), r.get_state()
    if case.get("precision") == "mixed":
        d = np.max(np.abs(qg - qr)) / np.max(np.abs(qr))
        print(f"mixed: state {d:.2e}, norms {np.max(np.abs(fg / fr - 1)):.2e}")
        assert d <= 1e-8 and np.max(np.abs(fg / fr - 1)) <= 1e-8
    else:
        assert np.array_equal(qg, qr)
        assert np.array_equal(fg, fr)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cc_fvresidual_flux_cache_equals_full_call(cc_mesh, precision):
    """uns_cc_fvresidual recomputes only the wall faces and their cells when
    nothing but the conserved state has changed since its last full call
    (the reference loop's RK stages 2 and 3); a call after any input change
    (here a same-precision set_precision) computes every face.  Both give
    the same residual bit for bit."""
    p = abi.make_params(flux="roe", grad="gg", m_inf=0.7, aoa_deg=2.0, precision=precision)
    cfl = mesh.cfl_schedule(p, 1, 15, "cc")
    a, b = CCSolver(cc_mesh, p), CCSolver(cc_mesh, p)
    for s in (a, b):
        s.iterate(cfl[:14], first_iter=True)
        s.con2prim(); s.avg_c2v(); s.time_step(float(cfl[14])); s.save_old(); s.gradient()
        s.fvresidual(); s.rk_stage(1)
    assert np.array_equal(a.get("res"), b.get("res"))
    a.fvresidual()                 # cached: wall faces only
    b.set_precision(precision)     # invalidates the cache
    b.fvresidual()                 # every face
    assert np.array_equal(a.get("res"), b.get("res"))
    assert np.array_equal(a.get_state(), b.get_state())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cc_autotune_keeps_results(cc_mesh, precision):
    """uns_cc_autotune times the kernels on scratch outputs and only changes
    launch geometry: the tuned handle's state is untouched by the tuning and
    its later steps equal an untuned handle's bit for bit."""
    p = abi.make_params(flux="roe", grad="gg", m_inf=0.7, aoa_deg=2.0, precision=precision)
    cfl = mesh.cfl_schedule(p, 1, 40, "cc")
    a, b = CCSolver(cc_mesh, p), CCSolver(cc_mesh, p)
    a.iterate(cfl[:20], first_iter=True)
    b.iterate(cfl[:20], first_iter=True)
    q0 = a.get_state()
    blocks = a.autotune(reps=2)
    assert set(blocks) == {"face", "vertex", "cell_grad"} and blocks["face"] in (64, 128, 256, 512)
    assert np.array_equal(a.get_state(), q0)
    fa = a.iterate(cfl[20:], first_iter=False)
    fb = b.iterate(cfl[20:], first_iter=False)
    assert np.array_equal(a.get_state(), b.get_state())
    assert np.array_equal(fa, fb)


@pytest.mark.parametrize("case", [dict(flux="roe", grad="gg"), dict(flux="rusanov", grad="lsqr")],
                         ids=["roe_gg", "rusanov_lsqr"])
def test_cc_routines_bit_exact_on_a_developed_state(cc_mesh, case):
    """Without pow in the path (inviscid, Roe or Rusanov), the FP64 routines
    perform the oracle's IEEE operations and give its values bit for bit:
    primitives, vertex and face values, radii, dt, gradient, limiter,
    residual and state, from a state with active limiters (30 oracle
    iterations from freestream)."""
    p = abi.make_params(m_inf=0.8, aoa_deg=1.25, **case)
    o = OracleCC(cc_mesh, p)
    cfl = mesh.cfl_schedule(p, 1, 31, "cc")
    for c in cfl[:30]:
        o.iteration(float(c))
    g = CCSolver(cc_mesh, p)
    g.set("qc", o.get("qc"))
    g.set("qp", o.get("qp"))
    g.set("phi", o.get("phi"))

    def same(name, a, b):
        assert np.array_equal(a, b), (name, float(np.max(np.abs(a - b))))

    for s in (g, o):
        s.con2prim()
    same("qp", g.get("qp"), o.get("qp"))
    for s in (g, o):
        s.avg_c2v()
    same("ptprim", g.get("ptprim"), o.get("ptprim"))
    for s in (g, o):
        s.time_step(float(cfl[30]))
    same("fla", g.get("fla"), o.get("fla"))
    same("dt", g.get("dt"), o.get("dt"))
    for s in (g, o):
        s.save_old()
        s.gradient()
    same("grad", g.get("grad"), o.get("grad"))
    same("phi", g.get("phi"), o.get("phi"))
    assert np.any(g.get("phi") < 1.0)  # the limiter is active somewhere
    for irk in (1, 2, 3):
        for s in (g, o):
            s.fvresidual()
        same("res", g.get("res"), o.get("res"))
        for s in (g, o):
            s.rk_stage(irk)
        same("qc", g.get("qc"), o.get("qc"))
