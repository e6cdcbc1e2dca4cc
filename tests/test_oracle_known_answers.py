"""Known-answer tests of the CPU oracle (no GPU).

The reference ships no golden vectors, so the oracle is pinned to analytic
answers the discretisation must reproduce:
  * freestream preservation away from boundaries, for every flux function;
  * Green-Gauss (interior cells), diamond-path GG and least-squares gradients
    are exact for linear fields;
  * the NCFVM least-squares gradient is exact for linear fields and the
    median-dual scheme preserves freestream at interior nodes;
  * host-side fault injection: non-positive states and a negative Roe sound
    speed are reported as status codes.
"""
import numpy as np
import pytest

from oracle import OracleCC, OracleNC, OracleError
from unsflow2d_gb300 import abi, mesh


@pytest.fixture(scope="module")
def cc():
    return mesh.CCMesh.airfoil(32, 16)


@pytest.fixture(scope="module")
def nc():
    return mesh.NCMesh.airfoil(32, 16)


def boundary_layers(m, layers):
    """Cells within `layers` face-neighbour steps of a boundary face."""
    noc, nfi = m["noc"], m["nfi"]
    near = np.zeros(noc, bool)
    near[m["fin"][nfi:]] = True
    fin, fout = m["fin"][:nfi], m["fout"][:nfi]
    for _ in range(layers - 1):
        grow = near.copy()
        grow[fout[near[fin]]] = True
        grow[fin[near[fout]]] = True
        near = grow
    return near


def prims_to_cons(q):
    rho, u, v, p = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    return np.stack([p / 0.4 + 0.5 * rho * (u * u + v * v), rho, rho * u, rho * v], axis=1)


def _first_residual(m, flux):
    o = OracleCC(m, abi.make_params(flux=flux, m_inf=0.5, aoa_deg=2.0))
    o.con2prim(); o.avg_c2v(); o.time_step(0.5); o.save_old(); o.gradient(); o.fvresidual()
    return o.get("res")


@pytest.mark.parametrize("flux", ["roe", "vanleer", "rusanov"])
def test_cc_freestream_preserved_in_interior(cc, flux):
    res = _first_residual(cc, flux)
    far = ~boundary_layers(cc.arrays, 3)
    scale = (1.0 / (1.4 * 0.25)) * cc["farea"].max()  # p_inf * face length
    assert far.sum() > 0.5 * cc["noc"]
    assert np.abs(res[far]).max() < 1e-12 * scale


def test_cc_ausm_unit_area_quirk(cc):
    """CCFVM's AUSM+-up scales by |n| of the unit normal (ausm_up_flux.F90:38),
    not the face length, so a closed cell does NOT preserve freestream."""
    res = _first_residual(cc, "ausm")
    far = ~boundary_layers(cc.arrays, 3)
    assert np.abs(res[far]).max() > 1e-3


def _linear_state(m, npts_key):
    x, y = m["cx"], m["cy"]
    q = np.stack([1.0 + 0.002 * x - 0.001 * y, 0.5 + 0.003 * y, 0.1 - 0.002 * x,
                  1.0 / (1.4 * 0.25) + 0.01 * x + 0.02 * y], axis=1)
    grad = np.array([[0.002, -0.001], [0.0, 0.003], [-0.002, 0.0], [0.01, 0.02]])
    return q, grad


@pytest.mark.parametrize("grad", ["gg", "ggfc", "lsqr"])
def test_cc_gradients_exact_for_linear_fields(cc, grad):
    m = cc.arrays
    p = abi.make_params(grad=grad, ilimit=0)
    o = OracleCC(cc, p)
    q, g = _linear_state(m, "noc")
    o.set_state(prims_to_cons(q))
    qp = np.zeros((m["noc"] + m["nbf"], 5))
    qp[:, :4] = q
    qp[:, 4] = q[:, 3] / (q[:, 0] * (1.0 / (1.4 * 0.25)))
    o.set("qp", qp)  # every cell incl. ghosts carries the linear field
    o.avg_c2v()
    o.gradient()
    got = o.get("grad")
    exact = np.broadcast_to(g, got.shape)
    if grad == "gg":
        # the boundary term of Gradient_GG has the opposite sign
        # (CCFVM/gradient.F90:135-136), so only interior cells are exact
        mask = ~boundary_layers(m, 1)
    else:
        mask = np.ones(m["noc"], bool)
    err = np.abs(got[mask] - exact[mask]).max() / np.abs(g).max()
    assert err < 1e-9, err


def test_cc_gradient_gg_boundary_sign_quirk(cc):
    m = cc.arrays
    o = OracleCC(cc, abi.make_params(grad="gg", ilimit=0))
    q, g = _linear_state(m, "noc")
    o.set_state(prims_to_cons(q))
    qp = np.zeros((m["noc"] + m["nbf"], 5)); qp[:, :4] = q
    o.set("qp", qp)
    o.avg_c2v(); o.gradient()
    got = o.get("grad")
    wall_cells = m["fin"][m["nfi"]:]
    assert np.abs(got[wall_cells] - g).max() > 1e-3  # visibly not exact there


def test_nc_lsq_exact_and_freestream(nc):
    m = nc.arrays
    p = abi.make_params(flux="vanleer", m_inf=0.8, aoa_deg=1.25)
    o = OracleNC(nc, p)
    x, y = m["px"], m["py"]
    q = np.stack([1.0 + 0.002 * x, 0.5 + 0.003 * y, 0.1 - 0.002 * x + 0.001 * y, 2.0 + 0.01 * x], axis=1)
    o.set_state(prims_to_cons(q))
    o.save_old()
    o.fvresidual(1.0)
    g = o.get("grad")
    exact = np.array([[0.002, 0.0], [0.0, 0.003], [-0.002, 0.001], [0.01, 0.0]])
    assert np.abs(g - exact).max() < 1e-9
    # freestream: interior nodes see a closed dual contour
    o2 = OracleNC(nc, p)
    o2.save_old(); o2.fvresidual(1.0)
    res = o2.get("res")
    onb = np.zeros(m["nop"], bool)
    bf = m["fbc"] != 0
    onb[m["fp1"][bf]] = True
    onb[m["fp2"][bf]] = True
    assert np.abs(res[~onb]).max() < 1e-12 * m["farea"].max() / (1.4 * 0.64)


def test_cc_positivity_fault_reported(cc):
    o = OracleCC(cc, abi.make_params())
    qc = o.get_state().copy()
    qc[7, 0] = -1.0  # negative energy -> negative pressure in cell 7
    o.set_state(qc)
    o.con2prim()
    with pytest.raises(OracleError, match="NONPOSITIVE"):
        o.check_positivity()


def test_cc_negative_roe_sound_speed_reported(cc):
    o = OracleCC(cc, abi.make_params(flux="roe"))
    qc = o.get_state().copy()
    qc[: cc["noc"], 0] = 1e-3  # energy far below kinetic: negative pressure everywhere
    o.set_state(qc)
    o.con2prim(); o.avg_c2v(); o.time_step(0.5); o.save_old()
    with pytest.raises(OracleError):
        o.gradient()
        o.fvresidual()


def test_oracle_runs_are_deterministic(cc):
    p = abi.make_params(flux="roe", grad="gg")
    a, b = OracleCC(cc, p), OracleCC(cc, p)
    cfl = mesh.cfl_schedule(p, 1, 5)
    fa = [a.iteration(c) for c in cfl]
    fb = [b.iteration(c) for c in cfl]
    assert fa == fb
    assert np.array_equal(a.get_state(), b.get_state())
