"""Device-side post-processing (uns_cc_find_cl_cd, uns_cc_screen_minmax,
uns_cc_tecplt; uns_nc_tecplt, uns_nc_screen_minmax) vs the oracle's
restatement of find_cl_cd, screen and tecplt (CCFVM/main.F90:187-480,
NCFVM/main.f90:115-233) after the same iterations on both.  The GPU state tracks the oracle's to
1e-12; the coefficients and wall rows are compared to 1e-10 of their scale,
the min/max diagnostics to 1e-12 (entropy: the math library's log10 / pow
differ in the last bits)."""
import numpy as np
import pytest

from oracle import OracleCC, OracleNC
from unsflow2d_gb300 import abi, mesh
from unsflow2d_gb300.solver import CCSolver, NCSolver

pytestmark = pytest.mark.gpu

CASES = {
    "euler": dict(flux="roe", grad="gg", m_inf=0.5, aoa_deg=2.0),
    "laminar_iso": dict(flux="roe", grad="ggfc", flow="laminar", iwall=0, rey=500.0, m_inf=0.5, aoa_deg=3.0),
    "laminar_adia": dict(flux="vanleer", grad="gg", flow="laminar", iwall=1, rey=5000.0, m_inf=0.5, aoa_deg=1.0),
}


@pytest.mark.parametrize("name", list(CASES))
def test_find_cl_cd_and_minmax_match_oracle(name):
    m = mesh.CCMesh.airfoil(24, 12)
    p = abi.make_params(**CASES[name])
    g, o = CCSolver(m, p), OracleCC(m, p)
    for c in mesh.cfl_schedule(p, 1, 30, "cc"):
        g.iteration(c)
        o.iteration(c)
    gc, gw = g.find_cl_cd(0.25, 0.0)
    oc, ow = o.find_cl_cd(0.25, 0.0)
    assert gw.shape == ow.shape and len(gw) == 24
    assert np.all(np.abs(gc - oc) <= 1e-10 * np.maximum(np.abs(oc), 1e-3)), (gc, oc)
    scale = np.maximum(np.abs(ow).max(axis=0), 1e-12)
    assert np.all(np.abs(gw - ow).max(axis=0) <= 1e-10 * scale), (np.abs(gw - ow).max(axis=0), scale)
    if CASES[name].get("flow") != "laminar":
        assert np.all(ow[:, 3] == 0.0)
    gm, om = g.screen_minmax(), o.screen_minmax()
    assert np.all(np.abs(gm - om) <= 1e-12 * np.maximum(np.abs(om), 1.0)), (gm, om)
    # flux-based coefficients agree with the solver's own force integral
    fx, fy = g.forces()
    a = np.deg2rad(CASES[name]["aoa_deg"])
    assert abs(gc[3] - (fy * np.cos(a) - fx * np.sin(a)) / 0.5) <= 1e-12 * abs(gc[3]) + 1e-15
    # tecplt's vertex table: averages, Mach, entropy, |V|, viscosity
    gt, ot = g.tecplt(), o.tecplt()
    scale = np.maximum(np.abs(ot).max(axis=0), 1e-300)
    assert np.all(np.abs(gt - ot).max(axis=0) <= 1e-12 * scale), (np.abs(gt - ot).max(axis=0) / scale)
    if CASES[name].get("flow") == "laminar":
        assert np.all(ot[:, 10] > 0.0)


@pytest.mark.parametrize("limiter", ["vkn", "barth_corrected"])
def test_nc_tecplt_and_screen_match_oracle(limiter):
    m = mesh.NCMesh.airfoil(24, 12)
    p = abi.make_params(flux="vanleer", limiter=limiter, time="lusgs", cfl_max=50.0, m_inf=0.8, aoa_deg=1.25)
    g, o = NCSolver(m, p), OracleNC(m, p)
    for c in mesh.cfl_schedule(p, 1, 20, "nc"):
        g.iteration(c)
        o.iteration(c)
    gt, ot = g.tecplt(), o.tecplt()
    scale = np.maximum(np.abs(ot).max(axis=0), 1e-300)
    assert np.all(np.abs(gt - ot).max(axis=0) <= 1e-12 * scale), (np.abs(gt - ot).max(axis=0) / scale)
    gm, om = g.screen_minmax(), o.screen_minmax()
    assert np.all(np.abs(gm - om) <= 1e-12 * np.maximum(np.abs(om), 1.0)), (gm, om)
