"""The contracted FP64 build (libunsflow_gpu_fma.so, UNSFLOW_FP64_FMA=1).

With multiply-add contraction the FP64 kernels round differently from the
reference's separate multiplies and adds, so they are no longer bit-exact;
they must still meet the parity criteria of the other tests (residuals 1e-12
of the flux scale, fields 1e-12 of their magnitude) and give the same FLO.RES
history to its printed digits.  The build is chosen per process, so each
check runs in a child process with the variable set.
"""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]

CHILD = r'''
import json, sys
sys.path.insert(0, %(root)r); sys.path.insert(0, %(root)r + "/oracle"); sys.path.insert(0, %(root)r + "/tests")
import numpy as np
from conftest import grad_err, inv_h_cc, inv_h_nc, rel_err, res_err
from oracle import OracleCC, OracleNC
from unsflow2d_gb300 import abi, mesh
from unsflow2d_gb300.solver import CCSolver, NCSolver
out = {"library": abi.gpu_library_name()}
abi.gpu_lib()
out["mapped"] = "libunsflow_gpu_fma.so" in open("/proc/self/maps").read()
# CCFVM, routine by routine over three iterations
m = mesh.CCMesh.airfoil(24, 12)
p = abi.make_params(flux="roe", grad="gg")
g, o = CCSolver(m, p), OracleCC(m, p)
e = {"res": 0.0, "qc": 0.0, "grad": 0.0, "phi": 0.0, "dt": 0.0}
c = 0.0
for it in range(1, 4):
    c = mesh.cfl_schedule(p, it, 1, "cc", c)[0]
    for s in (g, o):
        s.con2prim(); s.avg_c2v(); s.time_step(c); s.save_old(); s.gradient()
    e["grad"] = max(e["grad"], grad_err(g.get("grad"), o.get("grad"), o.get("qp")[:o.noc], inv_h_cc(m.arrays)))
    e["phi"] = max(e["phi"], rel_err(g.get("phi"), o.get("phi")))
    e["dt"] = max(e["dt"], rel_err(g.get("dt"), o.get("dt")))
    for irk in (1, 2, 3):
        for s in (g, o):
            s.fvresidual()
        e["res"] = max(e["res"], res_err(g.get("res"), o.get("res"), o.get("la"), o.get("qc")[:o.noc]))
        for s in (g, o):
            s.rk_stage(irk)
        e["qc"] = max(e["qc"], rel_err(g.get("qc"), o.get("qc")))
out["cc_routines"] = e
# CCFVM graph history, FLO.RES digits
g, o = CCSolver(m, p), OracleCC(m, p)
cfl = mesh.cfl_schedule(p, 1, 60, "cc")
fg = g.iterate(cfl, first_iter=True)
fo = np.array([o.iteration(x) for x in cfl])
flo = lambda f: ["%%6d%%16.6E" %% (i + 1, np.log10(x)) for i, x in enumerate(f)]
out["cc_history_lines_equal"] = flo(fg) == flo(fo)
out["cc_history_max_rel"] = float(np.max(np.abs(fg - fo) / fo))
out["cc_state_rel"] = rel_err(g.get_state(), o.get_state())
# NCFVM LU-SGS, three iterations
m = mesh.NCMesh.airfoil(24, 12)
p = abi.make_params(flux="ausm", limiter="barth_corrected", time="lusgs", cfl_max=50.0, m_inf=0.8, aoa_deg=1.25)
g, o = NCSolver(m, p), OracleNC(m, p)
e = {"res": 0.0, "qc": 0.0, "grad": 0.0}
for it in range(1, 4):
    c = mesh.cfl_schedule(p, it, 1, "nc")[0]
    for s in (g, o):
        s.save_old(); s.lusgs(c)
    e["grad"] = max(e["grad"], grad_err(g.get("grad"), o.get("grad"), o.get("qp"), inv_h_nc(m.arrays)))
    e["res"] = max(e["res"], res_err(g.get("res"), o.get("res"), o.get("la"), o.get("qc")))
    e["qc"] = max(e["qc"], rel_err(g.get("qc"), o.get("qc")))
out["nc_routines"] = e
print(json.dumps(out))
'''


@pytest.fixture(scope="module")
def fma_results():
    env = dict(os.environ, UNSFLOW_FP64_FMA="1")
    r = subprocess.run([sys.executable, "-c", CHILD % {"root": str(ROOT)}], capture_output=True, text=True, env=env,
                       timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


def test_fma_build_is_the_one_loaded(fma_results):
    assert fma_results["library"] == "unsflow_gpu_fma" and fma_results["mapped"]


def test_fma_cc_routines_within_parity_tolerance(fma_results):
    e = fma_results["cc_routines"]
    assert e["res"] <= 1e-12 and e["qc"] <= 1e-12 and e["grad"] <= 1e-12 and e["dt"] <= 1e-12, e
    assert e["phi"] <= 1e-10, e


def test_fma_cc_history_prints_the_same_flo_res(fma_results):
    assert fma_results["cc_history_lines_equal"], fma_results["cc_history_max_rel"]
    assert fma_results["cc_state_rel"] <= 1e-10


def test_fma_nc_lusgs_within_parity_tolerance(fma_results):
    e = fma_results["nc_routines"]
    assert e["res"] <= 1e-12 and e["qc"] <= 1e-12 and e["grad"] <= 1e-12, e
