"""Regenerate the golden fixtures in this directory (run from the repo root):

    python tests/golden/make_golden.py

Writes two small airfoil O-meshes as reference-format geometry.inp files
(cc_16x8.inp, nc_16x8.inp) and, for several solver settings, the CPU oracle's
residual history and final fields after a few iterations (golden.npz).  The
oracle is the serial restatement of the reference Fortran; the reference itself
ships no test vectors and cannot be compiled here, so these fixtures pin the
oracle against regressions and give the GPU tests fixed inputs (the mesh files
are read back, so both machines start from identical bits).
"""
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))

from unsflow2d_gb300 import abi, mesh  # noqa: E402

CC_CASES = {
    "cc_roe_gg_rk3": dict(flux="roe", grad="gg"),
    "cc_vanleer_lsqr_rk3": dict(flux="vanleer", grad="lsqr"),
    "cc_rusanov_ggfc_rk3": dict(flux="rusanov", grad="ggfc"),
    "cc_roe_gg_lusgs": dict(flux="roe", grad="gg", time="lusgs", cfl_type="ramp", cfl_min=0.5, cfl_max=5.0,
                            cfl_ramp_steps=10),
    "cc_laminar_ggfc_rk3": dict(flux="roe", grad="ggfc", flow="laminar", iwall=0, rey=500.0),
}
NC_CASES = {
    "nc_vanleer_vkn_rk3": dict(flux="vanleer", limiter="vkn", time="rk3", cfl_max=0.9, m_inf=0.6, aoa_deg=2.89),
    "nc_ausm_barth_lusgs": dict(flux="ausm", limiter="barth_corrected", time="lusgs", cfl_max=50.0, m_inf=0.8,
                                aoa_deg=1.25),
}
NITER = 5


def main():
    from oracle import OracleCC, OracleNC
    cc = mesh.CCMesh.airfoil(16, 8)
    nc = mesh.NCMesh.airfoil(16, 8)
    cc.write(HERE / "cc_16x8.inp")
    nc.write(HERE / "nc_16x8.inp")
    cc = mesh.CCMesh.read(HERE / "cc_16x8.inp")
    nc = mesh.NCMesh.read(HERE / "nc_16x8.inp")
    out = {}
    for name, case in CC_CASES.items():
        p = abi.make_params(**case)
        o = OracleCC(cc, p)
        cfl = mesh.cfl_schedule(p, 1, NITER, "cc")
        out[f"{name}/fres"] = np.array([o.iteration(c) for c in cfl])
        for f in ("qc", "qp", "res", "phi", "grad", "la"):
            out[f"{name}/{f}"] = o.get(f)
    for name, case in NC_CASES.items():
        p = abi.make_params(**case)
        o = OracleNC(nc, p)
        cfl = mesh.cfl_schedule(p, 1, NITER, "nc")
        out[f"{name}/fres"] = np.array([o.iteration(c) for c in cfl])
        for f in ("qc", "qp", "res", "phi", "grad", "la"):
            out[f"{name}/{f}"] = o.get(f)
    np.savez_compressed(HERE / "golden.npz", **out)
    print(f"wrote {len(out)} arrays")


if __name__ == "__main__":
    main()
