"""Golden fixtures (tests/golden, written by make_golden.py from the CPU oracle).

CPU: the oracle reproduces them (pins the oracle across x86 / Arm hosts).
GPU: the CUDA path reproduces them (1e-12 for states/residual norms, 1e-10 for
the ill-conditioned gradient / limiter fields).
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import OracleCC, OracleNC
from unsflow2d_gb300 import abi, mesh

HERE = Path(__file__).resolve().parent / "golden"
import importlib.util
_spec = importlib.util.spec_from_file_location("make_golden", HERE / "make_golden.py")
G = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(G)


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(HERE / "golden.npz"))


@pytest.fixture(scope="module")
def meshes():
    return mesh.CCMesh.read(HERE / "cc_16x8.inp"), mesh.NCMesh.read(HERE / "nc_16x8.inp")


def _inv_h(kind, m):
    from conftest import inv_h_cc, inv_h_nc
    return inv_h_cc(m.arrays) if kind == "cc" else inv_h_nc(m.arrays)


def _cases():
    return [(n, "cc", c) for n, c in G.CC_CASES.items()] + [(n, "nc", c) for n, c in G.NC_CASES.items()]


def _check(golden, name, run_fres, getter, gpu, inv_h):
    """Oracle on another host: 1e-13.  GPU: the parity criteria of conftest.py."""
    from conftest import grad_err, res_err
    ref = golden[f"{name}/fres"]
    fres = np.asarray(run_fres)
    if fres.ndim == 2:
        fres = fres[:, 0]
    if ref.ndim == 2:  # NCFVM rows: (L2, Linf)
        ref = ref[:, 0]
    rtol = 1e-12 if gpu else 1e-13
    assert np.allclose(fres, ref, rtol=1e-10 if gpu else 1e-13, atol=0), (name, fres, ref)
    G = {f: golden[f"{name}/{f}"] for f in ("qc", "qp", "res", "phi", "grad", "la")}
    n = len(G["res"])
    for f in ("qc", "phi", "la"):
        r, g = G[f], getter(f)
        scale = np.abs(r).reshape(len(r), -1).max(axis=0)
        err = (np.abs(g - r).reshape(len(r), -1).max(axis=0) / np.maximum(scale, 1e-300)).max()
        assert err <= (1e-10 if f == "phi" and gpu else rtol), (name, f, err)
    assert res_err(getter("res"), G["res"], G["la"], G["qc"][:n]) <= rtol, (name, "res")
    assert grad_err(getter("grad"), G["grad"], G["qp"][:n], inv_h) <= rtol, (name, "grad")


@pytest.mark.parametrize("name,kind,case", _cases(), ids=[c[0] for c in _cases()])
def test_oracle_matches_golden(golden, meshes, name, kind, case):
    m = meshes[0] if kind == "cc" else meshes[1]
    p = abi.make_params(**case)
    o = (OracleCC if kind == "cc" else OracleNC)(m, p)
    cfl = mesh.cfl_schedule(p, 1, G.NITER, kind)
    fres = [o.iteration(c) for c in cfl]
    _check(golden, name, fres, o.get, False, _inv_h(kind, m))


@pytest.mark.gpu
@pytest.mark.parametrize("name,kind,case", _cases(), ids=[c[0] for c in _cases()])
def test_gpu_matches_golden(golden, meshes, name, kind, case):
    from unsflow2d_gb300.solver import CCSolver, NCSolver
    m = meshes[0] if kind == "cc" else meshes[1]
    p = abi.make_params(**case)
    s = (CCSolver if kind == "cc" else NCSolver)(m, p)
    cfl = mesh.cfl_schedule(p, 1, G.NITER, kind)
    r = s.iterate(cfl, first_iter=True)
    fres = r if kind == "cc" else r[0]
    _check(golden, name, fres, s.get, True, _inv_h(kind, m))
