"""The reference main program (flo.inp + geometry.inp -> FLO.RES, FLO.DAT) on
the GPU library, driven by the C++ caller side: per-routine calls (mode 0)
and the graph-replayed fast path (mode 1) write the same history as the
oracle's main loop; a restart from FLO.DAT (Start 2) picks up the saved state.
"""
import numpy as np
import pytest

from oracle import OracleCC
from unsflow2d_gb300 import mesh

from test_host import FLO_CC

pytestmark = pytest.mark.gpu


def _case(tmp_path, start=1, max_iter=20):
    m = mesh.CCMesh.airfoil(32, 16)
    m.write(tmp_path / "geometry.inp")
    text = FLO_CC.format(flow="inviscid", cfl_type="tanh", cfl=0.9, tm="rk3")
    text = text.replace("Start     1", f"Start     {start}").replace("MaxIter   20", f"MaxIter   {max_iter}")
    (tmp_path / "flo.inp").write_text(text)
    return tmp_path / "flo.inp"


def _history(path):
    rows = [line.split() for line in path.read_text().splitlines()]
    return np.array([[float(x.replace("D", "E")) for x in r] for r in rows])


def test_main_modes_match_the_oracle_loop(tmp_path):
    flo = _case(tmp_path)
    out0, out1 = tmp_path / "m0", tmp_path / "m1"
    out0.mkdir()
    out1.mkdir()
    it0, _ = mesh.run_main(flo, out0, "cc", mode=0)
    it1, _ = mesh.run_main(flo, out1, "cc", mode=1)
    assert it0 == it1 == 20
    h0, h1 = _history(out0 / "FLO.RES"), _history(out1 / "FLO.RES")
    assert np.array_equal(h0, h1)
    p, _ = mesh.read_flo_inp(flo)
    o = OracleCC(mesh.CCMesh.read(tmp_path / "geometry.inp"), p)
    fo = np.array([o.iteration(c) for c in mesh.cfl_schedule(p, 1, 20, "cc")])
    assert np.allclose(h0[:, 1], np.log10(fo / fo[0]), rtol=0, atol=2e-6)  # e16.6 text
    assert (out0 / "FLO.DAT").exists()


def test_restart_from_flo_dat(tmp_path):
    flo = _case(tmp_path, start=1, max_iter=20)
    first = tmp_path / "first"
    first.mkdir()
    mesh.run_main(flo, first, "cc", mode=1)
    saved = (first / "FLO.DAT").read_text()
    (tmp_path / "FLO.DAT").write_text(saved)
    # Start 2 with no iterations writes back exactly the state it read
    flo = _case(tmp_path, start=2, max_iter=0)
    again = tmp_path / "again"
    again.mkdir()
    it, _ = mesh.run_main(flo, again, "cc", mode=1)
    assert it == 0 and (again / "FLO.DAT").read_text() == saved
    # ... and continues from it
    flo = _case(tmp_path, start=2, max_iter=5)
    cont = tmp_path / "cont"
    cont.mkdir()
    it, _ = mesh.run_main(flo, cont, "cc", mode=1)
    assert it == 5
    q0 = np.loadtxt(first / "FLO.DAT")
    q1 = np.loadtxt(cont / "FLO.DAT")
    assert np.isfinite(q1).all() and np.max(np.abs(q1 - q0)) < 0.1 * np.max(np.abs(q0))
