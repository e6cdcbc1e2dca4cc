"""The device-side failure statuses, each made to happen from the host.

The reference stops on a negative Roe-averaged sound speed
(CCFVM/roe_flux.F90:73-87) and on a non-positive density or pressure
(check_positivity, CCFVM/main.F90:358-414); its main loop ends when the
residual norm is not a number (main.F90:57).  Here the kernels record the
first such event in the handle's device error word and the next call that
reads it returns the status: UNS_ERR_NEG_SOUND_SPEED, UNS_ERR_NONPOSITIVE,
UNS_ERR_NAN.  The LU-SGS sweeps' waits are bounded: a sweep item that never
publishes (a test hook) makes its consumers give up at the wait limit with
UNS_ERR_TIMEOUT, and the handle stays usable.  Every fault here is a state
or a setting written from the host; no kernel is broken on purpose.
"""
import ctypes as C

import numpy as np
import pytest

from oracle import OracleCC, OracleError
from unsflow2d_gb300 import abi, mesh
from unsflow2d_gb300.solver import CCSolver, NCSolver

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def cc_mesh():
    return mesh.CCMesh.airfoil(24, 12)


@pytest.fixture(scope="module")
def nc_mesh():
    return mesh.NCMesh.airfoil(24, 12)


def _status(g, name, *args):
    lib = abi.gpu_lib()
    rc = getattr(lib, f"uns_{g.kind}_{name}")(g._h, *args)
    return rc, lib.uns_last_error().decode()


def test_cc_nonpositive_cell_is_reported_with_its_index(cc_mesh):
    p = abi.make_params(flux="roe", grad="gg")
    g, o = CCSolver(cc_mesh, p), OracleCC(cc_mesh, p)
    qc = g.get_state()
    qc[37, 0] = -1.0  # negative energy: negative pressure in cell 37
    for s in (g, o):
        s.set_state(qc)
        s.con2prim()
    bad = C.c_int(-5)
    rc, msg = _status(g, "check_positivity", C.byref(bad))
    assert rc == abi.UNS_ERR_NONPOSITIVE and bad.value == 37 and msg.endswith(" 37")
    with pytest.raises(OracleError, match="NONPOSITIVE"):
        o.check_positivity()
    # the error word was cleared when it was read: the handle goes on
    g.initialize()
    g.con2prim()
    assert _status(g, "check_positivity", C.byref(bad))[0] == abi.UNS_OK and bad.value == -1
    # the graph-replayed iteration checks positivity in its first kernel
    g.set_state(qc)
    with pytest.raises(abi.UnsError) as e:
        g.iterate(mesh.cfl_schedule(p, 1, 3, "cc"), first_iter=True)
    assert e.value.code == abi.UNS_ERR_NONPOSITIVE and "cell 37" in str(e.value)


def test_cc_negative_roe_sound_speed_is_reported(cc_mesh):
    """Energies far below the kinetic energy everywhere (the oracle's known
    answer for the same state raises too): the Roe flux finds a^2 <= 0."""
    p = abi.make_params(flux="roe", grad="gg")
    g, o = CCSolver(cc_mesh, p), OracleCC(cc_mesh, p)
    qc = g.get_state()
    qc[: cc_mesh.arrays["noc"], 0] = 1e-3
    g.set_state(qc)
    g.con2prim(); g.avg_c2v(); g.time_step(0.5); g.save_old(); g.gradient(); g.fvresidual()
    bad = C.c_int(-5)
    rc, msg = _status(g, "check_positivity", C.byref(bad))
    assert rc == abi.UNS_ERR_NEG_SOUND_SPEED, (rc, msg)
    face = int(msg.rsplit(" ", 1)[1])
    assert msg.startswith("Roe scheme: sonic speed is negative at face") and 0 <= face < len(cc_mesh.arrays["fin"])
    o.set_state(qc)
    o.con2prim(); o.avg_c2v(); o.time_step(0.5); o.save_old()
    with pytest.raises(OracleError):
        o.gradient()
        o.fvresidual()


@pytest.mark.parametrize("kind", ["cc", "nc"])
def test_nan_state_ends_the_iteration_with_nan_status(cc_mesh, nc_mesh, kind):
    if kind == "cc":
        p = abi.make_params(flux="roe", grad="gg")
        g = CCSolver(cc_mesh, p)
    else:
        p = abi.make_params(flux="vanleer", limiter="vkn", time="lusgs", cfl_max=50.0, m_inf=0.8, aoa_deg=1.25)
        g = NCSolver(nc_mesh, p)
    qc = g.get_state()
    qc[5, 2] = np.nan
    g.set_state(qc)
    with pytest.raises(abi.UnsError) as e:
        g.iterate(mesh.cfl_schedule(p, 1, 4, kind), first_iter=True)
    assert e.value.code == abi.UNS_ERR_NAN
    hist = e.value.history if kind == "cc" else e.value.history[0]
    assert len(hist) == 1 and np.isnan(hist[0])
    # the handle is usable again from a clean state
    g.initialize()
    r = g.iterate(mesh.cfl_schedule(p, 1, 2, kind), first_iter=True)
    assert np.isfinite(r if kind == "cc" else r[0]).all()


@pytest.mark.parametrize("kind", ["cc", "nc"])
def test_sweep_wait_runs_out_with_timeout_status(cc_mesh, nc_mesh, kind):
    """Node (cell) 0's forward item publishes nothing: its neighbours and its
    own backward item wait, give up after the wait limit (2e7 cycles, about
    10 ms) and the sweep returns UNS_ERR_TIMEOUT.  Cleared, the same handle
    then reproduces a fresh handle's iterations bit for bit."""
    if kind == "cc":
        p = abi.make_params(flux="roe", grad="gg", time="lusgs", cfl_max=5.0, cfl_type="ramp", cfl_min=0.5,
                            cfl_ramp_steps=10)
        S, m = CCSolver, cc_mesh
    else:
        p = abi.make_params(flux="vanleer", limiter="vkn", time="lusgs", cfl_max=50.0, m_inf=0.8, aoa_deg=1.25)
        S, m = NCSolver, nc_mesh
    g = S(m, p)
    cfl = mesh.cfl_schedule(p, 1, 3, kind)
    g.set_wait_limit(20_000_000)
    g.debug_unpublish(0, 0)
    with pytest.raises(abi.UnsError) as e:
        g.iterate(cfl, first_iter=True)
    assert e.value.code == abi.UNS_ERR_TIMEOUT
    g.debug_unpublish(-1, 0)
    g.set_wait_limit(4_000_000_000)
    g.initialize()
    fresh = S(m, p)
    a, b = g.iterate(cfl, first_iter=True), fresh.iterate(cfl, first_iter=True)
    a, b = (a, b) if kind == "cc" else (a[0], b[0])
    assert np.array_equal(a, b) and np.array_equal(g.get_state(), fresh.get_state())


def test_hooks_reject_bad_arguments(cc_mesh):
    g = CCSolver(cc_mesh, abi.make_params())
    lib = abi.gpu_lib()
    assert lib.uns_cc_set_wait_limit(g._h, 0) == abi.UNS_ERR_ARG
    assert lib.uns_cc_debug_unpublish(g._h, cc_mesh.arrays["noc"], 0) == abi.UNS_ERR_ARG
    assert lib.uns_cc_debug_unpublish(g._h, 0, 2) == abi.UNS_ERR_ARG
    assert lib.uns_nc_set_wait_limit(None, 10) == abi.UNS_ERR_ARG
