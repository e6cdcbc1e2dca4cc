"""Packed CCFVM cases (uns_cc_create_packed): one index space, one launch of
each kernel per iteration for every case; each case must evolve exactly as it
does alone (residual history and state bit-identical), in the FP64 and the
mixed form, with different mesh sizes, fluxes, Mach numbers, angles of attack
and stop levels."""
import numpy as np
import pytest

from unsflow2d_gb300 import abi, mesh
from unsflow2d_gb300.solver import CCPacked, CCSolver

pytestmark = pytest.mark.gpu

CASES = [
    ((24, 12), dict(flux="roe", m_inf=0.5, aoa_deg=2.0)),
    ((32, 16), dict(flux="rusanov", m_inf=0.7, aoa_deg=-1.0)),
    ((40, 20), dict(flux="vanleer", m_inf=0.3, aoa_deg=5.0, min_res=0.3)),  # stops early
    ((28, 14), dict(flux="roe", m_inf=0.8, aoa_deg=1.0)),
]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_packed_matches_cases_run_alone(precision):
    meshes = [mesh.CCMesh.airfoil(ni, nj) for (ni, nj), _ in CASES]
    params = [abi.make_params(precision=precision, **kw) for _, kw in CASES]
    packed = CCPacked(meshes, params)
    alone = [CCSolver(m, p) for m, p in zip(meshes, params)]
    for chunk, (first, n) in enumerate(((1, 25), (26, 15))):
        cfl = np.stack([mesh.cfl_schedule(p, first, n, "cc") for p in params])
        hist, done = packed.iterate(cfl, first_iter=(chunk == 0))
        for i, s in enumerate(alone):
            h = s.iterate(cfl[i], first_iter=(chunk == 0))
            assert done[i] == len(h), (chunk, i, done[i], len(h))
            assert np.array_equal(hist[i], h), (chunk, i)
            assert np.array_equal(packed.get_state(i), s.get_state()), (chunk, i)
    assert done[2] < 15 or len(hist[2]) < 25  # the min_res = 0.3 case stopped
    packed.close()


def test_packed_rejects_mixed_settings():
    m = mesh.CCMesh.airfoil(16, 8)
    with pytest.raises(abi.UnsError):
        CCPacked([m, m], [abi.make_params(grad="gg"), abi.make_params(grad="lsqr")])
    with pytest.raises(abi.UnsError):
        CCPacked([m], [abi.make_params(time="lusgs")])


def test_packed_forces_equal_cases_run_alone():
    """The per-case wall forces of a packed handle are the single-case
    handle's (the same face order, bit for bit)."""
    meshes = [mesh.CCMesh.airfoil(ni, nj) for (ni, nj), _ in CASES]
    params = [abi.make_params(**dict(kw, min_res=0.0)) for _, kw in CASES]
    packed = CCPacked(meshes, params)
    cfl = np.stack([mesh.cfl_schedule(p, 1, 20, "cc") for p in params])
    packed.iterate(cfl, first_iter=True)
    f = packed.forces([np.asarray(m.arrays["fbc"])[m.arrays["nfi"]:] for m in meshes])
    for i, (m, p) in enumerate(zip(meshes, params)):
        s = CCSolver(m, p)
        s.iterate(cfl[i], first_iter=True)
        assert (f[i, 0], f[i, 1]) == s.forces(), i


def test_packed_batch_converges_with_the_precision_ramp():
    """Three cases to a 1e-7 drop: the mixed form (FP32 fluxes) until every
    running case is at its FP32 floor, then FP64; and plain FP64.  Both reach
    the drop, and C_L, C_D agree to 1e-6."""
    sel = CASES[:2] + CASES[3:]
    meshes = [mesh.CCMesh.airfoil(ni, nj) for (ni, nj), _ in sel]
    fbc = [np.asarray(m.arrays["fbc"])[m.arrays["nfi"]:] for m in meshes]
    out = {}
    for form in ("mixed", "fp64"):
        params = [abi.make_params(**dict(kw, precision=form, min_res=1e-7)) for _, kw in sel]
        b = CCPacked(meshes, params)
        r = b.converge(params, 1e-7, 30000, switch_drop=1e-4 if form == "mixed" else None)
        assert all(x is not None for x in r["reached_at"]), (form, r["reached_at"], r["iterations"])
        if form == "mixed":
            assert r["switched_at"] is not None
        f = b.forces(fbc)
        a = np.deg2rad([kw["aoa_deg"] for _, kw in sel])
        out[form] = (2 * (f[:, 1] * np.cos(a) - f[:, 0] * np.sin(a)), 2 * (f[:, 0] * np.cos(a) + f[:, 1] * np.sin(a)))
        b.close()
    assert np.max(np.abs(out["mixed"][0] - out["fp64"][0])) < 1e-6
    assert np.max(np.abs(out["mixed"][1] - out["fp64"][1])) < 1e-6
