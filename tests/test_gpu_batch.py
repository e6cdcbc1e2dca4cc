"""Batched CCFVM instances (uns_cc_batch_*): one graph launch advances every
instance; each instance must evolve exactly as it does on its own."""
import numpy as np
import pytest

from unsflow2d_gb300 import abi, mesh
from unsflow2d_gb300.solver import CCBatch, CCSolver

pytestmark = pytest.mark.gpu

CASES = [
    ((24, 12), dict(flux="roe", m_inf=0.5, aoa_deg=2.0)),
    ((32, 16), dict(flux="rusanov", m_inf=0.7, aoa_deg=-1.0)),
    ((40, 20), dict(flux="vanleer", m_inf=0.3, aoa_deg=5.0, min_res=0.3)),  # stops early
    ((28, 14), dict(flux="roe", m_inf=0.8, aoa_deg=1.0, precision="mixed")),
]


def _make():
    out = []
    for (ni, nj), kw in CASES:
        m = mesh.CCMesh.airfoil(ni, nj)
        p = abi.make_params(**kw)
        out.append((m, p))
    return out


def _schedules(params, first, n):
    return np.stack([mesh.cfl_schedule(p, first, n, "cc") for p in params])


def test_batch_matches_instances_run_alone():
    setup = _make()
    params = [p for _, p in setup]
    batch_solvers = [CCSolver(m, p) for m, p in setup]
    alone = [CCSolver(m, p) for m, p in setup]
    batch = CCBatch(batch_solvers)
    for chunk, (first, n) in enumerate(((1, 25), (26, 15))):
        cfl = _schedules(params, first, n)
        hist, done = batch.iterate(cfl, first_iter=(chunk == 0))
        for i, s in enumerate(alone):
            h = s.iterate(cfl[i], first_iter=(chunk == 0))
            assert done[i] == len(h)
            assert np.array_equal(hist[i], h), (chunk, i)
            assert np.array_equal(batch_solvers[i].get_state(), s.get_state()), (chunk, i)
    assert done[2] < 15 or len(hist[2]) < 25  # the min_res = 0.3 instance stopped
    # a precision switch rebuilds the batch graph and still matches
    batch_solvers[0].set_precision("mixed")
    alone[0].set_precision("mixed")
    cfl = _schedules(params, 41, 10)
    hist, done = batch.iterate(cfl, first_iter=False)
    for i, s in enumerate(alone):
        h = s.iterate(cfl[i], first_iter=False)
        assert np.array_equal(hist[i], h) and np.array_equal(batch_solvers[i].get_state(), s.get_state()), i
    batch.close()


def test_batch_rejects_bad_handles():
    m, p = _make()[0]
    s = CCSolver(m, p)
    with pytest.raises(abi.UnsError):
        CCBatch([s, s])
