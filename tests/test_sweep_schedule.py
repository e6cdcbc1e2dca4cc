"""The LU-SGS sweeps' warp schedule (host side, no GPU).

The sweep kernels run each warp's list of items in order and poll the
records of an item's predecessors, so they finish only if the schedule is
deadlock-free: with every warp at its next item, some warp's next item must
always have all its predecessors done.  These tests run that execution on
the CPU, one item at a time, for the schedules uns_cc_create and
uns_nc_create build (the same host code, through uns_host_sweep_schedule),
and check the dependency levels against the graph of the reference's
sweeps: item (i, forward) needs (j, forward) for every neighbour j < i;
item (i, backward) needs (i, forward) and (j, backward) for every neighbour
j > i (CCFVM/lusgs.F90:245-318, NCFVM/lusgs.f90:48-124)."""
import ctypes as C

import numpy as np
import pytest

from unsflow2d_gb300 import abi, mesh

I32 = C.POINTER(C.c_int32)


def _schedule(off, nbr, nwarps):
    n = len(off) - 1
    lib = abi.host_lib()
    lib.uns_host_sweep_schedule.argtypes = [C.c_int, I32, I32, C.c_int, I32, I32, I32]
    off = np.ascontiguousarray(off, dtype=np.int32)
    nbr = np.ascontiguousarray(nbr, dtype=np.int32)
    woff = np.zeros(nwarps + 1, dtype=np.int32)
    items = np.zeros(2 * n, dtype=np.int32)
    lev = np.zeros(2, dtype=np.int32)
    p = lambda a: a.ctypes.data_as(I32)  # noqa: E731
    rc = lib.uns_host_sweep_schedule(n, p(off), p(nbr), nwarps, p(woff), p(items), p(lev))
    assert rc == 0, lib.uns_host_last_error()
    return woff, items, lev


def _preds(off, nbr, code):
    n = len(off) - 1
    i, pas = code >> 1, code & 1
    nb = [int(j) for j in nbr[off[i]:off[i + 1]] if 0 <= j < n]
    if pas == 0:
        return [2 * j for j in nb if j < i]
    return [2 * i] + [2 * j + 1 for j in nb if j > i]


def _levels(off, nbr):
    n = len(off) - 1
    lf, lb = [0] * n, [0] * n
    for i in range(n):
        lf[i] = max([lf[j] + 1 for j in nbr[off[i]:off[i + 1]] if 0 <= j < i], default=0)
    for i in reversed(range(n)):
        lb[i] = max([lb[j] + 1 for j in nbr[off[i]:off[i + 1]] if i < j < n], default=0)
    return (max(lf) + 1 if n else 0), (max(lb) + 1 if n else 0)


def _check(off, nbr, nwarps):
    """Every item once, and the warps' lists run to the end without a stall."""
    n = len(off) - 1
    woff, items, lev = _schedule(off, nbr, nwarps)
    assert woff[0] == 0 and woff[-1] == 2 * n and np.all(np.diff(woff) >= 0)
    assert np.array_equal(np.sort(items), np.arange(2 * n))
    done = np.zeros(2 * n, dtype=bool)
    head = woff[:-1].copy()
    preds = {int(c): _preds(off, nbr, int(c)) for c in items}
    left = 2 * n
    while left:
        moved = False
        for w in range(nwarps):
            while head[w] < woff[w + 1] and all(done[p] for p in preds[int(items[head[w]])]):
                done[items[head[w]]] = True
                head[w] += 1
                left -= 1
                moved = True
        assert moved, "the schedule stalls: every warp waits on an item queued behind another wait"
    assert tuple(lev) == _levels(off, nbr)
    return lev


def _nc_graph(m):
    a = m.arrays
    off, e, fp1, fp2 = a["v2f_off"], a["v2f"], a["fp1"], a["fp2"]
    nbr = np.empty(len(e), dtype=np.int32)
    for i in range(a["nop"]):
        for k in range(off[i], off[i + 1]):
            nbr[k] = fp1[e[k]] if fp2[e[k]] == i else fp2[e[k]]
    return off, nbr


def _cc_graph(m):
    a = m.arrays
    off, f, fin, fout = a["c2f_off"], a["c2f"], a["fin"], a["fout"]
    nbr = np.empty(len(f), dtype=np.int32)
    for i in range(a["noc"]):
        for k in range(off[i], off[i + 1]):
            nbr[k] = fin[f[k]] if fout[f[k]] == i else fout[f[k]]  # ghosts (>= noc) are ignored
    return off, nbr


@pytest.mark.parametrize("nwarps", [1, 7, 64, 608])
def test_nc_sweep_schedule_runs_without_a_stall(nwarps):
    off, nbr = _nc_graph(mesh.NCMesh.airfoil(32, 16))
    lev = _check(off, nbr, nwarps)
    assert lev[0] > 1 and lev[1] > 1


@pytest.mark.parametrize("nwarps", [1, 5, 96, 608])
def test_cc_sweep_schedule_runs_without_a_stall(nwarps):
    off, nbr = _cc_graph(mesh.CCMesh.airfoil(32, 16))
    _check(off, nbr, nwarps)


@pytest.mark.parametrize("seed", range(6))
def test_sweep_schedule_on_random_graphs(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 400))
    deg = rng.integers(0, 9, n)
    off = np.concatenate([[0], np.cumsum(deg)]).astype(np.int32)
    nbr = rng.integers(-3, n + 3, int(off[-1])).astype(np.int32)  # some entries outside [0, n): ignored
    _check(off, nbr, int(rng.integers(1, 40)))


def test_sweep_schedule_of_no_entities_and_bad_arguments():
    woff, items, lev = _schedule(np.zeros(1, dtype=np.int32), np.zeros(0, dtype=np.int32), 3)
    assert list(woff) == [0, 0, 0, 0] and len(items) == 0 and list(lev) == [0, 0]
    lib = abi.host_lib()
    bad = np.array([0, 2, 1], dtype=np.int32)
    z = np.zeros(8, dtype=np.int32)
    p = lambda a: a.ctypes.data_as(I32)  # noqa: E731
    assert lib.uns_host_sweep_schedule(2, p(bad), p(z), 2, p(z), p(z), p(z)) == abi.UNS_ERR_ARG
    assert lib.uns_host_sweep_schedule(2, p(np.array([0, 1, 2], dtype=np.int32)), p(z), 0, p(z), p(z), p(z)) \
        == abi.UNS_ERR_ARG
