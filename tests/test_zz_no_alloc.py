"""uns_residue_rms_noalloc: the residual norm without any device allocation.

It must return the same bits as uns_cc_residue for the same residual, call
after call (its scratch is a static device array reused by every call), and
refuse sizes beyond its static scratch before any device work.  The file is
named to be collected last, so the GPU case also runs after every other test
has used the device.
"""
import ctypes as C

import numpy as np
import pytest

from unsflow2d_gb300 import abi, mesh

MAX_CELLS = 4194304  # UNS_RMS_NOALLOC_MAX_CELLS in include/unsflow_gpu.h


def _noalloc(lib, ptr, n):
    out = C.c_double(-1.0)
    rc = lib.uns_residue_rms_noalloc(C.c_void_p(ptr), n, C.byref(out), None)
    return rc, out.value


def test_noalloc_rejects_bad_arguments_before_device_work():
    lib = abi.gpu_lib()
    fake = 1 << 20  # aligned, never dereferenced: every case is refused first
    assert _noalloc(lib, fake, MAX_CELLS + 1)[0] == abi.UNS_ERR_ARG
    assert _noalloc(lib, fake, 0)[0] == abi.UNS_ERR_ARG
    assert _noalloc(lib, fake, -5)[0] == abi.UNS_ERR_ARG
    assert _noalloc(lib, None, 10)[0] == abi.UNS_ERR_ARG
    assert _noalloc(lib, fake + 8, 10)[0] == abi.UNS_ERR_ARG  # not 32-byte aligned
    assert lib.uns_residue_rms_noalloc(C.c_void_p(fake), 10, None, None) == abi.UNS_ERR_ARG


@pytest.mark.gpu
def test_noalloc_matches_cc_residue_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    from unsflow2d_gb300.solver import CCSolver
    lib = abi.gpu_lib()
    m = mesh.CCMesh.airfoil(30, 14)  # 840 cells: not a multiple of the 256-cell block
    p = abi.make_params(flux="roe", grad="gg")
    s = CCSolver(m, p)
    cfl = mesh.cfl_schedule(p, 1, 2, "cc")
    for k in range(2):
        s.iteration(cfl[k])
        want = s.residue()
        res = torch.from_numpy(np.ascontiguousarray(s.get("res"))).cuda()
        torch.cuda.synchronize()
        rc, got = _noalloc(lib, res.data_ptr(), res.shape[0])
        abi.check(rc, lib, "uns_residue_rms_noalloc")
        assert got == want, (k, got, want)  # same reduction tree: same bits
        rc, again = _noalloc(lib, res.data_ptr(), res.shape[0])
        assert rc == abi.UNS_OK and again == got


@pytest.mark.gpu
def test_noalloc_at_the_size_limit():
    torch = pytest.importorskip("torch")
    lib = abi.gpu_lib()
    rng = np.random.default_rng(7)
    r = rng.standard_normal((MAX_CELLS, 4))
    res = torch.from_numpy(r).cuda()
    torch.cuda.synchronize()
    rc, got = _noalloc(lib, res.data_ptr(), MAX_CELLS)
    abi.check(rc, lib, "uns_residue_rms_noalloc")
    want = np.sqrt(np.sum(r * r) / MAX_CELLS / 4.0)
    assert abs(got - want) <= 1e-12 * want
    rc, tail = _noalloc(lib, res[1:].data_ptr(), MAX_CELLS - 1)
    assert rc == abi.UNS_OK
    want_tail = np.sqrt(np.sum(r[1:] * r[1:]) / (MAX_CELLS - 1) / 4.0)
    assert abs(tail - want_tail) <= 1e-12 * want_tail
