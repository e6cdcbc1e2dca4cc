"""The complex-step instance of the CCFVM oracle (oracle_cc_cs.cpp) against the
oracle itself: its real part is the oracle's iteration, and Im(G)/h for an
input x + i h u agrees with central differences of the oracle's iteration in
direction u (state and angle of attack), for inviscid and laminar flows.
This pins the complex-step reference that the adjoint's GPU tests use."""
import numpy as np
import pytest

from oracle import OracleCC, OracleCCComplexStep
from unsflow2d_gb300 import abi, mesh

CASES = {
    "euler": dict(flux="roe", grad="gg", m_inf=0.5, aoa_deg=2.0),
    "laminar": dict(flow="laminar", iwall=0, rey=5000.0, flux="roe", grad="ggfc", m_inf=0.5, aoa_deg=3.0),
}
CFL = 0.5
H = 1e-30


def _developed(m, p, n=40):
    """The flow after n iterations from freestream with the limiter on (an
    unlimited start from freestream produces negative states at the ghosts)."""
    o = OracleCC(m, p)
    for c in mesh.cfl_schedule(p, 1, n, "cc"):
        o.iteration(c)
    return o.get("qc"), o.get("qp"), o.get("phi")


def _oracle_step(m, p, qc, qp, phi, dq=0.0, dg=0.0):
    """One iteration from (qc + dq, qp + dg), after one from (qc, qp) that sets
    the face viscosity its time step reads (as in _cs_step)."""
    o = OracleCC(m, p)
    o.set("phi", phi)
    o.set("qc", qc)
    o.set("qp", qp)
    o.iteration(CFL)
    o.set("qc", qc + dq)
    o.set("qp", qp + dg)
    o.iteration(CFL)
    fx, fy = o.forces()
    return o.get("qc"), o.get("qp"), fx, fy


def _cs_step(m, p, qc, qp, phi, dq=None, dg=None, aoa_im=0.0):
    o = OracleCCComplexStep(m, p, aoa_im)
    o.set("phi", phi)
    o.set("qc", qc)
    o.set("qp", qp)
    o.iteration(CFL)
    o.set("qc", qc, dq)
    o.set("qp", qp, dg)
    o.iteration(CFL)
    fx, fy = o.forces()
    return o.get("qc"), o.get("qp"), fx, fy


@pytest.mark.parametrize("name", list(CASES))
def test_complex_step_matches_oracle_and_differences(name):
    m = mesh.CCMesh.airfoil(16, 8)
    qc, qp, phi = _developed(m, abi.make_params(**CASES[name]))
    p = abi.make_params(ilimit=0, **CASES[name])  # limiter frozen at phi, as in the adjoint
    rng = np.random.default_rng(1)
    noc = m.arrays["noc"]
    u = np.zeros_like(qc)
    u[:noc] = rng.standard_normal((noc, 4)) * np.abs(qc[:noc])
    ug = np.zeros_like(qp)
    ug[noc:] = rng.standard_normal(qp[noc:].shape) * np.abs(qp[noc:])
    c_qc, c_qp, cfx, cfy = _cs_step(m, p, qc, qp, phi, H * u, H * ug)
    r_qc, r_qp, rfx, rfy = _oracle_step(m, p, qc, qp, phi)
    # real part = the oracle
    assert np.max(np.abs(c_qc.real - r_qc)) <= 1e-12 * np.max(np.abs(r_qc))
    assert abs(cfx.real - rfx) <= 1e-11 * abs(rfx) + 1e-15
    # imaginary part / h = central differences
    e = 1e-6
    a_qc, a_qp, afx, _ = _oracle_step(m, p, qc, qp, phi, e * u, e * ug)
    b_qc, b_qp, bfx, _ = _oracle_step(m, p, qc, qp, phi, -e * u, -e * ug)
    d_cs = c_qc.imag[:noc] / H
    d_fd = (a_qc - b_qc)[:noc] / (2 * e)
    assert np.max(np.abs(d_cs - d_fd)) <= 1e-6 * np.max(np.abs(d_cs))
    assert abs(cfx.imag / H - (afx - bfx) / (2 * e)) <= 1e-6 * abs(cfx.imag / H)
    # angle of attack
    pa = abi.make_params(ilimit=0, **{**CASES[name], "aoa_deg": CASES[name]["aoa_deg"] + 1e-4})
    pb = abi.make_params(ilimit=0, **{**CASES[name], "aoa_deg": CASES[name]["aoa_deg"] - 1e-4})
    a_qc, _, _, _ = _oracle_step(m, pa, qc, qp, phi)
    b_qc, _, _, _ = _oracle_step(m, pb, qc, qp, phi)
    c_qc, _, _, _ = _cs_step(m, p, qc, qp, phi, aoa_im=H)
    d_fd = (a_qc - b_qc)[:noc] / (2 * np.deg2rad(1e-4))
    d_cs = c_qc.imag[:noc] / H
    assert np.max(np.abs(d_cs - d_fd)) <= 1e-6 * np.max(np.abs(d_cs))


@pytest.mark.parametrize("name", list(CASES))
def test_geometric_complex_step_matches_differences_of_the_oracle(name):
    """An imaginary perturbation of one geometric mesh array
    (oracle_cc_cs_set_geometry_im) against central differences of the oracle
    on meshes whose array is perturbed: Im(G)/h equals (G(A + eps d) -
    G(A - eps d)) / (2 eps), array by array: two iterations from a developed
    state, the second from the first's state with its imaginary part
    dropped, the geometry perturbed in both (the time step of the second
    reads the first's face viscosity)."""
    m = mesh.CCMesh.airfoil(16, 8)
    kw = CASES[name]
    p = abi.make_params(ilimit=0, min_res=1e-30, **kw)
    qc, qp, phi = _developed(m, abi.make_params(min_res=1e-30, **kw))
    noc = m.arrays["noc"]
    rng = np.random.default_rng(17)
    eps = 1e-7
    for field in ("fnx", "farea", "fcx", "cx", "cv", "r12", "v2c_wt", "px") + (("cov",) if kw["grad"] == "ggfc" else ()):
        x = np.asarray(m.arrays[field], dtype=np.float64)
        d = rng.standard_normal(x.shape) * (np.abs(x) + 1e-3 * np.mean(np.abs(x)))
        o = OracleCCComplexStep(m, p)
        o.set_geometry_im(field, H * d)  # before both iterations, as the differences perturb both
        o.set("phi", phi)
        o.set("qc", qc)
        o.set("qp", qp)
        o.iteration(CFL)  # sets the face viscosity the next time step reads
        q1, g1 = o.get("qc").real, o.get("qp").real
        o.set("qc", q1)
        o.set("qp", g1)
        o.iteration(CFL)
        cs = o.get("qc")[:noc].imag / H
        out = []
        for sgn in (1, -1):
            arr = dict(m.arrays)
            arr[field] = x + sgn * eps * d
            r = OracleCC(arr, p)
            r.set("phi", phi)
            r.set("qc", qc)
            r.set("qp", qp)
            r.iteration(CFL)
            r.set("qc", q1)
            r.set("qp", g1)
            r.iteration(CFL)
            out.append(r.get("qc")[:noc])
        fd = (out[0] - out[1]) / (2 * eps)
        # the differences' rounding floor is about ulp(q) / eps, 1e-9 of the state;
        # an array the iteration does not depend on (cv under GG-FC, where dt / cv
        # cancels the volume) has a zero derivative that the differences see as that
        scale = np.max(np.abs(cs))
        floor = 1e-8 * np.max(np.abs(q1))
        assert np.max(np.abs(cs - fd)) <= 1e-5 * scale + floor, (field, np.max(np.abs(cs - fd)), scale)
