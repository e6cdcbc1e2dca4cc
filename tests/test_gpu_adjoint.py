"""Discrete adjoint of the CCFVM RK3 iteration (uns_cc_adjoint_*).

At a converged state s* the adjoint runs the iteration G backwards:
uns_cc_adjoint_vjp returns G_s^T w + seed*J_s^T and G_alpha^T w + seed*J_alpha
for the flux-based C_L / C_D.  Checked here against central differences of the
GPU forward iteration itself (same limiter frozen at the converged phi):

* one transposed iteration: <w, dG/ds u> + seed <dJ/ds, u> (central difference,
  step 1e-6 relative per entry) equals <G_s^T w + seed J_s^T, u> for random
  w, u, and likewise for the angle of attack;
* the same transposed iteration against complex-step derivatives (step
  1e-30 i) of one iteration of the CPU oracle's complex-step instance at the
  converged state, which have no cancellation error: agreement to 1e-8;
* the total derivative dJ/dalpha of the adjoint solve equals the central
  difference of J between two solutions re-converged at alpha +- 5e-4 deg.

Inviscid (slip wall) and laminar (isothermal and adiabatic no-slip walls)
flows, the Roe, van Leer and Rusanov fluxes and the three gradients are
covered at converged states.  The CCFVM AUSM+-up flux (not scaled by the
face length -- a reference quirk) turns a cell non-positive on these meshes,
and a laminar flow with a non-GGFC convective gradient (the viscous step
recomputes the cell gradient inside each iteration) converges too slowly to
reach 1e-12, so neither has a converged state to differentiate; their
transposed iterations (AUSM+-up inviscid and laminar, laminar GG and LSQR)
are checked against the complex step at developed states instead, with the
oracle's local time step frozen as the adjoint's is.
"""
import numpy as np
import pytest

from unsflow2d_gb300 import abi, mesh
from unsflow2d_gb300.solver import CCSolver

pytestmark = pytest.mark.gpu

CFL = 0.8
CASES = {
    "euler_roe_gg": dict(flux="roe", grad="gg", m_inf=0.5, aoa_deg=2.0),
    "euler_roe_ggfc": dict(flux="roe", grad="ggfc", m_inf=0.5, aoa_deg=2.0),
    "euler_vanleer_lsqr": dict(flux="vanleer", grad="lsqr", m_inf=0.5, aoa_deg=2.0),
    "euler_rusanov_gg": dict(flux="rusanov", grad="gg", m_inf=0.5, aoa_deg=2.0),
    "laminar_roe_ggfc_iso": dict(flow="laminar", iwall=0, rey=5000.0, flux="roe", grad="ggfc", m_inf=0.5, aoa_deg=3.0),
    "laminar_roe_ggfc_adia": dict(flow="laminar", iwall=1, rey=5000.0, flux="roe", grad="ggfc", m_inf=0.5, aoa_deg=3.0),
}
_cache = {}


def _converge(s: CCSolver, target: float, chunk: int = 5000, max_iter: int = 300000) -> float:
    """Iterate until the raw residual norm is at most `target`; returns the last norm."""
    last, done = np.inf, 0
    while done < max_iter and last > target:
        h = s.iterate(np.full(chunk, CFL), first_iter=(done == 0))
        last = h[-1]
        done += chunk
    return last


def _frozen(m, kw, aoa=None):
    k = dict(kw)
    if aoa is not None:
        k["aoa_deg"] = aoa
    return CCSolver(m, abi.make_params(ilimit=0, min_res=1e-30, **k))


def _base(name):
    """Converged state of a case: limiter on while the flow develops, then phi frozen."""
    if name in _cache:
        return _cache[name]
    kw = CASES[name]
    m = mesh.CCMesh.airfoil(32, 16)
    p = abi.make_params(min_res=1e-30, **kw)
    s = CCSolver(m, p)
    r0 = s.iterate(mesh.cfl_schedule(p, 1, 600, "cc"), first_iter=True)[0]
    f = _frozen(m, kw)
    f.set("qc", s.get_state())
    f.set("qp", s.get("qp"))
    f.set("phi", s.get("phi"))
    target = 1e-12 * r0
    drop = _converge(f, target) / r0
    state = (f.get_state(), f.get("qp"), f.get("phi"))
    _cache[name] = (m, kw, f, state, drop, target)
    return _cache[name]


def _prime(s: CCSolver, state):
    """Load the converged state and run one iteration from it, so the face
    viscosity that the next iteration's time step reads is the converged
    one (a fresh handle holds zero there); then load the state again."""
    _load(s, state)
    s.iterate(np.array([CFL]), first_iter=True)
    _load(s, state)
    return s


def _load(s: CCSolver, state, dq=None, dg=None):
    qc, qp, phi = (x.copy() for x in state)
    noc = s.noc
    if dq is not None:
        qc[:noc] += dq
        qp[noc:] += dg
    s.set("qc", qc)
    s.set("qp", qp)
    s.set("phi", phi)


def _step(s: CCSolver):
    """One iteration G: returns (interior qc, ghost primitives + T, C_L, C_D)."""
    s.iterate(np.array([CFL]), first_iter=True)
    cl, cd = s.cl_cd()
    return s.get_state()[:s.noc], s.get("qp")[s.noc:], cl, cd


@pytest.mark.parametrize("name", list(CASES))
def test_vjp_matches_forward_differences(name):
    m, kw, f, state, drop, _ = _base(name)
    assert drop <= 1e-12, drop
    noc, nbf = f.noc, f.nbf
    qc0, qp0 = state[0][:noc], state[1][noc:]
    rng = np.random.default_rng(7)
    uq = rng.standard_normal(qc0.shape) * np.abs(qc0)
    ug = rng.standard_normal(qp0.shape) * np.abs(qp0)
    wq = rng.standard_normal((noc, 4))
    wg = rng.standard_normal((nbf, 5))
    seed = 0.7
    g = _prime(_frozen(m, kw), state)
    h = 1e-6
    _load(g, state, h * uq, h * ug)
    qa, ga, cla, cda = _step(g)
    _load(g, state, -h * uq, -h * ug)
    qb, gb, clb, cdb = _step(g)
    a = _frozen(m, kw)
    _load(a, state)
    a.adjoint_prepare(CFL)
    for obj, ja, jb in (("cl", cla, clb), ("cd", cda, cdb)):
        lhs = (np.sum(wq * (qa - qb)) + np.sum(wg * (ga - gb)) + seed * (ja - jb)) / (2 * h)
        oq, og, _ = a.adjoint_vjp(obj, seed, wq, wg)
        rhs = np.sum(oq * uq) + np.sum(og * ug)
        assert abs(lhs - rhs) <= 1e-6 * abs(lhs), (obj, lhs, rhs)
    # angle of attack (per radian)
    da = 1e-4
    gp_ = _prime(_frozen(m, kw, kw["aoa_deg"] + da), state)
    gm_ = _prime(_frozen(m, kw, kw["aoa_deg"] - da), state)
    qa, ga, cla, cda = _step(gp_)
    qb, gb, clb, cdb = _step(gm_)
    scale = 2 * np.deg2rad(da)
    for obj, ja, jb in (("cl", cla, clb), ("cd", cda, cdb)):
        lhs = (np.sum(wq * (qa - qb)) + np.sum(wg * (ga - gb)) + seed * (ja - jb)) / scale
        _, _, oa = a.adjoint_vjp(obj, seed, wq, wg)
        assert abs(lhs - oa) <= 1e-6 * max(abs(lhs), 1e-3), (obj, lhs, oa)


@pytest.mark.parametrize("name", ["euler_roe_gg", "laminar_roe_ggfc_iso"])
def test_total_derivative_matches_reconverged_differences(name):
    m, kw, f, state, _, target = _base(name)
    a = _frozen(m, kw)
    _load(a, state)
    cl0, cd0 = a.adjoint_prepare(CFL)
    da = 5e-4
    res = {}
    for sgn in (1, -1):
        s = _frozen(m, kw, kw["aoa_deg"] + sgn * da)
        _load(s, state)
        assert _converge(s, target) <= target
        s.iterate(np.array([CFL]), first_iter=True)
        res[sgn] = s.cl_cd()
    for k, obj in enumerate(("cl", "cd")):
        fd = (res[1][k] - res[-1][k]) / (2 * np.deg2rad(da))
        d, hist = a.adjoint_solve(obj, max_iter=300000, tol=1e-12)
        assert len(hist) < 300000 and np.isfinite(d)
        assert abs(d - fd) <= 2e-5 * abs(fd), (obj, d, fd)


@pytest.mark.parametrize("name", ["euler_roe_gg", "laminar_roe_ggfc_iso"])
def test_vjp_matches_complex_step(name):
    from oracle import OracleCCComplexStep
    m, kw, f, state, _, _ = _base(name)
    noc, nbf = f.noc, f.nbf
    qc, qp, phi = state
    rng = np.random.default_rng(11)
    uq = rng.standard_normal((noc, 4)) * np.abs(qc[:noc])
    ug = rng.standard_normal((nbf, 5)) * np.abs(qp[noc:])
    wq = rng.standard_normal((noc, 4))
    wg = rng.standard_normal((nbf, 5))
    seed = 0.7
    p = abi.make_params(ilimit=0, min_res=1e-30, **kw)
    H = 1e-30

    def cs_step(dq=None, dg=None, aoa_im=0.0):
        o = OracleCCComplexStep(m, p, aoa_im)
        o.set("phi", phi)
        o.set("qc", qc)
        o.set("qp", qp)
        o.iteration(CFL)  # sets the face viscosity that the next time step reads
        o.set("qc", qc, dq)
        o.set("qp", qp, dg)
        o.iteration(CFL)
        return o.get("qc")[:noc], o.get("qp")[noc:], o.forces()

    def coefficients(fx, fy, a):
        return {"cl": 2 * (fy * np.cos(a) - fx * np.sin(a)), "cd": 2 * (fx * np.cos(a) + fy * np.sin(a))}

    a = _frozen(m, kw)
    _load(a, state)
    a.adjoint_prepare(CFL)
    alpha = np.deg2rad(kw["aoa_deg"])
    dq = np.zeros_like(qc)
    dq[:noc] = H * uq
    dg = np.zeros_like(qp)
    dg[noc:] = H * ug
    cq, cg, (fx, fy) = cs_step(dq, dg)
    J = coefficients(fx, fy, alpha)
    for obj in ("cl", "cd"):
        lhs = (np.sum(wq * cq.imag) + np.sum(wg * cg.imag) + seed * J[obj].imag) / H
        oq, og, _ = a.adjoint_vjp(obj, seed, wq, wg)
        rhs = np.sum(oq * uq) + np.sum(og * ug)
        assert abs(lhs - rhs) <= 1e-8 * abs(lhs), (obj, lhs, rhs)
    cq, cg, (fx, fy) = cs_step(aoa_im=H)
    J = coefficients(fx, fy, alpha + 1j * H)
    for obj in ("cl", "cd"):
        lhs = (np.sum(wq * cq.imag) + np.sum(wg * cg.imag) + seed * J[obj].imag) / H
        _, _, oa = a.adjoint_vjp(obj, seed, wq, wg)
        assert abs(lhs - oa) <= 1e-8 * abs(lhs), (obj, lhs, oa)


#: Schemes with no converged state on these meshes (the AUSM+-up flux turns a
#: cell non-positive after about 110 iterations; the laminar flows with a
#: GG or LSQR convective gradient converge too slowly): their transposed
#: iteration is checked at a developed state after `iters` iterations instead.
DEVELOPED = {
    "euler_ausm_gg": (dict(flux="ausm", grad="gg", m_inf=0.5, aoa_deg=2.0), 60),
    "euler_ausm_lsqr": (dict(flux="ausm", grad="lsqr", m_inf=0.5, aoa_deg=2.0), 60),
    "laminar_roe_gg_iso": (dict(flow="laminar", iwall=0, rey=5000.0, flux="roe", grad="gg", m_inf=0.5, aoa_deg=3.0), 600),
    "laminar_vanleer_lsqr_adia": (dict(flow="laminar", iwall=1, rey=5000.0, flux="vanleer", grad="lsqr", m_inf=0.5,
                                       aoa_deg=3.0), 600),
    "laminar_ausm_ggfc_iso": (dict(flow="laminar", iwall=0, rey=5000.0, flux="ausm", grad="ggfc", m_inf=0.5,
                                   aoa_deg=3.0), 100),
}


@pytest.mark.parametrize("name", list(DEVELOPED))
def test_vjp_matches_complex_step_at_a_developed_state(name):
    """At any state the transposed iteration is the exact Jacobian of one
    iteration with the local time step held at its recorded value (the
    adjoint's linearisation; freezing it changes this derivative by about
    1e-3 here, so the check tells the two apart).  The complex-step oracle with its time step
    frozen computes the same directional derivative, so the dot products
    agree away from convergence too.  A viscous flow's uns_cc_adjoint_prepare
    runs one plain iteration before it records (for the face viscosity the
    time step reads), so there the linearisation point is G(s)."""
    from oracle import OracleCCComplexStep
    kw, iters = DEVELOPED[name]
    m = mesh.CCMesh.airfoil(32, 16)
    p = abi.make_params(min_res=1e-30, **kw)
    s = CCSolver(m, p)
    cfls = mesh.cfl_schedule(p, 1, iters + 1, "cc")
    s.iterate(cfls[:-1], first_iter=True)
    cfl = float(cfls[-1])  # the schedule's next CFL (still ramping up)
    state = (s.get_state(), s.get("qp"), s.get("phi"))
    noc, nbf = s.noc, s.nbf
    viscous = kw.get("flow") == "laminar"
    pf = abi.make_params(ilimit=0, min_res=1e-30, **kw)
    H = 1e-30

    def cs_instance(aoa_im=0.0):
        o = OracleCCComplexStep(m, pf, aoa_im)
        o.set("phi", state[2])
        o.set("qc", state[0])
        o.set("qp", state[1])
        if viscous:
            o.iteration(cfl)
        o.freeze_dt()
        return o

    base = cs_instance()
    qc1, qp1 = base.get("qc").real, base.get("qp").real
    rng = np.random.default_rng(23)
    uq = rng.standard_normal((noc, 4)) * np.abs(qc1[:noc])
    ug = rng.standard_normal((nbf, 5)) * np.abs(qp1[noc:])
    wq = rng.standard_normal((noc, 4))
    wg = rng.standard_normal((nbf, 5))
    seed = 0.7

    def cs_step(dq=None, dg=None, aoa_im=0.0):
        o = cs_instance(aoa_im)
        o.set("qc", qc1, dq)
        o.set("qp", qp1, dg)
        o.iteration(cfl)
        return o.get("qc")[:noc], o.get("qp")[noc:], o.forces()

    def coefficients(fx, fy, a):
        return {"cl": 2 * (fy * np.cos(a) - fx * np.sin(a)), "cd": 2 * (fx * np.cos(a) + fy * np.sin(a))}

    a = _frozen(m, kw)
    _load(a, state)
    a.adjoint_prepare(cfl)
    alpha = np.deg2rad(kw["aoa_deg"])
    dq = np.zeros_like(qc1)
    dq[:noc] = H * uq
    dg = np.zeros_like(qp1)
    dg[noc:] = H * ug
    cq, cg, (fx, fy) = cs_step(dq, dg)
    J = coefficients(fx, fy, alpha)
    for obj in ("cl", "cd"):
        lhs = (np.sum(wq * cq.imag) + np.sum(wg * cg.imag) + seed * J[obj].imag) / H
        oq, og, _ = a.adjoint_vjp(obj, seed, wq, wg)
        rhs = np.sum(oq * uq) + np.sum(og * ug)
        assert abs(lhs - rhs) <= 1e-8 * abs(lhs), (obj, lhs, rhs)
    cq, cg, (fx, fy) = cs_step(aoa_im=H)
    J = coefficients(fx, fy, alpha + 1j * H)
    for obj in ("cl", "cd"):
        lhs = (np.sum(wq * cq.imag) + np.sum(wg * cg.imag) + seed * J[obj].imag) / H
        _, _, oa = a.adjoint_vjp(obj, seed, wq, wg)
        assert abs(lhs - oa) <= 1e-8 * abs(lhs), (obj, lhs, oa)


def _geometry_vs_complex_step(m, kw, state, cfl, seed=0.7):
    """uns_cc_adjoint_geometry (G_X^T w + seed J_X^T for every geometric mesh
    array X) against complex-step derivatives of one oracle iteration with
    that array perturbed (dt / cv frozen, as the adjoint holds it), array by
    array, for random w.  Returns the per-array (adjoint, complex-step) pairs."""
    from oracle import OracleCCComplexStep
    arr = m.arrays
    noc, nbf = arr["noc"], arr["nbf"]
    viscous = kw.get("flow") == "laminar"
    pf = abi.make_params(ilimit=0, min_res=1e-30, **kw)
    H = 1e-30

    def instance():
        o = OracleCCComplexStep(m, pf)
        o.set("phi", state[2])
        o.set("qc", state[0])
        o.set("qp", state[1])
        if viscous:
            o.iteration(cfl)
        o.freeze_dt()
        return o

    base = instance()
    qc1, qp1 = base.get("qc").real, base.get("qp").real
    rng = np.random.default_rng(31)
    wq = rng.standard_normal((noc, 4))
    wg = rng.standard_normal((nbf, 5))
    a = _frozen(m, kw)
    _load(a, state)
    a.adjoint_prepare_geometry(cfl)
    out = a.adjoint_geometry("cl", seed, wq, wg)
    alpha = np.deg2rad(kw["aoa_deg"])
    pairs = {}
    for k in abi.CC_GEOM_FIELDS:
        x = np.asarray(arr[k], dtype=np.float64)
        d = rng.standard_normal(x.shape) * (np.abs(x) + 1e-3 * np.mean(np.abs(x)))
        o = instance()
        o.set_geometry_im(k, H * d)
        o.set("qc", qc1)
        o.set("qp", qp1)
        o.iteration(cfl)
        fx, fy = o.forces()
        cl = 2 * (fy * np.cos(alpha) - fx * np.sin(alpha))
        cs = (np.sum(wq * o.get("qc")[:noc].imag) + np.sum(wg * o.get("qp")[noc:].imag) + seed * cl.imag) / H
        pairs[k] = (float(np.dot(out[k], d)), float(cs))
    return pairs


GEOMETRY_CASES = ["euler_roe_gg", "euler_roe_ggfc", "euler_vanleer_lsqr", "laminar_roe_ggfc_iso", "laminar_roe_ggfc_adia"]


@pytest.mark.parametrize("name", GEOMETRY_CASES)
def test_geometry_vjp_matches_complex_step(name):
    """At the converged state: every geometric array's adjoint equals the
    complex-step derivative of one iteration, to 1e-8 of the summed terms."""
    m, kw, f, state, _, _ = _base(name)
    pairs = _geometry_vs_complex_step(m, kw, state, CFL)
    scale = sum(abs(c) for _, c in pairs.values())
    for k, (adj, cs) in pairs.items():
        assert abs(adj - cs) <= 1e-8 * scale, (k, adj, cs, scale)


@pytest.mark.parametrize("name", ["euler_ausm_gg", "euler_ausm_lsqr", "laminar_ausm_ggfc_iso"])
def test_geometry_vjp_matches_complex_step_at_a_developed_state(name):
    kw, iters = DEVELOPED[name]
    m = mesh.CCMesh.airfoil(32, 16)
    p = abi.make_params(min_res=1e-30, **kw)
    s = CCSolver(m, p)
    cfls = mesh.cfl_schedule(p, 1, iters + 1, "cc")
    s.iterate(cfls[:-1], first_iter=True)
    pairs = _geometry_vs_complex_step(m, kw, (s.get_state(), s.get("qp"), s.get("phi")), float(cfls[-1]))
    scale = sum(abs(c) for _, c in pairs.values())
    for k, (adj, cs) in pairs.items():
        assert abs(adj - cs) <= 1e-8 * scale, (k, adj, cs, scale)


def test_geometry_rejects_a_laminar_flow_with_a_stage_gradient():
    kw = DEVELOPED["laminar_roe_gg_iso"][0]
    a = _frozen(mesh.CCMesh.airfoil(16, 8), kw)
    with pytest.raises(abi.UnsError) as e:
        a.adjoint_prepare_geometry(CFL)
    assert e.value.code == abi.UNS_ERR_ARG


def test_geometry_entry_points_check_their_preconditions():
    kw = CASES["euler_roe_gg"]
    m = mesh.CCMesh.airfoil(16, 8)
    a = _frozen(m, kw)
    noc, nbf = a.noc, a.nbf
    with pytest.raises(abi.UnsError) as e:  # no geometric linearisation recorded
        a.adjoint_geometry("cl", 1.0, np.zeros((noc, 4)), np.zeros((nbf, 5)))
    assert e.value.code == abi.UNS_ERR_ARG
    a.adjoint_prepare(CFL)  # the state linearisation alone is not enough
    with pytest.raises(abi.UnsError) as e:
        a.adjoint_geometry("cl", 1.0, np.zeros((noc, 4)), np.zeros((nbf, 5)))
    assert e.value.code == abi.UNS_ERR_ARG
    import ctypes as C
    from unsflow2d_gb300.solver import CCPacked
    p = abi.make_params(ilimit=0, **kw)
    pk = CCPacked([m, m], [p, p])  # one case per handle: a packed handle is refused
    assert pk._lib.uns_cc_adjoint_prepare_geometry(pk._h, C.c_double(CFL), None, None) == abi.UNS_ERR_ARG
