"""Caller-side host logic (no GPU): mesh generator, geometry.inp round trip,
geometric invariants, flo.inp reader, CFL schedules, and the C-ABI surface."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from unsflow2d_gb300 import abi, mesh

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def cc():
    return mesh.CCMesh.airfoil(32, 16)


@pytest.fixture(scope="module")
def nc():
    return mesh.NCMesh.airfoil(32, 16)


def test_cc_counts_match_the_o_mesh_formula(cc):
    I, J = 32, 16
    assert cc["noc"] == 2 * I * J
    assert cc["nop"] == I * (J + 1)
    assert cc["nfi"] + cc["nbf"] == I * (J + 1) + 2 * I * J
    assert cc["nbf"] == 2 * I


def test_cc_geometry_invariants(cc):
    m = cc.arrays
    assert np.allclose(np.hypot(m["fnx"], m["fny"]), 1.0, atol=1e-14)
    assert (m["cv"] > 0).all() and (m["cov"] > 0).all() and (m["farea"] > 0).all()
    # normal points from `in` to `out` (ghosts included)
    d = np.stack([m["cx"][m["fout"]] - m["cx"][m["fin"]], m["cy"][m["fout"]] - m["cy"][m["fin"]]], 1)
    assert ((d[:, 0] * m["fnx"] + d[:, 1] * m["fny"]) > 0).all()
    # every interior cell is closed: sum of n*A over its faces (signed) = 0
    noc = m["noc"]
    s = np.zeros((noc, 2))
    for f in range(len(m["fin"])):
        a = m["farea"][f] * np.array([m["fnx"][f], m["fny"][f]])
        s[m["fin"][f]] += a
        if m["fout"][f] < noc:
            s[m["fout"][f]] -= a
    assert np.abs(s).max() < 1e-12
    # triangles: three faces each; ghost count = boundary faces
    assert (np.diff(m["c2f_off"]) == 3).all()
    assert (m["fout"][m["nfi"]:] == noc + np.arange(m["nbf"])).all()


def test_cc_bfs_renumbering(cc):
    """renumber (CCFVM/geometric.F90:247-356): a permutation starting at file cell 1,
    and every renumbered cell >0 has an interior neighbour with a smaller number."""
    nn = cc.newnum()
    m = cc.arrays
    assert sorted(nn.tolist()) == list(range(m["noc"]))
    assert nn[0] == 0
    nfi = m["nfi"]
    lowest = np.full(m["noc"], m["noc"])
    for a, b in zip(m["fin"][:nfi], m["fout"][:nfi]):
        lowest[a] = min(lowest[a], b)
        lowest[b] = min(lowest[b], a)
    assert (lowest[1:] < np.arange(1, m["noc"])).all()


def test_cc_pseudo_laplacian_weights_reproduce_linear_fields(cc):
    m = cc.arrays
    f = lambda x, y: 3.0 + 2.0 * x - 5.0 * y
    vals = f(m["cx"], m["cy"])
    off, idx, w = m["v2c_off"], m["v2c"], m["v2c_wt"]
    avg = np.array([np.dot(w[off[i]:off[i + 1]], vals[idx[off[i]:off[i + 1]]]) / w[off[i]:off[i + 1]].sum()
                    for i in range(m["nop"])])
    assert np.abs(avg - f(m["px"], m["py"])).max() < 1e-9


def test_nc_geometry_invariants(nc, cc):
    m = nc.arrays
    assert np.isclose(m["cv"].sum(), cc["cv"].sum(), rtol=1e-12)
    assert (m["cv"] > 0).all()
    assert np.allclose(np.hypot(m["fnx"], m["fny"]), 1.0, atol=1e-14)
    # interior dual cells are closed
    s = np.zeros((m["nop"], 2))
    for f in range(m["nof"]):
        a = m["farea"][f] * np.array([m["fnx"][f], m["fny"][f]])
        s[m["fp1"][f]] += a
        s[m["fp2"][f]] -= a
    onb = np.zeros(m["nop"], bool)
    onb[m["fp1"][m["fbc"] != 0]] = True
    onb[m["fp2"][m["fbc"] != 0]] = True
    assert np.abs(s[~onb]).max() < 1e-12
    nn = nc.newnum()
    assert sorted(nn.tolist()) == list(range(m["nop"])) and nn[0] == 0


def test_geometry_inp_round_trip(cc, nc, tmp_path):
    for m, cls in ((cc, mesh.CCMesh), (nc, mesh.NCMesh)):
        path = tmp_path / f"{m.kind}.inp"
        m.write(path)
        r = cls.read(path)
        for k, v in m.arrays.items():
            if isinstance(v, np.ndarray):
                assert np.array_equal(v, r.arrays[k]), (m.kind, k)


def test_truncated_geometry_file_is_an_io_error(cc, tmp_path):
    path = tmp_path / "g.inp"
    cc.write(path)
    lines = path.read_text().splitlines()
    path.write_text("\n".join(lines[: len(lines) // 2]) + "\n")
    with pytest.raises(abi.UnsError) as e:
        mesh.CCMesh.read(path)
    assert e.value.code == abi.UNS_ERR_IO


def test_inverted_cell_is_a_mesh_error(cc, tmp_path):
    path = tmp_path / "g.inp"
    cc.write(path)
    text = path.read_text().splitlines()
    nop = int(text[0].split()[0])
    # move point 1 far outside: its cells fold over
    parts = text[1].split()
    parts[1], parts[2] = "50.0", "50.0"
    text[1] = " ".join(parts)
    path.write_text("\n".join(text) + "\n")
    with pytest.raises(abi.UnsError) as e:
        mesh.CCMesh.read(path)
    assert e.value.code == abi.UNS_ERR_MESH
    assert nop > 0


FLO_CC = """Start     1
FlowType  {flow}  1 300
Mach      0.5
AOA       2.0
Reynolds  5000
CFL       {cfl_type}  0.1  {cfl} 500
Timemode  {tm}
GradType  gg
LastIter  0
MaxIter   20
MinRes    1.0e-8
SaveInt   1000
ScrInt    100
NoIso     30
Flux      roe
Limiter   1
irs       0
FarBC     0  0.0  0.0
GridFile  "geometry.inp"
"""


def test_flo_inp_reader_and_validation(tmp_path):
    f = tmp_path / "flo.inp"
    f.write_text(FLO_CC.format(flow="inviscid", cfl_type="tanh", cfl=0.9, tm="rk3"))
    p, grid = mesh.read_flo_inp(f)
    assert grid == "geometry.inp" and p.m_inf == 0.5 and p.cfl_max == 0.9 and p.max_iter == 20
    assert p.flux_type == abi.FLUX["roe"] and p.time_mode == abi.TIME["rk3"]
    for bad in (dict(flow="turbulent", cfl_type="tanh", cfl=0.9, tm="rk3"),
                dict(flow="inviscid", cfl_type="linear", cfl=0.9, tm="rk3"),
                dict(flow="inviscid", cfl_type="tanh", cfl=1.0, tm="rk3"),   # rk3 needs CFL < 1
                dict(flow="inviscid", cfl_type="tanh", cfl=0.9, tm="gmres")):
        f.write_text(FLO_CC.format(**bad))
        with pytest.raises(abi.UnsError) as e:
            mesh.read_flo_inp(f)
        assert e.value.code == abi.UNS_ERR_ARG
    f.write_text("Start 1\nFlowType inviscid 1 300\n")
    with pytest.raises(abi.UnsError) as e:
        mesh.read_flo_inp(f)
    assert e.value.code == abi.UNS_ERR_IO


def test_flo_dat_round_trip_and_format(tmp_path):
    """save_flow / read_flow: '(4e20.10)' lines, ten significant digits."""
    lib = abi.host_lib()
    rng = np.random.default_rng(3)
    q = rng.standard_normal((7, 4)) * 10.0 ** rng.integers(-30, 30, (7, 4))
    q[0, 0] = 0.0
    f = tmp_path / "FLO.DAT"
    D = C.POINTER(C.c_double)
    abi.check(lib.uns_host_save_flow(str(f).encode(), q.ctypes.data_as(D), 7), lib, "save_flow")
    lines = f.read_text().splitlines()
    assert len(lines) == 7 and all(len(x) == 80 for x in lines)
    assert lines[0][:20] == "    0.0000000000E+00"
    assert re.fullmatch(r"( *-?0\.\d{10}E[+-]\d{2}){4}", lines[1])
    back = np.zeros((7, 4))
    abi.check(lib.uns_host_read_flow(str(f).encode(), back.ctypes.data_as(D), 7), lib, "read_flow")
    assert np.allclose(back, q, rtol=5e-10, atol=0)
    # list-directed input also takes Fortran D exponents; a short file is an I/O error
    f.write_text("1.5D0 2 3 4\n")
    one = np.zeros((1, 4))
    abi.check(lib.uns_host_read_flow(str(f).encode(), one.ctypes.data_as(D), 1), lib, "read_flow")
    assert one.tolist() == [[1.5, 2.0, 3.0, 4.0]]
    assert lib.uns_host_read_flow(str(f).encode(), back.ctypes.data_as(D), 2) == abi.UNS_ERR_IO


def test_cfl_schedules():
    p = abi.make_params(cfl_type="tanh", cfl_max=0.9, cfl_ramp_steps=500)
    c = mesh.cfl_schedule(p, 1, 600)
    s = np.arange(1, 601) / 499.0
    assert np.allclose(c, 0.5 * 0.9 * (1 + np.tanh(s * 7 - 3.5)), rtol=1e-15)
    p = abi.make_params(cfl_type="ramp", cfl_min=0.1, cfl_max=5.0, cfl_ramp_steps=10, time="lusgs")
    c = mesh.cfl_schedule(p, 1, 15)
    assert np.isclose(c[9], 5.0) and (c[10:] == c[9]).all()
    n = mesh.cfl_schedule(abi.make_params(cfl_max=50.0), 1, 3, kind="nc")
    assert np.allclose(n, 0.5 * 50 * (1 + np.tanh(np.arange(1, 4) * 7 / 500 - 3.5)))


def _declared(header: Path) -> set[str]:
    text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
    return set(re.findall(r"^\s*(?:const\s+)?\w+[\s\*]+(uns_\w+)\s*\(", text, flags=re.M))


DRIVER = {"uns_host_cc_main", "uns_host_nc_main"}  # libunsflow_driver.so


def test_c_abi_exports_every_declared_symbol():
    gpu, host, drv = abi.gpu_lib(), abi.host_lib(), abi.driver_lib()
    for header, lib in (("unsflow_gpu.h", gpu), ("unsflow_host.h", host)):
        names = _declared(ROOT / "include" / header)
        assert len(names) > 10
        missing = [n for n in names if not hasattr(drv if n in DRIVER else lib, n)]
        assert not missing, (header, missing)


def test_host_library_needs_no_gpu_library():
    """The mesh / flo.inp / CFL library loads and works on its own (the CPU
    reference arm of the benchmark uses it without the GPU library)."""
    import subprocess
    import sys
    code = ("import sys; sys.path.insert(0, %r)\n"
            "from unsflow2d_gb300 import abi, mesh\n"
            "m = mesh.CCMesh.airfoil(8, 4)\n"
            "assert m.arrays['noc'] == 64\n"
            "maps = open('/proc/self/maps').read()\n"
            "assert 'libunsflow_host.so' in maps and 'libunsflow_gpu.so' not in maps, 'gpu library mapped'\n"
            % str(ROOT))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_gpu_create_validates_mesh_on_the_host(cc):
    """A corrupt index is rejected before any device call (works without a GPU)."""
    lib = abi.gpu_lib()
    arr = {k: (v.copy() if isinstance(v, np.ndarray) else v) for k, v in cc.arrays.items()}
    arr["fin"][5] = arr["noc"] + 100
    view, keep = abi.cc_view_from_arrays(arr)
    h = C.c_void_p()
    rc = lib.uns_cc_create(C.byref(view), C.byref(abi.make_params()), C.byref(h))
    assert rc == abi.UNS_ERR_MESH and not h.value
    assert b"out-of-range" in lib.uns_last_error()


def test_plot3d_ogrid_matches_the_generator(tmp_path):
    """MeshGen's plot3d input path: the generator's O-grid written as plot3d and
    read back gives the same CCFVM and NCFVM meshes (%.17g round-trips)."""
    path = tmp_path / "grid.grd"
    mesh.write_airfoil_plot3d(path, 16, 8, 0.12, 20.0, 1e-3)
    for cls in (mesh.CCMesh, mesh.NCMesh):
        a, b = cls.airfoil(16, 8, 0.12, 20.0, 1e-3).arrays, cls.plot3d(path).arrays
        assert sorted(a) == sorted(b)
        for k in a:
            if isinstance(a[k], np.ndarray):
                assert np.array_equal(a[k], b[k]), (cls.kind, k)
            else:
                assert a[k] == b[k], (cls.kind, k)


def test_plot3d_rejects_bad_grids(tmp_path):
    bad = tmp_path / "two_blocks.grd"
    bad.write_text("2\n5 2 1\n")
    with pytest.raises(abi.UnsError):
        mesh.CCMesh.plot3d(bad)
    # not an O-grid: the last i column does not repeat the first
    nx, ny = 6, 3
    xs = [float(i) for j in range(ny) for i in range(nx)]
    ys = [float(j) for j in range(ny) for i in range(nx)]
    open_grid = tmp_path / "open.grd"
    open_grid.write_text(f"1\n{nx} {ny} 1\n" + "\n".join(map(str, xs + ys + [0.0] * (nx * ny))) + "\n")
    with pytest.raises(abi.UnsError):
        mesh.CCMesh.plot3d(open_grid)


def test_tecplt_writer_layout(tmp_path):
    """tecplt.dat as the reference lays it out: header, N/E line, node rows
    of at most seven values, 1-based triangle vertex lists."""
    m = mesh.CCMesh.airfoil(8, 4)
    cells = mesh.cc_cell_vertices(m.arrays)
    assert cells.shape == (m.arrays["noc"], 3) and cells.min() == 0 and cells.max() < m.arrays["nop"]
    table = np.arange(m.arrays["nop"] * 11, dtype=float).reshape(-1, 11)
    path = tmp_path / "tecplt.dat"
    mesh.write_tecplt(path, table, [f"v{k}" for k in range(11)], cells)
    lines = path.read_text().splitlines()
    assert lines[2].strip() == "ZONE F=FEPOINT,ET=TRIANGLE"
    assert lines[3].strip() == f"N={m.arrays['nop']},E={m.arrays['noc']}"
    nodes = lines[4:4 + 2 * m.arrays["nop"]]
    vals = np.array([float(x) for ln in nodes for x in ln.split()]).reshape(-1, 11)
    assert np.array_equal(vals, table)
    elems = np.array([[int(x) for x in ln.split()] for ln in lines[4 + 2 * m.arrays["nop"]:]])
    assert np.array_equal(elems, cells + 1)


def test_moved_mesh_at_the_same_nodes_is_the_mesh(cc):
    a = cc.arrays
    m = cc.moved(a["px"], a["py"]).arrays
    for k in abi.CC_GEOM_FIELDS:  # centroids are recomputed as vertex means: rounding only
        assert np.allclose(m[k], a[k], rtol=1e-13, atol=1e-13), k
    for k in ("fp1", "fp2", "fin", "fout", "fbc", "c2f", "v2c"):
        assert np.array_equal(m[k], a[k]), k


def test_mesh_vjp_is_the_transpose_of_the_geometric_preprocessing(cc):
    """uns_host_cc_mesh_vjp against central differences of the host geometry
    (uns_host_cc_moved) in a random node direction, for random adjoints of
    every geometric array: <abar, dA/dX dX> = <Xbar, dX>."""
    a = cc.arrays
    rng = np.random.default_rng(3)
    sizes = abi.cc_geom_sizes(a)
    abar = {k: rng.standard_normal(n) for k, n in sizes.items()}
    gx, gy = cc.node_adjoint(abar)
    dpx, dpy = 1e-3 * rng.standard_normal(a["nop"]), 1e-3 * rng.standard_normal(a["nop"])
    rhs = np.dot(gx, dpx) + np.dot(gy, dpy)
    h = 1e-5
    mp = cc.moved(a["px"] + h * dpx, a["py"] + h * dpy).arrays
    mm = cc.moved(a["px"] - h * dpx, a["py"] - h * dpy).arrays
    terms = {k: np.dot(abar[k], (mp[k] - mm[k]) / (2 * h)) for k in sizes}
    lhs = sum(terms.values())
    assert abs(lhs - rhs) <= 1e-7 * abs(rhs), (lhs, rhs)
    # and array by array, against the scale of the whole product
    scale = sum(abs(t) for t in terms.values())
    for k in sizes:
        e = {kk: np.zeros(n) for kk, n in sizes.items()}
        e[k] = abar[k]
        x1, y1 = cc.node_adjoint(e)
        assert abs(terms[k] - (np.dot(x1, dpx) + np.dot(y1, dpy))) <= 1e-7 * scale, k


def test_mesh_vjp_rejects_a_mesh_whose_centroids_are_not_its_triangles(cc, tmp_path):
    """A geometry.inp keeps the file's cell centroids; one moved off its
    triangle's vertex mean makes the transposed geometry refuse the mesh."""
    path = tmp_path / "g.inp"
    cc.write(path)
    text = path.read_text().splitlines()
    nop, noc = (int(x) for x in text[0].split()[:2])
    row = nop + noc  # the last cell: an outer one, large enough to keep its face co-volumes positive
    parts = text[row].split()
    parts[1] = repr(float(parts[1]) + 1e-6)
    text[row] = " ".join(parts)
    path.write_text("\n".join(text) + "\n")
    m = mesh.CCMesh.read(path)
    with pytest.raises(abi.UnsError) as e:
        m.node_adjoint({k: np.zeros(n) for k, n in abi.cc_geom_sizes(m.arrays).items()})
    assert e.value.code == abi.UNS_ERR_MESH
    st, keep = abi.cc_mesh_adj(cc.arrays)
    gx, gy = np.zeros(cc.arrays["nop"]), np.zeros(cc.arrays["nop"])
    lib = abi.host_lib()
    assert lib.uns_host_cc_mesh_vjp(cc._h, None, gx.ctypes.data_as(abi._D), gy.ctypes.data_as(abi._D)) == abi.UNS_ERR_ARG


def test_moved_mesh_with_a_collapsed_cell_is_a_mesh_error(cc):
    a = cc.arrays
    px, py = a["px"].copy(), a["py"].copy()
    # put node 1 of the wall (the corner of triangles behind it) onto node 0
    px[1], py[1] = px[0], py[0]
    with pytest.raises(abi.UnsError) as e:
        cc.moved(px, py)
    assert e.value.code == abi.UNS_ERR_MESH


def test_mesh_vjp_accepts_the_plot3d_triangulation(tmp_path):
    path = tmp_path / "g.x"
    mesh.write_airfoil_plot3d(str(path), 24, 12)
    m = mesh.CCMesh.plot3d(str(path))
    rng = np.random.default_rng(5)
    abar = {k: rng.standard_normal(n) for k, n in abi.cc_geom_sizes(m.arrays).items()}
    gx, gy = m.node_adjoint(abar)
    assert np.isfinite(gx).all() and np.isfinite(gy).all()
