"""The bench's bookkeeping (CPU): launch counts per iteration, the launches
of each profiled phase and the algorithmic bytes of every kernel for the
step each form runs."""
import importlib.util
from pathlib import Path

import pytest

from unsflow2d_gb300 import abi, mesh

ROOT = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def bench():
    spec = importlib.util.spec_from_file_location("bench_under_test", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_cc_launch_counts(bench):
    p = abi.make_params
    # mixed Green-Gauss RK3: reset, begin, vertex, cell_grad_side, face_conv, wall cells, cell_res, res_final
    assert bench.cc_launches(p(precision="mixed", grad="gg")) == 8
    # FP64 RK3: + face pass, stage-1 gather and the stage 2-3 pass
    assert bench.cc_launches(p(grad="gg")) == 10
    assert bench.cc_launches(p(grad="ggfc")) == 11
    assert bench.cc_launches(p(precision="mixed", grad="lsqr")) == 9
    assert bench.cc_launches(p(grad="gg", time="lusgs")) == 12


def test_phase_launches(bench):
    one_pass = bench.launches_per_iter("cc", True, False, False, sides=True)
    assert one_pass["face_conv"] == 1 and one_pass["cell_res"] == 1 and one_pass["cell_rk23"] == 1
    assert one_pass["face_prim_spec"] == 0
    viscous = bench.launches_per_iter("cc", True, True)
    assert viscous["face_conv"] == 3 and viscous["cell_rk23"] == 0
    assert bench.launches_per_iter("nc", False, False) == {"grad_lim": 1, "edge": 1, "node_res": 1}


def test_algorithmic_bytes_cover_each_form(bench):
    m = mesh.CCMesh.airfoil(32, 16).arrays
    fp64 = bench.algorithmic_bytes("cc", m)
    mixed = bench.algorithmic_bytes("cc", m, True)
    sides = bench.algorithmic_bytes("cc", m, True, sides=True)
    for d in (fp64, mixed, sides):
        assert all(v > 0 for v in d.values())
    assert "face_prim_spec" in fp64 and "face_prim_spec" not in sides
    assert {"cell_grad", "face_conv", "cell_res", "cell_rk23"} <= set(sides)
    # the mixed kernels read FP32 copies: fewer bytes than the FP64 ones
    assert sides["face_conv"] < fp64["face_conv"] and sides["cell_res"] < fp64["cell_res"]
    n = mesh.NCMesh.airfoil(32, 16).arrays
    nc = bench.algorithmic_bytes("nc", n)
    assert {"grad_lim", "edge", "node_res", "lusgs_sweeps"} <= set(nc)


def _reference_arm(env_extra=None):
    import json
    import os
    import subprocess
    import sys
    env = dict(os.environ, **(env_extra or {}))
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--mesh", "48x24", "--steps", "3",
                        "--warmup", "1"], capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.strip()]
    return [json.loads(ln) for ln in lines]


def test_reference_arm_prints_one_line_with_the_contract_keys(bench):
    (d,) = _reference_arm()
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC and d["unit"] == bench.UNIT
    assert d["higher_is_better"] is True and d["dtype"] == "f64" and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] == 1
    assert d["cpu_baseline"]["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["steps"] >= 1 and d["ms_per_step"] > 0 and "48x24" in d["config"]["workload"]


def test_reference_arm_runs_on_rank_0_only():
    assert _reference_arm({"RANK": "1", "WORLD_SIZE": "2", "LOCAL_RANK": "1"}) == []
