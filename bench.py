#!/usr/bin/env python3
"""UNSFlow2D hot-path benchmark on GB300.

Workload (one "step" = one iteration of the solver main loop over the whole
mesh): NCFVM vertex-centred median-dual Euler on the analytic 12%-thick
4-digit airfoil, 1024x512 O-mesh split to 1,048,576 triangles (525,312 nodes),
Mach 0.8, alpha 1.25 deg, AUSM+-up flux, LSQ gradient + Barth limiter, LU-SGS
with CFL 50, FP64.  Metric: Mcell-iter/s (NCFVM counts nodes) -- whole-job
throughput, inputs resident in HBM.  `e2e` is the same metric through the
reference-facing per-routine C-ABI calls with the state copied host->device
and back every step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workload nc|cc|cc_mixed|nc_mixed]

Multi-GPU: N independent replicas (the LU-SGS sweep order is global, so the
path does not shard without changing results); value = all ranks' node
iterations / max rank time.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

from unsflow2d_gb300 import abi, mesh, replicas  # noqa: E402

METRIC = "Mcell-iter/s & time to 1e-8 residual drop: FP64 plain vs batched/mixed, 1 GB300"
UNIT = "Mcell-iter/s"

WORKLOADS = {
    "nc": dict(kind="nc", ni=1024, nj=512, dwall=1e-3,
               params=dict(m_inf=0.8, aoa_deg=1.25, flux="ausm", limiter="barth_corrected", time="lusgs", cfl_max=50.0,
                           min_res=0.0),
               desc="NCFVM median-dual Euler, 1024x512 O-mesh split to 1,048,576 triangles (525,312 nodes), "
                    "M0.8 a1.25, AUSM+-up, LSQ + Barth, LU-SGS CFL 50, FP64"),
    "nc_mixed": dict(kind="nc", ni=1024, nj=512, dwall=1e-3,
                     params=dict(m_inf=0.8, aoa_deg=1.25, flux="ausm", limiter="barth_corrected", time="lusgs", cfl_max=50.0,
                                 min_res=0.0, precision="mixed"),
                     desc="as nc with FP32 face reconstruction + flux, FP64 accumulation"),
    "nc_mixed_sweep": dict(kind="nc", ni=1024, nj=512, dwall=1e-3,
                           params=dict(m_inf=0.8, aoa_deg=1.25, flux="ausm", limiter="barth_corrected", time="lusgs",
                                       cfl_max=50.0, min_res=0.0, precision="mixed_sweep"),
                           desc="as nc with FP32 delta-form arithmetic inside the LU-SGS sweeps only (FP64 residual)"),
    "cc_small": dict(kind="cc", ni=128, nj=64, dwall=1e-3,
                     params=dict(m_inf=0.5, aoa_deg=2.0, flux="roe", grad="gg", time="rk3", cfl_max=0.9, min_res=0.0),
                     desc="CCFVM Euler, 128x64 O-mesh split to 16,384 triangles, M0.5 a2, Roe, GG + VKN, RK3 CFL 0.9, "
                          "FP64 (the reference's CPU-sized case; CFL 1.0 leaves RK3 undefined there)"),
    "cc_batched": dict(kind="cc_batch", n=256, tri=(5000, 200000), seed=20261203, dwall=1e-3, packed=True,
                       params=dict(flux="roe", grad="gg", time="rk3", cfl_max=0.9, min_res=0.0, precision="mixed"),
                       desc="256 CCFVM Euler instances packed into one index space, one launch of each kernel per "
                            "iteration for all of them: airfoil O-meshes with log-uniform 5k-200k triangles, Mach "
                            "U[0.3,0.85], alpha U[-2,6] deg, Roe or Rusanov, RK3 CFL 0.9, FP32 flux / FP64 "
                            "accumulation (seeded)"),
    "cc_batched_graphs": dict(kind="cc_batch", n=256, tri=(5000, 200000), seed=20261203, dwall=1e-3,
                              params=dict(flux="roe", grad="gg", time="rk3", cfl_max=0.9, min_res=0.0,
                                          precision="mixed"),
                              desc="the cc_batched instances as separate handles, one CUDA graph whose parallel "
                                   "branches are their own iterations (uns_cc_batch_*)"),
    "cc": dict(kind="cc", ni=2048, nj=1024, dwall=1e-3,
               params=dict(m_inf=0.75, aoa_deg=2.0, flux="roe", grad="gg", time="rk3", cfl_max=0.9, min_res=0.0),
               desc="CCFVM Euler, 2048x1024 O-mesh split to 4,194,304 triangles, M0.75 a2, Roe, GG + VKN, RK3, FP64"),
    "cc_mixed": dict(kind="cc", ni=2048, nj=1024, dwall=1e-3,
                     params=dict(m_inf=0.75, aoa_deg=2.0, flux="roe", grad="gg", time="rk3", cfl_max=0.9,
                                 min_res=0.0, precision="mixed"),
                     desc="as cc with FP32 face reconstruction + flux, FP64 accumulation"),
    # explicit RK3 from freestream on this mesh breaks down after ~250 steps
    # (the forward laminar start-up), so its timed region stays short
    "cc_adjoint": dict(kind="cc", ni=512, nj=256, dwall=2e-5, adjoint=True, max_timed_steps=100,
                       params=dict(m_inf=0.5, aoa_deg=3.0, rey=5000.0, flow="laminar", iwall=0, flux="roe",
                                   grad="ggfc", time="rk3", cfl_max=0.9, min_res=0.0),
                       desc="CCFVM laminar Navier-Stokes, Re 5000, M0.5 a3, Pr 0.72, Sutherland, 512x256 O-mesh with "
                            "2e-5c first wall spacing split to 262,144 triangles, Roe, GG-FC + VKN, RK3, FP64; "
                            "plus the discrete adjoint's transposed iteration (d C_L / d alpha)"),
}

# Kernels launched per iteration (our own; memsets excluded).
# CCFVM inviscid RK3 in FP64: reset_minmax, begin, vertex_avg, face_prim_spec, cell_grad,
# face_conv, cell_res (stage 1), cell_rk23_wall + cell_rk23 (stages 2-3), res_final.
# Mixed GG form: reset_minmax, begin, vertex_avg, cell_grad_side, face_conv,
# cell_rk23_wall (wall cells, stages 1-3), cell_res_mixed, res_final.
LAUNCHES = {("nc", "lusgs"): 9, ("nc", "rk3"): 11, ("cc", "rk3"): 10, ("cc", "lusgs"): 12, ("cc", "rk3_mixed_gg"): 8}


def cc_launches(p) -> int:
    """Kernels one CCFVM iteration launches (enqueue_iteration)."""
    ggfc = p.grad_type == abi.GRAD["ggfc"]
    rk3 = p.time_mode == abi.TIME["rk3"]
    mixed = p.precision == abi.PREC["mixed"]
    if not rk3:
        return LAUNCHES[("cc", "lusgs")] + (1 if ggfc else 0)
    if p.flow_type != abi.FLOW["laminar"]:
        if mixed and p.grad_type == abi.GRAD["gg"]:
            return LAUNCHES[("cc", "rk3_mixed_gg")]
        return LAUNCHES[("cc", "rk3")] + (1 if ggfc else 0) - (1 if mixed else 0)
    # reset_minmax, begin, vertex_avg, face_prim_spec, [face_ggfc], cell_grad,
    # 3 x (face_conv, cell_mul, [face_ggfc, (reset_minmax, begin), cell_grad], face_visc, cell_res), res_final
    per_stage = 4 + (0 if ggfc else 2 + (2 if p.ilimit else 0))
    return 5 + (1 if ggfc else 0) + 3 * per_stage + 1


def adjoint_cost(solver, w: dict, cfl: float, prof: dict) -> dict:
    """Device time of one transposed iteration of the discrete adjoint against
    one forward iteration and one residual evaluation, at the current state
    and CFL of the run (the per-iteration cost does not depend on convergence)."""
    import torch
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    cl, cd = solver.adjoint_prepare(cfl)
    prep = time.perf_counter() - t0
    solver.adjoint_solve("cl", max_iter=50, tol=0.0)  # warm-up (graph capture path)
    t = {}
    for n in (50, 250):
        t0 = time.perf_counter()
        solver.adjoint_solve("cl", max_iter=n, tol=0.0)
        t[n] = time.perf_counter() - t0
    per = (t[250] - t[50]) / 200 * 1e3
    # dC_L / d(wall-node y) of all wall nodes and the 16 Hicks-Henne amplitudes:
    # one transposed iteration with the geometric linearisation at the adjoint
    # vector, then the transposed geometric preprocessing on the host
    # (unsflow2d_gb300.shape, method "transposed")
    from unsflow2d_gb300 import shape
    lq, lg = solver.adjoint_get()
    case = shape.ShapeCase(w["ni"], w["nj"], w["params"], (solver.get_state(), solver.get("qp"), solver.get("phi")), cfl,
                           mesh_kw=dict(dwall=w["dwall"]))
    t0 = time.perf_counter()
    bumps = case.bump_gradient("cl", lq, lg)
    shape_s = time.perf_counter() - t0
    fwd = sum(prof.values())
    stage = sum(prof.get(k, 0.0) for k in ("face_conv", "viscous", "cell_res", "cirs")) / 3.0
    once = sum(v for k, v in prof.items() if k not in ("face_conv", "viscous", "cell_res", "cirs", "residue"))
    resid = once + stage
    return {"ms_per_transposed_iteration": round(per, 4), "ms_per_forward_iteration": round(fwd, 4),
            "ms_per_residual_evaluation": round(resid, 4),
            "ratio_to_forward_iteration": round(per / fwd, 3), "ratio_to_residual_evaluation": round(per / resid, 3),
            "prepare_s": round(prep, 3), "objective": "C_L", "CL": cl, "CD": cd,
            "shape_gradient_s": round(shape_s, 2), "shape_method": "transposed", "n_bumps": int(len(bumps)),
            "wall_nodes": int(w["ni"]),
            "timing": "host clock around uns_cc_adjoint_solve graphs of 50 and 250 transposed iterations (difference); "
                      "forward phases from CUDA events; a residual evaluation = con2prim, averages, gradient once + "
                      "one stage of flux, viscous flux and gather"}


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------- bytes model
def algorithmic_bytes(kind: str, m: dict, mixed: bool = False, sides: bool = False) -> dict:
    """Unique bytes each kernel must move per launch: every array it touches
    counted once at its full size, no credit for reuse.
    mixed: the CCFVM mixed form's kernels, which read FP32 copies; sides: its
    inviscid Green-Gauss RK3 step (k_cell_grad_side, wall cells through all
    three stages, one residual pass with the stages in closed form)."""
    if kind == "nc":
        N, E = m["nop"], m["nof"]
        B = int((m["fbc"] != 0).sum())
        return {
            "save_old": 96 * N,
            "grad_lim": 192 * N + 56 * E,
            "edge": 144 * N + 80 * E + 80 * B,
            "node_res": 60 * N + 56 * E + 80 * B,
            # per taken edge record R (2 per interior edge): 12 B of indices,
            # normal 16, length 8, la 8, qold 32 and its primitives 32 read;
            # 96 B written; per node the primitives of qold: 32 read, 32 written
            "sweep_prep": 204 * 2 * E + 64 * N,
            # per node: two items (schedule 16, diag 8, qold 32), res 32,
            # records written 2 x 64, qc 32; per record: 96 B read plus the
            # neighbour's 64 B record polled
            "lusgs_sweeps": 304 * N + 160 * 2 * E,
            "residue": 16 * ((N + 255) // 256),
        }
    N, F, P = m["noc"], m["nfi"] + m["nbf"], m["nop"]
    G = m["nbf"]
    W = int((np.asarray(m["fbc"])[m["nfi"]:] == 1001).sum())  # wall faces
    if mixed and sides:
        nnz = len(m["v2c"])
        nside = 2 * m["nfi"] + m["nbf"]
        return {
            "begin": 32 * N + 32 * N + 16 * N + 32 * N + 32 * G,
            "vertex_avg": 4 * P + 8 * nnz + 16 * (N + G) + 16 * P,
            # offsets, 32-byte cell-side records, vertex values, FP32 primitives (own and across), cv;
            # la, dt, dt/cv written; pack (phi read, 64 B written)
            "cell_grad": 4 * N + 32 * nside + 16 * P + 16 * N + 8 * N + 24 * N + 16 * N + 64 * N,
            "face_conv": 8 * F + 32 * F + 64 * N + 32 * F + 72 * G,
            # face lists, FP64 fluxes, qc read+write, res written, dt/cv, wall bits
            "cell_res": 16 * N + 32 * F + 64 * N + 32 * N + 8 * N + N // 8,
            # wall cells, stages 1-3: per wall face its neighbours, geometry, the pack of its cell, ghost
            # writes, wall force and flux; its cell's face lists, stored fluxes, state and residual
            "cell_rk23": (300 + 148 + 80) * W,
            "residue": 8 * ((N + 255) // 256),
        }
    if mixed:
        nnz = len(m["v2c"])
        return {
            # qc read; qold, qpf, qp written; ghost qp read for the limiter range
            "begin": 32 * N + 32 * N + 16 * N + 32 * N + 32 * G,
            # offsets, (cell, FP32 weight) per entry, FP32 primitives, FP32 vertex values
            "vertex_avg": 4 * P + 8 * nnz + 16 * (N + G) + 16 * P,
            # points, FP32 vertex values, FP32 normal+length; FP32 face values + radius, FP64 radius
            "face_prim_spec": 8 * F + 16 * P + 16 * F + 16 * F + 4 * F + 8 * F,
            # face lists, FP32 radii / normals / face values / offsets, neighbours, cv; la, dt, dt/cv, diag;
            # FP32 primitives; pack (phi read, 64 B written)
            "cell_grad": 4 * N + 8 * F + 4 * F + 16 * F + 16 * F + 16 * F + 8 * F + 8 * N + 32 * N + 16 * N + 16 * N + 64 * N,
            # neighbours, FP32 offsets + normal/length, two 64-byte packs (each cell once), FP64 flux written;
            # boundary: ghost writes and wall force
            "face_conv": 8 * F + 32 * F + 64 * N + 32 * F + 72 * G,
            # face lists, FP64 fluxes, qc read+write, qold, res, dt/cv
            "cell_res": 16 * N + 32 * F + 32 * N * 4 + 8 * N,
            # RK stages 2-3 in one pass: per cell the stored residual, qc read+write, qold, dt/cv and
            # its wall bit; per wall face its neighbours, geometry, the 64-byte pack of its cell, ghost
            # writes, wall force and flux, and its cell's face lists, stored fluxes and residual write
            "cell_rk23": 136 * N + N // 8 + (300 + 148) * W,
            "residue": 8 * ((N + 255) // 256),
        }
    return {
        "begin": 32 * N + 32 * N + 8 * N + 32 * N + 40 * G,
        "vertex_avg": 40 * (N + G) + 4 * P + 12 * len(m["v2c"]) + 40 * P,
        "face_prim_spec": 8 * F + 40 * P + 40 * F + 24 * F + 8 * F + 8 * F,
        "face_ggfc": 8 * F * 2 + 16 * P + 16 * (N + G) + 40 * P + 40 * (N + G) + 88 * F,
        "cell_grad": 4 * N + 12 * N + 8 * F + 40 * F + 24 * F + 16 * N + 64 * N + 32 * N + 40 * P + 16 * F + 32 * N * 2,
        "face_conv": 8 * F + 24 * F + 16 * F + 4 * G + 16 * (N + G) + 32 * (N + G) + 64 * N + 32 * N + 32 * F + 72 * G,
        "cell_res": 16 * N + 32 * F + 32 * N * 4 + 16 * N,
        "cell_rk23": 136 * N + N // 8 + (364 + 148) * W,
        "residue": 8 * ((N + 255) // 256),
    }


# DRAM traffic (dram__bytes_read.sum + dram__bytes_write.sum) per launch of
# the dominant kernels, per unit of the workload, from one ncu capture each
# (the NCFVM sweep's from the full-size launch list, the others from a
# quarter-size case, whose reads grow in proportion to the units; see the
# summaries under profiles/): scaled here to the benchmark's size.
TRAFFIC_PER_UNIT = {
    ("nc", "lusgs_sweeps", False): ((457.42e6 + 75.82e6) / 525312, "nodes", "profiles/nc_lusgs_1024x512_launches.md"),
    ("cc", "face_conv", False): (58.58e6 / 393728, "faces", "profiles/cc_fp64_512x256_full.md"),
    ("cc", "face_conv", True): (156.96e6 / 1573888, "faces", "profiles/cc_mixed_1024x512_full.md"),
    ("cc", "cell_res", True): (138.34e6 / 1048576, "cells", "profiles/cc_mixed_1024x512_full.md"),
    ("cc", "cell_grad", True): (261.72e6 / 1048576, "cells", "profiles/cc_mixed_1024x512_full.md"),
    ("cc", "cell_grad", False): (68.84e6 / 262144, "cells", "profiles/cc_fp64_512x256_full.md"),
}

# FP64-pipe utilisation (sm__pipe_fp64_cycles_active, fraction of peak while
# active) of the same kernels from the same captures: the second roofline
# fraction, the one that bounds the FP64 kernels.
FP64_PIPE = {
    ("nc", "lusgs_sweeps", False): (0.123, "profiles/nc_lusgs_512x256_full.md"),
    ("cc", "cell_grad", False): (0.845, "profiles/cc_fp64_512x256_full.md"),
    ("cc", "face_conv", False): (0.847, "profiles/cc_fp64_512x256_full.md"),
    ("cc", "cell_res", False): (0.799, "profiles/cc_fp64_512x256_full.md"),
    ("cc", "cell_grad", True): (0.198, "profiles/cc_mixed_1024x512_full.md"),
    ("cc", "face_conv", True): (0.354, "profiles/cc_mixed_1024x512_full.md"),
    ("cc", "cell_res", True): (0.755, "profiles/cc_mixed_1024x512_full.md"),
}


# Latency floor of one LU-SGS sweep item on the critical path, in cycles of
# the dependent FP64 chain from a predecessor's published values to this
# item's (measured per-operation latencies, profiles/gb300_fp64_issue_microbench.md:
# add / mul 76, divide 605): the edge term u*nx + v*ny, rho*un, *u, + p*n,
# *ds, - F(qold), - omega*la*dq, *0.5 (8 mul/add after the first product
# pair, 9 in all), one add of the edge sum, -res - sum, the division by the
# diagonal, qold + dq, con2prim's division, and the two operations by which
# the pressure (u*u + v*v, then three more) trails u and v where the next
# item first needs it.
FP64_ADD, FP64_DIV = 76.0, 605.0
SWEEP_ITEM_FLOOR_CYCLES = 9 * FP64_ADD + FP64_ADD + FP64_ADD + FP64_DIV + FP64_ADD + FP64_DIV + 2 * FP64_ADD


def launches_per_iter(kind: str, rk3: bool, laminar: bool, irs: bool = False, sides: bool = False) -> dict:
    """How many launches of each profiled phase one iteration makes.  An
    inviscid CCFVM RK3 step without smoothing computes its face fluxes once
    (stage 1) and runs stages 2 and 3 as one pass over the cells (cell_rk23),
    recomputing only the wall faces' fluxes; the mixed Green-Gauss step
    (sides) has no face pass and runs its wall cells as the cell_rk23 phase."""
    n = 3 if rk3 else 1
    if kind == "nc":
        return {"grad_lim": n, "edge": n, "node_res": n}
    if rk3 and not laminar and not irs:
        return {"face_conv": 1, "cell_res": 1, "cell_rk23": 1, "viscous": 0, "cirs": 0,
                "face_prim_spec": 0 if sides else 1}
    return {"face_conv": n, "cell_res": n, "viscous": n if laminar else 0, "cirs": n, "cell_rk23": 0}


# ---------------------------------------------------------------- accuracy
def lift_drag(fx: float, fy: float, aoa_deg: float) -> tuple[float, float]:
    """C_L, C_D of the flux-based wall force (unit chord; rho, |V| = 1)."""
    a = math.radians(aoa_deg)
    return (fy * math.cos(a) - fx * math.sin(a)) / 0.5, (fx * math.cos(a) + fy * math.sin(a)) / 0.5


def accuracy_vs_fp64(w: dict, m, solver, hist: np.ndarray) -> dict:
    """A mixed-form run against FP64 over the same iterations from freestream:
    the L2 residual norm histories, the final states and (CC) C_L / C_D."""
    from unsflow2d_gb300.solver import CCSolver, NCSolver
    kind = w["kind"]
    ref_params = {k: v for k, v in w["params"].items() if k != "precision"}
    p64 = abi.make_params(**ref_params)
    ref = (NCSolver if kind == "nc" else CCSolver)(m, p64)
    r = ref.iterate(cfl_list(p64, kind, 1, len(hist)), first_iter=True)
    h64 = np.asarray(r if kind == "cc" else r[0])
    q32, q64 = solver.get_state(), ref.get_state()
    out = {"iterations": int(len(hist)),
           "residual_l2_final": {"mixed": float(hist[-1]), "fp64": float(h64[-1]),
                                 "rel_diff": float(abs(hist[-1] - h64[-1]) / h64[-1])},
           "residual_l2_max_log10_diff": float(np.max(np.abs(np.log10(hist) - np.log10(h64)))),
           "state_rel_l2_diff": float(np.linalg.norm(q32 - q64) / np.linalg.norm(q64))}
    if kind == "cc":
        c32 = lift_drag(*solver.forces(), w["params"]["aoa_deg"])
        c64 = lift_drag(*ref.forces(), w["params"]["aoa_deg"])
        out["CL"] = {"mixed": c32[0], "fp64": c64[0], "abs_diff": abs(c32[0] - c64[0])}
        out["CD"] = {"mixed": c32[1], "fp64": c64[1], "abs_diff": abs(c32[1] - c64[1])}
    ref.close()
    return out


# ---------------------------------------------------------------- convergence
# Time to a 1e-8 drop of the normalised residual, from freestream, on the
# 128x64 mesh of the workload's family (the scheme has no multigrid: the
# 1024x512 NCFVM case drops only ~3e-2 in 4000 LU-SGS iterations, so a 1e-8
# drop there is hours of iterations; 128x64 takes ~7000).  FP64, and the fast
# form that still converges: NCFVM FP32 sweeps with the FP64 residual,
# CCFVM FP32 fluxes until their rounding floor, then FP64.
CONVERGE_MESH = (128, 64)


def time_to_drop(w: dict, target: float = 1e-8) -> dict:
    from unsflow2d_gb300.solver import CCSolver, NCSolver, converge
    kind = w["kind"]
    Mesh = mesh.CCMesh if kind == "cc" else mesh.NCMesh
    m = Mesh.airfoil(*CONVERGE_MESH, 0.12, 20.0, w["dwall"])
    base = {k: v for k, v in w["params"].items() if k not in ("min_res", "precision")}
    forms = [("fp64", None)] + ([("mixed_sweep", None)] if kind == "nc" else [("mixed", 1e-4)])
    out = {"mesh": f"{CONVERGE_MESH[0]}x{CONVERGE_MESH[1]}", "target_drop": target,
           "units": int(m.arrays["nop"] if kind == "nc" else m.arrays["noc"])}
    S = NCSolver if kind == "nc" else CCSolver
    nunits = out["units"]

    def rho_l2(s) -> float:  # L2 of the density residual (component 1 of the conserved order E, rho, rho u, rho v)
        r = s.get("res")[:nunits, 1]
        return float(np.sqrt(np.mean(r * r)))

    for prec, switch in forms:
        p = abi.make_params(precision=prec, min_res=target, **base)
        s0 = S(m, p)  # the first iteration alone: the density residual the drop is measured from
        s0.iterate(mesh.cfl_schedule(p, 1, 1, kind), first_iter=True)
        rho1 = rho_l2(s0)
        s0.close()
        s = S(m, p)
        t0 = time.perf_counter()
        r = converge(s, target, 60000 if kind == "cc" else 20000, switch_drop=switch)
        dt = time.perf_counter() - t0
        h = r["history"]
        out[prec] = {"seconds": round(dt, 3), "iterations": int(r["iterations"]), "reached": bool(h[-1] <= target),
                     "final_drop": float(h[-1]), "density_drop": rho_l2(s) / rho1,
                     "fp64_from_iteration": r["switched_at"]}
        s.close()
    return out


def converge_history(w: dict, max_iter: int, target: float, every: int = 500) -> dict:
    """The workload's case from freestream until the density residual has
    dropped by `target` or `max_iter` iterations: every `every` iterations the
    normalised all-variable residual (FLO.RES), the density-only drop and the
    wall time.  For solves far longer than a benchmark step."""
    from unsflow2d_gb300.solver import CCSolver, NCSolver
    kind = w["kind"]
    m = build_mesh(w)
    units = units_of(w, m)
    p = abi.make_params(**dict(w["params"], min_res=0.0))
    S = NCSolver if kind == "nc" else CCSolver
    s = S(m, p)
    rho = lambda: float(np.sqrt(np.mean(s.get("res")[:units, 1] ** 2)))
    first = True
    prev_cfl = 0.0
    it, f1, rho1 = 0, None, None
    rows = []
    t0 = time.perf_counter()
    while it < max_iter:
        n = 1 if first else min(every, max_iter - it)
        c = mesh.cfl_schedule(p, it + 1, n, kind, prev_cfl)
        prev_cfl = float(c[-1])
        r = s.iterate(c, first_iter=first)
        f = np.asarray(r if kind == "cc" else r[0])
        if first:
            f1, rho1, first = f[0], rho(), False
        it += len(f)
        d = rho() / rho1
        rows.append({"iteration": it, "drop": float(f[-1] / f1), "density_drop": d,
                     "seconds": round(time.perf_counter() - t0, 2)})
        if d <= target or not np.isfinite(f[-1]):
            break
    return {"workload": w["desc"], "units": int(units), "target_density_drop": target, "iterations": it,
            "reached": bool(rows and rows[-1]["density_drop"] <= target), "history": rows}


# ---------------------------------------------------------------- clocks
class ClockSampler:
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except (FileNotFoundError, OSError):
            self.p = None
        return self

    def __exit__(self, *exc):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self) -> dict:
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.count(",") >= 8]
        try:
            os.unlink(self.f.name)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for k, n in enumerate(names):
                if "Active" in r[5 + k] and "Not" not in r[5 + k]:
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


# ---------------------------------------------------------------- runs
def timed_steps(args, s_per_step: float) -> int:
    """`--steps`, raised where needed so the timed region lasts at least
    args.min_timed_s (the clock sampler's 200 ms period needs a few samples
    inside it), but to no more than args.max_steps."""
    need = getattr(args, "min_timed_s", 0.0)
    if need <= 0 or s_per_step <= 0:
        return args.steps
    n = max(args.steps, int(math.ceil(need / s_per_step)))
    cap = getattr(args, "max_steps", 0)
    return min(n, max(cap, args.steps)) if cap else n


def build_mesh(w):
    cls = mesh.NCMesh if w["kind"] == "nc" else mesh.CCMesh
    return cls.airfoil(w["ni"], w["nj"], 0.12, 20.0, w["dwall"])


def units_of(w, m) -> int:
    return m["nop"] if w["kind"] == "nc" else m["noc"]


def cfl_list(p, kind, first, n):
    return mesh.cfl_schedule(p, first, n, kind)


def batch_instances(w: dict):
    """The seeded instance set of the batched workload: (ni, nj, params)."""
    rng = np.random.default_rng(w["seed"])
    out = []
    for _ in range(w["n"]):
        tri = math.exp(rng.uniform(math.log(w["tri"][0]), math.log(w["tri"][1])))
        nj = max(4, int(round(math.sqrt(tri / 4.0))))  # 2 * ni * nj triangles, ni = 2 nj
        kw = dict(w["params"])
        kw.update(m_inf=float(rng.uniform(0.3, 0.85)), aoa_deg=float(rng.uniform(-2.0, 6.0)),
                  flux="roe" if rng.uniform() < 0.5 else "rusanov")
        out.append((2 * nj, nj, kw))
    return out


def batch_convergence(w: dict, count: int, max_iter: int = 20000, target: float = 1e-8, smallest: bool = False) -> dict:
    """A seeded subset of the batched workload's instances (`count` of them:
    spread evenly over the seeded list, so over the size range, or the
    smallest) run to a `target` drop of the normalised residual or `max_iter`
    iterations, twice on one packed handle each: the mixed form with the
    precision ramp (FP32 fluxes until every running case has reached its FP32
    floor, then FP64) and plain FP64.  Per instance: the iteration of the
    drop, the density residual's drop, C_L and C_D of both runs and their
    difference."""
    from unsflow2d_gb300.solver import CCPacked
    inst = batch_instances(w)
    if smallest:
        sel = sorted(inst, key=lambda x: x[0] * x[1])[:count]
    else:
        step = max(1, len(inst) // max(count, 1))
        sel = [inst[k] for k in range(0, len(inst), step)][:count]
    meshes = [mesh.CCMesh.airfoil(ni, nj, 0.12, 20.0, w["dwall"]) for ni, nj, _ in sel]
    fbc = [np.asarray(m.arrays["fbc"])[m.arrays["nfi"]:] for m in meshes]
    cells = np.array([int(m.arrays["noc"]) for m in meshes])
    runs = {}
    for form in ("mixed", "fp64"):
        params = [abi.make_params(**dict(kw, precision=form, min_res=target)) for _, _, kw in sel]
        b = CCPacked(meshes, params)
        import torch
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = b.converge(params, target, max_iter, switch_drop=1e-4 if form == "mixed" else None)
        secs = time.perf_counter() - t0
        f = b.forces(fbc)
        iters = np.array([ra if ra is not None else r["iterations"] for ra in r["reached_at"]])
        runs[form] = dict(r=r, secs=secs, cl_cd=[lift_drag(f[i, 0], f[i, 1], sel[i][2]["aoa_deg"]) for i in range(len(sel))],
                          mcell=float((cells * iters).sum() / secs / 1e6))
        b.close()
    per = []
    for i, (ni, nj, kw) in enumerate(sel):
        a, f = runs["mixed"], runs["fp64"]
        per.append({"triangles": int(cells[i]), "mesh": f"{ni}x{nj}", "mach": round(kw["m_inf"], 4),
                    "alpha_deg": round(kw["aoa_deg"], 3), "flux": kw["flux"],
                    "mixed_reached_at": a["r"]["reached_at"][i], "fp64_reached_at": f["r"]["reached_at"][i],
                    "mixed_final_drop": float(a["r"]["history"][i][-1]),
                    "mixed_density_drop": float(a["r"]["density_l2_last"][i] / a["r"]["density_l2_first"][i]),
                    "CL_mixed": a["cl_cd"][i][0], "CL_fp64": f["cl_cd"][i][0],
                    "CD_mixed": a["cl_cd"][i][1], "CD_fp64": f["cl_cd"][i][1],
                    "dCL": abs(a["cl_cd"][i][0] - f["cl_cd"][i][0]), "dCD": abs(a["cl_cd"][i][1] - f["cl_cd"][i][1])})
    both = [q for q in per if q["mixed_reached_at"] is not None and q["fp64_reached_at"] is not None]
    return {"instances": len(sel), "of": len(inst), "selection": "smallest" if smallest else "spread over the list",
            "target_drop": target, "max_iterations": max_iter,
            "reached": {"mixed_ramp": sum(q["mixed_reached_at"] is not None for q in per),
                        "fp64": sum(q["fp64_reached_at"] is not None for q in per)},
            "fp64_from_iteration": runs["mixed"]["r"]["switched_at"],
            "seconds": {"mixed_ramp": round(runs["mixed"]["secs"], 2), "fp64": round(runs["fp64"]["secs"], 2)},
            "mcell_iter_per_s": {"mixed_ramp": round(runs["mixed"]["mcell"], 1), "fp64": round(runs["fp64"]["mcell"], 1)},
            "time_ratio_fp64_over_mixed_ramp": round(runs["fp64"]["secs"] / runs["mixed"]["secs"], 3),
            "max_dCL_where_both_reached": max((q["dCL"] for q in both), default=None),
            "max_dCD_where_both_reached": max((q["dCD"] for q in both), default=None),
            "per_instance": per}


def run_batched(args, w, dist, rank, local_rank) -> dict | None:
    import torch
    from unsflow2d_gb300.solver import CCBatch, CCSolver

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    t0 = time.time()
    inst = batch_instances(w)
    meshes = [mesh.CCMesh.airfoil(ni, nj, 0.12, 20.0, w["dwall"]) for ni, nj, _ in inst]
    params = [abi.make_params(**kw) for _, _, kw in inst]
    packed = w.get("packed", False)
    if packed:  # one index space: one launch of each kernel for all instances
        from unsflow2d_gb300.solver import CCPacked
        batch = CCPacked(meshes, params)
        n_inst = batch.n
    else:  # one graph whose parallel branches are the instances' own iterations
        solvers = [CCSolver(m, p) for m, p in zip(meshes, params)]
        batch = CCBatch(solvers)
        n_inst = len(solvers)
    setup_s = time.time() - t0
    cells = int(sum(m.arrays["noc"] for m in meshes))
    it = 0

    def step(n):
        nonlocal it
        cfl = np.stack([mesh.cfl_schedule(p, it + 1, n, "cc") for p in params])
        hist, done = batch.iterate(cfl, first_iter=(it == 0))
        it += n
        if (done != n).any() or not all(np.isfinite(h).all() for h in hist):
            raise RuntimeError("an instance stopped or diverged")

    step(1)
    blocks = batch.autotune() if packed and not args.no_autotune else None  # launch geometry picked on the packed mesh
    t_w = time.perf_counter()
    nw = max(args.warmup - 1, 2)
    step(nw)
    args.steps = timed_steps(args, (time.perf_counter() - t_w) / nw)
    stream = torch.cuda.ExternalStream(batch.stream(), device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    replicas.barrier(dist, local_rank)
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clk:
        t_w = time.perf_counter()
        e0.record(stream)
        step(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t_w
    replicas.barrier(dist, local_rank)
    ms = e0.elapsed_time(e1)
    tot, secs = replicas.reduce_timing(dist, cells * args.steps, ms / 1e3, device=str(dev))
    tot_w, secs_w = replicas.reduce_timing(dist, cells * args.steps, wall, device=str(dev))
    nbytes = 0
    for m in meshes:
        b = algorithmic_bytes("cc", m.arrays, True, sides=True)
        nl = launches_per_iter("cc", True, False, sides=True)
        nbytes += sum(v * max(nl.get(k, 1), 1) for k, v in b.items() if k not in ("face_ggfc", "residue"))
    achieved = nbytes / (ms / 1e3 / args.steps) / 1e9
    peak, peak_src = peaks()
    clocks = clk.summary()
    # the face kernel of all cases: CUDA events around its launches (the
    # phase profile of the packed handle, after the timed region)
    face = None
    if packed:
        prof = batch.profile(float(params[0].cfl_max), reps=3)
        fb = sum(algorithmic_bytes("cc", m.arrays, True, sides=True)["face_conv"] for m in meshes)
        if prof.get("face_conv", 0.0) > 0:
            gbs = fb / (prof["face_conv"] * 1e-3) / 1e9
            face = {"kernel": "k_face_conv<float> (all cases, one launch)", "ms_per_launch": round(prof["face_conv"], 4),
                    "alg_MB_per_launch": round(fb / 1e6, 2), "achieved": round(gbs, 1), "peak": peak,
                    "unit": "GB/s", "frac": round(gbs / peak, 4),
                    "phases_ms": {k: round(v, 4) for k, v in prof.items()}}
    if rank != 0:
        return None
    n = n_inst
    launches = (LAUNCHES[("cc", "rk3_mixed_gg")] if packed else LAUNCHES[("cc", "rk3_mixed_gg")] * n) * args.steps
    path = ("uns_cc_packed_iterate" if packed else "uns_cc_batch_iterate") + \
        ": CFL schedules in, residual histories out, one call for all steps"
    return {
        "metric": METRIC, "value": round(tot / secs / 1e6, 3), "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32-face/f64-accumulate",
        "data": f"synthetic: {n} seeded analytic-airfoil O-meshes, uniform freestream starts",
        "config": {"workload": w["desc"], "instances": n, "units": cells, "global_batch": cells, "seq_len": 1,
                   "parallelism": f"replicas x{args.gpus}", "l2": f"inputs larger than L2: {cells} cells",
                   "setup_s": round(setup_s, 2), "block_sizes": blocks},
        "e2e": {"value": round(tot_w / secs_w / 1e6, 3), "unit": UNIT, "h2d_bytes_per_step": 8 * n,
                "d2h_bytes_per_step": 8 * n + 4 * n // max(args.steps, 1),
                "path": path},
        "gpu_launches": launches,
        "clocks": clocks,
        "roofline": {"bound": "hbm", "kernel": "whole batch iteration (all kernels of all instances)",
                     "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                     "traffic": None, "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
                     "face_kernel": face},
        # configuration 4's stop rule (1e-8 drop or 20k iterations) on a seeded
        # subset, and the smallest instances run on to the 1e-8 drop
        **({"convergence": batch_convergence(w, args.batch_converge),
            "convergence_to_1e-8": batch_convergence(w, 4, max_iter=150000, smallest=True)}
           if packed and args.batch_converge > 0 else {}),
    }


def run_ours(args, w, dist, rank, local_rank) -> dict | None:
    import torch
    from unsflow2d_gb300.solver import CCSolver, NCSolver

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    t0 = time.time()
    m = build_mesh(w)
    p = abi.make_params(**w["params"])
    S = NCSolver if w["kind"] == "nc" else CCSolver
    solver = S(m, p)
    setup_s = time.time() - t0
    units = units_of(w, m)
    kind = w["kind"]
    it = 0
    hist: list[float] = []

    def iterate(n):
        nonlocal it
        c = cfl_list(p, kind, it + 1, n)
        r = solver.iterate(c, first_iter=(it == 0))
        it += n
        f = r if kind == "cc" else r[0]
        if len(f) != n or not np.isfinite(f).all():
            raise RuntimeError(f"solver stopped or diverged: {len(f)} of {n} iterations, last norm {f[-1:]}")
        hist.extend(np.asarray(f).tolist())
        return r

    # CCFVM: launch geometry picked by the autotuner on this mesh after the
    # first step, before the rest of the warm-up (which re-captures the step)
    iterate(1)
    blocks = solver.autotune() if kind == "cc" and not args.no_autotune else None
    t_w = time.perf_counter()
    nw = max(args.warmup - 1, 2)
    iterate(nw)
    args.steps = timed_steps(args, (time.perf_counter() - t_w) / nw)
    stream = torch.cuda.ExternalStream(solver.stream(), device=dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    replicas.barrier(dist, local_rank)
    torch.cuda.synchronize()
    with ClockSampler(local_rank) as clk:
        e0.record(stream)
        iterate(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
    replicas.barrier(dist, local_rank)
    ms = e0.elapsed_time(e1)
    tot_units, secs = replicas.reduce_timing(dist, units * args.steps, ms / 1e3, device=str(dev))
    value = tot_units / secs / 1e6

    # Mixed forms: the same iterations in FP64 from the same start, compared.
    accuracy = None
    if p.precision != abi.PREC["fp64"] and rank == 0 and not args.no_accuracy:
        accuracy = accuracy_vs_fp64(w, m, solver, np.array(hist))

    # End to end through the per-routine C-ABI (the calls a Fortran driver
    # makes), with the state in pinned host memory copied in and out each step.
    lib = abi.gpu_lib()
    n_e2e = 0 if args.no_e2e else max(3, min(args.steps, 20))
    # two pinned host states used in turn: step k reads one and writes the other
    host = [torch.empty((solver.nstate, 4), dtype=torch.float64, pin_memory=True) for _ in range(2)]
    host[0].copy_(torch.from_numpy(solver.get_state()))
    h = solver._h
    dp = lambda t: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_double))
    fres = C.c_double()
    fresi, iresi = C.c_double(), C.c_int()
    cfls = cfl_list(p, kind, it + 1, n_e2e)
    replicas.barrier(dist, local_rank)
    torch.cuda.synchronize()
    t_e0 = time.perf_counter()
    lusgs = p.time_mode == abi.TIME["lusgs"]
    for k in range(n_e2e):
        c = float(cfls[k])
        host_in, host_out = host[k % 2], host[(k + 1) % 2]
        if kind == "nc":
            calls = [lambda: lib.uns_nc_set_state(h, dp(host_in)), lambda: lib.uns_nc_save_old(h)]
            if lusgs:
                calls.append(lambda: lib.uns_nc_lusgs(h, c))
            else:
                for irk in (1, 2, 3):
                    calls += [lambda: lib.uns_nc_fvresidual(h, c), lambda irk=irk: lib.uns_nc_rk_stage(h, irk)]
            calls += [lambda: lib.uns_nc_residue(h, C.byref(fres), C.byref(fresi), C.byref(iresi)),
                      lambda: lib.uns_nc_get_state(h, dp(host_out))]
        else:
            calls = [lambda: lib.uns_cc_set_state(h, dp(host_in)), lambda: lib.uns_cc_con2prim(h),
                     lambda: lib.uns_cc_avg_c2v(h), lambda: lib.uns_cc_time_step(h, c, None),
                     lambda: lib.uns_cc_save_old(h), lambda: lib.uns_cc_gradient(h)]
            if lusgs:
                calls.append(lambda: lib.uns_cc_lusgs(h))
            else:
                for irk in (1, 2, 3):
                    calls += [lambda: lib.uns_cc_fvresidual(h), lambda irk=irk: lib.uns_cc_rk_stage(h, irk)]
            calls += [lambda: lib.uns_cc_residue(h, C.byref(fres)), lambda: lib.uns_cc_get_state(h, dp(host_out))]
        for call in calls:
            rc = call()
            if rc:
                raise abi.UnsError(rc, lib.uns_last_error().decode())
    e2e_s = max(time.perf_counter() - t_e0, 1e-9)
    tot_e2e, e2e_s = replicas.reduce_timing(dist, units * n_e2e, e2e_s, device=str(dev))
    state_bytes = solver.nstate * 32
    e2e = {"value": tot_e2e / e2e_s / 1e6, "unit": UNIT, "h2d_bytes_per_step": state_bytes,
           "d2h_bytes_per_step": state_bytes + (24 if kind == "nc" else 8), "steps": n_e2e,
           "path": "per-routine C-ABI calls (reference main-loop order), pinned host state in/out each step"}

    # Per-kernel device times (CUDA events on the library stream) -> roofline.
    prof = solver.profile(float(cfl_list(p, kind, it + 1, 1)[0]), reps=3)
    mixed_cc = kind == "cc" and p.precision == abi.PREC["mixed"]
    sides = (mixed_cc and p.grad_type == abi.GRAD["gg"] and p.flow_type != abi.FLOW["laminar"]
             and p.time_mode == abi.TIME["rk3"] and p.irs == 0)
    nbytes = algorithmic_bytes(kind, m.arrays, mixed_cc, sides)
    peak, peak_src = peaks()
    dom = max(prof, key=prof.get)
    nl = launches_per_iter(kind, p.time_mode == abi.TIME["rk3"], p.flow_type == abi.FLOW["laminar"], p.irs != 0,
                           sides)
    per_launch = {k: v / max(nl.get(k, 1), 1) for k, v in prof.items()}  # ms per launch
    rl_kernel = max((k for k in nbytes if k in prof and prof[k] > 0), key=lambda k: prof[k])
    achieved = nbytes[rl_kernel] / (per_launch[rl_kernel] * 1e-3) / 1e9
    kernels = {k: {"ms_per_iter": round(v, 5), "launches_per_iter": nl.get(k, 1),
                   "alg_MB_per_launch": round(nbytes.get(k, 0) / 1e6, 2),
                   "GBps": round(nbytes[k] / (per_launch[k] * 1e-3) / 1e9, 1) if k in nbytes and v > 0 else None}
               for k, v in prof.items()}
    tr = TRAFFIC_PER_UNIT.get((kind, rl_kernel, mixed_cc))
    traffic = None
    if tr is not None:
        nunits = m["nop"] if tr[1] == "nodes" else (m["nfi"] + m["nbf"] if tr[1] == "faces" else m["noc"])
        traffic = round(tr[0] * nunits)

    clocks = clk.summary()
    if rank != 0:
        return None
    ws_mb = nbytes_total = sum(nbytes.values()) / 1e6
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(secs * 1e3 / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "gpu_library": abi.gpu_library_name(),
        "dtype": ("f64" if p.precision == abi.PREC["fp64"] else
                  "f64-residual/f32-sweep" if p.precision == abi.PREC["mixed_sweep"] else "f32-face/f64-accumulate"),
        "data": "synthetic: seeded analytic-airfoil O-mesh, uniform freestream start",
        "config": {"workload": w["desc"], "units": units, "edges_or_faces": int(m["nof"] if kind == "nc" else m["nfi"] + m["nbf"]),
                   "global_batch": units, "seq_len": 1, "parallelism": f"replicas x{args.gpus}",
                   "l2": f"inputs larger than L2: ~{ws_mb:.0f} MB of per-iteration arrays vs 129 MB L2, no flush",
                   "setup_s": round(setup_s, 2), "block_sizes": blocks},
        "e2e": e2e,
        "gpu_launches": (cc_launches(p) if kind == "cc" else
                         LAUNCHES[(kind, "lusgs" if p.time_mode == abi.TIME["lusgs"] else "rk3")]
                         + (1 if (kind, p.time_mode, p.precision) == ("nc", abi.TIME["lusgs"], abi.PREC["fp64"]) else 0))
                        * args.steps,
        "clocks": clocks,
        "roofline": {"bound": "hbm", "kernel": rl_kernel, "achieved": round(achieved, 1), "peak": peak,
                     "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": traffic,
                     "traffic_source": (f"ncu dram bytes per {tr[1][:-1]} x {tr[1]} ({tr[2]})" if tr else None),
                     "duration_ms": round(per_launch[rl_kernel], 4),
                     "timing": "CUDA events on the library stream around each phase, 3 iterations after the timed region",
                     "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured" else "fallback",
                     "dominant_phase": dom,
                     "fp64_pipe_frac": FP64_PIPE.get((kind, rl_kernel, mixed_cc), (None, None))[0],
                     "fp64_pipe_source": FP64_PIPE.get((kind, rl_kernel, mixed_cc), (None, None))[1]},
        "kernels": kernels,
    }
    if kind == "nc" and rl_kernel == "lusgs_sweeps":
        # the sweep is bound by its critical path, not by bytes: its time per
        # critical-path item against the FP64 latency floor of one item
        lf, lb = solver.sweep_levels()
        mhz = clocks.get("sm_mhz") or 2070.0
        per_item = per_launch[rl_kernel] * 1e3 / (lf + lb)
        floor = SWEEP_ITEM_FLOOR_CYCLES / mhz
        out["roofline"]["latency_floor"] = {
            "critical_path_items": lf + lb, "levels_forward": lf, "levels_backward": lb,
            "us_per_item": round(per_item, 3), "floor_us_per_item": round(floor, 3),
            "frac": round(floor / per_item, 3),
            "basis": "dependent FP64 chain of one item (9 mul/add of the edge term, the sum, two divisions, "
                     "the update, the pressure's lag) at the measured add 76 / divide 605 cycles, at the sampled SM clock"}
    if not args.no_cpu_baseline and args.gpus == 1:
        out["cpu_baseline"], out["parity"] = cpu_baseline(w, m, p, budget_s=args.cpu_budget)
    if accuracy is not None:
        out["accuracy_vs_fp64"] = accuracy
    if w.get("adjoint"):
        out["adjoint"] = adjoint_cost(solver, w, float(cfl_list(p, kind, it + 1, 1)[0]), prof)
    if not args.no_converge:
        out["time_to_1e-8"] = time_to_drop(w)
    return out


def cpu_baseline(w, m, p, budget_s=15.0) -> tuple[dict, dict]:
    """The oracle (serial C++ restatement of the reference) on this host, one
    core; then the same iterations from freestream on a fresh GPU handle,
    compared with the oracle's (the parity object of the bench line)."""
    sys.path.insert(0, str(ROOT / "oracle"))
    from oracle import OracleCC, OracleNC
    from unsflow2d_gb300.solver import CCSolver, NCSolver
    kind = w["kind"]
    O = OracleNC if kind == "nc" else OracleCC
    o = O(m, p)
    c = cfl_list(p, kind, 1, 64)
    first = lambda r: r[0] if isinstance(r, tuple) else r
    t0 = time.perf_counter()
    fo = [first(o.iteration(c[0]))]
    t1 = time.perf_counter() - t0
    n = max(1, min(63, int(budget_s / max(t1, 1e-6))))
    t0 = time.perf_counter()
    for k in range(n):
        fo.append(first(o.iteration(c[1 + k])))
    dt = time.perf_counter() - t0
    units = units_of(w, m)
    base = {"value": round(units * n / dt / 1e6, 4), "unit": UNIT, "cores": 1, "kind": "port",
            "host_cores": os.cpu_count(),
            "sample": f"{n} iterations of the full {units}-unit mesh after 1 untimed ({dt:.1f} s, serial oracle)"}
    g = (NCSolver if kind == "nc" else CCSolver)(m, p)
    fg = np.asarray(first(g.iterate(c[:n + 1], first_iter=True)))
    fo = np.asarray(fo)
    qg, qo = g.get_state(), o.get_state()
    rg, ro = g.get("res"), o.get("res")
    nu = len(ro)
    scale = np.asarray(o.get("la"))[:nu, None] * np.abs(qo[:nu]).max(axis=0)[None, :4]
    parity = {"iterations": int(n + 1), "units": int(units), "from": "uniform freestream, fresh GPU handle",
              "max_rel_state_err": float(np.max(np.abs(qg - qo)) / np.max(np.abs(qo))),
              "max_res_err": float(np.max(np.abs(rg[:nu] - ro) / np.maximum(scale, 1e-300))),
              "fres_max_rel_diff": float(np.max(np.abs(fg - fo) / np.abs(fo))),
              "state_bit_identical": bool(np.array_equal(qg, qo)),
              "criterion": "state 1e-12 of its max magnitude; residual 1e-12 of the flux scale lambda_i*max|q|",
              "oracle": "serial C++ restatement of the reference (oracle/), same mesh and inputs"}
    parity["pass"] = bool(parity["max_rel_state_err"] <= 1e-12 and parity["max_res_err"] <= 1e-12
                          and parity["fres_max_rel_diff"] <= 1e-12)
    g.close()
    o.close()
    return base, parity


def run_reference(args, w) -> dict:
    """The reference's CPU path: the Fortran reference cannot be built here (no
    Fortran compiler), so its serial C++ restatement (the oracle port) runs on
    the host cores; it is serial like the reference, so one thread."""
    m = build_mesh(w)
    p = abi.make_params(**w["params"])
    sys.path.insert(0, str(ROOT / "oracle"))
    from oracle import OracleCC, OracleNC
    O = OracleNC if w["kind"] == "nc" else OracleCC
    o = O(m, p)
    kind = w["kind"]
    units = units_of(w, m)
    nw = min(args.warmup, 10)  # about 0.3 s per full-mesh iteration on a Grace core
    c = cfl_list(p, kind, 1, nw + 200)
    for k in range(nw):
        o.iteration(c[k])
    t0 = time.perf_counter()
    o.iteration(c[nw])
    t_one = time.perf_counter() - t0
    n = max(1, min(args.steps, int(args.cpu_budget * 4 / max(t_one, 1e-6)))) - 1
    t0 = time.perf_counter()
    for k in range(n):
        o.iteration(c[nw + 1 + k])
    dt = time.perf_counter() - t0 + t_one
    n += 1
    v = units * n / dt / 1e6
    sample = f"{n} full-mesh iterations ({dt:.1f} s) of the serial oracle port"
    return {"metric": METRIC, "value": round(v, 4), "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
            "steps": n, "warmup": nw, "ms_per_step": round(dt * 1e3 / n, 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": w["desc"], "units": units},
            "cpu_baseline": {"value": round(v, 4), "unit": UNIT, "cores": 1, "kind": "port", "sample": sample,
                             "host_cores": os.cpu_count()},
            "e2e": {"value": round(v, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# The other benchmark configurations, measured in the same default run after
# the headline (one GPU): key -> workload.  "3_fp64" is configuration 3's mesh
# in the plain FP64 form, the denominator of the mixed and batched speed-ups.
CONFIG_RUNS = [("1", "cc_small"), ("2_mixed_sweep", "nc_mixed_sweep"), ("2_mixed", "nc_mixed"), ("3_fp64", "cc"),
               ("3", "cc_mixed"), ("4", "cc_batched"), ("5", "cc_adjoint")]
SUMMARY_KEYS = ("value", "unit", "ms_per_step", "steps", "dtype", "gpu_launches", "clocks", "roofline",
                "accuracy_vs_fp64", "adjoint", "time_to_1e-8", "convergence", "convergence_to_1e-8")


def run_configs(args, dist, rank, local_rank) -> dict:
    """Configurations 1, 3, 4 and 5, configuration 2's mixed forms (FP32 sweeps;
    FP32 residual and sweeps) and configuration 3's mesh in plain FP64,
    each timed like the headline: CUDA events on the library stream around
    `--steps` graph-replayed iterations after the warm-up, clocks sampled
    during the timed region.  No end-to-end leg and no CPU baseline here."""
    import copy
    out = {}
    for key, name in CONFIG_RUNS:
        a = copy.copy(args)
        a.no_e2e, a.no_cpu_baseline = True, True
        w = dict(WORKLOADS[name])
        a.min_timed_s = 0.6
        a.max_steps = w.get("max_timed_steps", 0)
        a.no_converge = name != "cc_small"  # configuration 1 is the time-to-drop mesh itself
        print(f"bench: configuration {key} ({name})", file=sys.stderr, flush=True)
        try:
            r = (run_batched if w["kind"] == "cc_batch" else run_ours)(a, w, dist, rank, local_rank)
        except (abi.UnsError, RuntimeError) as e:  # recorded, the other configurations still run
            out[key] = {"workload": w["desc"], "error": str(e)}
            continue
        if r is None:
            continue
        d = {"workload": w["desc"], "units": r["config"]["units"]}
        d.update({k: r[k] for k in SUMMARY_KEYS if k in r})
        if "kernels" in r:
            d["kernels_ms_per_iter"] = {k: v["ms_per_iter"] for k, v in r["kernels"].items()}
        if r["config"].get("block_sizes"):
            d["block_sizes"] = r["config"]["block_sizes"]
        out[key] = d
    # the FP64 forms again with multiply-add contraction (the other build of
    # the GPU library, chosen per process): the cost of bit-exactness
    fma = {}
    for key, name in (("2", "nc"), ("3_fp64", "cc")):
        cmd = [sys.executable, str(ROOT / "bench.py"), "--workload", name, "--steps", str(args.steps), "--warmup",
               str(args.warmup), "--no-configs", "--no-cpu-baseline", "--no-e2e", "--no-converge", "--no-accuracy"]
        r = subprocess.run(cmd, capture_output=True, text=True, env=dict(os.environ, UNSFLOW_FP64_FMA="1"),
                           timeout=1200)
        try:
            d = json.loads(r.stdout.strip().splitlines()[-1])
            fma[key] = {"workload": d["config"]["workload"], "gpu_library": d.get("gpu_library"), "value": d["value"],
                        "ms_per_step": d["ms_per_step"], "clocks": d["clocks"],
                        "kernels_ms_per_iter": {k: v["ms_per_iter"] for k, v in d["kernels"].items()}}
            plain_v = out.get(key, {}).get("value") if key != "2" else None
            if plain_v:
                fma[key]["speedup_vs_bit_exact"] = round(d["value"] / plain_v, 3)
        except Exception:
            fma[key] = {"error": (r.stderr or "")[-400:]}
    out["fp64_fma"] = fma
    plain = out.get("3_fp64", {}).get("value")
    if plain:
        for key in ("3", "4"):
            if key in out:
                out[key]["speedup_vs_plain_fp64"] = round(out[key]["value"] / plain, 3)
                out[key]["plain_fp64_reference"] = "configuration 3's 2048x1024 mesh in the plain FP64 form (key 3_fp64)"
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="nc", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-budget", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg (profiling runs)")
    ap.add_argument("--mesh", default=None, help="override the O-mesh size, e.g. 512x256 (profiling runs)")
    ap.add_argument("--no-converge", action="store_true", help="skip the time-to-1e-8 leg")
    ap.add_argument("--no-accuracy", action="store_true",
                    help="skip the mixed forms' FP64 comparison run (profiling runs)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default block sizes (profiling runs: no tuning launches before the captured ones)")
    ap.add_argument("--converge-history", type=int, default=0,
                    help="instead of the benchmark: run the workload from freestream for up to this many iterations "
                         "or a --target density drop, printing its residual history")
    ap.add_argument("--target", type=float, default=1e-10, help="density drop that ends --converge-history")
    ap.add_argument("--batch-converge", type=int, default=8,
                    help="instances of the batched workload run to a 1e-8 drop (mixed ramp and FP64); 0 skips it")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the other configurations that the default one-GPU run measures after the headline")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    rank, world, local_rank = replicas.dist_env()
    w = dict(WORKLOADS[args.workload])
    if args.mesh:
        w["ni"], w["nj"] = (int(x) for x in args.mesh.lower().split("x"))
        w["desc"] += f" [mesh overridden to {args.mesh}]"
    if args.impl == "reference":
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args, w)))
        return 0
    if args.converge_history > 0:
        print(json.dumps(converge_history(w, args.converge_history, args.target)))
        return 0
    dist = replicas.init("nccl")
    out = (run_batched if w["kind"] == "cc_batch" else run_ours)(args, w, dist, rank, local_rank)
    if args.gpus == 1 and args.workload == "nc" and not args.mesh and not args.no_configs:
        configs = run_configs(args, dist, rank, local_rank)
        if out is not None:
            out["configs"] = configs
            fma2 = configs.get("fp64_fma", {}).get("2", {})
            if fma2.get("value"):
                fma2["speedup_vs_bit_exact"] = round(fma2["value"] / out["value"], 3)
    if out is not None:
        print(json.dumps(out))
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
