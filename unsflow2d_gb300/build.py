"""In-tree build of the UNSFlow2D GB300 libraries.

    libunsflow_gpu.so   CUDA kernels + the drop-in C-ABI (include/unsflow_gpu.h),
                        sm_103a only, static CUDA runtime.
    libunsflow_host.so  caller side: geometry.inp / flo.inp, geometric
                        preprocessing, airfoil O-mesh generator, CFL schedules,
                        FLO.DAT I/O (include/unsflow_host.h); no GPU dependency.
    libunsflow_driver.so  the main programs (uns_host_*_main in unsflow_host.h)
                        on the two libraries above.
    libunsflow_gpu_fma.so the GPU library again with FP64 multiply-add
                        contraction: the same entry points, faster FP64
                        kernels, results within rounding of the bit-exact
                        build (chosen per process, UNSFLOW_FP64_FMA=1).

All three land in unsflow2d_gb300/lib/.  Translation units compile in parallel; host
code is built with -ffp-contract=off so x86 and Arm hosts round identically.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB = PKG / "lib"
OBJ = PKG / "_build"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# --fmad=false: no multiply-add contraction in device code, so the FP64 path
# performs the same IEEE operations, in the same order, as the reference
# expressions (and the CPU oracle, built with -ffp-contract=off).  Divisions
# and square roots are correctly rounded either way.
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I", str(INCLUDE), "-I", str(CSRC)]
# The contracted FP64 build: the compiler may fuse a multiply and an add into
# one FMA (one rounding instead of two).
NVCC_FMA_FLAGS = [f if f != "--fmad=false" else "--fmad=true" for f in NVCC_FLAGS]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
             "-I", str(INCLUDE), "-I", str(CSRC / "host")]

GPU_SOURCES = ["uns_api.cu", "uns_cc.cu", "uns_cc_adj.cu", "uns_cc_post.cu", "uns_nc.cu", "uns_noalloc.cu"]
HOST_SOURCES = ["host/host_mesh.cpp", "host/host_api.cpp", "host/host_shape.cpp"]
DRIVER_SOURCES = ["host/host_main.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _newer(target: Path, deps: list[Path]) -> bool:
    return target.exists() and all(target.stat().st_mtime >= d.stat().st_mtime for d in deps)


def _deps() -> list[Path]:
    return sorted(list(CSRC.rglob("*.cu")) + list(CSRC.rglob("*.cuh")) + list(CSRC.rglob("*.cpp")) +
                  list(CSRC.rglob("*.hpp")) + list(INCLUDE.glob("*.h")) + [Path(__file__)])


def build(force: bool = False, verbose: bool = False) -> dict[str, Path]:
    """Compile both libraries (incrementally unless force) and return their paths."""
    LIB.mkdir(exist_ok=True)
    OBJ.mkdir(exist_ok=True)
    gpu_so = LIB / "libunsflow_gpu.so"
    host_so = LIB / "libunsflow_host.so"
    driver_so = LIB / "libunsflow_driver.so"
    deps = _deps()
    fma_so = LIB / "libunsflow_gpu_fma.so"
    out = {"gpu": gpu_so, "host": host_so, "driver": driver_so, "gpu_fma": fma_so}
    (OBJ / "fma").mkdir(exist_ok=True)
    if not force and all(_newer(f, deps) for f in out.values()):
        return out
    nv = nvcc()
    jobs = []
    for src in GPU_SOURCES:
        o = OBJ / (Path(src).stem + ".o")
        jobs.append([nv, *ARCH, *NVCC_FLAGS, "-c", str(CSRC / src), "-o", str(o)])
    for src in GPU_SOURCES:
        o = OBJ / "fma" / (Path(src).stem + ".o")
        jobs.append([nv, *ARCH, *NVCC_FMA_FLAGS, "-c", str(CSRC / src), "-o", str(o)])
    for src in HOST_SOURCES + DRIVER_SOURCES:
        o = OBJ / (Path(src).stem + ".o")
        jobs.append(["g++", *CXX_FLAGS, "-c", str(CSRC / src), "-o", str(o)])
    with cf.ThreadPoolExecutor(max_workers=min(max(os.cpu_count() or 8, 8), len(jobs))) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    gpu_objs = [str(OBJ / (Path(s).stem + ".o")) for s in GPU_SOURCES]
    _run([nv, *ARCH, "-shared", "-Xcompiler", "-fPIC", *gpu_objs, "-o", str(gpu_so)])
    fma_objs = [str(OBJ / "fma" / (Path(s).stem + ".o")) for s in GPU_SOURCES]
    _run([nv, *ARCH, "-shared", "-Xcompiler", "-fPIC", *fma_objs, "-o", str(fma_so)])
    host_objs = [str(OBJ / (Path(s).stem + ".o")) for s in HOST_SOURCES]
    _run(["g++", "-shared", *host_objs, "-o", str(host_so)])
    drv_objs = [str(OBJ / (Path(s).stem + ".o")) for s in DRIVER_SOURCES]
    _run(["g++", "-shared", *drv_objs, "-L", str(LIB), "-lunsflow_host", "-lunsflow_gpu", "-Wl,-rpath,$ORIGIN",
          "-o", str(driver_so)])
    if verbose:
        print(f"built {gpu_so}, {host_so} and {driver_so}")
    return out


def ptxas_report() -> str:
    """Register / spill / shared-memory report of every kernel (-Xptxas -v)."""
    out = []
    for src in GPU_SOURCES:
        res = subprocess.run([nvcc(), *ARCH, *NVCC_FLAGS, "-Xptxas", "-v", "-c", str(CSRC / src),
                              "-o", os.devnull], capture_output=True, text=True)
        out.append(res.stderr)
    return "\n".join(out)


if __name__ == "__main__":
    if "--ptxas" in sys.argv:
        print(ptxas_report())
    else:
        build(force="--force" in sys.argv, verbose=True)
