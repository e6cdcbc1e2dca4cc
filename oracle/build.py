"""TEST INFRASTRUCTURE ONLY -- builds the CPU oracle (oracle/_build/liboracle.so).

The oracle restates the reference Fortran hot path in C++ (oracle_cc.cpp,
oracle_nc.cpp).  The reference itself is Fortran 90 and this image has no
Fortran compiler, so there is no oracle/_ref build: parity is unpinned by the
reference (see oracle.h).  -ffp-contract=off keeps the rounding identical on
x86 and Arm hosts.
"""
from __future__ import annotations

import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
OUT = HERE / "_build" / "liboracle.so"
SOURCES = [HERE / "oracle_cc.cpp", HERE / "oracle_cc_cs.cpp", HERE / "oracle_nc.cpp"]
DEPS = SOURCES + [HERE / "oracle_cc_body.inc", HERE / "oracle.h", ROOT / "include" / "unsflow_types.h", Path(__file__)]


def build(force: bool = False) -> Path:
    if not force and OUT.exists() and all(OUT.stat().st_mtime >= d.stat().st_mtime for d in DEPS):
        return OUT
    OUT.parent.mkdir(exist_ok=True)
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-Wall",
           "-I", str(ROOT / "include"), "-I", str(HERE), *map(str, SOURCES), "-o", str(OUT)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed:\n{res.stderr}")
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
