"""Builds the CPU oracle, oracle/_build/liboracle.so (TEST INFRASTRUCTURE ONLY).

g++ with OpenMP over oracle/*.cpp, contraction of a*b+c into FMA disabled so
that the FP32 structural predicates (cell coordinates, r^2 < h^2 thresholds)
round exactly like the CUDA kernels' single-rounded intrinsics.  Called by
__graft_entry__.build(), tests/conftest.py and oracle.lib() on first use; the
product package never imports anything under oracle/.
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "_build" / "liboracle.so"


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_oracle(force: bool = False) -> Path:
    srcs = sorted(HERE.glob("*.cpp"))
    if not force and not _stale(ORACLE_LIB, srcs + sorted(HERE.glob("*.h")) + [Path(__file__)]):
        return ORACLE_LIB
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    cxx = os.environ.get("CXX", "g++")
    tmp = ORACLE_LIB.with_suffix(".so.tmp")
    cmd = [cxx, "-O2", "-std=c++17", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
           *map(str, srcs), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


if __name__ == "__main__":
    print(build_oracle(force="--force" in os.sys.argv))
