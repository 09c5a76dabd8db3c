"""Builds the reference's own single-scale step kernels as a checker.

Compiles SPH2S_FINAL_SINGLE_SCALE/Solver.cu, unmodified, from the reference
checkout into oracle/_ref/ss_solver.cubin (sm_103a).  The reference is a
Windows / CUDA 5.0 / OpenGL program; only its device code is wanted, and the
translation unit needs a few header shims, written here into
oracle/_ref/shims/:
  * Windows.h: empty;
  * cuda_gl_interop.h: GL handle typedefs and two stub registration calls;
  * "OpenGL\\OpenGL.h" and "thrust\\*.h": the reference includes these with
    Windows path separators; the shims forward to the real headers;
  * prelude.h (force-included): std::powf for libstdc++, and a forward
    declaration of CUDA::SafeCall that MSVC's permissive lookup did not need.
The cubin is loaded on the GPU by oracle/ref_harness.cu, which build_harness()
compiles on a machine with a GPU (the cubin travels; the checkout need not).
Nothing here is run unless the reference checkout is present (cubin) or the
cubin is (harness); outputs go only to oracle/_ref/.  write_input /
read_output / time_reference_kernels drive the harness.
TEST INFRASTRUCTURE ONLY.
"""
from __future__ import annotations

import ctypes as C
import os
import re
import shutil
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
SHIMS = OUT / "shims"
CUBIN = OUT / "ss_solver.cubin"
HARNESS = OUT / "ref_harness"
HARNESS_CU = HERE / "ref_harness.cu"
REFERENCE = Path(os.environ.get("SPH2S_REFERENCE", "/root/reference"))
SOLVER_CU = REFERENCE / "SPH2S_FINAL_SINGLE_SCALE" / "Solver.cu"

SHIM_FILES = {
    "Windows.h": "",
    "cuda_gl_interop.h": (
        "#pragma once\n#include <cuda_runtime.h>\n"
        "typedef unsigned int GLuint;\ntypedef unsigned int GLenum;\n"
        "inline cudaError_t cudaGraphicsGLRegisterBuffer(struct cudaGraphicsResource**, GLuint,"
        " unsigned int) { return cudaErrorNotSupported; }\n"
        "inline cudaError_t cudaGraphicsGLRegisterImage(struct cudaGraphicsResource**, GLuint,"
        " GLenum, unsigned int) { return cudaErrorNotSupported; }\n"),
    "OpenGL\\OpenGL.h": '#pragma once\n#include "cuda_gl_interop.h"\n',
    "thrust\\fill.h": "#include <thrust/fill.h>\n",
    "thrust\\sort.h": "#include <thrust/sort.h>\n",
    "thrust\\device_ptr.h": "#include <thrust/device_ptr.h>\n",
    "thrust\\for_each.h": "#include <thrust/for_each.h>\n",
    "thrust\\iterator\\zip_iterator.h": "#include <thrust/iterator/zip_iterator.h>\n",
    "prelude.h": (
        "#pragma once\n#include <cmath>\n#include <cuda_runtime.h>\n"
        "namespace std { using ::powf; }\n"
        "namespace CUDA { inline void SafeCall(cudaError_t err, const char* filename,"
        " unsigned int line); }\n"),
}


def available() -> bool:
    return SOLVER_CU.exists()


def build(force: bool = False) -> Path | None:
    """Compiles the cubin when the reference checkout is present."""
    if not available():
        return CUBIN if CUBIN.exists() else None
    if CUBIN.exists() and not force and CUBIN.stat().st_mtime > SOLVER_CU.stat().st_mtime:
        return CUBIN
    SHIMS.mkdir(parents=True, exist_ok=True)
    for name, text in SHIM_FILES.items():
        (SHIMS / name).write_text(text)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    tmp = CUBIN.with_suffix(".tmp")
    cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
           "-I", str(SHIMS), "-include", str(SHIMS / "prelude.h"), str(SOLVER_CU), "-o", str(tmp)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference kernels failed to build: {' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, CUBIN)
    return CUBIN


def build_harness() -> Path:
    """Compiles oracle/ref_harness.cu for sm_103a (needs nvcc and libcuda)."""
    if HARNESS.exists() and HARNESS.stat().st_mtime > HARNESS_CU.stat().st_mtime:
        return HARNESS
    OUT.mkdir(parents=True, exist_ok=True)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    tmp = HARNESS.with_suffix(".tmp")
    cmd = [nvcc, "-O2", "-gencode", "arch=compute_103a,code=sm_103a", str(HARNESS_CU),
           "-o", str(tmp), "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"ref_harness failed to build: {' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, HARNESS)
    return HARNESS


def write_input(path, config, x, v, boundary, steps: int, dt: float) -> None:
    """Harness input: magic, SolverConfiguration bytes, counts, dt, x, v, boundary."""
    x = np.ascontiguousarray(x, np.float32)
    b = np.ascontiguousarray(boundary, np.float32).reshape(-1, 3)
    with open(path, "wb") as f:
        f.write(b"SPHREF01")
        f.write(C.string_at(C.addressof(config), C.sizeof(config)))
        f.write(np.array([x.shape[0], b.shape[0], steps], np.uint32).tobytes())
        f.write(np.array([dt], np.float32).tobytes())
        f.write(x.tobytes())
        f.write(np.ascontiguousarray(v, np.float32).tobytes())
        f.write(b.tobytes())


def read_output(path) -> dict:
    raw = Path(path).read_bytes()
    assert raw[:8] == b"SPHOUT01"
    n, nc = np.frombuffer(raw[8:16], np.uint32)
    off = 16
    out = {}
    for name, dt, count in [("ids1", np.uint32, n), ("hash1", np.uint32, n),
                            ("cell_start1", np.uint32, nc), ("cell_end1", np.uint32, nc),
                            ("rho1", np.float32, n), ("p1", np.float32, n),
                            ("acc1", np.float32, 3 * n), ("x_end", np.float32, 3 * n),
                            ("v_end", np.float32, 3 * n), ("ids_end", np.uint32, n)]:
        nbytes = int(count) * 4
        out[name] = np.frombuffer(raw[off:off + nbytes], dt).copy()
        off += nbytes
    for k in ("acc1", "x_end", "v_end"):
        out[k] = out[k].reshape(-1, 3)
    return out


def run_harness(config, x, v, boundary, steps: int, dt: float, warmup: int | None = None):
    """Runs the reference kernels; returns (outputs, ms per timed step or None)."""
    if not CUBIN.exists():
        raise FileNotFoundError(f"{CUBIN} is missing (built where the reference checkout is)")
    exe = build_harness()
    with tempfile.TemporaryDirectory() as tmp:
        fin, fout = Path(tmp) / "in.bin", Path(tmp) / "out.bin"
        write_input(fin, config, x, v, boundary, steps, dt)
        cmd = [str(exe), str(CUBIN), str(fin), str(fout)]
        if warmup is not None:
            cmd += ["--time", str(int(warmup))]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"ref_harness failed ({r.returncode}): {r.stderr.strip()}")
        m = re.search(r"ref_harness_ms_per_step\s+([0-9.eE+-]+)", r.stdout)
        return read_output(fout), (float(m.group(1)) if m else None)


def time_reference_kernels(config, x, boundary, steps: int, dt: float, warmup: int) -> float:
    """ms per whole reference step (CUDA events), starting from rest."""
    _, ms = run_harness(config, x, np.zeros_like(x), boundary, steps, dt, warmup=max(1, warmup))
    return ms


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
