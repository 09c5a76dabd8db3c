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
The cubin is loaded on the GPU by oracle/ref_harness.cu.  Nothing here is run
unless the reference checkout is present; outputs go only to oracle/_ref/.
TEST INFRASTRUCTURE ONLY.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"
SHIMS = OUT / "shims"
CUBIN = OUT / "ss_solver.cubin"
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


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
