"""Builds the reference's own step kernels as a checker, and drives them.

Compiles, unmodified, from a reference checkout named by the environment
variable SPH2S_REFERENCE (the directory holding SPH2S_FINAL_SINGLE_SCALE/ etc.):
  SPH2S_FINAL_SINGLE_SCALE/Solver.cu           -> oracle/_ref/ss_solver.cubin
  SPH2S_FINAL_TWO_SCALE/Solver.cu              -> oracle/_ref/ts_solver.cubin
  SPH2S_FINAL_TWO_SCALE_COUPLED/Solver.cu      -> oracle/_ref/cp_solver.cubin
for sm_103a.  The reference is a Windows / CUDA 5.0 / OpenGL program; only its
device code is wanted, and the translation units need a few header shims,
written here into oracle/_ref/shims/:
  * Windows.h: empty;
  * cuda_gl_interop.h: GL handle typedefs and two stub registration calls;
  * "OpenGL\\OpenGL.h" and "thrust\\*.h": the reference includes these with
    Windows path separators; the shims forward to the real headers;
  * prelude.h (force-included): std::powf for libstdc++, and a forward
    declaration of CUDA::SafeCall that MSVC's permissive lookup did not need.
The cubins are loaded on the GPU by oracle/ref_harness.cu (single scale) and
oracle/ref_harness_ts.cu (two scale, coupled), which build_harness() compiles on
a machine with a GPU (the cubins travel; the checkout need not).  Nothing here
runs unless SPH2S_REFERENCE is set (cubins) or the cubins exist (harnesses);
outputs go only to oracle/_ref/.

  SPH2S_REFERENCE=<checkout> python -m oracle.ref_build      builds the cubins

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
CUBIN_TS = OUT / "ts_solver.cubin"
CUBIN_CP = OUT / "cp_solver.cubin"
HARNESS = OUT / "ref_harness"
HARNESS_CU = HERE / "ref_harness.cu"
HARNESS_TS = OUT / "ref_harness_ts"
HARNESS_TS_CU = HERE / "ref_harness_ts.cu"
PROJECTS = {CUBIN: "SPH2S_FINAL_SINGLE_SCALE", CUBIN_TS: "SPH2S_FINAL_TWO_SCALE",
            CUBIN_CP: "SPH2S_FINAL_TWO_SCALE_COUPLED"}


def reference_root() -> Path | None:
    r = os.environ.get("SPH2S_REFERENCE")
    return Path(r) if r else None


def solver_cu(cubin: Path) -> Path | None:
    root = reference_root()
    return None if root is None else root / PROJECTS[cubin] / "Solver.cu"

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
    src = solver_cu(CUBIN)
    return src is not None and src.exists()


def build(force: bool = False) -> list[Path]:
    """Compiles the three cubins when a reference checkout is configured."""
    if not available():
        return [c for c in PROJECTS if c.exists()]
    SHIMS.mkdir(parents=True, exist_ok=True)
    for name, text in SHIM_FILES.items():
        (SHIMS / name).write_text(text)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    built = []
    for cubin in PROJECTS:
        src = solver_cu(cubin)
        if cubin.exists() and not force and cubin.stat().st_mtime > src.stat().st_mtime:
            built.append(cubin)
            continue
        tmp = cubin.with_suffix(".tmp")
        cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
               "-I", str(SHIMS), "-include", str(SHIMS / "prelude.h"), str(src), "-o", str(tmp)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"reference kernels failed to build: {' '.join(cmd)}\n{r.stderr}")
        os.replace(tmp, cubin)
        built.append(cubin)
    return built


def _build_exe(src: Path, exe: Path) -> Path:
    if exe.exists() and exe.stat().st_mtime > src.stat().st_mtime:
        return exe
    OUT.mkdir(parents=True, exist_ok=True)
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    tmp = exe.with_suffix(".tmp")
    cmd = [nvcc, "-O2", "-gencode", "arch=compute_103a,code=sm_103a", str(src), "-o", str(tmp),
           "-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"{src.name} failed to build: {' '.join(cmd)}\n{r.stderr}")
    os.replace(tmp, exe)
    return exe


def build_harness() -> Path:
    """Compiles oracle/ref_harness.cu for sm_103a (needs nvcc and libcuda)."""
    return _build_exe(HARNESS_CU, HARNESS)


def build_harness_ts() -> Path:
    """Compiles oracle/ref_harness_ts.cu for sm_103a (needs nvcc and libcuda)."""
    return _build_exe(HARNESS_TS_CU, HARNESS_TS)


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


# ---- two-scale and coupled projects (oracle/ref_harness_ts.cu) ----------------

MODE_BLENDED, MODE_COUPLED = 0, 1


def ts_config_bytes(cfg, mode: int) -> bytes:
    """SolverConfiguration of the two-scale project (TS Solver.h:52-61, 100 bytes)
    or of the coupled one (CP Solver.h:50-58, 96 bytes: no BlendIncrement),
    from an object with the sph_config2 field names."""
    f = [cfg.effective_radius[0], cfg.effective_radius[1], cfg.fluid_particle_mass[0],
         cfg.fluid_particle_mass[1], cfg.boundary_particle_mass, cfg.rest_density,
         cfg.bulk_modulus, cfg.viscosity, cfg.speed_sound, cfg.tension_coefficient]
    if mode == MODE_BLENDED:
        f.append(cfg.blend_increment)
    b = np.array(f, np.float32).tobytes()
    for g in (cfg.grid[0], cfg.grid[1]):
        b += np.array(list(g.origin), np.float32).tobytes()
        b += np.array(list(g.dims), np.int32).tobytes()
        b += np.array([g.spacing], np.float32).tobytes()
    return b


def write_input_ts(path, mode, cfg, pops, boundary, caps, steps: int, dt: float) -> None:
    """pops = [low, high], each a dict of x (n,3), v (n,3), lam (n), state (n)."""
    cb = ts_config_bytes(cfg, mode)
    b = np.ascontiguousarray(boundary, np.float32).reshape(-1, 3)
    n = [np.asarray(p["x"]).reshape(-1, 3).shape[0] for p in pops]
    with open(path, "wb") as f:
        f.write(b"SPHTSI01")
        f.write(np.array([mode, len(cb)], np.uint32).tobytes())
        f.write(cb)
        f.write(np.array([n[0], n[1], b.shape[0], caps[0], caps[1], steps], np.uint32).tobytes())
        f.write(np.array([dt], np.float32).tobytes())
        for p, k in zip(pops, n):
            f.write(np.ascontiguousarray(p["x"], np.float32).reshape(k, 3).tobytes())
            f.write(np.ascontiguousarray(p["v"], np.float32).reshape(k, 3).tobytes())
            f.write(np.ascontiguousarray(p["lam"], np.float32).reshape(k).tobytes())
            f.write(np.ascontiguousarray(p["state"], np.int32).reshape(k).tobytes())
        f.write(b.tobytes())


def read_output_ts(path) -> list[dict]:
    """Per recorded step: {"fields": [low, high], "post": [low, high],
    "high_survivors", "slot_overlap"}.  fields[r]: sorted order of the step's
    force pass (pid, hash, rho, p, acc, colour, state, lam); post[r]: the
    particles listed active after the step, in list order (pid, x, v, state,
    lam)."""
    raw = Path(path).read_bytes()
    assert raw[:8] == b"SPHTSO01"
    off = 8

    def take(dt, count):
        nonlocal off
        a = np.frombuffer(raw, dt, count=int(count), offset=off).copy()
        off += a.nbytes
        return a

    mode, rec = take(np.uint32, 2)
    steps = []
    for _ in range(int(rec)):
        fields = []
        for _r in range(2):
            n = int(take(np.uint32, 1)[0])
            fields.append({"pid": take(np.uint32, n), "hash": take(np.uint32, n),
                           "rho": take(np.float32, n), "p": take(np.float32, n),
                           "acc": take(np.float32, 3 * n).reshape(n, 3),
                           "colour": take(np.float32, n), "state": take(np.int32, n),
                           "lam": take(np.float32, n)})
        post = []
        for _r in range(2):
            count, slots = (int(v) for v in take(np.uint32, 2))
            active = take(np.uint32, count).astype(np.int64)
            x = take(np.float32, 3 * slots).reshape(slots, 3)
            v = take(np.float32, 3 * slots).reshape(slots, 3)
            st = take(np.int32, slots)
            lam = take(np.float32, slots)
            pid = take(np.uint32, slots)
            post.append({"pid": pid[active], "x": x[active], "v": v[active],
                         "state": st[active], "lam": lam[active]})
        hs, ov = (int(v) for v in take(np.uint32, 2))
        steps.append({"fields": fields, "post": post, "high_survivors": hs, "slot_overlap": ov})
    return steps


def run_harness_ts(mode, cfg, pops, boundary, caps, steps: int, dt: float,
                   warmup: int | None = None):
    """Runs the reference's two-scale (mode 0) or coupled (mode 1) kernels;
    returns (recorded steps, ms per timed step or None, end counts or None)."""
    cubin = CUBIN_TS if mode == MODE_BLENDED else CUBIN_CP
    if not cubin.exists():
        raise FileNotFoundError(f"{cubin} is missing (built where the reference checkout is)")
    exe = build_harness_ts()
    with tempfile.TemporaryDirectory() as tmp:
        fin, fout = Path(tmp) / "in.bin", Path(tmp) / "out.bin"
        write_input_ts(fin, mode, cfg, pops, boundary, caps, steps, dt)
        cmd = [str(exe), str(cubin), str(fin), str(fout)]
        if warmup is not None:
            cmd += ["--time", str(int(warmup))]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"ref_harness_ts failed ({r.returncode}): {r.stderr.strip()}")
        m = re.search(r"ref_harness_ms_per_step\s+([0-9.eE+-]+)", r.stdout)
        c = re.search(r"ref_harness_counts\s+(\d+)\s+(\d+)", r.stdout)
        return (read_output_ts(fout), float(m.group(1)) if m else None,
                (int(c.group(1)), int(c.group(2))) if c else None)


if __name__ == "__main__":
    if not available():
        sys.exit("set SPH2S_REFERENCE to the reference checkout")
    for c in build(force="--force" in sys.argv):
        print(c)
