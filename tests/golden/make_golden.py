"""Generates tests/golden/ref_*.npz: outputs of the reference's own kernels.

The reference (segfault11/SPH2S_FINAL) ships no tests or fixtures and cannot
run as a program here (CUDA 5.0 / Windows / OpenGL).  Its single-scale device
code does compile for sm_103a (oracle/ref_build.py -> oracle/_ref/ss_solver.cubin);
oracle/ref_harness.cu replays the reference's host orchestration around those
kernels.  This script writes the inputs of two seeded scenes, runs the harness
on a GPU, and stores inputs and outputs:

  ref_block8_rest.npz     8^3 jittered block at s = 1/16, at rest, 20 steps, dt 1e-4
  ref_block16_moving.npz  16^3 jittered block at s = 1/64, v ~ N(0, 0.1^2), 20 steps, dt 1e-4

Usage (on a machine with a GPU, after oracle/ref_build.py built the cubin
where the reference checkout is present):
  nvcc -O2 -gencode arch=compute_103a,code=sm_103a oracle/ref_harness.cu \
       -o oracle/_ref/ref_harness -lcuda
  python tests/golden/make_golden.py --out tests/golden
"""
from __future__ import annotations

import argparse
import ctypes as C
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from sph2s_final_gb300 import scenes  # noqa: E402

HARNESS = ROOT / "oracle" / "_ref" / "ref_harness"
CUBIN = ROOT / "oracle" / "_ref" / "ss_solver.cubin"
STEPS = 20


def cases():
    a = scenes.small_scene(8, seed=0)
    yield "ref_block8_rest", a, np.zeros_like(a.fluid.positions)
    b, _ = scenes.differentiable_scene((16, 16, 16))
    v = np.random.default_rng(3).normal(0.0, 0.1, b.fluid.positions.shape).astype(np.float32)
    yield "ref_block16_moving", b, v


def write_input(path, sc, v, steps, dt):
    x = np.ascontiguousarray(sc.fluid.positions, np.float32)
    b = np.ascontiguousarray(sc.boundary.positions, np.float32)
    with open(path, "wb") as f:
        f.write(b"SPHREF01")
        f.write(C.string_at(C.addressof(sc.config), C.sizeof(sc.config)))
        f.write(np.array([x.shape[0], b.shape[0], steps], np.uint32).tobytes())
        f.write(np.array([dt], np.float32).tobytes())
        f.write(x.tobytes())
        f.write(np.ascontiguousarray(v, np.float32).tobytes())
        f.write(b.tobytes())


def read_output(path):
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
    out["acc1"] = out["acc1"].reshape(-1, 3)
    out["x_end"] = out["x_end"].reshape(-1, 3)
    out["v_end"] = out["v_end"].reshape(-1, 3)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(Path(__file__).resolve().parent))
    args = ap.parse_args()
    out_dir = Path(args.out)
    out_dir.mkdir(parents=True, exist_ok=True)
    if not HARNESS.exists() or not CUBIN.exists():
        raise SystemExit("build oracle/_ref/ss_solver.cubin and oracle/_ref/ref_harness first")
    with tempfile.TemporaryDirectory() as tmp:
        for name, sc, v in cases():
            fin, fout = Path(tmp) / f"{name}.in", Path(tmp) / f"{name}.out"
            write_input(fin, sc, v, STEPS, sc.dt)
            subprocess.run([str(HARNESS), str(CUBIN), str(fin), str(fout)], check=True)
            res = read_output(fout)
            np.savez_compressed(out_dir / f"{name}.npz", x0=sc.fluid.positions, v0=v,
                                steps=STEPS, dt=np.float32(sc.dt), spacing=np.float32(sc.spacing),
                                **res)
            print(name, sc.fluid.num_particles, "->", out_dir / f"{name}.npz")


if __name__ == "__main__":
    main()
