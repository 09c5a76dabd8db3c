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
where the reference checkout is present; the harness is compiled on first use):
  python tests/golden/make_golden.py --out tests/golden
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import ref_build  # noqa: E402
from sph2s_final_gb300 import scenes  # noqa: E402

STEPS = 20


def cases():
    a = scenes.small_scene(8, seed=0)
    yield "ref_block8_rest", a, np.zeros_like(a.fluid.positions)
    b, _ = scenes.differentiable_scene((16, 16, 16))
    v = np.random.default_rng(3).normal(0.0, 0.1, b.fluid.positions.shape).astype(np.float32)
    yield "ref_block16_moving", b, v


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(Path(__file__).resolve().parent))
    args = ap.parse_args()
    out_dir = Path(args.out)
    out_dir.mkdir(parents=True, exist_ok=True)
    for name, sc, v in cases():
        res, _ = ref_build.run_harness(sc.config, sc.fluid.positions, v, sc.boundary.positions,
                                       STEPS, sc.dt)
        np.savez_compressed(out_dir / f"{name}.npz", x0=sc.fluid.positions, v0=v,
                            steps=STEPS, dt=np.float32(sc.dt), spacing=np.float32(sc.spacing),
                            **res)
        print(name, sc.fluid.num_particles, "->", out_dir / f"{name}.npz")


if __name__ == "__main__":
    main()
