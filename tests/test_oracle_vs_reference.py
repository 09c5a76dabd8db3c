"""Pins the FP64 oracle to outputs of the reference's own kernels (CPU only).

tests/golden/ref_*.npz hold what SPH2S_FINAL_SINGLE_SCALE/Solver.cu's kernels,
compiled unmodified and driven through the reference's host sequence
(oracle/ref_harness.cu), produced on a GB300 for two seeded scenes; the
script that made them is tests/golden/make_golden.py.  Checked here:
  * the reference's hashes (Solver.cu:40-83) and its sorted order
    (thrust::sort_by_key, Solver.cu:1110-1115) equal the oracle's linear cell
    index and a stable sort of it, bit for bit; its cell ranges
    (Solver.cu:478-534) follow from them;
  * the reference's FP32 densities and accelerations of the first step agree
    with the oracle's FP64 ones to 1e-5 (measured ~3e-7);
  * positions after 20 steps agree to 1e-6 (measured ~2e-7).
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as O
from sph2s_final_gb300 import scenes

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = ["ref_block8_rest", "ref_block16_moving"]


def scene_for(name):
    if name == "ref_block8_rest":
        return scenes.small_scene(8, seed=0)
    return scenes.differentiable_scene((16, 16, 16))[0]


@pytest.fixture(params=CASES)
def case(request):
    z = np.load(GOLDEN / f"{request.param}.npz")
    sc = scene_for(request.param)
    np.testing.assert_array_equal(sc.fluid.positions, z["x0"])
    return sc, z


def test_reference_hashes_sorted_order_and_cell_ranges(case):
    sc, z = case
    g = sc.config.grid
    _, lin = O.cell_keys(g, z["x0"])
    perm = np.argsort(lin, kind="stable")
    np.testing.assert_array_equal(perm, z["ids1"])
    np.testing.assert_array_equal(lin[perm], z["hash1"])
    nc = g.dims[0] * g.dims[1] * g.dims[2]
    start = np.full(nc, 0xFFFFFFFF, np.uint64)
    end = np.full(nc, 0xFFFFFFFF, np.uint64)
    hs = lin[perm]
    first = np.r_[True, hs[1:] != hs[:-1]]
    last = np.r_[hs[1:] != hs[:-1], True]
    start[hs[first]] = np.nonzero(first)[0]
    end[hs[last]] = np.nonzero(last)[0] + 1
    np.testing.assert_array_equal(start.astype(np.uint32), z["cell_start1"])
    np.testing.assert_array_equal(end.astype(np.uint32), z["cell_end1"])


def test_reference_first_step_fields(case):
    sc, z = case
    f = O.ss_fields(sc.config, z["x0"], z["v0"], sc.boundary.positions)
    ids = z["ids1"]
    rho = f["rho"][ids]
    assert (np.abs(z["rho1"] - rho) / rho).max() <= 1e-5
    p = sc.config.bulk_modulus * (rho - sc.config.rest_density)
    assert np.abs(z["p1"] - p).max() <= 1e-5 * np.abs(rho).max() * sc.config.bulk_modulus
    acc = f["acc"][ids]
    assert np.abs(z["acc1"] - acc).max() / np.abs(acc).max() <= 1e-5


def test_reference_rollout_positions(case):
    sc, z = case
    ro = O.SSRollout(sc.config, z["x0"], sc.boundary.positions, z["v0"])
    ro.advance(float(z["dt"]), int(z["steps"]))
    st = ro.state()
    xo = np.empty_like(st["x"])
    xo[st["ids"]] = st["x"]
    xr = np.empty_like(z["x_end"], dtype=np.float64)
    xr[z["ids_end"]] = z["x_end"]
    assert np.abs(xo - xr).max() <= 1e-6
