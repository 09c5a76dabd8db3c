"""Batched scenes (sphb_*): every scene of a batch must evolve exactly as the
single-scale solver evolves it alone (same keys, order and device code), so
the comparison with per-scene solvers is bit-exact; the per-scene solver is
itself checked against the FP64 oracle in test_gpu_single_scale.py."""
import numpy as np
import pytest

from sph2s_final_gb300 import scenes
from sph2s_final_gb300.batched import Batch
from sph2s_final_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def small_batch(num=6, seed=7):
    return scenes.batched_scenes(num=num, seed=seed, n_min=512, n_max=20000)


def per_scene(sc, steps, dt):
    with Solver(sc.fluid, sc.boundary, sc.config) as s:
        s.advance(dt, steps)
        return {"x": s.positions("sorted"), "v": s.velocities("sorted"),
                "rho": s.densities("sorted"), "xb": s.positions("by_id")}


def test_batch_equals_per_scene_solvers_bit_exact():
    scs = small_batch()
    dt, steps = scs[0].dt, 40
    with Batch([(s.fluid.positions, s.boundary.positions, s.config) for s in scs]) as b:
        b.advance(dt, steps)
        for k, sc in enumerate(scs):
            want = per_scene(sc, steps, dt)
            got = b.scene(k, "sorted")
            np.testing.assert_array_equal(got["x"], want["x"])
            np.testing.assert_array_equal(got["v"], want["v"])
            np.testing.assert_array_equal(got["rho"], want["rho"])
            np.testing.assert_array_equal(b.scene(k, "by_id")["x"], want["xb"])


def test_autotune_changes_launch_shape_not_results():
    scs = small_batch(num=5, seed=9)
    dt = scs[0].dt
    items = [(s.fluid.positions, s.boundary.positions, s.config) for s in scs]
    with Batch(items) as a, Batch(items) as b:
        choice = b.autotune(dt)
        assert choice["density_block"] in (128, 256, 512)
        a.advance(dt, 20)
        b.advance(dt, 20)
        for k in range(len(scs)):
            np.testing.assert_array_equal(a.scene(k)["x"], b.scene(k)["x"])


def test_full_256_scene_batch_steps_and_matches_per_scene():
    scs = scenes.batched_scenes()
    assert len(scs) == 256
    dt = scs[0].dt
    with Batch([(s.fluid.positions, s.boundary.positions, s.config) for s in scs]) as b:
        assert b.total_particles == sum(s.fluid.num_particles for s in scs)
        b.advance(dt, 5)
        b.sync()
        for k in (0, 17, 255):
            want = per_scene(scs[k], 5, dt)
            np.testing.assert_array_equal(b.scene(k)["x"], want["x"])
        x = b.scene(100)["x"]
        assert np.isfinite(x).all()


def test_coherent_batch_sort_equals_per_scene_solvers():
    """From 131,072 particles a batch sorts coherently (only the particles that
    changed cell are radix-sorted); the per-scene solvers of these small scenes
    sort from scratch.  60 steps must agree bit for bit."""
    scs = scenes.batched_scenes(num=8, seed=11, n_min=20000, n_max=40000)
    assert sum(s.fluid.num_particles for s in scs) >= 131072
    dt, steps = scs[0].dt, 60
    with Batch([(s.fluid.positions, s.boundary.positions, s.config) for s in scs]) as b:
        b.advance(dt, steps)
        for k, sc in enumerate(scs):
            want = per_scene(sc, steps, dt)
            got = b.scene(k, "sorted")
            np.testing.assert_array_equal(got["x"], want["x"])
            np.testing.assert_array_equal(got["v"], want["v"])
            np.testing.assert_array_equal(got["rho"], want["rho"])
