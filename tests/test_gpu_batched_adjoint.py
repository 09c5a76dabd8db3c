"""Batched differentiable rollout (sphb_rollout_*): every scene's loss, splat
field and gradients (initial velocities, initial positions, viscosity) equal,
bit for bit, those of a single-scale solver rollout on that scene — whose
gradients are checked against finite differences and the FP64 oracle in
tests/test_gpu_adjoint.py."""
import numpy as np
import pytest

from sph2s_final_gb300 import scenes
from sph2s_final_gb300.autograd import node_grid
from sph2s_final_gb300.batched import Batch
from sph2s_final_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def make_case(num=5, steps=24, K=7, seed=11):
    scs = scenes.batched_scenes(num, seed=seed, n_min=512, n_max=6000, dt=1e-4)
    rng = np.random.default_rng(seed)
    v0 = [rng.normal(0, 0.1, (sc.fluid.num_particles, 3)).astype(np.float32) for sc in scs]
    mu = rng.uniform(1.0, 6.0, num).astype(np.float32)
    dims = [(16, 16, 16), (12, 12, 12), (16, 8, 16), (10, 10, 10), (16, 16, 16)]
    nodes = [node_grid(dims[k % len(dims)]) for k in range(num)]
    targets = [rng.uniform(0, 800, n.dims[0] * n.dims[1] * n.dims[2]).astype(np.float32)
               for n in nodes]
    return scs, v0, mu, nodes, targets, steps, K


def per_scene(sc, v0, mu, nodes, target, steps, K):
    with Solver(sc.fluid, sc.boundary, sc.config) as s:
        s.rollout_forward(v0, float(mu), sc.dt, steps, K)
        field, loss = s.rollout_density_loss(nodes, target)
        gv, gx, gm = s.rollout_backward()
    return field, loss, gv, gx, gm


def test_batched_rollout_equals_per_scene_rollouts():
    scs, v0, mu, nodes, targets, steps, K = make_case()
    dt = scs[0].dt
    with Batch([(sc.fluid.positions, sc.boundary.positions, sc.config) for sc in scs]) as b:
        b.rollout_forward(v0, mu, dt, steps, K)
        fields, losses = b.rollout_density_loss(nodes, targets)
        gv, gx, gm = b.rollout_backward()
        # a second backward after a fresh forward + loss gives the same answer
        b.rollout_forward(v0, mu, dt, steps, K)
        b.rollout_density_loss(nodes, targets)
        gv2, _, gm2 = b.rollout_backward()
    for k, sc in enumerate(scs):
        f, L, sv, sx, sm = per_scene(sc, v0[k], mu[k], nodes[k], targets[k], steps, K)
        np.testing.assert_array_equal(fields[k], f)
        assert losses[k] == L
        np.testing.assert_array_equal(gv[k], sv)
        np.testing.assert_array_equal(gx[k], sx)
        assert gm[k] == sm, (k, gm[k], sm)
        np.testing.assert_array_equal(gv2[k], sv)
        assert gm2[k] == sm
        assert np.abs(sv).max() > 0 and sm != 0.0


def test_batched_rollout_after_autotune_and_checkpoint_change():
    """Block-size choices of the autotuner and another checkpoint interval leave
    the per-scene gradients unchanged (same per-particle code, same tape)."""
    scs, v0, mu, nodes, targets, steps, _ = make_case(num=3, steps=15, seed=5)
    dt = scs[0].dt
    with Batch([(sc.fluid.positions, sc.boundary.positions, sc.config) for sc in scs]) as b:
        b.autotune(dt)
        b.rollout_forward(v0, mu, dt, steps, 4)
        b.rollout_density_loss(nodes, targets)
        gv, _, gm = b.rollout_backward()
    for k, sc in enumerate(scs):
        _, _, sv, _, sm = per_scene(sc, v0[k], mu[k], nodes[k], targets[k], steps, 15)
        np.testing.assert_array_equal(gv[k], sv)
        assert gm[k] == sm


def test_batched_backward_needs_forward_and_loss():
    scs, v0, mu, nodes, targets, steps, K = make_case(num=2, steps=4, K=2)
    from sph2s_final_gb300._abi import SphError
    with Batch([(sc.fluid.positions, sc.boundary.positions, sc.config) for sc in scs]) as b:
        with pytest.raises(SphError, match="SPH_E_INVALID"):
            b.rollout_backward()
        b.rollout_forward(v0, mu, scs[0].dt, steps, K)
        with pytest.raises(SphError, match="SPH_E_INVALID"):
            b.rollout_backward()
