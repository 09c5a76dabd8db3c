"""The single-scale step computes the boundary force in its own pass, beside
the density pass, from the near-boundary particles the cell-range kernel lists
and each cell's static candidate list; the batched step still scans the
boundary stencil inside its force pass.  Both must give the same bits (the
candidate lists are a superset of every particle's boundary neighbours, in
the order of the full scan), so a one-scene batch, whose other kernels are
the single-scale ones, must stay identical to the solver -- also for fluid
particles outside the grid's box (clamped into edge cells, which walk the
stencil instead of the lists), a grid far from the origin, and a non-cubic
grid whose cells are larger than h."""
import numpy as np
import pytest

from sph2s_final_gb300.batched import Batch
from sph2s_final_gb300.solver import Grid, ParticleData, Solver, SolverConfiguration

pytestmark = pytest.mark.gpu


def solver_and_batch_agree(x, b, cfg, dt, steps):
    with Solver(ParticleData(x), ParticleData(b), cfg) as s, Batch([(x, b, cfg)]) as bt:
        for _ in range(3):
            s.advance(dt, steps)
            bt.advance(dt, steps)
            got = bt.scene(0, "sorted")
            np.testing.assert_array_equal(got["x"], s.positions("sorted"))
            np.testing.assert_array_equal(got["v"], s.velocities("sorted"))
        d = s.debug_step_fields()
        return int(d["nbr_boundary"].sum())


def test_boundary_pass_with_particles_outside_the_box():
    h = 1.0 / 16
    g = Grid.make_grid((0, 0, 0), (1, 1, 1), h)
    cfg = SolverConfiguration.direct(h, (h / 2) ** 3 * 1000, 1000.0, 30.0, 5.0, 88.1472, 0.8, g)
    shell = ParticleData.create_particle_box_canvas(Grid.make_grid((0, 0, 0), (1, 1, 1), h / 2), 5)
    rng = np.random.default_rng(15)
    inside = rng.uniform(0.0, 1.0, (3000, 3))
    outside = rng.uniform(0.0, 1.0, (600, 3))
    for k in range(600):  # through a face, an edge or a corner, up to 2 h deep
        for a in rng.choice(3, size=1 + k % 3, replace=False):
            dpt = rng.uniform(0.0, 2.0 * h)
            outside[k, a] = -dpt if rng.random() < 0.5 else 1.0 + dpt
    x = np.concatenate([inside, outside]).astype(np.float32)
    assert solver_and_batch_agree(x, shell.positions, cfg, 2e-4, 4) > 100


def test_boundary_pass_far_from_the_origin():
    h = 1.0 / 16
    o = (1000.0, 1000.0, 1000.0)
    g = Grid.make_grid(o, (1001.0, 1001.0, 1001.0), h)
    cfg = SolverConfiguration.direct(h, (h / 2) ** 3 * 1000, 1000.0, 30.0, 5.0, 88.1472, 0.8, g)
    shell = ParticleData.create_particle_box_canvas(Grid.make_grid(o, (1001.0, 1001.0, 1001.0), h / 2), 3)
    rng = np.random.default_rng(16)
    x = (np.float32(1000.0) + rng.uniform(0.0, 1.0, (3000, 3))).astype(np.float32)
    assert solver_and_batch_agree(x, shell.positions, cfg, 2e-4, 4) > 100


def test_boundary_pass_non_cubic_grid_with_an_inner_wall():
    """Cells of 0.0203 for h = 0.015 (stencils of two or three cells per axis)
    and a second boundary box standing inside the grid."""
    g = Grid.make_grid((-0.1, -0.1, -0.2), (1.7, 1.6, 0.6), 0.0203)
    cfg = SolverConfiguration.direct(0.015, 0.0075 ** 3 * 1000, 1000.0, 30.0, 5.0, 88.1472, 0.8, g)
    fluid = ParticleData.create_particle_box(Grid.make_grid((0.04, 0.04, 0.0), (0.35, 0.45, 0.3), 0.0075))
    outer = ParticleData.create_particle_box_canvas(Grid.make_grid((0.0, 0.0, -0.1), (1.6, 1.5, 0.5), 0.015), 2)
    inner = ParticleData.create_particle_box_canvas(Grid.make_grid((0.36, 0.0, 0.0), (0.42, 0.3, 0.3), 0.015), 2)
    b = np.concatenate([outer.positions, inner.positions]).astype(np.float32)
    assert solver_and_batch_agree(fluid.positions, b, cfg, 1e-4, 10) > 100
