"""Seeded synthetic dam-break scenes (the workloads the solver is measured on).

A scene is a fluid lattice block in the unit box, jittered uniformly by
+-0.01 spacing per component, plus the hollow 5-layer boundary shell of the
box built like ParticleData::CreateParticleBoxCanvas.  Constants follow the
reference's single-scale driver (SPH2S_FINAL_SINGLE_SCALE/main.cpp:234-246:
rest density 1000, K 30, mu 5, c 88.1472, sigma 0.8), with the support h = 2s
and mass 1000 s^3 given directly instead of derived from a neighbour count.

  dam_break(1/64)            32^3 = 32,768 particles, 32^3 cells, dt 1e-4
  dam_break(1/256)           128^3 = 2,097,152 particles, 128^3 cells, dt 2.5e-5
  dam_break(1/64, (32,64,32)) 65,536 particles (64 lattice sites along y)
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .solver import Grid, ParticleData, SolverConfiguration

REST_DENSITY = 1000.0
BULK_MODULUS = 30.0
VISCOSITY = 5.0
SPEED_SOUND = 88.1472
TENSION = 0.8


@dataclass
class Scene:
    fluid: ParticleData
    boundary: ParticleData
    config: object
    dt: float
    spacing: float


def lattice_block(spacing: float, dims) -> np.ndarray:
    """Lattice origin + (i, j, k) * s for i < dims (CreateParticleBox on dims)."""
    g = Grid.make_grid_dims((0.0, 0.0, 0.0), dims, spacing)
    return ParticleData.create_particle_box(g).positions


def jitter(pos: np.ndarray, spacing: float, amount: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    j = rng.uniform(-amount * spacing, amount * spacing, size=pos.shape)
    return (pos.astype(np.float64) + j).astype(np.float32)


def dam_break(spacing: float, fluid_dims=None, seed: int = 0, jitter_amount: float = 0.01,
              h_over_s: float = 2.0, border: int = 5, dt: float | None = None,
              viscosity: float = VISCOSITY, bulk_modulus: float = BULK_MODULUS) -> Scene:
    s = float(np.float32(spacing))
    if fluid_dims is None:
        k = int(round(0.5 / s))
        fluid_dims = (k, k, k)
    fluid = jitter(lattice_block(s, fluid_dims), s, jitter_amount, seed)
    box = Grid.make_grid((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), s)
    boundary = ParticleData.create_particle_box_canvas(box, border)
    h = float(np.float32(h_over_s * s))
    grid = Grid.make_grid((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), h)
    mass = float(np.float32(REST_DENSITY * s ** 3))
    cfg = SolverConfiguration.direct(h, mass, REST_DENSITY, bulk_modulus, viscosity, SPEED_SOUND,
                                     TENSION, grid)
    if dt is None:
        dt = 1e-4 if s >= 1.0 / 64 else 2.5e-5
    return Scene(ParticleData(fluid), boundary, cfg, dt, s)


def small_scene(k: int = 8, seed: int = 0) -> Scene:
    """A k^3 block at spacing 1/(2k) in the unit box (fast parity cases)."""
    return dam_break(0.5 / k, (k, k, k), seed=seed, dt=1e-4)


@dataclass
class TwoScaleScene:
    low: ParticleData
    boundary: ParticleData
    config: object
    dt: float
    spacing: float


def two_scale_dam_break(spacing: float = 1 / 128, fluid_dims=None, seed: int = 0,
                        jitter_amount: float = 0.01, slab=(0.35, 0.65), axis: int = 0,
                        blend_increment: float = 0.0125, dt: float = 2.5e-5,
                        border: int = 5) -> TwoScaleScene:
    """Coarse dam break with a refinement slab: LOW support h = 2s, mass
    1000 s^3; HIGH support h/2, mass m/8; LOW grid spacing h, HIGH grid h/2
    over the unit box; slab lo < x[axis] < hi drives split and merge."""
    from .two_scale import SolverConfiguration2
    s = float(np.float32(spacing))
    if fluid_dims is None:
        k = int(round(0.5 / s))
        fluid_dims = (k, k, k)
    low = jitter(lattice_block(s, fluid_dims), s, jitter_amount, seed)
    box = Grid.make_grid((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), s)
    boundary = ParticleData.create_particle_box_canvas(box, border)
    h = float(np.float32(2.0 * s))
    g0 = Grid.make_grid((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), h)
    g1 = Grid.make_grid((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), float(np.float32(0.5) * np.float32(h)))
    mass = float(np.float32(REST_DENSITY * s ** 3))
    cfg = SolverConfiguration2.direct(h, mass, REST_DENSITY, BULK_MODULUS, VISCOSITY, SPEED_SOUND,
                                      TENSION, blend_increment, g0, g1, refine_axis=axis,
                                      refine_lo=slab[0], refine_hi=slab[1])
    return TwoScaleScene(ParticleData(low), boundary, cfg, dt, s)


def batched_scenes(num: int = 256, seed: int = 2, n_min: int = 4096, n_max: int = 131072,
                   dt: float = 5e-5):
    """Independent dam breaks with log-uniform particle counts in [n_min, n_max]:
    lattice side k = round(n^(1/3)) in [0, 0.5]^3 at s = 0.5/k, h = 2s, each in
    its own unit box and grid; viscosity and stiffness scaled per scene by
    U[0.5, 2].  One dt for all scenes (5e-5 keeps dt/s <= 6.4e-3, the ratio of
    the 32^3 and 128^3 single-scale cases, down to the finest scene)."""
    rng = np.random.default_rng(seed)
    n = np.exp(rng.uniform(np.log(n_min), np.log(n_max), num))
    mu_scale = rng.uniform(0.5, 2.0, num)
    k_scale = rng.uniform(0.5, 2.0, num)
    out = []
    for i in range(num):
        k = int(round(n[i] ** (1.0 / 3.0)))
        sc = dam_break(0.5 / k, (k, k, k), seed=seed * 100003 + i, dt=dt,
                       viscosity=VISCOSITY * float(mu_scale[i]),
                       bulk_modulus=BULK_MODULUS * float(k_scale[i]))
        out.append(sc)
    return out


def differentiable_scene(lattice=(32, 64, 32), spacing: float = 1 / 64, seed: int = 0):
    """The differentiable-rollout workload: a 32 x 64 x 32 lattice (64 along y)
    at s = 1/64 (65,536 particles), h = 2s, dt = 1e-4; target initial
    velocities N(0, 0.1^2) per component (seed 1)."""
    sc = dam_break(spacing, lattice, seed=seed, dt=1e-4)
    rng = np.random.default_rng(1)
    v_target = rng.normal(0.0, 0.1, (sc.fluid.num_particles, 3)).astype(np.float32)
    return sc, v_target
