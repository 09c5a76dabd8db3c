"""The seeded dam-break scenes, restated in numpy for the reference arm.

TEST INFRASTRUCTURE ONLY.  bench.py's reference arm builds its workload here,
so that it runs the oracle and the reference's own kernels without loading
anything of the product (libsph2s.so or the sph2s_final_gb300 package).
tests/test_scenes_ref.py checks every array and configuration field against
the product's scene builders byte for byte.

  make_grid        Grid::MakeGrid              SPH2S_FINAL_SINGLE_SCALE/Grid.h:16-35
  particle_box     CreateParticleBox           SPH2S_FINAL_SINGLE_SCALE/ParticleData.cpp:129-163
  particle_canvas  CreateParticleBoxCanvas     SPH2S_FINAL_SINGLE_SCALE/ParticleData.cpp:165-209

All lattice arithmetic is FP32 without contraction (origin + float(i) *
spacing), as in the reference's host code.  Constants: rest density 1000,
K 30, mu 5, c 88.1472, sigma 0.8 (SPH2S_FINAL_SINGLE_SCALE/main.cpp:234-246),
support h = 2s and mass 1000 s^3 given directly.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

REST_DENSITY = 1000.0
BULK_MODULUS = 30.0
VISCOSITY = 5.0
SPEED_SOUND = 88.1472
TENSION = 0.8


class OGrid(C.Structure):  # Grid (Grid.h:55-58); the oracle's OGrid
    _fields_ = [("origin", C.c_float * 3), ("dims", C.c_int32 * 3), ("spacing", C.c_float)]


class OConfig(C.Structure):  # SolverConfiguration (Solver.h:50-60) + XSPH epsilon; the oracle's OConfig
    _fields_ = [("effective_radius", C.c_float), ("fluid_particle_mass", C.c_float),
                ("boundary_particle_mass", C.c_float), ("rest_density", C.c_float),
                ("bulk_modulus", C.c_float), ("viscosity", C.c_float),
                ("speed_sound", C.c_float), ("tension_coefficient", C.c_float),
                ("xsph_coeff", C.c_float), ("grid", OGrid)]


@dataclass
class RefScene:
    fluid: np.ndarray
    boundary: np.ndarray
    config: OConfig
    dt: float
    spacing: float


def make_grid(origin, end, spacing: float) -> OGrid:
    g = OGrid()
    s = np.float32(spacing)
    for a in range(3):
        o, e = np.float32(origin[a]), np.float32(end[a])
        g.origin[a] = float(o)
        g.dims[a] = int(np.ceil(np.float32(np.float32(e - o) / s)))
    g.spacing = float(s)
    return g


def _coords(g: OGrid, lo, hi):
    """origin + float(i) * spacing for i in [lo[a], hi[a]), x fastest."""
    s = np.float32(g.spacing)
    axes = [np.float32(g.origin[a]) + np.arange(lo[a], hi[a]).astype(np.float32) * s
            for a in range(3)]
    z, y, x = np.meshgrid(axes[2], axes[1], axes[0], indexing="ij")
    return np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1).astype(np.float32)


def particle_box(g: OGrid) -> np.ndarray:
    return _coords(g, (0, 0, 0), tuple(g.dims))


def particle_canvas(g: OGrid, border: int) -> np.ndarray:
    d = tuple(g.dims)
    xyz = _coords(g, (-border,) * 3, tuple(v + border for v in d))
    i = np.arange(-border, d[0] + border)
    j = np.arange(-border, d[1] + border)
    k = np.arange(-border, d[2] + border)
    kk, jj, ii = np.meshgrid(k, j, i, indexing="ij")
    inside = ((ii >= 0) & (ii < d[0]) & (jj >= 0) & (jj < d[1]) & (kk >= 0) & (kk < d[2])).ravel()
    return np.ascontiguousarray(xyz[~inside])


def jitter(pos: np.ndarray, spacing: float, amount: float, seed: int) -> np.ndarray:
    rng = np.random.default_rng(seed)
    j = rng.uniform(-amount * spacing, amount * spacing, size=pos.shape)
    return (pos.astype(np.float64) + j).astype(np.float32)


def dam_break(spacing: float, fluid_dims=None, seed: int = 0, jitter_amount: float = 0.01,
              border: int = 5, dt: float | None = None) -> RefScene:
    """The jittered fluid block at the box corner and the 5-layer shell of [0,1]^3."""
    s = float(np.float32(spacing))
    if fluid_dims is None:
        k = int(round(0.5 / s))
        fluid_dims = (k, k, k)
    lat = OGrid()
    lat.dims[:] = [int(v) for v in fluid_dims]
    lat.spacing = s
    fluid = jitter(particle_box(lat), s, jitter_amount, seed)
    boundary = particle_canvas(make_grid((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), s), border)
    h = float(np.float32(2.0 * s))
    cfg = OConfig()
    cfg.effective_radius = h
    cfg.fluid_particle_mass = float(np.float32(REST_DENSITY * s ** 3))
    cfg.boundary_particle_mass = cfg.fluid_particle_mass
    cfg.rest_density = REST_DENSITY
    cfg.bulk_modulus = BULK_MODULUS
    cfg.viscosity = VISCOSITY
    cfg.speed_sound = SPEED_SOUND
    cfg.tension_coefficient = TENSION
    cfg.xsph_coeff = 0.0
    cfg.grid = make_grid((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), h)
    if dt is None:
        dt = 1e-4 if s >= 1.0 / 64 else 2.5e-5
    return RefScene(fluid, boundary, cfg, dt, s)
