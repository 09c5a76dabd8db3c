"""Host-side mirror of the reference's Solver / ParticleData surface.

Reference names, argument meaning and error behaviour are kept:

  Grid.make_grid / Grid.compute_num_grid_cells    SPH2S_FINAL_SINGLE_SCALE/Grid.h:11-46
  SolverConfiguration.make_configuration          SPH2S_FINAL_SINGLE_SCALE/Solver.h:15-48
  ParticleData.create_particle_box(_canvas), union SPH2S_FINAL_SINGLE_SCALE/ParticleData.cpp:68-209
  Solver(fluid, boundary, config).advance(dt)     SPH2S_FINAL_SINGLE_SCALE/Solver.h:113-121

ParticleData is headless: positions live in a float32 (N, 3) array instead of
an OpenGL VBO (the reference maps its VBOs into CUDA each step,
ParticleData.cpp:47-66).  Every computation runs in libsph2s.so through the C
ABI; errors raise SphError (the reference throws std::runtime_error).
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import _abi, state_io
from ._abi import check, fptr, lib, sph_config, sph_grid, uptr

ORDER = {"sorted": _abi.SPH_ORDER_SORTED, "by_id": _abi.SPH_ORDER_BY_ID}
INTEGRATORS = {"symplectic_euler": 0, "xsph": 1}


class Grid:
    """Grid::MakeGrid / ComputeNumGridCells / ComputeVolume."""

    @staticmethod
    def make_grid(origin, end, spacing: float) -> sph_grid:
        g = sph_grid()
        o = (C.c_float * 3)(*map(float, origin))
        e = (C.c_float * 3)(*map(float, end))
        check(lib().sph_make_grid(o, e, C.c_float(spacing), C.byref(g)))
        return g

    @staticmethod
    def make_grid_dims(origin, dims, spacing: float) -> sph_grid:
        """Grid::MakeGrid(origin, int3 dimensions, spacing), Grid.h:37-46."""
        g = sph_grid()
        g.origin[:] = [float(v) for v in origin]
        g.dims[:] = [int(v) for v in dims]
        g.spacing = float(np.float32(spacing))
        return g

    @staticmethod
    def compute_num_grid_cells(g: sph_grid) -> int:
        return int(lib().sph_grid_num_cells(C.byref(g)))

    @staticmethod
    def compute_volume(g: sph_grid) -> float:
        """Grid::ComputeVolume (Grid.h:48-54), FP32 like the reference."""
        s = np.float32(g.spacing)
        n = np.float32(g.dims[0] * g.dims[1] * g.dims[2])
        return float(np.float32(n * s * s * s))


class SolverConfiguration:
    @staticmethod
    def make_configuration(origin, end, volume, num_particles, avg_particles, rest_density,
                           bulk_modulus, viscosity, speed_sound, tension_coefficient,
                           epsilon) -> sph_config:
        c = sph_config()
        o = (C.c_float * 3)(*map(float, origin))
        e = (C.c_float * 3)(*map(float, end))
        check(lib().sph_make_configuration(o, e, volume, num_particles, avg_particles,
                                           rest_density, bulk_modulus, viscosity, speed_sound,
                                           tension_coefficient, epsilon, C.byref(c)))
        return c

    @staticmethod
    def direct(h, mass, rest_density, bulk_modulus, viscosity, speed_sound, tension_coefficient,
               grid: sph_grid, boundary_mass=None, epsilon=0.0) -> sph_config:
        """All constants explicit (h and m given directly rather than derived)."""
        c = sph_config()
        c.effective_radius = h
        c.fluid_particle_mass = mass
        c.boundary_particle_mass = mass if boundary_mass is None else boundary_mass
        c.rest_density = rest_density
        c.bulk_modulus = bulk_modulus
        c.viscosity = viscosity
        c.speed_sound = speed_sound
        c.tension_coefficient = tension_coefficient
        c.xsph_coeff = epsilon
        c.grid = grid
        return c


@dataclass
class ParticleData:
    """Headless ParticleData: float32 positions (N, 3)."""

    positions: np.ndarray

    @property
    def num_particles(self) -> int:
        return int(self.positions.shape[0])

    max_particles = num_particles

    @staticmethod
    def create_particle_box(g: sph_grid) -> "ParticleData":
        n = C.c_uint32()
        check(lib().sph_particle_box(C.byref(g), None, 0, C.byref(n)))
        out = np.empty((n.value, 3), np.float32)
        check(lib().sph_particle_box(C.byref(g), fptr(out), n.value, C.byref(n)))
        return ParticleData(out)

    @staticmethod
    def create_particle_box_canvas(g: sph_grid, border: int) -> "ParticleData":
        n = C.c_uint32()
        check(lib().sph_particle_box_canvas(C.byref(g), border, None, 0, C.byref(n)))
        out = np.empty((n.value, 3), np.float32)
        check(lib().sph_particle_box_canvas(C.byref(g), border, fptr(out), n.value, C.byref(n)))
        return ParticleData(out)

    @staticmethod
    def union(a: "ParticleData", b: "ParticleData") -> "ParticleData":
        """ParticleData::Union (ParticleData.cpp:68-127): concatenation."""
        if a is None or b is None:
            return None
        return ParticleData(np.concatenate([a.positions, b.positions]).astype(np.float32))


def _as_xyz(a, n: int, what: str) -> np.ndarray:
    arr = np.ascontiguousarray(a, dtype=np.float32).reshape(-1, 3)
    if arr.shape[0] != n:
        raise ValueError(f"{what}: expected {n} rows, got {arr.shape[0]}")
    return arr


class Solver:
    """Single-scale WCSPH solver on the GPU (Solver, SPH2S_FINAL_SINGLE_SCALE/Solver.h:62-132)."""

    def __init__(self, fluid: ParticleData, boundary: ParticleData | None, config: sph_config,
                 velocities=None):
        self.config = config
        fx = np.ascontiguousarray(fluid.positions, np.float32)
        bx = (np.ascontiguousarray(boundary.positions, np.float32) if boundary is not None
              else np.zeros((0, 3), np.float32))
        v = None if velocities is None else _as_xyz(velocities, fx.shape[0], "velocities")
        h = C.c_void_p()
        check(lib().sph_create(C.byref(config), fptr(fx), fx.shape[0], fptr(bx), bx.shape[0],
                               fptr(v), C.byref(h)))
        self._h = h
        self.num_fluid = fx.shape[0]
        self.num_boundary = bx.shape[0]

    def bind(self) -> None:
        """Solver::Bind: a no-op here; every handle carries its own configuration."""

    def advance(self, dt: float, steps: int = 1) -> None:
        check(lib().sph_advance(self._h, C.c_float(dt), int(steps)))

    def sync(self) -> None:
        check(lib().sph_sync(self._h))

    def positions(self, order: str = "sorted") -> np.ndarray:
        out = np.empty((self.num_fluid, 3), np.float32)
        check(lib().sph_get_positions(self._h, fptr(out), ORDER[order]))
        return out

    def velocities(self, order: str = "sorted") -> np.ndarray:
        out = np.empty((self.num_fluid, 3), np.float32)
        check(lib().sph_get_velocities(self._h, fptr(out), ORDER[order]))
        return out

    def densities(self, order: str = "sorted") -> np.ndarray:
        out = np.empty(self.num_fluid, np.float32)
        check(lib().sph_get_densities(self._h, fptr(out), ORDER[order]))
        return out

    def read_device(self, field: str, device_ptr: int, order: str = "sorted") -> None:
        """Enqueues a copy of "positions", "velocities" (3 floats per particle)
        or "densities" into caller-owned device memory at `device_ptr`, on the
        solver's stream (order later work after `stream` or call sync())."""
        fn = {"positions": lib().sph_get_positions_device,
              "velocities": lib().sph_get_velocities_device,
              "densities": lib().sph_get_densities_device}[field]
        check(fn(self._h, C.c_void_p(device_ptr), ORDER[order]))

    def ids(self) -> np.ndarray:
        out = np.empty(self.num_fluid, np.uint32)
        check(lib().sph_get_ids(self._h, uptr(out)))
        return out

    def set_velocities(self, v, order: str = "by_id") -> None:
        a = _as_xyz(v, self.num_fluid, "velocities")
        check(lib().sph_set_velocities(self._h, fptr(a), ORDER[order]))

    @property
    def stream(self) -> int:
        return lib().sph_stream(self._h) or 0

    def debug_step_fields(self) -> dict:
        """Structure and fields of the next step for the current state (no advance)."""
        n = self.num_fluid
        nc = Grid.compute_num_grid_cells(self.config.grid)
        r = {
            "keys": np.empty(n, np.uint32), "ids": np.empty(n, np.uint32),
            "cell_start": np.empty(nc, np.uint32), "cell_end": np.empty(nc, np.uint32),
            "nbr_fluid": np.empty(n, np.uint32), "nbr_boundary": np.empty(n, np.uint32),
            "rho": np.empty(n, np.float32), "acc": np.empty((n, 3), np.float32),
        }
        check(lib().sph_debug_step_fields(
            self._h, uptr(r["keys"]), uptr(r["ids"]), uptr(r["cell_start"]), uptr(r["cell_end"]),
            uptr(r["nbr_fluid"]), uptr(r["nbr_boundary"]), fptr(r["rho"]), fptr(r["acc"])))
        return r

    # ---- differentiable rollout ------------------------------------------
    def rollout_forward(self, v0, viscosity: float, dt: float, steps: int,
                        checkpoint_every: int = 20) -> None:
        v = None if v0 is None else _as_xyz(v0, self.num_fluid, "v0")
        check(lib().sph_rollout_forward(self._h, fptr(v), C.c_float(viscosity), C.c_float(dt),
                                        int(steps), int(checkpoint_every)))

    def rollout_density_loss(self, nodes: sph_grid, target=None):
        """Splat field on the node grid, and the loss against `target` if given."""
        nn = Grid.compute_num_grid_cells(nodes)
        field = np.empty(nn, np.float32)
        t = None if target is None else np.ascontiguousarray(target, np.float32).reshape(-1)
        loss = C.c_double(0.0)
        check(lib().sph_rollout_density_loss(self._h, C.byref(nodes), fptr(t), fptr(field),
                                             C.byref(loss)))
        return field, (loss.value if t is not None else None)

    def rollout_backward(self):
        gv = np.empty((self.num_fluid, 3), np.float32)
        gx = np.empty((self.num_fluid, 3), np.float32)
        gmu = C.c_double(0.0)
        check(lib().sph_rollout_backward(self._h, fptr(gv), fptr(gx), C.byref(gmu)))
        return gv, gx, gmu.value

    def profile_phases(self, dt: float, steps: int) -> dict:
        """Mean ms per step of (neighbourhood, density, force+integrate), CUDA events."""
        ms = np.zeros(3, np.float32)
        check(lib().sph_profile_phases(self._h, C.c_float(dt), int(steps), fptr(ms)))
        return {"neighborhood": float(ms[0]), "density": float(ms[1]), "force": float(ms[2])}

    def debug_force_lookback_timeout(self, on: bool) -> None:
        check(lib().sph_debug_force_lookback_timeout(self._h, 1 if on else 0))

    SORT_MODES = {"auto": 0, "full": 1, "coherent": 2}

    def debug_sort_mode(self, mode: str) -> None:
        """Test hook: how each step sorts ("auto", "full" = from scratch,
        "coherent" = only the particles that changed cell); same results."""
        check(lib().sph_debug_sort_mode(self._h, self.SORT_MODES[mode]))

    def positions_async(self, out: np.ndarray, order: str = "sorted") -> None:
        """Enqueues a readback of the positions into `out` (float32 (n, 3), best
        pinned); valid after sync().  The copy overlaps the next steps."""
        assert out.dtype == np.float32 and out.shape == (self.num_fluid, 3) and \
            out.flags.c_contiguous
        check(lib().sph_get_positions_async(self._h, fptr(out), ORDER[order]))

    def set_integrator(self, integrator: str) -> None:
        """"symplectic_euler" (integrateD, the default) or "xsph" (integrateXSPHD,
        Solver.cu:757-853, per-component correction, eps = config.xsph_coeff)."""
        check(lib().sph_set_integrator(self._h, INTEGRATORS[integrator]))

    # ---- headless state I/O (state_io.py describes the formats) ----
    @property
    def step_count(self) -> int:
        v = C.c_uint64()
        check(lib().sph_step_count(self._h, C.byref(v)))
        return v.value

    def save_state(self, path=None) -> bytes:
        """The complete state as bytes; also written atomically to `path` if given."""
        need = C.c_uint64()
        check(lib().sph_save_state(self._h, None, 0, C.byref(need)))
        buf = (C.c_ubyte * need.value)()
        check(lib().sph_save_state(self._h, buf, need.value, C.byref(need)))
        data = bytes(buf)
        if path is not None:
            state_io.write_bytes(path, data)
        return data

    @classmethod
    def from_state(cls, src) -> "Solver":
        """Resumes from bytes or a file written by save_state."""
        data = state_io.read_bytes(src)
        h = C.c_void_p()
        check(lib().sph_create_from_state(data, len(data), C.byref(h)))
        self = cls.__new__(cls)
        self._h = h
        self.config = sph_config.from_buffer_copy(data, 24)
        nf, nb = C.c_uint32(), C.c_uint32()
        check(lib().sph_counts(h, C.byref(nf), C.byref(nb)))
        self.num_fluid, self.num_boundary = nf.value, nb.value
        return self

    def write_frame(self, path, fields=state_io.FIELD_POSITIONS | state_io.FIELD_DENSITIES,
                    append: bool = True) -> None:
        check(lib().sph_write_frame(self._h, os.fsencode(path), int(fields), 1 if append else 0))

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().sph_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


def sort_passes_for(g: sph_grid) -> int:
    """8-bit digit passes the onesweep sort runs for this grid's Morton keys."""
    dmax = max(g.dims[0], g.dims[1], g.dims[2])
    b = 1
    while (1 << b) < dmax:
        b += 1
    return max(1, (3 * b + 7) // 8)
