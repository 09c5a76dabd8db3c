"""Host-side mirror of the reference's two-scale Solver.

  SolverConfiguration2.make_configuration   SPH2S_FINAL_TWO_SCALE/Solver.h:16-50
  Solver2(low, high, boundary, config)      SPH2S_FINAL_TWO_SCALE/Solver.h:121-130
  Solver2.advance(dt)                       SPH2S_FINAL_TWO_SCALE/Solver.cu:1568-1614

Everything runs in libsph2s.so through the C ABI (sph2_* entry points).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _abi, state_io
from ._abi import check, fptr, lib, sph_config2, sph_grid, uptr

LOW, HIGH = 0, 1
STAT_NAMES = ("splits", "merges", "removed_low", "removed_high", "faded_in_low", "faded_in_high")


class SolverConfiguration2:
    @staticmethod
    def make_configuration(origin, end, volume, num_particles, avg_particles, rest_density,
                           bulk_modulus, viscosity, speed_sound, tension_coefficient,
                           blend_increment) -> sph_config2:
        c = sph_config2()
        o = (C.c_float * 3)(*map(float, origin))
        e = (C.c_float * 3)(*map(float, end))
        check(lib().sph_make_configuration2(o, e, volume, num_particles, avg_particles,
                                            rest_density, bulk_modulus, viscosity, speed_sound,
                                            tension_coefficient, blend_increment, C.byref(c)))
        return c

    @staticmethod
    def direct(h, mass, rest_density, bulk_modulus, viscosity, speed_sound, tension_coefficient,
               blend_increment, grid_low: sph_grid, grid_high: sph_grid, refine_axis=-1,
               refine_lo=0.0, refine_hi=0.0, boundary_mass=None) -> sph_config2:
        c = sph_config2()
        h32 = np.float32(h)
        m32 = np.float32(mass)
        c.effective_radius[:] = [float(h32), float(np.float32(0.5) * h32)]
        c.fluid_particle_mass[:] = [float(m32), float(np.float32(1.0 / 8.0) * m32)]
        c.boundary_particle_mass = float(m32) if boundary_mass is None else boundary_mass
        c.rest_density = rest_density
        c.bulk_modulus = bulk_modulus
        c.viscosity = viscosity
        c.speed_sound = speed_sound
        c.tension_coefficient = tension_coefficient
        c.blend_increment = blend_increment
        c.grid[0] = grid_low
        c.grid[1] = grid_high
        c.refine_axis = refine_axis
        c.refine_lo = refine_lo
        c.refine_hi = refine_hi
        return c


class Solver2:
    """Two-scale WCSPH solver on the GPU (SPH2S_FINAL_TWO_SCALE/Solver.h:64-144)."""

    def __init__(self, low, high, boundary, config: sph_config2, capacity_low: int = 0,
                 capacity_high: int = 0):
        self.config = config
        arrs = []
        for p in (low, high, boundary):
            a = np.zeros((0, 3), np.float32) if p is None else np.ascontiguousarray(
                getattr(p, "positions", p), np.float32).reshape(-1, 3)
            arrs.append(a)
        h = C.c_void_p()
        check(lib().sph2_create(C.byref(config), fptr(arrs[0]), arrs[0].shape[0], fptr(arrs[1]),
                                arrs[1].shape[0], fptr(arrs[2]), arrs[2].shape[0], capacity_low,
                                capacity_high, C.byref(h)))
        self._h = h

    def advance(self, dt: float, steps: int = 1) -> None:
        check(lib().sph2_advance(self._h, C.c_float(dt), int(steps)))

    def counts(self) -> dict:
        v = [C.c_uint32() for _ in range(4)]
        check(lib().sph2_counts(self._h, *[C.byref(x) for x in v]))
        return {"low": v[0].value, "high": v[1].value, "boundary": v[2].value,
                "groups": v[3].value}

    def next_ids(self) -> tuple:
        lo, hi = C.c_uint32(), C.c_uint32()
        check(lib().sph2_next_ids(self._h, C.byref(lo), C.byref(hi)))
        return lo.value, hi.value

    def last_stats(self) -> dict:
        s = np.zeros(6, np.uint32)
        check(lib().sph2_last_stats(self._h, uptr(s)))
        return dict(zip(STAT_NAMES, map(int, s)))

    def state(self, population: int) -> dict:
        n = self.counts()["low" if population == LOW else "high"]
        r = {"x": np.empty((n, 3), np.float32), "v": np.empty((n, 3), np.float32),
             "lam": np.empty(n, np.float32), "state": np.empty(n, np.int32),
             "group": np.empty(n, np.uint32), "ids": np.empty(n, np.uint32)}
        check(lib().sph2_get_state(self._h, population, fptr(r["x"]), fptr(r["v"]),
                                   fptr(r["lam"]), r["state"].ctypes.data_as(C.POINTER(C.c_int32)),
                                   uptr(r["group"]), uptr(r["ids"])))
        return r

    def read_positions_device(self, population: int, device_ptr: int) -> None:
        """Enqueues a copy of one population's positions (current order, 3 floats
        per particle) into caller-owned device memory on the solver's stream."""
        check(lib().sph2_get_positions_device(self._h, population, C.c_void_p(device_ptr)))

    def read_states_device(self, population: int, device_ptr: int) -> None:
        """Enqueues a copy of one population's state bits (int32, current order)
        into caller-owned device memory on the solver's stream."""
        check(lib().sph2_get_states_device(self._h, population, C.c_void_p(device_ptr)))

    def debug_step_fields(self, population: int) -> dict:
        n = self.counts()["low" if population == LOW else "high"]
        r = {"ids": np.empty(n, np.uint32), "rho": np.empty(n, np.float32),
             "acc": np.empty((n, 3), np.float32), "nbr_same": np.empty(n, np.uint32),
             "nbr_compl": np.empty(n, np.uint32), "nbr_boundary": np.empty(n, np.uint32)}
        check(lib().sph2_debug_step_fields(self._h, population, uptr(r["ids"]), fptr(r["rho"]),
                                           fptr(r["acc"]), uptr(r["nbr_same"]),
                                           uptr(r["nbr_compl"]), uptr(r["nbr_boundary"])))
        return r

    def set_color_output(self, on: bool = True) -> None:
        """Colour / energy output of the force pass (dColorValues), off by default."""
        check(lib().sph2_set_color_output(self._h, 1 if on else 0))

    def colors(self, population: int):
        """Last step's colour values of one population in that step's sorted
        order, with the persistent ids."""
        n = C.c_uint32()
        check(lib().sph2_get_colors(self._h, population, None, None, C.byref(n)))
        col = np.empty(n.value, np.float32)
        ids = np.empty(n.value, np.uint32)
        check(lib().sph2_get_colors(self._h, population, fptr(col), uptr(ids), C.byref(n)))
        return col, ids

    # ---- headless state I/O (state_io.py describes the formats) ----
    @property
    def step_count(self) -> int:
        v = C.c_uint64()
        check(lib().sph2_step_count(self._h, C.byref(v)))
        return v.value

    def save_state(self, path=None) -> bytes:
        """The complete two-scale state as bytes; also written atomically to `path`."""
        need = C.c_uint64()
        check(lib().sph2_save_state(self._h, None, 0, C.byref(need)))
        buf = (C.c_ubyte * need.value)()
        check(lib().sph2_save_state(self._h, buf, need.value, C.byref(need)))
        data = bytes(buf)
        if path is not None:
            state_io.write_bytes(path, data)
        return data

    @classmethod
    def from_state(cls, src) -> "Solver2":
        data = state_io.read_bytes(src)
        h = C.c_void_p()
        check(lib().sph2_create_from_state(data, len(data), C.byref(h)))
        self = cls.__new__(cls)
        self._h = h
        self.config = sph_config2.from_buffer_copy(data, 24)
        return self

    def write_frame(self, path, fields=state_io.FIELD_POSITIONS | state_io.FIELD_BLEND,
                    append: bool = True) -> None:
        check(lib().sph2_write_frame(self._h, os.fsencode(path), int(fields), 1 if append else 0))

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().sph2_destroy(self._h)
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
