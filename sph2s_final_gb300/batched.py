"""Host-side wrapper of a batch of independent single-scale scenes (sphb_*).

Each scene is what `Solver(fluid, boundary, config)` would step on its own;
the batch steps all of them with one launch per kernel per step.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._abi import check, fptr, lib, sph_scene_desc

ORDER = {"sorted": 0, "by_id": 1}


class Batch:
    def __init__(self, scenes):
        """scenes: iterable of (fluid_xyz, boundary_xyz, config[, velocities])."""
        self._keep = []
        descs = (sph_scene_desc * len(scenes))()
        self.sizes = []
        for k, sc in enumerate(scenes):
            fx = np.ascontiguousarray(sc[0], np.float32).reshape(-1, 3)
            bx = np.ascontiguousarray(sc[1], np.float32).reshape(-1, 3)
            v = None if len(sc) < 4 or sc[3] is None else np.ascontiguousarray(sc[3], np.float32)
            self._keep += [fx, bx, v]
            descs[k].fluid_xyz = fptr(fx)
            descs[k].n_fluid = fx.shape[0]
            descs[k].boundary_xyz = fptr(bx)
            descs[k].n_boundary = bx.shape[0]
            descs[k].velocity_xyz = fptr(v)
            descs[k].config = sc[2]
            self.sizes.append(fx.shape[0])
        h = C.c_void_p()
        check(lib().sphb_create(descs, len(scenes), C.byref(h)))
        self._keep = None
        self._h = h

    @property
    def num_scenes(self) -> int:
        return len(self.sizes)

    @property
    def total_particles(self) -> int:
        return int(sum(self.sizes))

    def advance(self, dt: float, steps: int = 1) -> None:
        check(lib().sphb_advance(self._h, C.c_float(dt), int(steps)))

    def sync(self) -> None:
        check(lib().sphb_sync(self._h))

    @property
    def stream(self) -> int:
        return lib().sphb_stream(self._h) or 0

    def scene(self, s: int, order: str = "sorted") -> dict:
        n = self.sizes[s]
        r = {"x": np.empty((n, 3), np.float32), "v": np.empty((n, 3), np.float32),
             "rho": np.empty(n, np.float32)}
        check(lib().sphb_get_scene(self._h, s, fptr(r["x"]), fptr(r["v"]), fptr(r["rho"]),
                                   ORDER[order]))
        return r

    def autotune(self, dt: float) -> dict:
        c = (C.c_int32 * 3)()
        check(lib().sphb_autotune(self._h, C.c_float(dt), c))
        return {"density_block": c[0], "force_block": c[1], "blocks_per_sm": c[2]}

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().sphb_destroy(self._h)
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
