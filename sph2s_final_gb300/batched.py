"""Host-side wrapper of a batch of independent single-scale scenes (sphb_*).

Each scene is what `Solver(fluid, boundary, config)` would step on its own;
the batch steps all of them with one launch per kernel per step.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._abi import check, fptr, lib, sph_grid, sph_scene_desc

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

    # ---- batched differentiable rollout (every scene at once) ----
    def _split(self, packed, width):
        out, o = [], 0
        for n in self.sizes:
            out.append(packed[o:o + n].reshape((n,) + width))
            o += n
        return out

    def rollout_forward(self, v0=None, viscosity=None, dt: float = 1e-4, steps: int = 200,
                        checkpoint_every: int = 20) -> None:
        """v0: per-scene (n_s, 3) arrays (creation order) or None; viscosity: per scene."""
        vp = None
        if v0 is not None:
            vp = np.ascontiguousarray(np.concatenate(
                [np.asarray(v, np.float32).reshape(-1, 3) for v in v0]), np.float32)
            assert vp.shape[0] == self.total_particles
        mu = None if viscosity is None else np.ascontiguousarray(viscosity, np.float32)
        if mu is not None:
            assert mu.shape == (self.num_scenes,)
        check(lib().sphb_rollout_forward(self._h, fptr(vp), fptr(mu), C.c_float(dt), int(steps),
                                         int(checkpoint_every)))

    def rollout_density_loss(self, nodes, targets=None):
        """nodes: one sph_grid per scene; targets: per-scene node arrays (or None).
        Returns (per-scene fields, per-scene losses or None)."""
        grids = (sph_grid * self.num_scenes)(*nodes)
        counts = [g.dims[0] * g.dims[1] * g.dims[2] for g in nodes]
        field = np.empty(sum(counts), np.float32)
        t = None
        if targets is not None:
            t = np.ascontiguousarray(np.concatenate(
                [np.asarray(x, np.float32).ravel() for x in targets]), np.float32)
        loss = np.zeros(self.num_scenes, np.float64)
        check(lib().sphb_rollout_density_loss(self._h, grids, fptr(t), fptr(field),
                                              loss.ctypes.data_as(C.POINTER(C.c_double))))
        fields, o = [], 0
        for c in counts:
            fields.append(field[o:o + c])
            o += c
        return fields, (loss if targets is not None else None)

    def rollout_backward(self):
        """Per-scene gradients: (d L_s / d v0_s list, d L_s / d x0_s list, d L_s / d mu_s)."""
        n = self.total_particles
        gv = np.empty((n, 3), np.float32)
        gx = np.empty((n, 3), np.float32)
        gm = np.zeros(self.num_scenes, np.float64)
        check(lib().sphb_rollout_backward(self._h, fptr(gv), fptr(gx),
                                          gm.ctypes.data_as(C.POINTER(C.c_double))))
        return self._split(gv, (3,)), self._split(gx, (3,)), gm

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
