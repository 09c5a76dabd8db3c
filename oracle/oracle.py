"""ctypes wrapper of the FP64 CPU oracle (oracle/sph_oracle.cpp).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_build" / "liboracle.so"

_f = C.POINTER(C.c_float)
_d = C.POINTER(C.c_double)
_u = C.POINTER(C.c_uint32)
_i = C.POINTER(C.c_int32)
_lib = None


def _ptr(a, t):
    return None if a is None else a.ctypes.data_as(t)


def lib():
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            from .build import build_oracle
            build_oracle()
        l = C.CDLL(str(LIB_PATH))
        l.or_thresh_sq.restype = C.c_float
        l.or_thresh_sq.argtypes = [C.c_float]
        l.or_num_threads.restype = C.c_int
        l.or_set_num_threads.argtypes = [C.c_int]
        l.or_morton_bits.restype = C.c_int
        l.or_morton_bits.argtypes = [C.c_void_p]
        l.or_cell_keys.argtypes = [C.c_void_p, _f, C.c_uint32, _u, _u]
        l.or_stencil.argtypes = [C.c_void_p, _f, C.c_uint32, C.c_float, _i, _i]
        l.or_neighborhood.argtypes = [C.c_void_p, _f, C.c_uint32, _u, _u, _u, _u]
        l.or_ss_fields.argtypes = [C.c_void_p, _f, _f, C.c_uint32, _f, C.c_uint32, _d, _d, _u, _u]
        l.or_ss_xsph_step.argtypes = [C.c_void_p, _f, _f, C.c_uint32, _f, C.c_uint32, C.c_double,
                                      C.c_double, _d, _d]
        l.or_ss_create.restype = C.c_void_p
        l.or_ss_create.argtypes = [C.c_void_p, _f, C.c_uint32, _f, C.c_uint32, _f]
        l.or_ss_advance.argtypes = [C.c_void_p, C.c_double, C.c_int]
        l.or_ss_get.argtypes = [C.c_void_p, _d, _d, _d, _u]
        l.or_ss_destroy.argtypes = [C.c_void_p]
        _lib = l
    return _lib


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def thresh_sq(h: float) -> float:
    return float(lib().or_thresh_sq(h))


def set_threads(n: int) -> None:
    lib().or_set_num_threads(int(n))


def num_threads() -> int:
    return int(lib().or_num_threads())


def cell_keys(grid, xyz):
    x = f32(xyz)
    n = x.shape[0]
    keys = np.empty(n, np.uint32)
    lin = np.empty(n, np.uint32)
    lib().or_cell_keys(C.byref(grid), _ptr(x, _f), n, _ptr(keys, _u), _ptr(lin, _u))
    return keys, lin


def stencil(grid, xyz, h):
    x = f32(xyz)
    n = x.shape[0]
    cs = np.empty((n, 3), np.int32)
    ce = np.empty((n, 3), np.int32)
    lib().or_stencil(C.byref(grid), _ptr(x, _f), n, C.c_float(h), _ptr(cs, _i), _ptr(ce, _i))
    return cs, ce


def neighborhood(grid, xyz):
    """Stable Morton sort of xyz (in its given order) and the cell table."""
    x = f32(xyz)
    n = x.shape[0]
    nc = grid.dims[0] * grid.dims[1] * grid.dims[2]
    perm = np.empty(n, np.uint32)
    keys = np.empty(n, np.uint32)
    cs = np.empty(nc, np.uint32)
    ce = np.empty(nc, np.uint32)
    lib().or_neighborhood(C.byref(grid), _ptr(x, _f), n, _ptr(perm, _u), _ptr(keys, _u),
                          _ptr(cs, _u), _ptr(ce, _u))
    return {"perm": perm, "keys": keys, "cell_start": cs, "cell_end": ce}


def ss_fields(config, fluid_xyz, fluid_vel, boundary_xyz):
    """Density, acceleration and neighbour counts (input order) for one state."""
    x = f32(fluid_xyz)
    v = None if fluid_vel is None else f32(fluid_vel)
    b = f32(boundary_xyz)
    n = x.shape[0]
    rho = np.empty(n, np.float64)
    acc = np.empty((n, 3), np.float64)
    nf = np.empty(n, np.uint32)
    nb = np.empty(n, np.uint32)
    lib().or_ss_fields(C.byref(config), _ptr(x, _f), _ptr(v, _f), n, _ptr(b, _f), b.shape[0],
                       _ptr(rho, _d), _ptr(acc, _d), _ptr(nf, _u), _ptr(nb, _u))
    return {"rho": rho, "acc": acc, "nbr_fluid": nf, "nbr_boundary": nb}


def ss_xsph_step(config, fluid_xyz, fluid_vel, boundary_xyz, dt, eps):
    """One XSPH-integrator step (Solver.cu:757-853, per-component correction) from
    one state; next positions and velocities in input order (float64)."""
    x = f32(fluid_xyz)
    v = None if fluid_vel is None else f32(fluid_vel)
    b = f32(boundary_xyz)
    n = x.shape[0]
    xo = np.empty((n, 3), np.float64)
    vo = np.empty((n, 3), np.float64)
    lib().or_ss_xsph_step(C.byref(config), _ptr(x, _f), _ptr(v, _f), n, _ptr(b, _f), b.shape[0],
                          dt, eps, _ptr(xo, _d), _ptr(vo, _d))
    return xo, vo


class SSRollout:
    """FP64 single-scale rollout (state kept in double, sorted order)."""

    def __init__(self, config, fluid_xyz, boundary_xyz, vel=None):
        self.config = config
        x = f32(fluid_xyz)
        b = f32(boundary_xyz)
        v = None if vel is None else f32(vel)
        self.n = x.shape[0]
        self._h = lib().or_ss_create(C.byref(config), _ptr(x, _f), self.n, _ptr(b, _f),
                                     b.shape[0], _ptr(v, _f))

    def advance(self, dt: float, steps: int = 1) -> None:
        lib().or_ss_advance(self._h, dt, steps)

    def state(self):
        n = self.n
        x = np.empty((n, 3)); v = np.empty((n, 3)); rho = np.empty(n); ids = np.empty(n, np.uint32)
        lib().or_ss_get(self._h, _ptr(x, _d), _ptr(v, _d), _ptr(rho, _d), _ptr(ids, _u))
        return {"x": x, "v": v, "rho": rho, "ids": ids}

    def close(self):
        if self._h:
            lib().or_ss_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def splat_loss(config, x, nodes_dims=(32, 32, 32), target=None):
    """FP64 Poly6 splat of positions x (n,3) on the cell centres of a grid over
    the unit box (G_n = m sum_i W(|y_n - x_i|), r < h), and the mean squared
    error against `target` if given.  Test infrastructure for finite
    differences of the differentiable rollout."""
    x = np.asarray(x, np.float64)
    h = float(np.float32(config.effective_radius))
    m = float(np.float32(config.fluid_particle_mass))
    c6 = 315.0 / (64.0 * np.pi * h ** 9)
    d = np.array(nodes_dims)
    sp = 1.0 / d[0]
    base = np.floor(x / sp - 0.5).astype(np.int64)
    field = np.zeros(int(np.prod(d)))
    offs = np.arange(-1, 3)
    for ox in offs:
        for oy in offs:
            for oz in offs:
                idx = base + np.array([ox, oy, oz])
                ok = np.all((idx >= 0) & (idx < d), axis=1)
                y = (idx + 0.5) * sp
                r2 = ((x - y) ** 2).sum(1)
                w = np.where(ok & (r2 < h * h), (h * h - r2) ** 3, 0.0)
                lin = idx[:, 0] + d[0] * (idx[:, 1] + d[1] * idx[:, 2])
                np.add.at(field, lin[ok], w[ok])
    field *= m * c6
    if target is None:
        return field, None
    return field, float(((field - np.asarray(target, np.float64)) ** 2).mean())
