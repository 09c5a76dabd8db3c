"""ctypes wrapper of the two-scale FP64 oracle (oracle/sph_oracle_ts.cpp).

TEST INFRASTRUCTURE ONLY; the product never imports it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from .oracle import lib as _base_lib

_f = C.POINTER(C.c_float)
_d = C.POINTER(C.c_double)
_u = C.POINTER(C.c_uint32)
_i = C.POINTER(C.c_int32)
_b = C.POINTER(C.c_uint8)
_ready = False


def lib():
    global _ready
    l = _base_lib()
    if not _ready:
        l.or_ts_create.restype = C.c_void_p
        l.or_ts_create.argtypes = [C.c_void_p, _f, C.c_uint32, _u, C.POINTER(_f), C.POINTER(_f),
                                   C.POINTER(_f), C.POINTER(_i), C.POINTER(_u), C.POINTER(_u),
                                   C.c_uint32, _u]
        l.or_ts_advance.argtypes = [C.c_void_p, C.c_double, C.c_int]
        l.or_ts_step_fields.argtypes = [C.c_void_p, C.c_double, C.POINTER(_d), C.POINTER(_d),
                                        C.POINTER(_u), C.POINTER(_u), C.POINTER(_u), C.POINTER(_u),
                                        C.POINTER(_d), C.POINTER(_d)]
        l.or_ts_counts.argtypes = [C.c_void_p, _u, _u, _u]
        l.or_ts_last_stats.argtypes = [C.c_void_p, _u]
        l.or_ts_get.argtypes = [C.c_void_p, C.c_int, _d, _d, _f, _i, _u, _u]
        l.or_ts_destroy.argtypes = [C.c_void_p]
        l.or_ts_decide.argtypes = [C.c_void_p, _u, C.POINTER(_f), C.POINTER(_f), C.POINTER(_i),
                                   C.POINTER(_u), C.c_uint32, _u, C.POINTER(_b), C.POINTER(_i),
                                   C.POINTER(_f), C.POINTER(_u)]
        _ready = True
    return l


def _pp(arrs, t):
    return (t * 2)(*[a.ctypes.data_as(t) if a is not None else None for a in arrs])


class TSRollout:
    """Two-scale FP64 rollout.  `pops` = [low, high], each a dict with float
    arrays x (n,3) and optional v (n,3), lam (n), state (n), group (n), ids (n)."""

    def __init__(self, config, boundary_xyz, pops, group_base=0, pid_base=None):
        self.config = config
        self._keep = []

        def arr(p, k, dt, shape):
            if p.get(k) is None:
                return None
            a = np.ascontiguousarray(p[k], dt).reshape(shape)
            self._keep.append(a)
            return a

        n = np.array([np.asarray(p["x"]).reshape(-1, 3).shape[0] for p in pops], np.uint32)
        xs = [arr(p, "x", np.float32, (-1, 3)) for p in pops]
        vs = [arr(p, "v", np.float32, (-1, 3)) for p in pops]
        ls = [arr(p, "lam", np.float32, (-1,)) for p in pops]
        ss = [arr(p, "state", np.int32, (-1,)) for p in pops]
        gs = [arr(p, "group", np.uint32, (-1,)) for p in pops]
        ids = [arr(p, "ids", np.uint32, (-1,)) for p in pops]
        b = np.ascontiguousarray(boundary_xyz, np.float32).reshape(-1, 3)
        pb = None if pid_base is None else np.asarray(pid_base, np.uint32)
        self._h = lib().or_ts_create(
            C.byref(config), b.ctypes.data_as(_f), b.shape[0], n.ctypes.data_as(_u), _pp(xs, _f),
            _pp(vs, _f), _pp(ls, _f), _pp(ss, _i), _pp(gs, _u), _pp(ids, _u), group_base,
            None if pb is None else pb.ctypes.data_as(_u))

    def counts(self):
        v = [C.c_uint32() for _ in range(3)]
        lib().or_ts_counts(self._h, *[C.byref(x) for x in v])
        return {"low": v[0].value, "high": v[1].value, "groups": v[2].value}

    def advance(self, dt, steps=1):
        lib().or_ts_advance(self._h, dt, steps)

    def step_fields(self, dt):
        """One step; fields of the sorted pre-step populations."""
        c = self.counts()
        n = [c["low"], c["high"]]
        out = {k: [None, None] for k in ("rho", "acc", "nbr_same", "nbr_compl", "nbr_bnd", "ids",
                                         "colour", "dist_cm")}
        for r in range(2):
            out["rho"][r] = np.empty(n[r])
            out["acc"][r] = np.empty((n[r], 3))
            out["colour"][r] = np.empty(n[r])
            out["dist_cm"][r] = np.empty(n[r])
            for k in ("nbr_same", "nbr_compl", "nbr_bnd", "ids"):
                out[k][r] = np.empty(n[r], np.uint32)
        lib().or_ts_step_fields(self._h, dt, _pp(out["rho"], _d), _pp(out["acc"], _d),
                                _pp(out["nbr_same"], _u), _pp(out["nbr_compl"], _u),
                                _pp(out["nbr_bnd"], _u), _pp(out["ids"], _u),
                                _pp(out["colour"], _d), _pp(out["dist_cm"], _d))
        return out

    def last_stats(self):
        s = np.zeros(6, np.uint32)
        lib().or_ts_last_stats(self._h, s.ctypes.data_as(_u))
        return dict(zip(("splits", "merges", "removed_low", "removed_high", "faded_in_low",
                         "faded_in_high"), map(int, s)))

    def state(self, r):
        n = self.counts()["low" if r == 0 else "high"]
        x = np.empty((n, 3)); v = np.empty((n, 3)); lam = np.empty(n, np.float32)
        st = np.empty(n, np.int32); g = np.empty(n, np.uint32); ids = np.empty(n, np.uint32)
        lib().or_ts_get(self._h, r, x.ctypes.data_as(_d), v.ctypes.data_as(_d),
                        lam.ctypes.data_as(_f), st.ctypes.data_as(_i), g.ctypes.data_as(_u),
                        ids.ctypes.data_as(_u))
        return {"x": x, "v": v, "lam": lam, "state": st, "group": g, "ids": ids}

    def close(self):
        if self._h:
            lib().or_ts_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


STAT_NAMES = ("splits", "merges", "removed_low", "removed_high", "faded_in_low", "faded_in_high")


def decide(config, pops, group_base):
    """The state-machine decisions of one slab-trigger step from the
    start-of-step state (or_ts_decide): the six counters and, per population,
    keep flags and the state bits, blend coefficients and group ids the
    particles leave the step with.  pops = [low, high] dicts of x (n,3), lam,
    state, group."""
    arr = []
    for p in pops:
        arr.append({"x": np.ascontiguousarray(p["x"], np.float32).reshape(-1, 3),
                    "lam": np.ascontiguousarray(p["lam"], np.float32),
                    "state": np.ascontiguousarray(p["state"], np.int32),
                    "group": np.ascontiguousarray(p["group"], np.uint32)})
    n = np.array([a["x"].shape[0] for a in arr], np.uint32)
    out = [{"keep": np.empty(k, np.uint8), "state": np.empty(k, np.int32),
            "lam": np.empty(k, np.float32), "group": np.empty(k, np.uint32)} for k in n]
    stats = np.zeros(6, np.uint32)
    lib().or_ts_decide(C.byref(config), n.ctypes.data_as(_u),
                       _pp([a["x"] for a in arr], _f), _pp([a["lam"] for a in arr], _f),
                       _pp([a["state"] for a in arr], _i), _pp([a["group"] for a in arr], _u),
                       int(group_base), stats.ctypes.data_as(_u),
                       _pp([o["keep"] for o in out], _b), _pp([o["state"] for o in out], _i),
                       _pp([o["lam"] for o in out], _f), _pp([o["group"] for o in out], _u))
    return dict(zip(STAT_NAMES, map(int, stats))), out
