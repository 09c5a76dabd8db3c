"""Test helpers for two-scale fixtures: solvers and oracles started from an
arbitrary two-population state, and the golden files of the reference's own
two-scale / coupled kernels (tests/golden/ref_ts_*.npz, ref_cp_*.npz, made by
tests/golden/make_golden_ts.py).

A GPU solver is seeded through the public state format: sph2_create with the
positions, sph2_save_state, the velocities, blend coefficients and state bits
patched into the buffer (particles are in creation order there, the creation
index in pos.w), the checksum recomputed, sph2_create_from_state.
"""
from __future__ import annotations

import ctypes as C
import struct
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"
CHILD_PID_BASE = 0x40000000  # ids the reference harness gives split children


def fnv_words(data: bytes) -> int:
    """Word-wise FNV-1a of the state format (csrc/state_format.h)."""
    pad = (-len(data)) % 8
    w = np.frombuffer(data + b"\0" * pad, np.uint64)
    h = 0xCBF29CE484222325
    for x in w.tolist():
        h = ((h ^ x) * 0x100000001B3) & 0xFFFFFFFFFFFFFFFF
    return h


def config_from_golden(g):
    from sph2s_final_gb300._abi import sph_config2, sph_grid
    c = sph_config2()
    c.effective_radius[:] = [float(v) for v in g["cfg_h"]]
    c.fluid_particle_mass[:] = [float(v) for v in g["cfg_m"]]
    (c.boundary_particle_mass, c.rest_density, c.bulk_modulus, c.viscosity, c.speed_sound,
     c.tension_coefficient, c.blend_increment) = [float(v) for v in g["cfg_scalars"]]
    for r in range(2):
        gr = sph_grid()
        gr.origin[:] = [float(v) for v in g["cfg_origin"][r]]
        gr.dims[:] = [int(v) for v in g["cfg_dims"][r]]
        gr.spacing = float(g["cfg_spacing"][r])
        c.grid[r] = gr
    c.refine_axis = -1
    c.mode = int(g["mode"])
    return c


def load(name: str) -> dict:
    with np.load(GOLDEN / f"{name}.npz") as f:
        return {k: f[k] for k in f.files}


def pre_state(g: dict, t: int) -> list[dict]:
    """The state step t starts from: the input for t = 0, else the particles the
    reference listed active after step t-1.  Each population: x, v, lam, state
    and the harness ids `pid`."""
    out = []
    for tag in ("low", "high"):
        if t == 0:
            x = g[f"in_{tag}_x"]
            pid = np.arange(x.shape[0], dtype=np.uint32)
            p = {"x": x, "v": g[f"in_{tag}_v"], "lam": g[f"in_{tag}_lam"],
                 "state": g[f"in_{tag}_state"], "pid": pid}
        else:
            k = f"s{t - 1}_{tag}_post_"
            p = {"x": g[k + "x"], "v": g[k + "v"], "lam": g[k + "lam"], "state": g[k + "state"],
                 "pid": g[k + "pid"]}
        out.append({kk: np.ascontiguousarray(vv) for kk, vv in p.items()})
    return out


def solver_from_pops(config, pops, boundary, caps=None):
    """A GPU Solver2 whose populations are exactly `pops` (creation order = array
    order, so persistent id i = element i)."""
    from sph2s_final_gb300._abi import sph_config2
    from sph2s_final_gb300.two_scale import Solver2
    nl, nh = pops[0]["x"].shape[0], pops[1]["x"].shape[0]
    if caps is None:
        caps = (nl + 1024, nh + 8 * nl + 1024)
    with Solver2(pops[0]["x"], pops[1]["x"], boundary, config, caps[0], caps[1]) as s:
        data = bytearray(s.save_state())
    off = 24 + C.sizeof(sph_config2) + 24 + 16
    for p in pops:
        n = p["x"].shape[0]
        pos = np.frombuffer(data, np.float32, 4 * n, off).reshape(n, 4)
        assert np.array_equal(pos[:, 3].view(np.uint32), np.arange(n, dtype=np.uint32))
        vel = np.zeros((n, 4), np.float32)
        vel[:, :3] = p["v"]
        vel[:, 3] = p["lam"]
        data[off + 16 * n: off + 32 * n] = vel.tobytes()
        data[off + 32 * n: off + 36 * n] = np.ascontiguousarray(p["state"], np.int32).tobytes()
        off += 40 * n
    body = bytes(data[:-8])
    data[-8:] = struct.pack("<Q", fnv_words(body))
    return Solver2.from_state(bytes(data))


def oracle_from_pops(config, pops, boundary):
    """The FP64 oracle started from `pops` (ids = array positions)."""
    from oracle.oracle_ts import TSRollout
    arr = []
    for p in pops:
        n = p["x"].shape[0]
        arr.append({"x": p["x"], "v": p["v"], "lam": p["lam"], "state": p["state"],
                    "ids": np.arange(n, dtype=np.uint32),
                    "group": np.full(n, 0xFFFFFFFF, np.uint32)})
    return TSRollout(config, boundary, arr, group_base=0,
                     pid_base=[pops[0]["x"].shape[0], pops[1]["x"].shape[0]])


def by_pid(values, ids, pid_of_id):
    """values indexed by dense ids -> dict harness pid -> value row."""
    return dict(zip(pid_of_id[ids].tolist(), values))


def match_children(ref_x, got_x, tol=2e-6):
    """Pairs the reference's split children with ours by position (the
    reference appends them in atomicAdd order).  Returns the permutation p with
    got_x[p[i]] matching ref_x[i]; asserts a bijection within tol."""
    from scipy.spatial import cKDTree
    assert ref_x.shape == got_x.shape, (ref_x.shape, got_x.shape)
    if ref_x.shape[0] == 0:
        return np.zeros(0, np.int64)
    d, p = cKDTree(np.asarray(got_x, np.float64)).query(np.asarray(ref_x, np.float64))
    assert np.unique(p).size == p.size, "children do not pair one to one"
    assert d.max() <= tol, f"child position mismatch {d.max():.3e}"
    return p
