"""Generates tests/golden/ref_ts_*.npz and ref_cp_*.npz: outputs of the
reference's own two-scale and coupled kernels.

The reference's two-scale project (SPH2S_FINAL_TWO_SCALE/Solver.cu) and its
coupled variant (SPH2S_FINAL_TWO_SCALE_COUPLED/Solver.cu) compile unmodified
for sm_103a (oracle/ref_build.py -> oracle/_ref/ts_solver.cubin,
cp_solver.cubin); oracle/ref_harness_ts.cu replays their Solver::Advance
around those kernels.  This script builds seeded two-population scenes, runs
the harness on a GPU and stores inputs and per-step outputs:

  ref_ts_mixed    blended step: a coarse block (s = 1/32, h = 1/16) beside and
                  overlapping a fine block (s = 1/64, h/2), 2-layer boundary
                  shell of the unit box, dt 2.5e-4, 4 steps.  Initial states
                  cover every branch of the blend / state machine
                  (TS Solver.cu:1229-1289): normal, fading out (some reach
                  lambda <= 0 in each step), fading in (some complete),
                  marked for split (LOW: 8 children each; HIGH: left alone),
                  and the renderer's surface bit 8 combined with each.
  ref_ts_clamp    the same scene with 3% of the particles at 0.75-2x the
                  velocity clamp 0.8 h_r / dt (TS Solver.cu:1212-1223), 2 steps.
  ref_cp_mixed    coupled step (two fixed populations), the mixed scene's
                  positions and velocities, 3 steps.

Every case is checked to have no HIGH slot overlap (children written over
HIGH survivors, a hazard of the reference's list compaction; the scenes keep
every HIGH particle alive).

Usage (on a machine with a GPU, with the cubins built where the reference
checkout is; the harness is compiled on first use):
  python tests/golden/make_golden_ts.py --out tests/golden
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import ref_build  # noqa: E402
from sph2s_final_gb300 import scenes  # noqa: E402
from sph2s_final_gb300.solver import Grid, ParticleData  # noqa: E402
from sph2s_final_gb300.two_scale import SolverConfiguration2  # noqa: E402

S = 1.0 / 32.0


def base_scene(seed: int = 11):
    """Coarse 10 x 8 x 10 block at s, fine 12 x 16 x 20 block at s/2 from x = 0.25
    (overlapping the coarse block's last two layers), 2-layer boundary shell."""
    s = float(np.float32(S))
    low = scenes.jitter(scenes.lattice_block(s, (10, 8, 10)), s, 0.01, seed)
    hs = float(np.float32(0.5) * np.float32(s))
    high = scenes.jitter(scenes.lattice_block(hs, (12, 16, 20)), hs, 0.01, seed + 1)
    high[:, 0] += np.float32(0.25)
    box = Grid.make_grid((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), s)
    boundary = ParticleData.create_particle_box_canvas(box, 2).positions
    h = float(np.float32(2.0 * s))
    g0 = Grid.make_grid((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), h)
    g1 = Grid.make_grid((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), float(np.float32(0.5) * np.float32(h)))
    mass = float(np.float32(scenes.REST_DENSITY * s ** 3))
    cfg = SolverConfiguration2.direct(h, mass, scenes.REST_DENSITY, scenes.BULK_MODULUS,
                                      scenes.VISCOSITY, scenes.SPEED_SOUND, scenes.TENSION,
                                      0.0125, g0, g1, refine_axis=-1)
    return low, high, boundary, cfg


def mixed_states(low, high, rng):
    """States and blend coefficients reaching every branch of the state machine."""
    nl, nh = low.shape[0], high.shape[0]
    sl = np.zeros(nl, np.int32)
    ll = np.ones(nl, np.float32)
    over = low[:, 0] >= 0.245
    u = rng.random(nl)
    sl[over] = 1
    lo_lam = np.where(rng.random(nl) < 0.5, rng.uniform(0.001, 0.06, nl), rng.uniform(0.06, 0.6, nl))
    ll[over] = lo_lam[over]
    rest = ~over
    pick = [(0.12, 3, None), (0.20, 2, (0.5, 1.0)), (0.24, 8, None), (0.26, 11, None),
            (0.28, 9, (0.2, 1.0)), (0.30, 10, (0.5, 1.0))]
    lo = 0.0
    for hi, st, lam in pick:
        m = rest & (u >= lo) & (u < hi)
        sl[m] = st
        if lam is not None:
            ll[m] = rng.uniform(lam[0], lam[1], int(m.sum()))
        lo = hi
    sh = np.full(nh, 4, np.int32)
    lh = np.ones(nh, np.float32)
    over_h = high[:, 0] < 0.3125
    sh[over_h] = 6
    lh[over_h] = rng.uniform(0.3, 1.0, int(over_h.sum()))
    u = rng.random(nh)
    m5 = ~over_h & (u < 0.10)
    sh[m5] = 5
    lh[m5] = rng.uniform(0.3, 1.0, int(m5.sum()))
    sh[~over_h & (u >= 0.10) & (u < 0.12)] = 7
    sh[~over_h & (u >= 0.12) & (u < 0.14)] = 12
    return sl, ll, sh, lh


def cases():
    low, high, boundary, cfg = base_scene()
    rng = np.random.default_rng(5)
    sl, ll, sh, lh = mixed_states(low, high, rng)
    vl = rng.normal(0.0, 0.3, low.shape).astype(np.float32)
    vh = rng.normal(0.0, 0.3, high.shape).astype(np.float32)
    pops = [{"x": low, "v": vl, "lam": ll, "state": sl}, {"x": high, "v": vh, "lam": lh, "state": sh}]
    yield "ref_ts_mixed", ref_build.MODE_BLENDED, cfg, pops, boundary, 4, 2.5e-4

    dt = 2.5e-4
    fast = []
    for r, p in enumerate(pops):
        vmax = 0.8 * cfg.effective_radius[r] / dt
        v = p["v"].copy()
        pick = rng.random(v.shape[0]) < 0.03
        d = rng.normal(size=(int(pick.sum()), 3))
        d /= np.linalg.norm(d, axis=1, keepdims=True)
        v[pick] = (d * rng.uniform(0.75, 2.0, (int(pick.sum()), 1)) * vmax).astype(np.float32)
        fast.append(dict(p, v=v))
    yield "ref_ts_clamp", ref_build.MODE_BLENDED, cfg, fast, boundary, 2, dt

    cp = [dict(p, lam=np.ones_like(p["lam"]), state=np.full_like(p["state"], 4 * r))
          for r, p in enumerate(pops)]
    yield "ref_cp_mixed", ref_build.MODE_COUPLED, cfg, cp, boundary, 3, 2.5e-4


def config_arrays(cfg):
    return {"cfg_h": np.array(cfg.effective_radius[:], np.float32),
            "cfg_m": np.array(cfg.fluid_particle_mass[:], np.float32),
            "cfg_scalars": np.array([cfg.boundary_particle_mass, cfg.rest_density,
                                     cfg.bulk_modulus, cfg.viscosity, cfg.speed_sound,
                                     cfg.tension_coefficient, cfg.blend_increment], np.float32),
            "cfg_origin": np.array([list(g.origin) for g in cfg.grid], np.float32),
            "cfg_dims": np.array([list(g.dims) for g in cfg.grid], np.int32),
            "cfg_spacing": np.array([g.spacing for g in cfg.grid], np.float32)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(Path(__file__).resolve().parent))
    args = ap.parse_args()
    out_dir = Path(args.out)
    out_dir.mkdir(parents=True, exist_ok=True)
    for name, mode, cfg, pops, boundary, steps, dt in cases():
        nl, nh = pops[0]["x"].shape[0], pops[1]["x"].shape[0]
        caps = (nl + 64, nh + 8 * nl + 64)
        rec, _, _ = ref_build.run_harness_ts(mode, cfg, pops, boundary, caps, steps, dt)
        assert len(rec) == steps
        assert all(r["slot_overlap"] == 0 for r in rec), name
        arrs = {"mode": np.int32(mode), "steps": np.int32(steps), "dt": np.float32(dt),
                "boundary": np.asarray(boundary, np.float32), **config_arrays(cfg)}
        for r, tag in ((0, "low"), (1, "high")):
            for k in ("x", "v", "lam", "state"):
                arrs[f"in_{tag}_{k}"] = pops[r][k]
        for t, st in enumerate(rec):
            arrs[f"s{t}_high_survivors"] = np.uint32(st["high_survivors"])
            for r, tag in ((0, "low"), (1, "high")):
                for k, v in st["fields"][r].items():
                    arrs[f"s{t}_{tag}_f_{k}"] = v
                for k, v in st["post"][r].items():
                    arrs[f"s{t}_{tag}_post_{k}"] = v
        np.savez_compressed(out_dir / f"{name}.npz", **arrs)
        counts = [(len(s["post"][0]["pid"]), len(s["post"][1]["pid"])) for s in rec]
        print(name, nl, nh, "->", counts, out_dir / f"{name}.npz")


if __name__ == "__main__":
    main()
