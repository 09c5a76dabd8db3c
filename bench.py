"""Throughput of the SPH2S single-scale step on GB300 (particle-steps/s).

Default workload: the 2M-particle dam break (2,097,152 fluid + 2,043,880
boundary particles, 128^3 cells, dt 2.5e-5), 100 warm-up + 1,000 timed steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload c1|c0] [--no-cpu-baseline]

`value` is device-timed (CUDA events on the solver's stream, state resident in
HBM); `e2e` goes through the public API (sph_create from host arrays, then per
step sph_advance + a device->host read of the positions into pinned memory).
`--impl reference` times the CPU restatement of the reference step (the
reference has no CPU path of its own and its CUDA 5.0/OpenGL program cannot
run here) on the host cores, and beside it the reference's own step kernels
rebuilt for this GPU (`reference_gpu`); that arm builds its scene with
oracle/scenes_ref.py and loads nothing of the product.  With N > 1 each rank
runs an independent replica (the path does not shard; there is no collective).

Roofline arithmetic (density and force passes, per launch):
  bytes  density 16 + 4 + 8 C/N B per particle (positions in, density out,
         cell table); force + integrate 72 + 16 C/N + 16 B_touched/N
  flops  density 8 per candidate (3 sub, r^2 as mul + 2 fma) + 4 per neighbour
         (Poly6 (h^2-r^2)^3 accumulated); force 38 per fluid neighbour
         (distance, rsqrt, spiky, Laplacian, Poly6 tension, 2 x 3 fma) + 16 per
         boundary neighbour; fma counted as 2.  Candidates (particles in the
         stencil cells) and neighbours are counted exactly for the timed
         state: candidates by a summed-area table of the cell occupancy in
         numpy, neighbours from the solver's own debug pass.
  peaks  HBM: MEASURED_PEAKS.json hbm_gbs; FP32: SMs x 128 lanes x 2 x the
         SM clock sampled during the timed region.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "particle-steps/s"
UNIT = "particle-steps/s"


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=100)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["c1", "c0", "c1m"], default="c1")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--profile-steps", type=int, default=200)
    ap.add_argument("--no-extras", action="store_true", help="skip the batched and adjoint measurements")
    ap.add_argument("--batched-steps", type=int, default=500)
    return ap.parse_args()


WORKLOADS = {
    "c1": (1 / 256, "dam break 2,097,152 fluid + 2,043,880 boundary, s=1/256, h=2s, 128^3 cells, "
                    "dt=2.5e-5"),
    "c0": (1 / 64, "dam break 32,768 fluid + 143,080 boundary, s=1/64, h=2s, 32^3 cells, dt=1e-4"),
    # a mid-size case for one-kernel ncu captures: above the 129 MB L2, far below the 2M case
    "c1m": (1 / 160, "dam break 512,000 fluid + 817,000 boundary, s=1/160, h=2s, 80^3 cells, "
                     "dt=2.5e-5"),
}


def workload(name: str):
    """The product's scene builders (libsph2s.so)."""
    from sph2s_final_gb300 import scenes
    spacing, desc = WORKLOADS[name]
    return scenes.dam_break(spacing), desc


def workload_reference(name: str):
    """The same scene restated in numpy (byte-identical, tests/test_scenes_ref.py),
    so the reference arm loads nothing of the product."""
    from oracle import scenes_ref
    spacing, desc = WORKLOADS[name]
    r = scenes_ref.dam_break(spacing)

    class _P:  # ParticleData-like view
        def __init__(self, a):
            self.positions = a
            self.num_particles = int(a.shape[0])

    class _S:
        pass
    sc = _S()
    sc.fluid, sc.boundary, sc.config, sc.dt, sc.spacing = _P(r.fluid), _P(r.boundary), r.config, r.dt, r.spacing
    return sc, desc


# Device bytes a step touches per fluid particle (state and step copies 64, density /
# aux 12, force records 16, neighbour lists ~136 used, keys and sort scratch ~24, the
# coherent sort's flags and previous keys ~8), per cell (fluid and boundary tables,
# 16) and per boundary particle (16).
STEP_BYTES_PER_PARTICLE, STEP_BYTES_PER_CELL, STEP_BYTES_PER_BOUNDARY = 260, 16, 16


def l2_bytes() -> tuple[int, str]:
    """The GPU's L2 size (cudaDevAttrL2CacheSize through torch), else the GB300's 129 MB."""
    try:
        import torch
        if torch.cuda.is_available():
            return int(torch.cuda.get_device_properties(0).L2_cache_size), "queried"
    except Exception:
        pass
    return 129 * 2**20, "nominal"


def config_for(desc: str, ws: int, sc) -> dict:
    """The `config` object of both arms' lines: the workload and whether its per-step
    data exceeds L2 (then no flush is needed between timed steps)."""
    g = sc.config.grid
    cells = int(g.dims[0]) * int(g.dims[1]) * int(g.dims[2])
    ws_bytes = (STEP_BYTES_PER_PARTICLE * sc.fluid.num_particles + STEP_BYTES_PER_CELL * cells
                + STEP_BYTES_PER_BOUNDARY * sc.boundary.num_particles)
    l2, how = l2_bytes()
    rel = "> L2, no flush needed" if ws_bytes > l2 else "fits in L2 (a parity-size case, not flushed)"
    return {"workload": desc, "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
            "l2": f"per-step data ~{ws_bytes / 2**20:.0f} MiB, L2 {l2 / 2**20:.0f} MiB ({how}): {rel}"}


def dist_env():
    """(world size, rank, local rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def physical_gpu_index(local: int) -> str:
    vis = os.environ.get("CUDA_VISIBLE_DEVICES")
    if vis:
        parts = [p.strip() for p in vis.split(",") if p.strip()]
        if local < len(parts):
            return parts[local]
    return str(local)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: str):
        self.gpu = gpu
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200", "-i", self.gpu], stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        time.sleep(0.3)

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.3)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in Path(self.path).read_text().splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
                power.append(float(p[3]))
            except ValueError:
                continue
            for nm, val in zip(names, p[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "power_w_max": max(power), "samples": len(sm), "reasons": sorted(reasons)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def committed_metric(name: str, kernel: str, wl: str):
    """A per-launch figure `name` of `kernel` on workload `wl` from the committed
    ncu summaries under profiles/ (lines "name: kernel wl value")."""
    pat = re.compile(rf"{re.escape(name)}:\s*{re.escape(kernel)}\s+{wl}\s+([0-9.eE+]+)")
    for f in sorted((ROOT / "profiles").glob("*.md")):
        m = pat.search(f.read_text())
        if m:
            return float(m.group(1))
    return None


def _cell_coord(x, o, s, d, off=0.0):
    """clamp(trunc(((x + off) - o) / s), 0, d - 1) in FP32, as the kernels."""
    t = (x.astype(np.float32) + np.float32(off)) - np.float32(o)
    t = t / np.float32(s)
    t = np.clip(t, np.float32(-1.0), np.float32(d))
    return np.clip(np.trunc(t).astype(np.int64), 0, d - 1)


def stencil_candidates(grid, h, query, source):
    """Per query particle: source particles in the cells of its stencil
    [cell(x - h), cell(x + h)] (self included), by a summed-area table."""
    d = [int(v) for v in grid.dims]
    o = [float(v) for v in grid.origin]
    s = float(grid.spacing)
    src = np.asarray(source, np.float32)
    cx, cy, cz = (_cell_coord(src[:, a], o[a], s, d[a]) for a in range(3))
    occ = np.zeros((d[2] + 1, d[1] + 1, d[0] + 1), np.int64)
    np.add.at(occ, (cz + 1, cy + 1, cx + 1), 1)
    sat = occ.cumsum(0).cumsum(1).cumsum(2)
    q = np.asarray(query, np.float32)
    lo = [_cell_coord(q[:, a], o[a], s, d[a], -h) for a in range(3)]
    hi = [_cell_coord(q[:, a], o[a], s, d[a], h) + 1 for a in range(3)]
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    return (sat[z1, y1, x1] - sat[z0, y1, x1] - sat[z1, y0, x1] - sat[z1, y1, x0]
            + sat[z0, y0, x1] + sat[z0, y1, x0] + sat[z1, y0, x0] - sat[z0, y0, x0])


def boundary_touched(sc) -> int:
    """Boundary particles in a cell that the stencil of some fluid particle covers."""
    g = sc.config.grid
    d = [int(v) for v in g.dims]
    o = [float(v) for v in g.origin]
    h = float(sc.config.effective_radius)
    f = np.asarray(sc.fluid.positions, np.float32)
    cover = np.zeros((d[2], d[1], d[0]), bool)
    lo = [_cell_coord(f[:, a], o[a], float(g.spacing), d[a], -h) for a in range(3)]
    hi = [_cell_coord(f[:, a], o[a], float(g.spacing), d[a], h) for a in range(3)]
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                cover[np.minimum(lo[2] + dz, hi[2]), np.minimum(lo[1] + dy, hi[1]),
                      np.minimum(lo[0] + dx, hi[0])] = True
    b = np.asarray(sc.boundary.positions, np.float32)
    bc = [_cell_coord(b[:, a], o[a], float(g.spacing), d[a]) for a in range(3)]
    return int(cover[bc[2], bc[1], bc[0]].sum())


FLOPS_DENS_CAND, FLOPS_DENS_NBR = 8, 4
FLOPS_FORCE_NBR, FLOPS_FORCE_BND = 38, 16


def step_work(scene_list, positions=None, nbr_per_candidate=None):
    """Whole single-scale steps of a list of scenes: algorithmic bytes
    (192 + 16 P) n + 40 C + 16 B_touched per scene (hash 24, sort 4 + 16 P with
    P = 3 digit passes, reorder + cell table 72 n + 16 C, density 20 n + 8 C,
    force + integrate 72 n + 16 C + 16 B_touched) and FP32 flops from exact
    candidate counts; neighbours per candidate are the measured ratio of the
    2M-particle step when given (the batch has no per-scene debug pass)."""
    algo, flops = 0, 0
    for k, sc in enumerate(scene_list):
        x = sc.fluid.positions if positions is None else positions[k]
        n = len(x)
        cells = int(np.prod(list(sc.config.grid.dims)))
        algo += 240 * n + 40 * cells + 16 * boundary_touched(sc)
        cand = int(stencil_candidates(sc.config.grid, float(sc.config.effective_radius), x, x).sum())
        ratio = nbr_per_candidate or 0.155
        nbr = cand * ratio
        flops += FLOPS_DENS_CAND * cand + FLOPS_DENS_NBR * nbr + FLOPS_FORCE_NBR * (nbr - n)
    return algo, flops


def fp32_peak_tflops(sm_mhz):
    import torch
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = sm_mhz or 2070.0
    return sms * 128 * 2 * mhz * 1e6 / 1e12, sms, mhz


def pass_roofline(name, ms, algo_bytes, flops, peak_gbs, peak_kind, peak_tf, sms, mhz, wl):
    gbs = algo_bytes / (ms * 1e-3) / 1e9
    tf = flops / (ms * 1e-3) / 1e12
    fb, ff = gbs / peak_gbs, tf / peak_tf
    out = {"ms": ms, "algorithmic_bytes_per_launch": int(algo_bytes), "achieved_gbs": gbs,
           "hbm_frac": fb, "flops_per_launch": int(flops), "achieved_tflops": tf,
           "fp32_peak_tflops": peak_tf, "fp32_frac": ff,
           "binds": "fp32 issue" if ff >= fb else "hbm",
           "traffic": committed_metric("traffic_bytes_per_launch", name, wl),
           "issue_active_pct": committed_metric("issue_active_pct", name, wl),
           "peaks": f"HBM {peak_gbs:.0f} GB/s ({peak_kind}); FP32 {sms} SMs x 128 x 2 x "
                    f"{mhz:.0f} MHz (sampled)"}
    return out


def cpu_baseline(sc, seconds: float):
    from oracle import oracle as O
    O.set_threads(os.cpu_count() or 1)
    cores = O.num_threads()
    ro = O.SSRollout(sc.config, sc.fluid.positions, sc.boundary.positions)
    t0 = time.perf_counter()
    ro.advance(sc.dt, 1)
    t1 = time.perf_counter()
    steps = max(1, int(seconds / max(t1 - t0, 1e-6)))
    t2 = time.perf_counter()
    ro.advance(sc.dt, steps)
    t3 = time.perf_counter()
    ro.close()
    n = sc.fluid.num_particles
    return {"value": n * steps / (t3 - t2), "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"FP64 oracle (C++/OpenMP) on the same scene, {steps} steps after 1 warm-up step"}


def cpu_baseline_c0(steps: int = 1000):
    """The FP64 oracle over the whole 1,000-step 32,768-particle case on the host cores."""
    from oracle import oracle as O
    from sph2s_final_gb300 import scenes
    sc = scenes.dam_break(1 / 64)
    O.set_threads(os.cpu_count() or 1)
    ro = O.SSRollout(sc.config, sc.fluid.positions, sc.boundary.positions)
    t0 = time.perf_counter()
    ro.advance(sc.dt, steps)
    el = time.perf_counter() - t0
    ro.close()
    n = sc.fluid.num_particles
    return {"value": n * steps / el, "unit": UNIT, "cores": O.num_threads(), "kind": "port",
            "seconds": el, "sample": f"FP64 oracle, dam break 32,768 fluid + 143,080 boundary, "
                                     f"all {steps} steps at dt 1e-4"}


def measure_batched(steps: int, warmup: int = 3, peaks=None, ratio=None):
    """256 independent scenes (9.4M fluid particles): one batch stepped with one
    launch per kernel per step, against the same scenes stepped one after
    another by per-scene solvers (each with its own CUDA graph)."""
    import torch

    from sph2s_final_gb300 import scenes
    from sph2s_final_gb300.batched import Batch
    from sph2s_final_gb300.solver import Solver

    scs = scenes.batched_scenes()
    dt = scs[0].dt
    items = [(s.fluid.positions, s.boundary.positions, s.config) for s in scs]
    n = sum(s.fluid.num_particles for s in scs)
    with Batch(items) as b:
        choice = b.autotune(dt)
        b.advance(dt, warmup)
        b.sync()
        st = torch.cuda.ExternalStream(b.stream)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        b.advance(dt, steps)
        e1.record(st)
        b.sync()
        batched_ms = e0.elapsed_time(e1)
    solvers = [Solver(s.fluid, s.boundary, s.config) for s in scs]
    for s in solvers:
        s.advance(dt, warmup)
        s.sync()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in solvers:
        s.advance(dt, steps)
        s.sync()
    serial_ms = 1e3 * (time.perf_counter() - t0)
    xs = [s.positions() for s in solvers]
    for s in solvers:
        s.close()
    out = {"scenes": len(scs), "fluid_particles": n, "steps": steps, "dt": dt,
           "batched_ms": batched_ms, "per_scene_serial_ms": serial_ms,
           "speedup": serial_ms / batched_ms,
           "batched_particle_steps_per_s": n * steps / (batched_ms * 1e-3),
           "per_scene_particle_steps_per_s": n * steps / (serial_ms * 1e-3),
           "autotune": choice,
           "timing": "batched: CUDA events on the batch stream; per-scene: host clock, "
                     "each scene synchronised before the next starts"}
    if peaks is not None:
        algo, flops = step_work(scs, xs, ratio)
        out["roofline"] = pass_roofline("batched_step", batched_ms / steps, algo, flops, *peaks,
                                        "c4")
        out["roofline"]["note"] = ("whole batched step; bytes by the single-scale per-pass "
                                   "formulas summed over the scenes; flops from exact candidate "
                                   "counts of the final state, neighbours at the 2M step's "
                                   "measured neighbours per candidate")
    return out


def measure_adjoint(steps: int = 200, every: int = 20, reps: int = 3, peaks=None, ratio=None):
    """65,536-particle differentiable rollout (T steps, checkpoints every K):
    forward (with checkpoints) and backward (segment recompute + adjoint
    kernels) wall time per rollout, synchronous calls, best of `reps`."""
    import torch

    from sph2s_final_gb300 import scenes
    from sph2s_final_gb300.autograd import node_grid
    from sph2s_final_gb300.solver import Solver

    sc, vt = scenes.differentiable_scene()
    with Solver(sc.fluid, sc.boundary, sc.config) as s:
        s.rollout_forward(vt, 5.0, sc.dt, steps, every)
        target, _ = s.rollout_density_loss(node_grid())
        v0 = np.zeros_like(vt)
        fw, bw, plain = [], [], []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            s.rollout_forward(v0, 5.0, sc.dt, steps, every)
            t1 = time.perf_counter()
            _, loss = s.rollout_density_loss(node_grid(), target)
            t2 = time.perf_counter()
            s.rollout_backward()
            t3 = time.perf_counter()
            fw.append(t1 - t0)
            bw.append(t3 - t2)
            s.sync()
            t4 = time.perf_counter()
            s.advance(sc.dt, steps)
            s.sync()
            plain.append(time.perf_counter() - t4)
        xs = [s.positions()]
    f, b, p = min(fw), min(bw), min(plain)
    out = {"particles": sc.fluid.num_particles, "steps": steps, "checkpoint_every": every,
           "forward_ms": 1e3 * f, "backward_ms": 1e3 * b, "plain_forward_ms": 1e3 * p,
           "adjoint_over_forward": b / f, "adjoint_over_plain_forward": b / p,
           "loss": loss, "timing": "host clock around synchronous calls, best of 3"}
    if peaks is not None:
        n = sc.fluid.num_particles
        algo, flops = step_work([sc], xs, ratio)
        # backward per step: the segment's forward recomputed with its tape written
        # (310 B per particle), then the adjoint integrate / force / density passes,
        # which read the tape and the same records as their forward passes
        bw_algo = 2 * algo + 2 * 310 * n
        out["roofline_forward"] = pass_roofline("rollout_forward", 1e3 * f / steps, algo, flops,
                                                *peaks, "c3")
        out["roofline_backward"] = pass_roofline("rollout_backward", 1e3 * b / steps, bw_algo,
                                                 3 * flops, *peaks, "c3")
        out["roofline_backward"]["note"] = ("per step, estimated: recompute (one forward step + "
                                            "310 B/particle of tape) + adjoint passes (one more "
                                            "step's bytes + the tape read; twice the forward flops)")
    return out


def measure_batched_adjoint(num: int = 64, steps: int = 100, every: int = 20, reps: int = 2):
    """Batched differentiable rollout over the first `num` scenes of the 256-scene
    batch: forward (checkpoints), per-scene splat loss on a 32^3 node grid, and
    backward, against the same rollouts run scene after scene by single-scale
    solvers.  Host clock around synchronous calls, best of `reps`."""
    import torch

    from sph2s_final_gb300 import scenes
    from sph2s_final_gb300.autograd import node_grid
    from sph2s_final_gb300.batched import Batch
    from sph2s_final_gb300.solver import Solver

    scs = scenes.batched_scenes()[:num]
    dt = scs[0].dt
    n = sum(s.fluid.num_particles for s in scs)
    rng = np.random.default_rng(1)
    vt = [rng.normal(0.0, 0.1, (s.fluid.num_particles, 3)).astype(np.float32) for s in scs]
    v0 = [np.zeros_like(v) for v in vt]
    mu = np.array([s.config.viscosity for s in scs], np.float32)
    nodes = [node_grid() for _ in scs]
    with Batch([(s.fluid.positions, s.boundary.positions, s.config) for s in scs]) as b:
        b.autotune(dt)
        b.rollout_forward(vt, mu, dt, steps, every)
        targets, _ = b.rollout_density_loss(nodes)
        fw, bw = [], []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            b.rollout_forward(v0, mu, dt, steps, every)
            b.rollout_density_loss(nodes, targets)
            t1 = time.perf_counter()
            b.rollout_backward()
            fw.append(t1 - t0)
            bw.append(time.perf_counter() - t1)
    solvers = [Solver(s.fluid, s.boundary, s.config) for s in scs]

    def serial_pass():
        for k, so in enumerate(solvers):
            so.rollout_forward(v0[k], float(mu[k]), dt, steps, every)
            so.rollout_density_loss(nodes[k], targets[k])
            so.rollout_backward()

    serial_pass()  # allocates every solver's tape
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    serial_pass()
    serial = time.perf_counter() - t0
    for so in solvers:
        so.close()
    f, bk = min(fw), min(bw)
    return {"scenes": num, "fluid_particles": n, "steps": steps, "checkpoint_every": every,
            "forward_and_loss_ms": 1e3 * f, "backward_ms": 1e3 * bk,
            "adjoint_over_forward": bk / f,
            "per_scene_serial_ms": 1e3 * serial, "speedup": serial / (f + bk),
            "timing": "host clock around synchronous calls; batched best of 2; per-scene "
                      "solvers (tapes allocated in an untimed pass) run forward, loss and "
                      "backward one scene after another"}


def measure_two_scale(steps: int = 300, warmup: int = 20, peaks=None):
    """Two-scale dam break (262,144 coarse particles at s = 1/128, refinement slab
    0.35 < x < 0.65, blend increment 0.0125 per step, dt = 2.5e-5): wall time per
    step of sph2_advance (synchronous: populations are read back every step, as
    the reference reads its counts) and particle-steps/s over both populations,
    with the split / merge activity seen.  The reference's own two-scale kernels
    (SPH2S_FINAL_TWO_SCALE/Solver.cu, oracle/ref_harness_ts.cu) are timed from the
    same state, the populations at the start of the timed window."""
    from oracle import ref_build
    from sph2s_final_gb300 import scenes
    from sph2s_final_gb300.two_scale import HIGH, LOW, Solver2

    sc = scenes.two_scale_dam_break(1 / 128)
    with Solver2(sc.low, None, sc.boundary, sc.config) as s:
        # the first step splits every coarse particle in the slab (8 children each)
        t0 = time.perf_counter()
        s.advance(sc.dt, 1)
        split_ms = 1e3 * (time.perf_counter() - t0)
        split_stats = s.last_stats()
        s.advance(sc.dt, warmup - 1)
        start = [s.state(LOW), s.state(HIGH)]
        dbg = [s.debug_step_fields(LOW), s.debug_step_fields(HIGH)]
        part_steps, splits, merges = 0, 0, 0
        t0 = time.perf_counter()
        for _ in range(steps):
            c = s.counts()
            part_steps += c["low"] + c["high"]
            s.advance(sc.dt, 1)
            st = s.last_stats()
            splits += st["splits"]
            merges += st["merges"]
        el = time.perf_counter() - t0
        c = s.counts()
    ms = 1e3 * el / steps
    out = {"workload": "two-scale dam break, 262,144 coarse + fine children, slab 0.35<x<0.65, "
                       "dt 2.5e-5", "steps": steps, "warmup": warmup,
           "ms_per_step": ms, "particle_steps_per_s": part_steps / el,
           "start_low": len(start[0]["ids"]), "start_high": len(start[1]["ids"]),
           "final_low": c["low"], "final_high": c["high"], "splits": splits, "merges": merges,
           "first_step": {"ms": split_ms, **split_stats},
           "timing": "host clock around synchronous sph2_advance calls"}
    if peaks is not None:
        # whole-step roofline of the step at the start of the timed window
        peak_gbs, peak_kind, peak_tf, sms, mhz = peaks
        g = sc.config.grid
        h = [float(sc.config.effective_radius[0]), float(sc.config.effective_radius[1])]
        pos = [st["x"] for st in start]
        cand = 0
        for r in (LOW, HIGH):
            if len(pos[r]) == 0:
                continue
            cand += int(stencil_candidates(g[r], h[r], pos[r], pos[r]).sum())
            if len(pos[1 - r]):
                cand += int(stencil_candidates(g[1 - r], h[0], pos[r], pos[1 - r]).sum())
        nbr = sum(int(d["nbr_same"].sum() + d["nbr_compl"].sum()) for d in dbg)
        bnd = sum(int(d["nbr_boundary"].sum()) for d in dbg)
        nparts = sum(len(p) for p in pos)
        flops = (FLOPS_DENS_CAND * cand + FLOPS_DENS_NBR * nbr + FLOPS_FORCE_NBR * nbr
                 + FLOPS_FORCE_BND * bnd)
        cells = sum(int(np.prod(list(gg.dims))) for gg in g)
        # per particle: state in (pos, vel, state, group 40 B), sorted copies out and in
        # (80 B), keys / values (16 B), density and force records (36 B), next state
        # out (40 B), compaction (12 B); cell tables 16 B per cell
        algo = 224 * nparts + 16 * cells
        out["roofline"] = pass_roofline("two_scale_step", ms, algo, flops, peak_gbs, peak_kind,
                                        peak_tf, sms, mhz, "c2")
        out["roofline"]["note"] = ("whole step; bytes 224 per particle + 16 per cell (state in, "
                                   "sorted copies, keys, records, next state); flops from exact "
                                   "candidate counts (same and complementary stencils) and the "
                                   "solver's neighbour counts")
    try:
        if not ref_build.CUBIN_TS.exists():
            raise FileNotFoundError("oracle/_ref/ts_solver.cubin not built")
        pops = [{"x": st["x"], "v": st["v"], "lam": st["lam"], "state": st["state"]}
                for st in start]
        caps = (len(pops[0]["x"]) + 1024, len(pops[1]["x"]) + 8 * len(pops[0]["x"]) + 1024)
        _, rms, ends = ref_build.run_harness_ts(ref_build.MODE_BLENDED, sc.config, pops,
                                               sc.boundary.positions, caps, steps, sc.dt,
                                               warmup=5)
        n0 = len(pops[0]["x"]) + len(pops[1]["x"])
        n1 = ends[0] + ends[1]
        out["reference_gpu"] = {
            "ms_per_step": rms, "particle_steps_per_s": 0.5 * (n0 + n1) / (rms * 1e-3),
            "end_low": ends[0], "end_high": ends[1], "speedup_ours": rms / ms,
            "kind": "reference kernels (SPH2S_FINAL_TWO_SCALE/Solver.cu, unmodified, sm_103a) "
                    "and its host sequence (thrust sort, per-step count reads) from our state "
                    "after the warm-up; the reference has no split trigger and no merge, so its "
                    "populations only fade; CUDA events around whole steps"}
    except Exception as e:  # reported, not fatal
        out["reference_gpu"] = {"unavailable": f"{type(e).__name__}: {str(e).splitlines()[0][:200]}"}
    return out


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    sc, desc = workload_reference(args.workload)
    from oracle import oracle as O
    O.set_threads(os.cpu_count() or 1)
    cores = O.num_threads()
    n = sc.fluid.num_particles
    ro = O.SSRollout(sc.config, sc.fluid.positions, sc.boundary.positions)
    t0 = time.perf_counter()
    ro.advance(sc.dt, 1)
    one = time.perf_counter() - t0
    budget = 90.0
    warm = min(args.warmup, max(0, int(0.2 * budget / one)))
    steps = max(1, min(args.steps, int(budget / one)))
    ro.advance(sc.dt, warm)
    t0 = time.perf_counter()
    ro.advance(sc.dt, steps)
    el = time.perf_counter() - t0
    ro.close()
    v = n * steps / el
    ref_gpu = reference_kernels_on_gpu(sc, args)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws,
        "steps": steps, "steps_requested": args.steps, "warmup": warm + 1,
        "ms_per_step": 1e3 * el / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded dam break)",
        "config": config_for(desc, ws, sc),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"FP64 CPU restatement of the reference step (the reference has "
                                   f"no CPU path), {steps} of {args.steps} requested steps"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "reference_gpu": ref_gpu,
    }
    print(json.dumps(line), flush=True)


def reference_kernels_on_gpu(sc, args):
    """The reference's own step kernels (its Solver.cu compiled for sm_103a) and its
    host sequence (thrust::sort_by_key per step), timed with CUDA events on this GPU."""
    from oracle import ref_build
    try:
        if not ref_build.CUBIN.exists():
            return {"unavailable": "reference kernels not built (oracle/_ref/ss_solver.cubin "
                                   "is made where the reference checkout is present)"}
        ms = ref_build.time_reference_kernels(sc.config, sc.fluid.positions,
                                              sc.boundary.positions, args.steps, sc.dt,
                                              args.warmup)
    except Exception as e:  # reported, not fatal: the CPU port above is the arm's value
        return {"unavailable": f"{type(e).__name__}: {str(e).splitlines()[0][:200]}"}
    n = sc.fluid.num_particles
    return {"value": n / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "steps": args.steps,
            "warmup": max(1, args.warmup),
            "kind": "reference kernels (SPH2S_FINAL_SINGLE_SCALE/Solver.cu, unmodified, sm_103a) "
                    "+ its thrust sort, the same steps and warm-up as our arm, CUDA events "
                    "around whole steps"}


def run_ours(args):
    import torch
    import torch.distributed as dist

    from sph2s_final_gb300.build import build_library
    from sph2s_final_gb300.solver import Solver
    from sph2s_final_gb300.solver import sort_passes_for

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    build_library()
    sc, desc = workload(args.workload)
    n, nb = sc.fluid.num_particles, sc.boundary.num_particles
    solver = Solver(sc.fluid, sc.boundary, sc.config)
    stream = torch.cuda.ExternalStream(solver.stream)

    from sph2s_final_gb300 import replicas
    barrier = replicas.barrier

    solver.advance(sc.dt, args.warmup)
    solver.sync()
    clocks = ClockSampler(physical_gpu_index(local))
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    solver.advance(sc.dt, args.steps)
    e1.record(stream)
    solver.sync()
    torch.cuda.synchronize()
    barrier()
    ms = replicas.max_over_ranks(e0.elapsed_time(e1), device="cuda")
    clk = clocks.stop()
    value = replicas.throughput(ws * n * args.steps, ms)

    # per-phase kernel durations: the step graph with event nodes between phases
    phases = solver.profile_phases(sc.dt, max(1, min(args.profile_steps, args.steps)))
    # exact work of the state the phases ended on (debug pass, no advance)
    dbg = solver.debug_step_fields()
    xs = solver.positions()
    solver.close()
    cand = int(stencil_candidates(sc.config.grid, float(sc.config.effective_radius), xs, xs).sum())
    nbr_self = int(dbg["nbr_fluid"].sum())          # r < h, self included (density)
    nbr_bnd = int(dbg["nbr_boundary"].sum())
    work = {"candidates": cand, "fluid_neighbours_with_self": nbr_self,
            "boundary_neighbours": nbr_bnd}

    # end to end through the public API: create from host arrays, then per step
    # advance + positions read back into pinned host memory (sph_get_positions_async:
    # the copy of step k overlaps step k+1; two pinned buffers alternate), and a
    # final sync that waits for the last copy.
    pinned = [torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]
    barrier()
    t0 = time.perf_counter()
    s2 = Solver(sc.fluid, sc.boundary, sc.config)
    tc = time.perf_counter()
    for k in range(args.steps):
        s2.advance(sc.dt, 1)
        s2.positions_async(pinned[k & 1])
    s2.sync()
    t1 = time.perf_counter()
    s2.close()
    e2e_s = replicas.max_over_ranks(t1 - t0, device="cuda")
    e2e = {"value": replicas.throughput(ws * n * args.steps, 1e3 * e2e_s), "unit": UNIT,
           "h2d_bytes_per_step": int(round((12 * n + 12 * nb) / args.steps)),
           "d2h_bytes_per_step": 12 * n,
           "create_ms": 1e3 * (tc - t0), "steps_ms": 1e3 * (t1 - tc)}

    if rank != 0:
        if ws > 1:
            dist.destroy_process_group()
        return

    peak, peak_kind = measured_peaks()
    peak_tf, sms, mhz = fp32_peak_tflops(clk.get("sm_mhz"))
    ncells = sc.config.grid.dims[0] * sc.config.grid.dims[1] * sc.config.grid.dims[2]
    btouch = boundary_touched(sc)
    dens_bytes = 20 * n + 8 * ncells
    force_bytes = 72 * n + 16 * ncells + 16 * btouch
    dens_flops = FLOPS_DENS_CAND * cand + FLOPS_DENS_NBR * nbr_self
    force_flops = FLOPS_FORCE_NBR * (nbr_self - n) + FLOPS_FORCE_BND * nbr_bnd
    dens = pass_roofline("density_kernel", phases["density"], dens_bytes, dens_flops, peak,
                         peak_kind, peak_tf, sms, mhz, args.workload)
    force = pass_roofline("force_kernel", phases["force"], force_bytes, force_flops, peak,
                          peak_kind, peak_tf, sms, mhz, args.workload)
    roofline = {"bound": "hbm", "kernel": "density_kernel (the dominant kernel)",
                "achieved": dens["achieved_gbs"], "peak": peak, "unit": "GB/s",
                "frac": dens["hbm_frac"], "peak_source": f"{peak_kind} hbm_gbs",
                "traffic": dens["traffic"], "algorithmic_bytes_per_launch": dens_bytes,
                "density": dens, "force": force, "work": work,
                "note": "bytes and FP32 fractions per pass; 'binds' names the larger one",
                "phase_ms": phases,
                "phase_sum_ms": phases["neighborhood"] + phases["density"] + phases["force"]}
    passes = sort_passes_for(sc.config.grid)
    # kernels per step: from 131,072 particles the step sorts coherently (keys and
    # flags, offsets, compaction, digit offsets, the passes, placement, cell
    # ranges), below from scratch (hash, digit offsets, the passes, gather);
    # then the boundary force pass beside density, density and force
    coherent = sc.fluid.num_particles >= 131072
    launches = ((9 if coherent else 6) + passes) * args.steps
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded dam break)",
        "config": config_for(desc, ws, sc),
        "clocks": clk, "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
    }
    if ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(sc, args.cpu_seconds)
        line["cpu_baseline_c0"] = cpu_baseline_c0()
    if ws == 1 and not args.no_extras:
        pk = (peak, peak_kind, peak_tf, sms, mhz)
        ratio = (nbr_self - n) / max(1, cand)  # neighbours per candidate of the 2M step
        line["batched"] = measure_batched(args.batched_steps, peaks=pk, ratio=ratio)
        line["adjoint"] = measure_adjoint(peaks=pk, ratio=ratio)
        line["batched_adjoint"] = measure_batched_adjoint()
        line["two_scale"] = measure_two_scale(peaks=pk)
    print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
