"""Throughput of the SPH2S single-scale step on GB300 (particle-steps/s).

Default workload: the 2M-particle dam break (2,097,152 fluid + 2,043,880
boundary particles, 128^3 cells, dt 2.5e-5), 100 warm-up + 1,000 timed steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload c1|c0] [--no-cpu-baseline]

`value` is device-timed (CUDA events on the solver's stream, state resident in
HBM); `e2e` goes through the public API (sph_create from host arrays, then per
step sph_advance + a device->host read of the positions into pinned memory).
`--impl reference` times the CPU restatement of the reference step (the
reference has no CPU path of its own and its CUDA 5.0/OpenGL build cannot run
here) on the host cores.  With N > 1 each rank runs an independent replica
(the path does not shard; there is no collective).
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
    ap.add_argument("--workload", choices=["c1", "c0"], default="c1")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--profile-steps", type=int, default=200)
    ap.add_argument("--no-extras", action="store_true", help="skip the batched and adjoint measurements")
    ap.add_argument("--batched-steps", type=int, default=500)
    return ap.parse_args()


def workload(name: str):
    from sph2s_final_gb300 import scenes
    if name == "c1":
        sc = scenes.dam_break(1 / 256)
        desc = "dam break 2,097,152 fluid + 2,043,880 boundary, s=1/256, h=2s, 128^3 cells, dt=2.5e-5"
    else:
        sc = scenes.dam_break(1 / 64)
        desc = "dam break 32,768 fluid + 143,080 boundary, s=1/64, h=2s, 32^3 cells, dt=1e-4"
    return sc, desc


def dist_env():
    from sph2s_final_gb300 import replicas
    return replicas.world()


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


def committed_traffic(kernel: str, wl: str):
    """Per-launch DRAM bytes of `kernel` on workload `wl` from the committed ncu summaries."""
    pat = re.compile(rf"traffic_bytes_per_launch:\s*{re.escape(kernel)}\s+{wl}\s+([0-9.eE+]+)")
    for f in sorted((ROOT / "profiles").glob("*.md")):
        m = pat.search(f.read_text())
        if m:
            return float(m.group(1))
    return None


def boundary_touched(sc) -> int:
    """Boundary particles within one cell (Chebyshev) of a fluid-occupied cell."""
    from oracle import oracle as O  # host-side counting only
    g = sc.config.grid
    _, lf = O.cell_keys(g, sc.fluid.positions)
    _, lb = O.cell_keys(g, sc.boundary.positions)
    d = np.array(g.dims[:])
    occ = np.zeros(d[::-1], bool)
    cz, rem = np.divmod(lf, d[0] * d[1])
    cy, cx = np.divmod(rem, d[0])
    occ[cz, cy, cx] = True
    dil = occ.copy()
    for ax in range(3):
        for sh in (-1, 1):
            dil |= np.roll(occ, sh, axis=ax)  # roll wraps, but edges are clamped cells anyway
    bz, rem = np.divmod(lb, d[0] * d[1])
    by, bx = np.divmod(rem, d[0])
    return int(dil[bz, by, bx].sum())


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


def measure_batched(steps: int, warmup: int = 3):
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
    for s in solvers:
        s.close()
    return {"scenes": len(scs), "fluid_particles": n, "steps": steps, "dt": dt,
            "batched_ms": batched_ms, "per_scene_serial_ms": serial_ms,
            "speedup": serial_ms / batched_ms,
            "batched_particle_steps_per_s": n * steps / (batched_ms * 1e-3),
            "per_scene_particle_steps_per_s": n * steps / (serial_ms * 1e-3),
            "autotune": choice,
            "timing": "batched: CUDA events on the batch stream; per-scene: host clock, "
                      "each scene synchronised before the next starts"}


def measure_adjoint(steps: int = 200, every: int = 20, reps: int = 3):
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
    f, b, p = min(fw), min(bw), min(plain)
    return {"particles": sc.fluid.num_particles, "steps": steps, "checkpoint_every": every,
            "forward_ms": 1e3 * f, "backward_ms": 1e3 * b, "plain_forward_ms": 1e3 * p,
            "adjoint_over_forward": b / f, "adjoint_over_plain_forward": b / p,
            "loss": loss, "timing": "host clock around synchronous calls, best of 3"}


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


def measure_two_scale(steps: int = 300, warmup: int = 20):
    """Two-scale dam break (262,144 coarse particles at s = 1/128, refinement slab
    0.35 < x < 0.65, blend increment 0.0125 per step, dt = 2.5e-5): wall time per
    step of sph2_advance (synchronous: populations are read back every step) and
    particle-steps/s over both populations, with the split / merge activity seen."""
    from sph2s_final_gb300 import scenes
    from sph2s_final_gb300.two_scale import Solver2

    sc = scenes.two_scale_dam_break(1 / 128)
    with Solver2(sc.low, None, sc.boundary, sc.config) as s:
        s.advance(sc.dt, warmup)
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
    return {"workload": "two-scale dam break, 262,144 coarse + fine children, slab 0.35<x<0.65, "
                        "dt 2.5e-5", "steps": steps, "warmup": warmup,
            "ms_per_step": 1e3 * el / steps, "particle_steps_per_s": part_steps / el,
            "final_low": c["low"], "final_high": c["high"], "splits": splits, "merges": merges,
            "timing": "host clock around synchronous sph2_advance calls"}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    sc, desc = workload(args.workload)
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
        "config": {"workload": desc},
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
            "kind": "reference kernels (Solver.cu, unmodified, sm_103a) + its thrust sort, "
                    "CUDA events around whole steps"}


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

    # per-phase kernel durations (CUDA events on the solver's stream)
    phases = solver.profile_phases(sc.dt, max(1, min(args.profile_steps, args.steps)))
    solver.close()

    # end to end through the public API: create from host arrays, then per step
    # advance + positions read back into pinned host memory (sph_get_positions_async:
    # the copy of step k overlaps step k+1; two pinned buffers alternate), and a
    # final sync that waits for the last copy.
    pinned = [torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy() for _ in range(2)]
    barrier()
    t0 = time.perf_counter()
    s2 = Solver(sc.fluid, sc.boundary, sc.config)
    for k in range(args.steps):
        s2.advance(sc.dt, 1)
        s2.positions_async(pinned[k & 1])
    s2.sync()
    t1 = time.perf_counter()
    s2.close()
    e2e_s = replicas.max_over_ranks(t1 - t0, device="cuda")
    e2e = {"value": replicas.throughput(ws * n * args.steps, 1e3 * e2e_s), "unit": UNIT,
           "h2d_bytes_per_step": int(round((32 * n + 16 * nb) / args.steps)),
           "d2h_bytes_per_step": 12 * n}

    if rank != 0:
        if ws > 1:
            dist.destroy_process_group()
        return

    peak, peak_kind = measured_peaks()
    ncells = sc.config.grid.dims[0] * sc.config.grid.dims[1] * sc.config.grid.dims[2]
    btouch = boundary_touched(sc)
    force_bytes = 72 * n + 16 * ncells + 16 * btouch
    dens_bytes = 28 * n + 8 * ncells
    force_ms, dens_ms = phases["force"], phases["density"]
    achieved = dens_bytes / (dens_ms * 1e-3) / 1e9
    f_achieved = force_bytes / (force_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": "density_kernel (the dominant kernel)",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": f"{peak_kind} hbm_gbs",
                "traffic": committed_traffic("density_kernel", args.workload),
                "algorithmic_bytes_per_launch": dens_bytes,
                "note": "density and force are FP32-issue / load-latency bound (~216 candidate "
                        "tests per particle); HBM fraction by compulsory bytes",
                "force_kernel": {"ms": force_ms, "achieved": f_achieved, "frac": f_achieved / peak,
                                 "algorithmic_bytes_per_launch": force_bytes,
                                 "traffic": committed_traffic("force_kernel", args.workload)},
                "phase_ms": phases}
    passes = sort_passes_for(sc.config.grid)
    # kernels per step: from 131,072 particles the step sorts coherently (keys and
    # flags, offsets, compaction, digit offsets, the passes, placement, cell
    # ranges), below from scratch (hash, digit offsets, the passes, gather);
    # then density and force
    coherent = sc.fluid.num_particles >= 131072
    launches = ((8 if coherent else 5) + passes) * args.steps
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded dam break)",
        "config": {"workload": desc, "parallelism": f"replicas x{ws}" if ws > 1 else "single GPU",
                   "l2": "working set ~0.3 GB > 129 MB L2 (no flush needed)"},
        "clocks": clk, "e2e": e2e, "gpu_launches": launches, "roofline": roofline,
    }
    if ws == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(sc, args.cpu_seconds)
    if ws == 1 and not args.no_extras:
        line["batched"] = measure_batched(args.batched_steps)
        line["adjoint"] = measure_adjoint()
        line["batched_adjoint"] = measure_batched_adjoint()
        line["two_scale"] = measure_two_scale()
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
