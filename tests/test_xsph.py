"""XSPH integrator variant (integrateXSPHD, SPH2S_FINAL_SINGLE_SCALE/Solver.cu:757-853,
with the per-component correction).

CPU: the oracle's XSPH step against a direct numpy restatement of the formula
and, at eps = 0, against its own symplectic Euler step.  GPU (through the C
ABI): one step from an identical state against the oracle, including
coincident particles (picked up from the home cell) and a crowded particle
whose list overflows (stencil rescan), and bit-identical resume of an XSPH
solver from a saved state.
"""
import numpy as np
import pytest

from oracle import oracle as O
from sph2s_final_gb300 import scenes
from sph2s_final_gb300.solver import Grid, ParticleData, Solver, SolverConfiguration


def xsph_config(eps):
    sc = scenes.dam_break(1 / 32)
    sc.config.xsph_coeff = eps
    return sc


def test_oracle_xsph_at_zero_eps_is_the_euler_step():
    sc = xsph_config(0.0)
    v = np.random.default_rng(1).normal(0, 0.2, (sc.fluid.num_particles, 3)).astype(np.float32)
    xo, vo = O.ss_xsph_step(sc.config, sc.fluid.positions, v, sc.boundary.positions, sc.dt, 0.0)
    ro = O.SSRollout(sc.config, sc.fluid.positions, sc.boundary.positions, v)
    ro.advance(sc.dt, 1)
    st = ro.state()
    np.testing.assert_allclose(xo[st["ids"]], st["x"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(vo[st["ids"]], st["v"], rtol=0, atol=1e-13)


def test_oracle_xsph_matches_the_formula():
    """Random cloud, no pair within 1e-4 h of the cutoff (so the FP32 predicate
    equals the exact one); the correction restated with numpy in double."""
    rng = np.random.default_rng(7)
    g = Grid.make_grid((0, 0, 0), (1, 1, 1), 0.1)
    cfg = SolverConfiguration.direct(0.1, 0.02, 1000.0, 30.0, 5.0, 88.1472, 0.8, g)
    h = np.float64(np.float32(0.1))
    while True:
        x = rng.uniform(0.3, 0.6, (60, 3)).astype(np.float32)
        d = np.sqrt(((x[:, None, :].astype(np.float64) - x[None]) ** 2).sum(-1))
        if np.abs(d - h).min() > 1e-4 * h:
            break
    v = rng.normal(0, 0.3, (60, 3)).astype(np.float32)
    eps, dt = 0.4, 1e-3
    f = O.ss_fields(cfg, x, v, np.zeros((0, 3), np.float32))
    vp = v.astype(np.float64) + dt * f["acc"]
    poly6 = 315.0 / (64.0 * np.pi * h ** 9)
    w = np.where(d < h, poly6 * (h * h - d * d) ** 3, 0.0) * float(np.float32(0.02)) / f["rho"][None]
    corr = (w[:, :, None] * (vp[None, :, :] - vp[:, None, :])).sum(1)
    v2 = vp + eps * corr
    x2 = x.astype(np.float64) + dt * v2
    xo, vo = O.ss_xsph_step(cfg, x, v, np.zeros((0, 3), np.float32), dt, eps)
    np.testing.assert_allclose(vo, v2, rtol=0, atol=1e-12)
    np.testing.assert_allclose(xo, x2, rtol=0, atol=1e-14)


def gpu_vs_oracle(cfg, x, v, b, dt, eps, steps_before=0):
    cfg.xsph_coeff = eps
    with Solver(ParticleData(x), ParticleData(b), cfg, velocities=v) as s:
        s.set_integrator("xsph")
        s.advance(dt, steps_before)
        x0, v0 = s.positions("by_id"), s.velocities("by_id")
        s.advance(dt, 1)
        xg, vg = s.positions("by_id"), s.velocities("by_id")
    xo, vo = O.ss_xsph_step(cfg, x0, v0, b, dt, eps)
    dx = np.abs(xg - xo).max()
    dv = np.abs(vg - vo).max() / max(1.0, np.abs(vo).max())
    return dx, dv


@pytest.mark.gpu
def test_gpu_xsph_step_matches_oracle():
    sc = xsph_config(0.5)
    v = np.random.default_rng(2).normal(0, 0.2, (sc.fluid.num_particles, 3)).astype(np.float32)
    dx, dv = gpu_vs_oracle(sc.config, sc.fluid.positions, v, sc.boundary.positions, sc.dt, 0.5,
                           steps_before=5)
    assert dx <= 1e-6 and dv <= 1e-5, (dx, dv)


@pytest.mark.gpu
def test_gpu_xsph_coincident_and_crowded_particles():
    """Two coincident pairs (distance 0, different velocities) and a ball of 90
    particles around one point (more than 64 neighbours: stencil rescan)."""
    sc = scenes.small_scene(8)
    rng = np.random.default_rng(3)
    x = sc.fluid.positions.copy()
    x[10] = x[11]
    x[200] = x[201]
    ball = (np.float32([0.7, 0.7, 0.7]) + rng.uniform(-0.02, 0.02, (90, 3))).astype(np.float32)
    x = np.concatenate([x, ball])
    v = rng.normal(0, 0.3, x.shape).astype(np.float32)
    dx, dv = gpu_vs_oracle(sc.config, x, v, sc.boundary.positions, sc.dt, 0.7)
    assert dx <= 1e-6 and dv <= 1e-5, (dx, dv)


@pytest.mark.gpu
def test_gpu_xsph_resume_is_bit_identical():
    sc = xsph_config(0.3)
    with Solver(sc.fluid, sc.boundary, sc.config) as a:
        a.set_integrator("xsph")
        a.advance(sc.dt, 10)
        with Solver.from_state(a.save_state()) as b:
            a.advance(sc.dt, 20)
            b.advance(sc.dt, 20)
            np.testing.assert_array_equal(a.positions(), b.positions())
            np.testing.assert_array_equal(a.velocities(), b.velocities())


@pytest.mark.gpu
def test_gpu_switching_back_to_euler():
    sc = xsph_config(0.3)
    with Solver(sc.fluid, sc.boundary, sc.config) as a, \
            Solver(sc.fluid, sc.boundary, sc.config) as b:
        a.set_integrator("xsph")
        a.set_integrator("symplectic_euler")
        a.advance(sc.dt, 5)
        b.advance(sc.dt, 5)
        np.testing.assert_array_equal(a.positions(), b.positions())
