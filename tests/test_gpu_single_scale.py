"""Single-scale parity: the CUDA path (through the C ABI) against the FP64 oracle.

Bars:
  * cell keys, sorted order, cell ranges, neighbour counts: bit-exact;
  * per-step density: |rho - rho_oracle| / rho_oracle <= 1e-5 per particle;
  * per-step acceleration: max_i |a_i - a_oracle,i| / max_i |a_oracle,i| <= 1e-5;
  * 1,000-step rollouts (chaotic): mean and max density, kinetic energy and
    centre of mass within 1 % of the FP64 rollout.
Per-step checks start from the GPU's own FP32 state, fed to the oracle.
"""
import numpy as np
import pytest

from oracle import oracle as O
from sph2s_final_gb300 import scenes
from sph2s_final_gb300._abi import SPH_E_TIMEOUT, SphError
from sph2s_final_gb300.solver import Grid, ParticleData, Solver, SolverConfiguration

pytestmark = pytest.mark.gpu

RHO_TOL = 1e-5
ACC_TOL = 1e-5


def check_step_against_oracle(solver, cfg, boundary_xyz, acc_tol=ACC_TOL, rho_tol=RHO_TOL):
    x = solver.positions("sorted")
    v = solver.velocities("sorted")
    ids = solver.ids()
    d = solver.debug_step_fields()
    nb = O.neighborhood(cfg.grid, x)
    perm = nb["perm"]
    np.testing.assert_array_equal(d["keys"], nb["keys"])
    np.testing.assert_array_equal(d["ids"], ids[perm])
    np.testing.assert_array_equal(d["cell_start"], nb["cell_start"])
    np.testing.assert_array_equal(d["cell_end"], nb["cell_end"])
    f = O.ss_fields(cfg, x, v, boundary_xyz)
    np.testing.assert_array_equal(d["nbr_fluid"], f["nbr_fluid"][perm])
    np.testing.assert_array_equal(d["nbr_boundary"], f["nbr_boundary"][perm])
    rho_o = f["rho"][perm]
    rel = np.abs(d["rho"] - rho_o) / np.abs(rho_o)
    assert rel.max() <= rho_tol, rel.max()
    acc_o = f["acc"][perm]
    err = np.abs(d["acc"] - acc_o).max() / np.abs(acc_o).max()
    assert err <= acc_tol, err
    return {"rho_rel_max": float(rel.max()), "acc_rel_maxnorm": float(err)}


@pytest.fixture(scope="module")
def c0():
    return scenes.dam_break(1 / 64)


def test_c0_initial_step_parity(c0):
    with Solver(c0.fluid, c0.boundary, c0.config) as s:
        check_step_against_oracle(s, c0.config, c0.boundary.positions)


def test_c0_parity_after_steps_with_random_velocities(c0):
    rng = np.random.default_rng(3)
    v0 = rng.normal(0, 0.1, (c0.fluid.num_particles, 3)).astype(np.float32)
    with Solver(c0.fluid, c0.boundary, c0.config, velocities=v0) as s:
        check_step_against_oracle(s, c0.config, c0.boundary.positions)
        for _ in range(3):
            s.advance(c0.dt, 50)
            check_step_against_oracle(s, c0.config, c0.boundary.positions)


def test_one_step_state_matches_oracle_step(c0):
    """A full step (sort, density, force, integrate) from identical state."""
    with Solver(c0.fluid, c0.boundary, c0.config) as s:
        s.advance(c0.dt, 5)
        x, v, ids = s.positions(), s.velocities(), s.ids()
        ro = O.SSRollout(c0.config, x, c0.boundary.positions, v)
        ro.advance(c0.dt, 1)
        s.advance(c0.dt, 1)
        st = ro.state()
        np.testing.assert_array_equal(s.ids(), ids[st["ids"]])
        dv = np.abs(s.velocities() - st["v"]).max()
        dx = np.abs(s.positions() - st["x"]).max()
        assert dv <= 1e-5 * max(1.0, np.abs(st["v"]).max()), dv
        assert dx <= 1e-6, dx
        np.testing.assert_allclose(s.densities(), st["rho"], rtol=RHO_TOL)


def test_by_id_readback_roundtrip(c0):
    with Solver(c0.fluid, c0.boundary, c0.config) as s:
        np.testing.assert_array_equal(s.positions("by_id"), c0.fluid.positions)
        s.advance(c0.dt, 3)
        ids = s.ids()
        assert np.array_equal(np.sort(ids), np.arange(c0.fluid.num_particles))
        xs, xb = s.positions("sorted"), s.positions("by_id")
        np.testing.assert_array_equal(xb[ids], xs)
        rs, rb = s.densities("sorted"), s.densities("by_id")
        np.testing.assert_array_equal(rb[ids], rs)
        vb = s.velocities("by_id")
        s.set_velocities(vb, "by_id")
        np.testing.assert_array_equal(s.velocities("by_id"), vb)


@pytest.mark.slow
def test_c0_rollout_1000_steps_statistics(c0):
    steps = 1000
    with Solver(c0.fluid, c0.boundary, c0.config) as s:
        s.advance(c0.dt, steps)
        x, v, rho = s.positions(), s.velocities(), s.densities()
    ro = O.SSRollout(c0.config, c0.fluid.positions, c0.boundary.positions)
    ro.advance(c0.dt, steps)
    st = ro.state()
    assert np.isfinite(x).all() and np.isfinite(st["x"]).all()
    rel = lambda a, b: abs(a - b) / abs(b)
    assert rel(rho.mean(), st["rho"].mean()) <= 0.01
    assert rel(rho.max(), st["rho"].max()) <= 0.01
    ke_g = 0.5 * (v.astype(np.float64) ** 2).sum()
    ke_o = 0.5 * (st["v"] ** 2).sum()
    assert rel(ke_g, ke_o) <= 0.01
    com_g, com_o = x.astype(np.float64).mean(0), st["x"].mean(0)
    assert np.linalg.norm(com_g - com_o) / np.linalg.norm(com_o) <= 0.01


def test_edge_cases_empty_single_clamped_coincident():
    g = Grid.make_grid((0, 0, 0), (1, 1, 1), 0.125)
    cfg = SolverConfiguration.direct(0.125, 0.01, 1000.0, 30.0, 5.0, 88.1472, 0.8, g)
    empty = np.zeros((0, 3), np.float32)
    # empty fluid, empty boundary
    with Solver(ParticleData(empty), ParticleData(empty), cfg) as s:
        s.advance(1e-4, 3)
        assert s.positions().shape == (0, 3)
    # single particle, no boundary: free fall
    with Solver(ParticleData(np.array([[0.5, 0.5, 0.5]], np.float32)), None, cfg) as s:
        s.advance(1e-3, 10)
        v = s.velocities()
        np.testing.assert_allclose(v[0], [0, -9.81 * 1e-2, 0], rtol=1e-5, atol=1e-7)
    # particles outside the grid (clamped into edge cells), coincident pairs, a crowded cell
    rng = np.random.default_rng(11)
    x = np.concatenate([
        rng.uniform(-0.3, 1.3, (400, 3)),
        np.repeat(rng.uniform(0, 1, (20, 3)), 3, axis=0),
        rng.uniform(0.5, 0.56, (300, 3)),
    ]).astype(np.float32)
    b = rng.uniform(-0.2, 1.2, (500, 3)).astype(np.float32)
    with Solver(ParticleData(x), ParticleData(b), cfg) as s:
        check_step_against_oracle(s, cfg, b)
        s.advance(1e-5, 5)
        check_step_against_oracle(s, cfg, b)


def test_boundary_depth_cut_with_particles_outside_the_box():
    """The boundary scan of a cell stops at the first boundary particle deeper
    outside the grid's box than the fluid particle can reach.  A five-layer
    shell around the box (the layers outside the grid pile up in the edge
    cells) and fluid particles outside the box, up to 2.5 h deep, beside
    faces, edges and corners: boundary neighbour counts bit-exact and
    accelerations as the full scan gives them (the oracle)."""
    h = 1.0 / 16
    g = Grid.make_grid((0, 0, 0), (1, 1, 1), h)
    cfg = SolverConfiguration.direct(h, (h / 2) ** 3 * 1000, 1000.0, 30.0, 5.0, 88.1472, 0.8, g)
    shell = ParticleData.create_particle_box_canvas(Grid.make_grid((0, 0, 0), (1, 1, 1), h / 2), 5)
    rng = np.random.default_rng(5)
    inside = rng.uniform(0.0, 1.0, (1500, 3))
    depth = rng.uniform(0.0, 2.5 * h, (900, 1))
    outside = rng.uniform(0.0, 1.0, (900, 3))
    for k in range(900):  # push 1, 2 or 3 coordinates out through a face, edge or corner
        axes = rng.choice(3, size=1 + k % 3, replace=False)
        for a in axes:
            outside[k, a] = -depth[k, 0] if rng.random() < 0.5 else 1.0 + depth[k, 0]
    x = np.concatenate([inside, outside]).astype(np.float32)
    with Solver(ParticleData(x), shell, cfg) as s:
        check_step_against_oracle(s, cfg, shell.positions)
        d = s.debug_step_fields()
        assert d["nbr_boundary"].max() > 20  # particles deep in the shell


def test_boundary_scan_without_depth_cut_far_from_the_origin():
    """A grid at x ~ 1000 with h = 1/16: the depth classes (h/16) would sit
    near the coordinates' rounding, so the presort leaves them out and every
    boundary cell is scanned in full; parity as everywhere else."""
    h = 1.0 / 16
    o = (1000.0, 1000.0, 1000.0)
    g = Grid.make_grid(o, (1001.0, 1001.0, 1001.0), h)
    cfg = SolverConfiguration.direct(h, (h / 2) ** 3 * 1000, 1000.0, 30.0, 5.0, 88.1472, 0.8, g)
    shell = ParticleData.create_particle_box_canvas(Grid.make_grid(o, (1001.0, 1001.0, 1001.0), h / 2), 3)
    rng = np.random.default_rng(6)
    x = (np.float32(1000.0) + rng.uniform(-0.1, 1.1, (1500, 3))).astype(np.float32)
    with Solver(ParticleData(x), shell, cfg) as s:
        check_step_against_oracle(s, cfg, shell.positions)


def test_non_cubic_grid_and_non_power_of_two_dims():
    g = Grid.make_grid((-0.1, -0.1, -0.2), (1.7, 1.6, 0.6), 0.0203)
    cfg = SolverConfiguration.direct(0.0203, 0.0075 ** 3 * 1000, 1000.0, 30.0, 5.0, 88.1472, 0.8, g)
    pg = Grid.make_grid((0.04, 0.04, 0.0), (0.35, 0.75, 0.4), 0.0075)
    fluid = ParticleData.create_particle_box(pg)
    bg = Grid.make_grid((0.0, 0.0, -0.1), (1.6, 1.5, 0.5), 0.015)
    bnd = ParticleData.create_particle_box_canvas(bg, 2)
    with Solver(fluid, bnd, cfg) as s:
        check_step_against_oracle(s, cfg, bnd.positions)
        s.advance(1e-4, 20)
        check_step_against_oracle(s, cfg, bnd.positions)


def test_lookback_timeout_reports_error_and_recovers(c0):
    with Solver(c0.fluid, c0.boundary, c0.config) as s:
        s.debug_force_lookback_timeout(True)
        s.advance(c0.dt, 1)
        with pytest.raises(SphError) as e:
            s.sync()
        assert e.value.code == SPH_E_TIMEOUT
        s.debug_force_lookback_timeout(False)
    with Solver(c0.fluid, c0.boundary, c0.config) as s:  # a fresh handle is unaffected
        s.advance(c0.dt, 2)
        s.sync()


@pytest.mark.parametrize("spacing,sigma", [(64, 0.1), (64, 3.0), (64, 30.0), (128, 10.0)])
def test_coherent_sort_equals_sorting_from_scratch(c0, spacing, sigma):
    """The step sorts only the particles that changed cell since the last step
    and merges them into the rest; the permutation must equal a from-scratch
    stable sort every step, from a few movers per step (sigma 0.1 m/s) to most
    particles (30 m/s: about h/10 per step), including the first step, where
    every particle counts as moved.  At 262,144 particles and 10 m/s more than
    12,288 particles change cell per step, past what one block sorts."""
    sc = c0 if spacing == 64 else scenes.dam_break(1 / spacing)
    rng = np.random.default_rng(11)
    v0 = rng.normal(0, sigma, (sc.fluid.num_particles, 3)).astype(np.float32)
    runs = []
    for mode in ("coherent", "full"):
        s = Solver(sc.fluid, sc.boundary, sc.config, velocities=v0)
        s.debug_sort_mode(mode)
        runs.append(s)
    try:
        for k in range(6):
            for s in runs:
                s.advance(sc.dt, 1 if k == 0 else 25)
            a, b = runs
            np.testing.assert_array_equal(a.ids(), b.ids())
            np.testing.assert_array_equal(a.positions("sorted"), b.positions("sorted"))
            np.testing.assert_array_equal(a.velocities("sorted"), b.velocities("sorted"))
            np.testing.assert_array_equal(a.densities("sorted"), b.densities("sorted"))
        if spacing == 64 and sigma <= 3.0:  # structure and fields against the oracle
            assert np.isfinite(runs[0].positions("sorted")).all()
            check_step_against_oracle(runs[0], sc.config, sc.boundary.positions)
    finally:
        for s in runs:
            s.close()


def test_c1_full_size_structure_and_fields():
    """2,097,152 particles: bit-exact structure and per-step fields at full size."""
    c1 = scenes.dam_break(1 / 256)
    assert c1.fluid.num_particles == 2097152 and c1.boundary.num_particles == 2043880
    with Solver(c1.fluid, c1.boundary, c1.config) as s:
        s.advance(c1.dt, 2)
        r = check_step_against_oracle(s, c1.config, c1.boundary.positions)
        d = s.debug_step_fields()
        assert np.all(np.diff(d["keys"].astype(np.int64)) >= 0)
        assert np.array_equal(np.sort(d["ids"]), np.arange(c1.fluid.num_particles))
    print(r)
