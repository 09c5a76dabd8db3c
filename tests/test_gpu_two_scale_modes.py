"""Two-scale modes beyond the slab-triggered blended solver, through the C ABI
against the FP64 oracle from identical state:
  * coupled fixed populations (SPH2S_FINAL_TWO_SCALE_COUPLED): neighbour
    counts bit-exact, densities / accelerations <= 1e-5, populations, states
    and blend coefficients unchanged; with an empty fine population it is the
    single-scale step;
  * the colour / energy output (dColorValues) of both populations;
  * the surface split trigger (density deficit): split, merge, removal and
    fade-in counts and the next populations bit-exact.
"""
import ctypes as C
import struct

import numpy as np
import pytest

from oracle.oracle_ts import TSRollout
from sph2s_final_gb300 import scenes
from sph2s_final_gb300._abi import sph_config2
from sph2s_final_gb300.solver import Solver
from sph2s_final_gb300.two_scale import HIGH, LOW, Solver2

pytestmark = pytest.mark.gpu

RHO_TOL = 1e-5
ACC_TOL = 1e-5


def oracle_from(s, sc):
    pops = [s.state(LOW), s.state(HIGH)]
    nl, nh = s.next_ids()
    return TSRollout(sc.config, sc.boundary.positions, pops, group_base=s.counts()["groups"],
                     pid_base=[nl, nh])


def compare_step(s, sc, surf_rho=None):
    """One step of GPU and oracle from the GPU's state; returns the oracle fields."""
    ro = oracle_from(s, sc)
    dbg = [s.debug_step_fields(LOW), s.debug_step_fields(HIGH)]
    of = ro.step_fields(sc.dt)
    for r in (LOW, HIGH):
        d = dbg[r]
        if d["ids"].size == 0:
            continue
        np.testing.assert_array_equal(d["ids"], of["ids"][r])
        np.testing.assert_array_equal(d["nbr_same"], of["nbr_same"][r])
        np.testing.assert_array_equal(d["nbr_compl"], of["nbr_compl"][r])
        np.testing.assert_array_equal(d["nbr_boundary"], of["nbr_bnd"][r])
        rel = np.abs(d["rho"] - of["rho"][r]) / np.abs(of["rho"][r])
        assert rel.max() <= RHO_TOL, (r, rel.max())
        err = np.abs(d["acc"] - of["acc"][r]).max() / np.abs(of["acc"][r]).max()
        assert err <= ACC_TOL, (r, err)
        if surf_rho is not None:  # a density this close to the trigger could flip a decision
            near = np.abs(of["rho"][r] / surf_rho - 1.0) < 1e-5
            assert not near.any(), "density within 1e-5 of the surface trigger"
    s.advance(sc.dt, 1)
    assert s.last_stats() == ro.last_stats()
    c, oc = s.counts(), ro.counts()
    assert (c["low"], c["high"], c["groups"]) == (oc["low"], oc["high"], oc["groups"])
    for r in (LOW, HIGH):
        g, o = s.state(r), ro.state(r)
        np.testing.assert_array_equal(g["ids"], o["ids"])
        np.testing.assert_array_equal(g["state"], o["state"])
        np.testing.assert_array_equal(g["group"], o["group"])
        np.testing.assert_array_equal(g["lam"], o["lam"])
        if g["x"].size:
            assert np.abs(g["x"] - o["x"]).max() <= 2e-6
            vs = max(1.0, np.abs(o["v"]).max())
            assert np.abs(g["v"] - o["v"]).max() <= 1e-4 * vs
    return of, ro.last_stats()


def coupled_scene():
    sc = scenes.two_scale_dam_break(1 / 32, dt=1e-4)
    sc.config.mode = 1  # SPH2_MODE_COUPLED
    rng = np.random.default_rng(8)
    high = rng.uniform(0.05, 0.3, (4000, 3)).astype(np.float32)
    return sc, high


def test_coupled_mode_matches_oracle_and_keeps_populations():
    sc, high = coupled_scene()
    with Solver2(sc.low, high, sc.boundary, sc.config) as s:
        n0 = s.counts()
        s.advance(sc.dt, 3)
        for _ in range(3):
            _, st = compare_step(s, sc)
            assert st == {"splits": 0, "merges": 0, "removed_low": 0, "removed_high": 0,
                          "faded_in_low": 0, "faded_in_high": 0}
        assert s.counts() == n0
        hs = s.state(HIGH)
        assert (hs["state"] == 4).all() and (hs["lam"] == 1.0).all()


def word_fnv1a(data: bytes) -> int:
    h = 0xcbf29ce484222325
    pad = data + b"\0" * (-len(data) % 8)
    for (w,) in struct.iter_unpack("<Q", pad):
        h = ((h ^ w) * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
    return h


def with_high_lambda(state: bytes, lam: float) -> bytes:
    """A two-scale state (layout in csrc/two_scale.cu) with every HIGH blend
    coefficient replaced, re-checksummed."""
    b = bytearray(state[:-8])
    off = 24 + C.sizeof(sph_config2)
    n_low, n_high = struct.unpack_from("<II", b, off)
    off += 24 + 16 + 40 * n_low  # counts, capacities, the LOW arrays
    vel = np.frombuffer(b, np.float32, 4 * n_high, off + 16 * n_high).reshape(n_high, 4).copy()
    vel[:, 3] = lam
    b[off + 16 * n_high: off + 32 * n_high] = vel.tobytes()
    return bytes(b) + struct.pack("<Q", word_fnv1a(bytes(b)))


def test_coupled_mode_ignores_blend_coefficients():
    """Coupled sums are unweighted: HIGH blend coefficients of 0.3 instead of 1
    change nothing (the same state in blended mode does change)."""
    sc, high = coupled_scene()
    with Solver2(sc.low, high, sc.boundary, sc.config) as a:
        a.advance(sc.dt, 2)
        st = a.save_state()
        with Solver2.from_state(with_high_lambda(st, 0.3)) as b:
            assert (b.state(HIGH)["lam"] == np.float32(0.3)).all()
            a.advance(sc.dt, 3)
            b.advance(sc.dt, 3)
            for r in (LOW, HIGH):
                np.testing.assert_array_equal(a.state(r)["x"], b.state(r)["x"])
                np.testing.assert_array_equal(a.state(r)["v"], b.state(r)["v"])
    sc.config.mode = 0
    sc.config.refine_axis = -1
    with Solver2(sc.low, high, sc.boundary, sc.config) as a:
        a.advance(sc.dt, 2)
        with Solver2.from_state(with_high_lambda(a.save_state(), 0.3)) as b:
            a.advance(sc.dt, 3)
            b.advance(sc.dt, 3)
            assert not np.array_equal(a.state(LOW)["x"], b.state(LOW)["x"])


def test_coupled_mode_without_fine_particles_is_the_single_scale_step():
    sc = scenes.two_scale_dam_break(1 / 32, dt=1e-4)
    sc.config.mode = 1
    ss = scenes.dam_break(1 / 32, dt=1e-4)
    with Solver2(sc.low, None, sc.boundary, sc.config) as a, \
            Solver(sc.low, sc.boundary, ss.config) as b:
        a.advance(sc.dt, 5)
        b.advance(sc.dt, 5)
        st = a.state(LOW)
        order = np.argsort(st["ids"])
        np.testing.assert_allclose(st["x"][order], b.positions("by_id"), rtol=0, atol=1e-6)
        np.testing.assert_allclose(st["v"][order], b.velocities("by_id"), rtol=0, atol=1e-4)


def test_colour_output_matches_oracle():
    sc = scenes.two_scale_dam_break(1 / 32, dt=1e-4)
    with Solver2(sc.low, None, sc.boundary, sc.config) as s:
        s.set_color_output(True)
        s.advance(sc.dt, 6)  # splits have produced a fine population
        assert s.counts()["high"] > 0
        ro = oracle_from(s, sc)
        of = ro.step_fields(sc.dt)
        s.advance(sc.dt, 1)
        for r in (LOW, HIGH):
            col, ids = s.colors(r)
            np.testing.assert_array_equal(ids, of["ids"][r])
            ok = np.abs(of["dist_cm"][r] - 0.0025) > 1e-6
            assert ok.mean() > 0.99
            err = np.abs(col[ok] - of["colour"][r][ok]).max()
            assert err <= 1e-4, (r, err)
            if r == LOW:  # both branches of the colour rule occur
                assert (col == np.float32(0.3)).any() and (col != np.float32(0.3)).any()
        s.set_color_output(False)
        s.advance(sc.dt, 1)
        assert s.colors(LOW)[0].size == 0


def test_surface_trigger_split_and_merge_match_oracle():
    sc = scenes.two_scale_dam_break(1 / 32, dt=2e-4, blend_increment=0.25)
    sc.config.split_trigger = 1  # SPH2_SPLIT_SURFACE
    sc.config.surface_density = 900.0
    with Solver2(sc.low, None, sc.boundary, sc.config) as s:
        splits = merges = 0
        for k in range(40):
            if k % 4 == 0:
                _, st = compare_step(s, sc, surf_rho=900.0)
            else:
                s.advance(sc.dt, 1)
                st = s.last_stats()
            splits += st["splits"]
            merges += st["merges"]
        assert splits > 0
        # split particles are LOW particles below the surface density
        assert s.counts()["high"] > 0


def test_surface_trigger_bad_density_rejected():
    from sph2s_final_gb300._abi import SphError
    sc = scenes.two_scale_dam_break(1 / 32)
    sc.config.split_trigger = 1
    sc.config.surface_density = 0.0
    with pytest.raises(SphError, match="SPH_E_INVALID"):
        Solver2(sc.low, None, sc.boundary, sc.config)
