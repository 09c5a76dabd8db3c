"""Headless state save / resume and frame records on the GPU.

A solver created from a saved state must continue bit for bit like the solver
it was saved from (the next sort is stable with respect to the stored order,
so the order is part of the state): positions, velocities, densities and
persistent ids after further steps are compared with array_equal, for the
single-scale step and for the two-scale step across splits, fades and merges.
"""
import numpy as np
import pytest

from sph2s_final_gb300 import scenes, state_io
from sph2s_final_gb300._abi import SphError
from sph2s_final_gb300.solver import ParticleData, Solver
from sph2s_final_gb300.two_scale import HIGH, LOW, Solver2

pytestmark = pytest.mark.gpu


def test_single_scale_resume_is_bit_identical(tmp_path):
    sc = scenes.dam_break(1 / 32)
    v0 = np.random.default_rng(5).normal(0, 0.1, (sc.fluid.num_particles, 3)).astype(np.float32)
    with Solver(sc.fluid, sc.boundary, sc.config, velocities=v0) as a:
        a.advance(sc.dt, 37)
        path = tmp_path / "state.bin"
        data = a.save_state(path)
        assert state_io.state_info(data)["step"] == 37 == a.step_count
        with Solver.from_state(path) as b:
            assert b.step_count == 37
            assert (b.num_fluid, b.num_boundary) == (a.num_fluid, a.num_boundary)
            assert b.save_state() == data  # save -> load -> save round trip
            a.advance(sc.dt, 50)
            b.advance(sc.dt, 50)
            np.testing.assert_array_equal(a.positions(), b.positions())
            np.testing.assert_array_equal(a.velocities(), b.velocities())
            np.testing.assert_array_equal(a.densities(), b.densities())
            np.testing.assert_array_equal(a.ids(), b.ids())
            assert b.step_count == 87


def test_single_scale_state_of_fresh_and_empty_solvers():
    sc = scenes.small_scene(6)
    with Solver(sc.fluid, sc.boundary, sc.config) as a:
        with Solver.from_state(a.save_state()) as b:
            a.advance(sc.dt, 3)
            b.advance(sc.dt, 3)
            np.testing.assert_array_equal(a.positions("by_id"), b.positions("by_id"))
    empty = scenes.small_scene(6)
    with Solver(ParticleData(np.zeros((0, 3), np.float32)), None, empty.config) as a:
        with Solver.from_state(a.save_state()) as b:
            assert b.num_fluid == 0 and b.num_boundary == 0


def test_corrupt_state_raises():
    sc = scenes.small_scene(6)
    with Solver(sc.fluid, sc.boundary, sc.config) as a:
        data = bytearray(a.save_state())
    data[len(data) // 2] ^= 1
    with pytest.raises(SphError, match="SPH_E_INVALID"):
        Solver.from_state(bytes(data))


def test_frames_record_positions_and_densities_by_id(tmp_path):
    sc = scenes.small_scene(8)
    path = tmp_path / "frames.bin"
    fields = state_io.FIELD_POSITIONS | state_io.FIELD_VELOCITIES | state_io.FIELD_DENSITIES
    want = []
    with Solver(sc.fluid, sc.boundary, sc.config) as s:
        for k in range(3):
            s.advance(sc.dt, 5)
            s.write_frame(path, fields, append=k > 0)
            want.append((s.positions("by_id"), s.velocities("by_id"), s.densities("by_id")))
        with pytest.raises(SphError, match="SPH_E_INVALID"):
            s.write_frame(path, state_io.FIELD_BLEND)
        with pytest.raises(SphError, match="SPH_E_IO"):
            s.write_frame(tmp_path / "missing_dir" / "f.bin")
    fr = state_io.read_frames(path)
    assert [f["step"] for f in fr] == [5, 10, 15]
    for f, (x, v, r) in zip(fr, want):
        np.testing.assert_array_equal(f["positions"], x)
        np.testing.assert_array_equal(f["velocities"], v)
        np.testing.assert_array_equal(f["densities"], r)


def ts_snapshot(s):
    return [s.state(LOW), s.state(HIGH)], s.counts(), s.next_ids(), s.last_stats()


def test_two_scale_resume_is_bit_identical_through_split_and_merge(tmp_path):
    sc = scenes.two_scale_dam_break(1 / 32, dt=2e-4, slab=(0.40, 0.485), blend_increment=0.25)
    with Solver2(sc.low, None, sc.boundary, sc.config) as a:
        a.advance(sc.dt, 30)
        assert a.counts()["high"] > 0 and a.counts()["groups"] > 0
        path = tmp_path / "ts.bin"
        data = a.save_state(path)
        with Solver2.from_state(path) as b:
            assert b.step_count == 30 and b.save_state() == data
            merges = 0
            for _ in range(40):
                a.advance(sc.dt, 1)
                b.advance(sc.dt, 1)
                pa, ca, ia, sa = ts_snapshot(a)
                pb, cb, ib, sb = ts_snapshot(b)
                assert (ca, ia, sa) == (cb, ib, sb)
                for r in (LOW, HIGH):
                    for k in ("x", "v", "lam", "state", "group", "ids"):
                        np.testing.assert_array_equal(pa[r][k], pb[r][k])
                merges += sa["merges"]
            assert merges > 0


def test_two_scale_frames(tmp_path):
    sc = scenes.two_scale_dam_break(1 / 32, dt=1e-4)
    path = tmp_path / "ts_frames.bin"
    with Solver2(sc.low, None, sc.boundary, sc.config) as s:
        s.advance(sc.dt, 2)
        s.write_frame(path, state_io.FIELD_POSITIONS | state_io.FIELD_BLEND, append=False)
        st = [s.state(LOW), s.state(HIGH)]
        with pytest.raises(SphError, match="SPH_E_INVALID"):
            s.write_frame(path, state_io.FIELD_DENSITIES)
    (f,) = state_io.read_frames(path)
    assert f["kind"] == 2 and f["step"] == 2 and f["high"]["n"] > 0
    for name, r in (("low", LOW), ("high", HIGH)):
        np.testing.assert_array_equal(f[name]["ids"], st[r]["ids"])
        np.testing.assert_array_equal(f[name]["positions"], st[r]["x"])
        np.testing.assert_array_equal(f[name]["lambda"], st[r]["lam"])
        np.testing.assert_array_equal(f[name]["state"], st[r]["state"])
