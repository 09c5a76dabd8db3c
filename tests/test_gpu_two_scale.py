"""Two-scale parity: the CUDA path (sph2_* C ABI) against the FP64 oracle.

From an identical state (the GPU's FP32 state fed to the oracle), one step:
  * sorted order, same-population, complementary and boundary neighbour
    counts of both populations: bit-exact;
  * densities <= 1e-5 relative per particle, accelerations <= 1e-5 max-norm
    relative;
  * split, merge, removal and fade-in counts, the next populations' sizes,
    states, blend coefficients, group ids and persistent ids: bit-exact;
  * next positions and velocities within FP32 tolerance.
"""
import numpy as np
import pytest

from oracle.oracle_ts import TSRollout
from sph2s_final_gb300._abi import SphError
from sph2s_final_gb300 import scenes
from sph2s_final_gb300.two_scale import HIGH, LOW, Solver2

pytestmark = pytest.mark.gpu

RHO_TOL = 1e-5
ACC_TOL = 1e-5


def oracle_from_gpu(s, sc):
    pops = [s.state(LOW), s.state(HIGH)]
    nl, nh = s.next_ids()
    ro = TSRollout(sc.config, sc.boundary.positions, pops, group_base=s.counts()["groups"],
                   pid_base=[nl, nh])
    return ro, pops


def check_step(s, sc):
    """Compares one step of GPU and oracle from the GPU's current state."""
    ro, pre = oracle_from_gpu(s, sc)
    dbg = [s.debug_step_fields(LOW), s.debug_step_fields(HIGH)]
    of = ro.step_fields(sc.dt)  # the oracle's step (also advances it)
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
    return ro.last_stats()


@pytest.fixture(scope="module")
def small():
    return scenes.two_scale_dam_break(1 / 32, dt=1e-4)


def test_first_step_splits_the_slab(small):
    with Solver2(small.low, None, small.boundary, small.config) as s:
        st = check_step(s, small)
        assert st["splits"] > 0
        assert s.counts()["high"] == 8 * st["splits"]


def test_capacity_overflow_is_reported_and_the_device_stays_usable(small):
    """A HIGH capacity below the first step's children: the step reports
    SPH_E_CAPACITY (the device error word comes back with the step's counts),
    the population is cut at its capacity (every write is checked against it),
    and a fresh solver on the same device then steps as the oracle does."""
    with Solver2(small.low, None, small.boundary, small.config, capacity_high=64) as s:
        with pytest.raises(SphError, match="SPH_E_CAPACITY"):
            s.advance(small.dt, 1)
        assert s.counts()["high"] <= 64
    with Solver2(small.low, None, small.boundary, small.config) as s:
        assert check_step(s, small)["splits"] > 8


def test_fading_and_removal_steps_match(small):
    """Steps 1..3, then around step 80 where split parents reach lambda 0."""
    with Solver2(small.low, None, small.boundary, small.config) as s:
        s.advance(small.dt, 1)
        for _ in range(3):
            check_step(s, small)
        s.advance(small.dt, 75)
        seen_removal = False
        for _ in range(4):
            st = check_step(s, small)
            seen_removal |= st["removed_low"] > 0
        assert seen_removal


def test_merge_path_matches():
    """A slab that the fine particles leave quickly: merges occur and match."""
    sc = scenes.two_scale_dam_break(1 / 32, dt=2e-4, slab=(0.40, 0.485), blend_increment=0.25)
    with Solver2(sc.low, None, sc.boundary, sc.config) as s:
        merges = 0
        s.advance(sc.dt, 44)
        for k in range(24):
            st = check_step(s, sc)
            merges += st["merges"]
        assert merges > 0


SLAB_RUNS = {
    # a narrow slab that fine particles cross both ways: every event occurs
    "crossing": (dict(spacing=1 / 32, dt=2e-4, slab=(0.40, 0.485), blend_increment=0.25),
                 ("splits", "merges", "removed_low", "removed_high", "faded_in_low",
                  "faded_in_high")),
    # the 262,144-particle two-scale configuration's slab 0.35 < x < 0.65 and
    # blend increment 0.0125 at 32,768 coarse particles (dt scaled with h)
    "c2_slab": (dict(spacing=1 / 64, dt=5e-5), ("splits", "removed_low", "faded_in_high")),
}


@pytest.mark.parametrize("run", sorted(SLAB_RUNS))
def test_split_merge_counts_every_step_for_1000_steps(run):
    """1,000 consecutive steps: before every step the oracle takes the GPU's
    state; after it the split, merge, removal and fade-in counts, population
    sizes, persistent ids, states, blend coefficients and group ids match bit
    for bit."""
    kw, seen = SLAB_RUNS[run]
    kw = dict(kw)
    sc = scenes.two_scale_dam_break(kw.pop("spacing"), **kw)
    totals = dict.fromkeys(("splits", "merges", "removed_low", "removed_high", "faded_in_low",
                            "faded_in_high"), 0)
    with Solver2(sc.low, None, sc.boundary, sc.config) as s:
        for k in range(1000):
            ro, _ = oracle_from_gpu(s, sc)
            ro.advance(sc.dt, 1)
            s.advance(sc.dt, 1)
            st = s.last_stats()
            assert st == ro.last_stats(), k
            c, oc = s.counts(), ro.counts()
            assert (c["low"], c["high"], c["groups"]) == (oc["low"], oc["high"], oc["groups"]), k
            for r in (LOW, HIGH):
                g, o = s.state(r), ro.state(r)
                for key in ("ids", "state", "group", "lam"):
                    np.testing.assert_array_equal(g[key], o[key], err_msg=f"step {k} {key}")
            ro.close()
            for key, v in st.items():
                totals[key] += v
    assert all(totals[key] > 0 for key in seen), totals


def test_without_refinement_is_two_independent_populations(small):
    cfg = small.config
    cfg.refine_axis = -1
    rng = np.random.default_rng(4)
    high = rng.uniform(0.55, 0.7, (3000, 3)).astype(np.float32)
    with Solver2(small.low, high, small.boundary, cfg) as s:
        for _ in range(3):
            st = check_step(s, small)
            assert st["splits"] == 0 and st["merges"] == 0
    cfg.refine_axis = 0


def test_c2_scale_first_steps():
    """262,144 coarse particles, the slab 0.35 < x < 0.65: the first steps at full size."""
    sc = scenes.two_scale_dam_break(1 / 128)
    assert sc.low.num_particles == 262144 and sc.boundary.num_particles == 530920
    with Solver2(sc.low, None, sc.boundary, sc.config) as s:
        st = check_step(s, sc)
        assert st["splits"] > 70000
        check_step(s, sc)
