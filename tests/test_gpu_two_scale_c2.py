"""The 262,144-particle two-scale dam break (refinement slab 0.35 < x < 0.65,
blend increment 0.0125 per step, dt 2.5e-5) at full size over 1,000 steps.

Every step, from the GPU's own start-of-step state, the oracle's decision rules
(oracle/sph_oracle_ts.cpp or_ts_decide: slab split, group merge on the
fixed-point centroid, fade-out removal, fade-in completion; TS Solver.cu:
1229-1289) predict the step's split / merge / removal / fade-in counts and, by
persistent id, the state bits, blend coefficients and group ids every
surviving particle leaves the step with; the GPU's step must match them bit
for bit, and its children and merged particles must be exactly the predicted
number, with state 6 / lambda 0 and state 2 / lambda 0.  These decisions
depend on the state only, not on the physics, so they are checked at full
size on every step; the physics (densities, accelerations, the next state)
is checked against the full FP64 oracle step, from the GPU's state, every
100 steps at full size, and free-running 1,000-step rollouts of both are
compared by mass, centre of mass, kinetic energy and mean density (1 %).
"""
import numpy as np
import pytest

from oracle import oracle_ts
from sph2s_final_gb300 import scenes
from sph2s_final_gb300.two_scale import HIGH, LOW, Solver2

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

STEPS = 1000


def _by_id(ids, *arrays):
    o = np.argsort(ids, kind="stable")
    return (ids[o],) + tuple(np.asarray(a)[o] for a in arrays)


def check_decisions(sc, pre, group_base, stats, post):
    want, dec = oracle_ts.decide(sc.config, pre, group_base)
    assert stats == want, (stats, want)
    for r in (LOW, HIGH):
        keep = dec[r]["keep"].astype(bool)
        ids_pre = pre[r]["ids"]
        new = ~np.isin(post[r]["ids"], ids_pre)
        # survivors: the same ids, state bits, lambdas and groups as decided
        a = _by_id(ids_pre[keep], dec[r]["state"][keep], dec[r]["lam"][keep], dec[r]["group"][keep])
        b = _by_id(post[r]["ids"][~new], post[r]["state"][~new], post[r]["lam"][~new],
                   post[r]["group"][~new])
        for x, y, what in zip(a, b, ("ids", "state", "lam", "group")):
            np.testing.assert_array_equal(y, x, err_msg=f"population {r}: {what}")
        born = int(new.sum())
        if r == HIGH:
            assert born == 8 * want["splits"]
            assert np.all(post[r]["state"][new] == 6) and np.all(post[r]["lam"][new] == 0.0)
        else:
            assert born == want["merges"]
            assert np.all(post[r]["state"][new] == 2) and np.all(post[r]["lam"][new] == 0.0)


def check_physics(s, sc):
    """One step against the FP64 oracle from the GPU's state (densities and
    accelerations <= 1e-5, the next state's ids / states / lambdas / groups
    bit-exact, positions <= 2e-6)."""
    pops = [s.state(LOW), s.state(HIGH)]
    nl, nh = s.next_ids()
    ro = oracle_ts.TSRollout(sc.config, sc.boundary.positions, pops,
                             group_base=s.counts()["groups"], pid_base=[nl, nh])
    try:
        dbg = [s.debug_step_fields(LOW), s.debug_step_fields(HIGH)]
        of = ro.step_fields(sc.dt)
        for r in (LOW, HIGH):
            d = dbg[r]
            if d["ids"].size == 0:
                continue
            np.testing.assert_array_equal(d["ids"], of["ids"][r])
            np.testing.assert_array_equal(d["nbr_same"], of["nbr_same"][r])
            np.testing.assert_array_equal(d["nbr_compl"], of["nbr_compl"][r])
            rel = np.abs(d["rho"] - of["rho"][r]) / np.abs(of["rho"][r])
            assert rel.max() <= 1e-5, (r, rel.max())
            err = np.abs(d["acc"] - of["acc"][r]).max() / np.abs(of["acc"][r]).max()
            assert err <= 1e-5, (r, err)
        s.advance(sc.dt, 1)
        assert s.last_stats() == ro.last_stats()
        for r in (LOW, HIGH):
            g, o = s.state(r), ro.state(r)
            for key in ("ids", "state", "group", "lam"):
                np.testing.assert_array_equal(g[key], o[key])
            if g["x"].size:
                assert np.abs(g["x"] - o["x"]).max() <= 2e-6
    finally:
        ro.close()


def test_c2_full_size_every_step_for_1000_steps():
    sc = scenes.two_scale_dam_break(1 / 128)
    assert sc.low.num_particles == 262144
    totals = dict.fromkeys(oracle_ts.STAT_NAMES, 0)
    peak_high = 0
    with Solver2(sc.low, None, sc.boundary, sc.config) as s:
        for k in range(STEPS):
            if k % 100 == 50:
                check_physics(s, sc)  # advances one step itself
                continue
            pre = [s.state(LOW), s.state(HIGH)]
            gb = s.counts()["groups"]
            s.advance(sc.dt, 1)
            stats = s.last_stats()
            post = [s.state(LOW), s.state(HIGH)]
            check_decisions(sc, pre, gb, stats, post)
            for key, v in stats.items():
                totals[key] += v
            peak_high = max(peak_high, len(post[HIGH]["ids"]))
    # the run splits most of the slab, fades split parents out and children in
    assert totals["splits"] > 70000 and totals["removed_low"] > 70000, totals
    assert totals["faded_in_high"] > 500000, totals
    assert peak_high > 500000


def _stats(pops, masses):
    """Mass-weighted centre of mass, kinetic energy per unit mass and particle
    counts of both populations (blend-weighted mass)."""
    m_tot, com, ke = 0.0, np.zeros(3), 0.0
    for p, m in zip(pops, masses):
        w = m * np.asarray(p["lam"], np.float64)
        x = np.asarray(p["x"], np.float64)
        v = np.asarray(p["v"], np.float64)
        m_tot += w.sum()
        com += (w[:, None] * x).sum(0)
        ke += 0.5 * (w * (v * v).sum(1)).sum()
    return com / m_tot, ke / m_tot, m_tot


def test_c2_full_size_1000_step_statistics():
    """Free-running rollouts of the GPU and of the FP64 oracle from the same
    state (999 steps, then the 1,000th step's density pass): blend-weighted
    mass, centre of mass and kinetic energy within 1 %, mean density within 1 %."""
    sc = scenes.two_scale_dam_break(1 / 128)
    masses = [float(sc.config.fluid_particle_mass[0]), float(sc.config.fluid_particle_mass[1])]
    with Solver2(sc.low, None, sc.boundary, sc.config) as s:
        ro = oracle_ts.TSRollout(sc.config, sc.boundary.positions,
                                 [s.state(LOW), s.state(HIGH)], group_base=0,
                                 pid_base=list(s.next_ids()))
        try:
            s.advance(sc.dt, STEPS - 1)
            ro.advance(sc.dt, STEPS - 1)
            gpu = [s.state(LOW), s.state(HIGH)]
            ora = [ro.state(LOW), ro.state(HIGH)]
            # densities of the 1,000th step (no advance on the GPU side)
            g_rho = [s.debug_step_fields(r)["rho"] for r in (LOW, HIGH)]
            o_rho = ro.step_fields(sc.dt)["rho"]
        finally:
            ro.close()
    gc, gk, gm = _stats(gpu, masses)
    oc, ok, om = _stats(ora, masses)
    assert abs(gm - om) <= 0.01 * om
    assert np.abs(gc - oc).max() <= 0.01 * np.abs(oc).max()
    assert abs(gk - ok) <= 0.01 * ok
    g_mean = np.concatenate(g_rho).mean()
    o_mean = np.concatenate(o_rho).mean()
    assert abs(g_mean - o_mean) <= 0.01 * o_mean
    assert ok > 0 and len(gpu[HIGH]["ids"]) > 500000
