"""Two-scale and coupled parity pinned to the reference's own kernels.

tests/golden/ref_ts_mixed.npz, ref_ts_clamp.npz and ref_cp_mixed.npz hold the
inputs and per-step outputs of SPH2S_FINAL_TWO_SCALE/Solver.cu and
SPH2S_FINAL_TWO_SCALE_COUPLED/Solver.cu, compiled unmodified and replayed by
oracle/ref_harness_ts.cu (tests/golden/make_golden_ts.py).  Every step t is
checked from the state the reference itself started it from (the input for
t = 0, the reference's state after step t-1 otherwise), so each comparison is
one step from an identical state:

  * densities <= 1e-5 relative per particle, accelerations <= 1e-5 max-norm
    relative per population (TS Solver.cu:732-1083: lambda-weighted sums,
    averaged complementary kernels, LOW-radius / LOW-mass boundary);
  * colour / energy values <= 1e-4 (Solver.cu:1050-1075), particles within
    1e-6 of the 0.0025 mass-centre switch excepted;
  * after the step (Solver.cu:1163-1289): the set of surviving particles,
    their state bits and blend coefficients exactly, positions <= 1e-6,
    velocities (with the clamp |v| <= 0.8 h_r / dt) <= 1e-5 relative; the
    split children (8 per marked LOW particle, Solver.cu:541-586) paired with
    the reference's by position (<= 2e-6), with state 6, lambda 0 and the
    parent's velocity.

The CPU tests check the FP64 oracle (oracle/sph_oracle_ts.cpp) against the
fixtures; the GPU tests check the CUDA path through the C ABI.
"""
import numpy as np
import pytest

import ts_seed as T

CASES = {"ref_ts_mixed": 4, "ref_ts_clamp": 2, "ref_cp_mixed": 3}
PARAMS = [(c, t) for c, n in CASES.items() for t in range(n)]
RHO_TOL = 1e-5
ACC_TOL = 1e-5
COLOUR_TOL = 1e-4
X_TOL = 1e-6
V_TOL = 1e-5


def _golden(name):
    p = T.GOLDEN / f"{name}.npz"
    if not p.exists():
        pytest.skip(f"{p.name} not generated")
    return T.load(name)


def check_fields(g, t, pre, got):
    """got[r] = dict(ids (dense pre index), rho, acc[, colour, dist_cm]) per population."""
    for r, tag in ((0, "low"), (1, "high")):
        f = {k[len(f"s{t}_{tag}_f_"):]: v for k, v in g.items() if k.startswith(f"s{t}_{tag}_f_")}
        n = f["pid"].size
        gr = got[r]
        assert gr["ids"].size == n, (tag, gr["ids"].size, n)
        if n == 0:
            continue
        pid = pre[r]["pid"][gr["ids"]]
        order = np.argsort(pid)
        ro = np.argsort(f["pid"])
        assert np.array_equal(pid[order], f["pid"][ro]), f"{tag}: particle sets differ"
        rho = np.asarray(gr["rho"], np.float64)[order]
        rrho = f["rho"][ro].astype(np.float64)
        rel = np.abs(rho - rrho) / np.abs(rrho)
        assert rel.max() <= RHO_TOL, (tag, "rho", rel.max())
        acc = np.asarray(gr["acc"], np.float64)[order]
        racc = f["acc"][ro].astype(np.float64)
        err = np.abs(acc - racc).max() / np.abs(racc).max()
        assert err <= ACC_TOL, (tag, "acc", err)
        if "colour" in gr and int(g["mode"]) == 0:
            col = np.asarray(gr["colour"], np.float64)[order]
            keep = np.abs(np.asarray(gr["dist_cm"])[order] - 0.0025) > 1e-6
            d = np.abs(col - f["colour"][ro])[keep]
            assert d.max() <= COLOUR_TOL, (tag, "colour", d.max())


def check_post(g, t, pre, post, dt):
    """post[r] = dict(ids, x, v, lam, state): ids < len(pre[r]) are survivors
    (dense pre index), larger ids are particles born in the step."""
    for r, tag in ((0, "low"), (1, "high")):
        k = f"s{t}_{tag}_post_"
        rp = {kk: g[k + kk] for kk in ("pid", "x", "v", "lam", "state")}
        npre = pre[r]["pid"].size
        born_ref = ~np.isin(rp["pid"], pre[r]["pid"])
        q = post[r]
        born = q["ids"] >= npre
        # survivors: identical sets, states, lambdas; positions and velocities
        sp = pre[r]["pid"][q["ids"][~born]]
        o = np.argsort(sp)
        ro = np.argsort(rp["pid"][~born_ref])
        assert np.array_equal(sp[o], rp["pid"][~born_ref][ro]), f"{tag}: survivor sets differ"
        sel = lambda a, m, oo: np.asarray(a)[m][oo]  # noqa: E731
        assert np.array_equal(sel(q["state"], ~born, o), sel(rp["state"], ~born_ref, ro)), tag
        assert np.array_equal(sel(q["lam"], ~born, o), sel(rp["lam"], ~born_ref, ro)), tag
        dx = np.abs(sel(q["x"], ~born, o) - sel(rp["x"], ~born_ref, ro)).max(initial=0.0)
        assert dx <= X_TOL, (tag, "x", dx)
        rv = sel(rp["v"], ~born_ref, ro).astype(np.float64)
        dv = np.abs(sel(q["v"], ~born, o) - rv) / np.maximum(1.0, np.abs(rv))
        assert dv.max(initial=0.0) <= V_TOL, (tag, "v", dv.max(initial=0.0))
        if int(g["mode"]) == 0:  # the clamp held for every survivor
            vmax = 0.8 * float(g["cfg_h"][r]) / dt
            assert np.linalg.norm(rv, axis=1).max(initial=0.0) <= vmax * (1 + 1e-6)
        # children born in the step
        p = T.match_children(rp["x"][born_ref], np.asarray(q["x"])[born])
        assert np.array_equal(np.asarray(q["state"])[born][p], rp["state"][born_ref])
        assert np.array_equal(np.asarray(q["lam"])[born][p], rp["lam"][born_ref])
        dv = np.abs(np.asarray(q["v"])[born][p] - rp["v"][born_ref]).max(initial=0.0)
        assert dv <= V_TOL * max(1.0, np.abs(rp["v"]).max(initial=0.0)), (tag, "child v", dv)


# ---- FP64 oracle against the reference (CPU) --------------------------------

@pytest.mark.parametrize("case,t", PARAMS)
def test_oracle_matches_reference_kernels(case, t):
    g = _golden(case)
    cfg = T.config_from_golden(g)
    dt = float(g["dt"])
    pre = T.pre_state(g, t)
    ro = T.oracle_from_pops(cfg, pre, g["boundary"])
    try:
        of = ro.step_fields(dt)
        got = [{"ids": of["ids"][r], "rho": of["rho"][r], "acc": of["acc"][r],
                "colour": of["colour"][r], "dist_cm": of["dist_cm"][r]} for r in range(2)]
        check_fields(g, t, pre, got)
        post = [ro.state(r) for r in range(2)]
        check_post(g, t, pre, post, dt)
    finally:
        ro.close()


def test_fixtures_cover_the_state_machine():
    """The blended fixtures exercise removal, fade-in completion and splits in
    their first step, and the clamp case clamps."""
    g = _golden("ref_ts_mixed")
    pre = T.pre_state(g, 0)
    post_low = g["s0_low_post_pid"]
    removed = np.setdiff1d(pre[0]["pid"], post_low).size
    assert removed > 0
    born = np.sum(g["s0_high_post_pid"] >= T.CHILD_PID_BASE)
    splits = int(np.sum((pre[0]["state"] & 3) == 3))
    assert splits > 0 and born == 8 * splits
    for r, tag in ((0, "low"), (1, "high")):  # fade-in completions (state &3: 2 -> 0, lambda 1)
        before = dict(zip(pre[r]["pid"].tolist(), pre[r]["state"].tolist()))
        after = zip(g[f"s0_{tag}_post_pid"].tolist(), g[f"s0_{tag}_post_state"].tolist(),
                    g[f"s0_{tag}_post_lam"].tolist())
        done = [p for p, st, lam in after if p in before and (before[p] & 3) == 2
                and (st & 3) == 0 and lam == 1.0]
        assert len(done) > 0, tag
    c = _golden("ref_ts_clamp")
    dt = float(c["dt"])
    for r, tag in ((0, "low"), (1, "high")):
        vmax = 0.8 * float(c["cfg_h"][r]) / dt
        sp = np.linalg.norm(c[f"s0_{tag}_post_v"].astype(np.float64), axis=1)
        assert np.sum(sp > 0.999 * vmax) > 0, tag


# ---- CUDA path against the reference (GPU) ----------------------------------

@pytest.mark.gpu
@pytest.mark.parametrize("case,t", PARAMS)
def test_gpu_matches_reference_kernels(case, t):
    from sph2s_final_gb300.two_scale import HIGH, LOW
    g = _golden(case)
    cfg = T.config_from_golden(g)
    dt = float(g["dt"])
    pre = T.pre_state(g, t)
    ro = T.oracle_from_pops(cfg, pre, g["boundary"])  # only for the colour switch distance
    try:
        of = ro.step_fields(dt)
    finally:
        ro.close()
    s = T.solver_from_pops(cfg, pre, g["boundary"])
    try:
        dbg = [s.debug_step_fields(LOW), s.debug_step_fields(HIGH)]
        if int(g["mode"]) == 0:
            s.set_color_output(True)
        s.advance(dt, 1)
        got = []
        for r in (LOW, HIGH):
            d = dbg[r]
            e = {"ids": d["ids"], "rho": d["rho"], "acc": d["acc"]}
            if int(g["mode"]) == 0 and d["ids"].size:
                col, cid = s.colors(r)
                assert np.array_equal(cid, d["ids"])
                dist = dict(zip(of["ids"][r].tolist(), of["dist_cm"][r]))
                e["colour"] = col
                e["dist_cm"] = np.array([dist[i] for i in cid.tolist()])
            got.append(e)
        check_fields(g, t, pre, got)
        check_post(g, t, pre, [s.state(LOW), s.state(HIGH)], dt)
    finally:
        s.close()
