"""bench.py's work counts for the roofline: stencil candidates by summed-area
table equal a direct count over the same stencil rule (the oracle's stencil),
including particles outside the grid (clamped cells)."""
import numpy as np

import bench
from oracle import oracle as O
from sph2s_final_gb300 import scenes


def test_stencil_candidates_match_direct_count():
    sc = scenes.dam_break(1 / 16)
    x = sc.fluid.positions.copy()
    rng = np.random.default_rng(4)
    x[:20] = rng.uniform(-0.1, 1.1, (20, 3)).astype(np.float32)  # some outside the grid
    g = sc.config.grid
    h = float(sc.config.effective_radius)
    got = bench.stencil_candidates(g, h, x, x)
    cs, ce = O.stencil(g, x, h)
    _, lin = O.cell_keys(g, x)
    d = np.array(g.dims[:])
    cz, rem = np.divmod(lin.astype(np.int64), d[0] * d[1])
    cy, cx = np.divmod(rem, d[0])
    want = np.array([np.sum((cx >= cs[i, 0]) & (cx <= ce[i, 0]) & (cy >= cs[i, 1]) & (cy <= ce[i, 1])
                            & (cz >= cs[i, 2]) & (cz <= ce[i, 2])) for i in range(len(x))])
    np.testing.assert_array_equal(got, want)


def test_reference_workload_loads_no_product_code():
    import subprocess
    import sys
    code = ("import sys, bench; sc, d = bench.workload_reference('c0'); "
            "assert not any(m.startswith('sph2s_final_gb300') for m in sys.modules), "
            "sorted(m for m in sys.modules if m.startswith('sph2s'))")
    r = subprocess.run([sys.executable, "-c", code], cwd=bench.ROOT, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_config_states_whether_the_step_data_exceeds_l2():
    """Timed steps need inputs larger than L2 or a flush between them: the headline
    2M case says it exceeds L2, the 32,768-particle parity case says it fits; both arms
    emit the same config for the same workload."""
    big, d1 = bench.workload_reference("c1")
    small, d0 = bench.workload_reference("c0")
    assert "> L2, no flush needed" in bench.config_for(d1, 1, big)["l2"]
    assert "fits in L2" in bench.config_for(d0, 1, small)["l2"]
    ours, d = bench.workload("c0")
    assert bench.config_for(d, 1, ours) == bench.config_for(d0, 1, small)


def test_committed_ncu_figures_cover_the_single_scale_passes():
    """The roofline block reads each pass's measured DRAM traffic and issue-active
    share from the committed ncu summaries; every pass and workload it reports on
    has both, and the traffic is at least the pass's algorithmic bytes (20 bytes
    per particle + 8 per cell for density, 72 + 16 for force, at 2,097,152
    particles in 128^3 cells and 512,000 in 80^3)."""
    sizes = {"c1": (2097152, 128 ** 3), "c1m": (512000, 80 ** 3)}
    per = {"density_kernel": (20, 8), "force_kernel": (72, 16)}
    for wl, (n, cells) in sizes.items():
        for kernel, (bp, bc) in per.items():
            traffic = bench.committed_metric("traffic_bytes_per_launch", kernel, wl)
            issue = bench.committed_metric("issue_active_pct", kernel, wl)
            assert traffic is not None and issue is not None, (kernel, wl)
            assert traffic >= bp * n + bc * cells, (kernel, wl, traffic)
            assert 0.0 < issue <= 100.0
