"""sph_get_positions_async: readbacks enqueued after every step, copied on a
second stream while later steps run, equal the synchronous readback of the
same step, in both orders, with more readbacks in flight than staging buffers."""
import numpy as np
import pytest
import torch

from sph2s_final_gb300 import scenes
from sph2s_final_gb300.solver import Solver

pytestmark = pytest.mark.gpu


def test_async_readback_matches_sync_readback():
    sc = scenes.dam_break(1 / 32)
    n = sc.fluid.num_particles
    steps = 6
    bufs = [torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
            for _ in range(steps)]
    want = []
    with Solver(sc.fluid, sc.boundary, sc.config) as ref:
        for k in range(steps):
            ref.advance(sc.dt, 1)
            want.append(ref.positions("by_id" if k % 2 else "sorted"))
    with Solver(sc.fluid, sc.boundary, sc.config) as s:
        for k in range(steps):
            s.advance(sc.dt, 1)
            s.positions_async(bufs[k], "by_id" if k % 2 else "sorted")
        s.sync()
        for k in range(steps):
            np.testing.assert_array_equal(bufs[k], want[k])
        # a synchronous readback after async ones still works
        np.testing.assert_array_equal(s.positions("by_id"), want[-1])
