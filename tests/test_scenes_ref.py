"""The reference arm's numpy scene builder (oracle/scenes_ref.py) equals the
product's builders (libsph2s.so through scenes.py) byte for byte, so both
arms of bench.py measure the same workload."""
import ctypes as C

import numpy as np
import pytest

from oracle import scenes_ref as R
from sph2s_final_gb300 import scenes
from sph2s_final_gb300._abi import sph_config


@pytest.mark.parametrize("spacing,dims", [(1 / 64, None), (1 / 32, (10, 8, 10)), (1 / 256, None),
                                          (0.5 / 11, (11, 11, 11))])
def test_dam_break_identical(spacing, dims):
    a = scenes.dam_break(spacing, dims)
    b = R.dam_break(spacing, dims)
    assert a.fluid.positions.tobytes() == b.fluid.tobytes()
    assert a.boundary.positions.tobytes() == b.boundary.tobytes()
    assert C.sizeof(sph_config) == C.sizeof(R.OConfig)
    assert bytes(a.config) == bytes(b.config)
    assert a.dt == b.dt and a.spacing == b.spacing


def test_grid_and_canvas_identical():
    from sph2s_final_gb300.solver import Grid, ParticleData
    for o, e, s in [((0, 0, 0), (1, 1, 1), 0.03), ((-0.2, 0.1, 0.0), (0.7, 0.35, 1.3), 0.0625)]:
        g1, g2 = Grid.make_grid(o, e, s), R.make_grid(o, e, s)
        assert bytes(g1) == bytes(g2)
        for border in (0, 1, 3):
            c1 = ParticleData.create_particle_box_canvas(g1, border).positions
            assert c1.tobytes() == R.particle_canvas(g2, border).tobytes()
        assert ParticleData.create_particle_box(g1).positions.tobytes() == R.particle_box(g2).tobytes()
