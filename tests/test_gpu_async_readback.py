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


def test_device_readback_matches_host_readback():
    """sph_get_positions/_velocities/_densities_device write the host readback's
    arrays into caller-owned device memory, in both orders; sph2's positions
    and state bits likewise; a host destination is refused before any kernel
    runs."""
    from sph2s_final_gb300 import _abi
    from sph2s_final_gb300.two_scale import HIGH, LOW, Solver2
    sc = scenes.dam_break(1 / 32)
    n = sc.fluid.num_particles
    with Solver(sc.fluid, sc.boundary, sc.config) as s:
        s.advance(sc.dt, 7)
        stream = torch.cuda.ExternalStream(s.stream)
        for order in ("sorted", "by_id"):
            want = {"positions": s.positions(order), "velocities": s.velocities(order),
                    "densities": s.densities(order)}
            for field, w in want.items():
                d = torch.full(w.shape, float("nan"), dtype=torch.float32, device="cuda")
                torch.cuda.synchronize()
                s.read_device(field, d.data_ptr(), order)
                with torch.cuda.stream(stream):
                    got = d.cpu().numpy()
                np.testing.assert_array_equal(got, w, err_msg=f"{field} {order}")
        host = np.zeros((n, 3), np.float32)
        rc = _abi.lib().sph_get_positions_device(s._h, host.ctypes.data, 0)
        assert rc == _abi.SPH_E_INVALID and b"device memory" in _abi.lib().sph_last_error()
    ts = scenes.two_scale_dam_break(1 / 32, dt=1e-4)
    with Solver2(ts.low, None, ts.boundary, ts.config) as s2:
        s2.advance(ts.dt, 3)
        for pop in (LOW, HIGH):
            w = s2.state(pop)["x"]
            d = torch.empty(w.shape, dtype=torch.float32, device="cuda")
            s2.read_positions_device(pop, d.data_ptr())
            torch.cuda.synchronize()
            np.testing.assert_array_equal(d.cpu().numpy(), w)
            ws = s2.state(pop)["state"]
            ds = torch.empty(ws.shape, dtype=torch.int32, device="cuda")
            s2.read_states_device(pop, ds.data_ptr())
            torch.cuda.synchronize()
            np.testing.assert_array_equal(ds.cpu().numpy(), ws)
