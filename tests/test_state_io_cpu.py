"""State and frame formats without a GPU: the frame reader, the state header
parser, and sph_create_from_state / sph2_create_from_state rejecting broken
buffers (validation happens before any device call)."""
import ctypes as C
import struct

import numpy as np
import pytest

from sph2s_final_gb300 import _abi, state_io
from sph2s_final_gb300.solver import Grid, SolverConfiguration


def word_fnv1a(data: bytes) -> int:
    """The state checksum: FNV-1a over little-endian 64-bit words, tail zero-padded."""
    h = 0xcbf29ce484222325
    pad = data + b"\0" * (-len(data) % 8)
    for (w,) in struct.iter_unpack("<Q", pad):
        h = ((h ^ w) * 0x100000001b3) & 0xFFFFFFFFFFFFFFFF
    return h


def single_scale_state(ids, nb=2, step=7, version=1):
    """A well-formed single-scale state (by the layout in csrc/state_io.cu)."""
    g = Grid.make_grid((0, 0, 0), (1, 1, 1), 0.25)
    cfg = SolverConfiguration.direct(0.25, 1.0, 1000.0, 30.0, 5.0, 88.1472, 0.8, g)
    n = len(ids)
    rng = np.random.default_rng(0)
    pos = rng.uniform(0.1, 0.9, (n, 4)).astype(np.float32)
    pos[:, 3] = np.asarray(ids, np.uint32).view(np.float32)
    vel = np.zeros((n, 4), np.float32)
    bpos = rng.uniform(0.0, 1.0, (nb, 4)).astype(np.float32)
    body = (b"SPHSTAT1" + struct.pack("<IIQ", version, 1, step)
            + C.string_at(C.addressof(cfg), C.sizeof(cfg)) + struct.pack("<IIII", n, nb, 0, 0)
            + pos.tobytes() + vel.tobytes() + pos.tobytes() + bpos.tobytes())
    return body + struct.pack("<Q", word_fnv1a(body))


def create_rc(data: bytes) -> tuple[int, str]:
    h = C.c_void_p()
    rc = _abi.lib().sph_create_from_state(data, len(data), C.byref(h))
    assert not h.value
    return rc, _abi.lib().sph_last_error().decode()


def test_checksum_matches_the_library():
    """A state built here passes the library's checksum: its rejection names the
    id check, which runs after magic, version, kind, size and checksum."""
    rc, msg = create_rc(single_scale_state([0, 1, 1, 3]))
    assert rc == _abi.SPH_E_INVALID and "permutation" in msg


@pytest.mark.parametrize("mutate", ["magic", "version", "kind", "checksum", "truncate", "empty"])
def test_broken_state_is_rejected(mutate):
    data = bytearray(single_scale_state([2, 0, 1, 3]))
    if mutate == "magic":
        data[0:8] = b"SPHSTAT2"
    elif mutate == "version":
        data[8] = 2
    elif mutate == "kind":
        data[12] = 2
    elif mutate == "checksum":
        data[200] ^= 0x40
    elif mutate == "truncate":
        data = data[:-20]
    else:
        data = bytearray()
    rc, msg = create_rc(bytes(data))
    assert rc == _abi.SPH_E_INVALID, msg


def test_two_scale_entry_rejects_a_single_scale_state():
    data = single_scale_state([0, 1])
    h = C.c_void_p()
    rc = _abi.lib().sph2_create_from_state(data, len(data), C.byref(h))
    assert rc == _abi.SPH_E_INVALID and not h.value


def test_state_info():
    info = state_io.state_info(single_scale_state([0], step=123))
    assert info == {"version": 1, "kind": 1, "step": 123}
    with pytest.raises(ValueError):
        state_io.state_info(b"nope")


def test_read_frames(tmp_path):
    """Two single-scale records and one two-scale record, written by hand."""
    p = tmp_path / "f.bin"
    x = np.arange(12, dtype=np.float32).reshape(4, 3)
    rho = np.array([1000, 1001, 999, 998], np.float32)
    rec1 = b"SPHFRM01" + struct.pack("<IIQII", 1, 5, 10, 4, 0) + x.tobytes() + rho.tobytes()
    rec2 = b"SPHFRM01" + struct.pack("<IIQII", 1, 2, 11, 4, 0) + (x + 1).tobytes()
    ids = np.array([3, 4], np.uint32)
    lam = np.array([0.5, 1.0], np.float32)
    st = np.array([6, 4], np.int32)
    rec3 = (b"SPHFRM01" + struct.pack("<IIQII", 2, 9, 12, 0, 2) + b""  # LOW empty
            + ids.tobytes() + x[:2].tobytes() + lam.tobytes() + st.tobytes())
    p.write_bytes(rec1 + rec2 + rec3)
    fr = state_io.read_frames(p)
    assert [f["step"] for f in fr] == [10, 11, 12]
    np.testing.assert_array_equal(fr[0]["positions"], x)
    np.testing.assert_array_equal(fr[0]["densities"], rho)
    np.testing.assert_array_equal(fr[1]["velocities"], x + 1)
    assert fr[2]["low"]["n"] == 0
    np.testing.assert_array_equal(fr[2]["high"]["ids"], ids)
    np.testing.assert_array_equal(fr[2]["high"]["positions"], x[:2])
    np.testing.assert_array_equal(fr[2]["high"]["state"], st)
    p.write_bytes(rec1[:-3])
    with pytest.raises(ValueError):
        state_io.read_frames(p)


def test_write_bytes_is_atomic(tmp_path):
    p = tmp_path / "s.bin"
    state_io.write_bytes(p, b"abc")
    assert p.read_bytes() == b"abc" and not (tmp_path / "s.bin.tmp").exists()
