"""Headless state save / resume and frame records.

The reference's only output is the OpenGL vertex buffer it renders
(ParticleData::Map/Unmap, SPH2S_FINAL_SINGLE_SCALE/ParticleData.cpp:47-66)
and the rendered pixels VideoWriter writes (VideoWriter/VideoWriter.cpp:41-49).
Here the solver state is serialised by libsph2s.so (sph_save_state /
sph_create_from_state and the sph2_* pair) into a self-checking binary
buffer, and frame records of selected per-particle fields are appended to a
file (sph_write_frame / sph2_write_frame).  This module holds the pieces that
need no GPU: file helpers and a numpy reader for frame files.

Formats (little-endian):
  state  "SPHSTAT1" | u32 version | u32 kind (1 single, 2 two-scale) | u64 step
         | body | u64 checksum
  frame  "SPHFRM01" | u32 kind | u32 fields | u64 step | u32 count[2] | arrays
    kind 1: count = (n, 0); positions f32[n,3], velocities f32[n,3],
            densities f32[n] (those in `fields`), in persistent-id order.
    kind 2: count = (n_low, n_high); per population: ids u32[n], then
            positions, velocities f32[n,3], blend f32[n] + state i32[n].
"""
from __future__ import annotations

import os
import struct
from pathlib import Path

import numpy as np

FIELD_POSITIONS = 1
FIELD_VELOCITIES = 2
FIELD_DENSITIES = 4
FIELD_BLEND = 8

STATE_MAGIC = b"SPHSTAT1"
FRAME_MAGIC = b"SPHFRM01"
KIND_SINGLE_SCALE = 1
KIND_TWO_SCALE = 2


def state_info(data: bytes) -> dict:
    """Kind, version and step of a state buffer (no validation of the body)."""
    if len(data) < 24 or data[:8] != STATE_MAGIC:
        raise ValueError("not a SPHSTAT1 state")
    version, kind, step = struct.unpack_from("<IIQ", data, 8)
    return {"version": version, "kind": kind, "step": step}


def read_bytes(src) -> bytes:
    """A state given as bytes-like or as a file path."""
    if isinstance(src, (bytes, bytearray, memoryview)):
        return bytes(src)
    return Path(os.fspath(src)).read_bytes()


def write_bytes(path, data: bytes) -> None:
    """Writes atomically: a crash never leaves a truncated state behind."""
    path = Path(os.fspath(path))
    tmp = path.with_name(path.name + ".tmp")
    tmp.write_bytes(data)
    os.replace(tmp, path)


def _take(buf, off, dtype, count):
    a = np.frombuffer(buf, dtype=dtype, count=count, offset=off)
    return a.copy(), off + a.nbytes


def read_frames(path) -> list[dict]:
    """All frame records of a file written by sph_write_frame / sph2_write_frame."""
    buf = Path(os.fspath(path)).read_bytes()
    frames, off = [], 0
    while off < len(buf):
        if len(buf) - off < 32 or buf[off:off + 8] != FRAME_MAGIC:
            raise ValueError(f"corrupt frame record at byte {off}")
        kind, fields, step = struct.unpack_from("<IIQ", buf, off + 8)
        n0, n1 = struct.unpack_from("<II", buf, off + 24)
        off += 32
        fr = {"kind": kind, "fields": fields, "step": step}
        if kind == KIND_SINGLE_SCALE:
            fr["n"] = n0
            if fields & FIELD_POSITIONS:
                a, off = _take(buf, off, np.float32, 3 * n0)
                fr["positions"] = a.reshape(n0, 3)
            if fields & FIELD_VELOCITIES:
                a, off = _take(buf, off, np.float32, 3 * n0)
                fr["velocities"] = a.reshape(n0, 3)
            if fields & FIELD_DENSITIES:
                fr["densities"], off = _take(buf, off, np.float32, n0)
        elif kind == KIND_TWO_SCALE:
            for name, n in (("low", n0), ("high", n1)):
                p = {"n": n}
                p["ids"], off = _take(buf, off, np.uint32, n)
                if fields & FIELD_POSITIONS:
                    a, off = _take(buf, off, np.float32, 3 * n)
                    p["positions"] = a.reshape(n, 3)
                if fields & FIELD_VELOCITIES:
                    a, off = _take(buf, off, np.float32, 3 * n)
                    p["velocities"] = a.reshape(n, 3)
                if fields & FIELD_BLEND:
                    p["lambda"], off = _take(buf, off, np.float32, n)
                    p["state"], off = _take(buf, off, np.int32, n)
                fr[name] = p
        else:
            raise ValueError(f"unknown frame kind {kind}")
        frames.append(fr)
    return frames
