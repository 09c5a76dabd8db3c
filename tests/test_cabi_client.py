"""The C ABI from compiled code: tests/cabi_client.cpp is the reference-side
adapter (the `Solver` class that forwards to include/sph2s.h) driving a scene
built with the ABI's grid, particle-box and configuration builders.

CPU: the header compiles as C99 and as C++17 with warnings as errors, and the
client links against libsph2s.so.  GPU: the client's run equals the same run
through the Python binding bit for bit (same library, same inputs)."""
import ctypes as C
import shutil
import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

from sph2s_final_gb300 import _abi
from sph2s_final_gb300.solver import ParticleData, Solver

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "sph2s_final_gb300"


def compiler(name):
    exe = shutil.which(name)
    if not exe:
        pytest.skip(f"{name} not found")
    return exe


def build_client(tmp_path):
    _abi.lib()  # the library is built (raises with the build command otherwise)
    exe = tmp_path / "cabi_client"
    cmd = [compiler("g++"), "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror",
           "-I", str(ROOT / "include"), str(ROOT / "tests" / "cabi_client.cpp"),
           "-L", str(PKG), "-lsph2s", f"-Wl,-rpath,{PKG}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_header_compiles_as_c(tmp_path):
    src = tmp_path / "h.c"
    src.write_text('#include "sph2s.h"\nint main(void) { sph_grid g; (void)g; return SPH_OK; }\n')
    r = subprocess.run([compiler("gcc"), "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic",
                        "-I", str(ROOT / "include"), "-c", str(src), "-o", str(tmp_path / "h.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_client_compiles_and_links(tmp_path):
    assert build_client(tmp_path).exists()


def read_run(path):
    data = path.read_bytes()
    nf, nb, steps = struct.unpack_from("<III", data, 0)
    (dt,) = struct.unpack_from("<f", data, 12)
    off = 16
    cfg = _abi.sph_config.from_buffer_copy(data, off)
    off += C.sizeof(_abi.sph_config)

    def take(count):
        nonlocal off
        a = np.frombuffer(data, np.float32, count, off).copy()
        off += 4 * count
        return a

    fluid = take(3 * nf).reshape(nf, 3)
    boundary = take(3 * nb).reshape(nb, 3)
    x = take(3 * nf).reshape(nf, 3)
    rho = take(nf)
    assert off == len(data)
    return cfg, fluid, boundary, steps, dt, x, rho


@pytest.mark.gpu
def test_client_run_equals_python_binding(tmp_path):
    exe = build_client(tmp_path)
    out = tmp_path / "run.bin"
    r = subprocess.run([str(exe), str(out), "25"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    cfg, fluid, boundary, steps, dt, x, rho = read_run(out)
    assert fluid.shape == (4096, 3) and steps == 25 and np.isfinite(x).all()
    with Solver(ParticleData(fluid), ParticleData(boundary), cfg) as s:
        s.advance(dt, steps)
        np.testing.assert_array_equal(s.positions("by_id"), x)
        np.testing.assert_array_equal(s.densities("by_id"), rho)
    assert np.abs(x - fluid).max() > 0  # the client did step the scene
