"""The C ABI from compiled code: tests/cabi_client.cpp and tests/cabi_client2.cpp
are the reference-side adapters (the single-scale and two-scale `Solver`
classes that forward to include/sph2s.h), each driving a scene built with the
ABI's grid, particle-box and configuration builders; tests/cabi_client3.cpp is
the reference's own host-program flow (initSim / display) on the header-only
drop-in include/sph2s_solver.hpp (Grid, SolverConfiguration, ParticleData with
device arrays, Solver(ParticleData*, ParticleData*, const SolverConfiguration*)),
and tests/cabi_client4.cpp the two-scale program's flow on
include/sph2s_solver2.hpp (Solver(low, high, boundary, config), ParticleData
with dPositions, dStates and NumParticles kept current by every Advance).

CPU: the header compiles as C99 and as C++17 with warnings as errors, and both
clients link against libsph2s.so.  GPU: each client's run equals the same run
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
from sph2s_final_gb300.two_scale import HIGH, LOW, STAT_NAMES, Solver2

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "sph2s_final_gb300"


def compiler(name):
    exe = shutil.which(name)
    if not exe:
        pytest.skip(f"{name} not found")
    return exe


CUDA_HOME = Path("/usr/local/cuda")


def build_client(tmp_path, name="cabi_client"):
    _abi.lib()  # the library is built (raises with the build command otherwise)
    exe = tmp_path / name
    cmd = [compiler("g++"), "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror",
           "-I", str(ROOT / "include"), str(ROOT / "tests" / f"{name}.cpp"),
           "-L", str(PKG), "-lsph2s", f"-Wl,-rpath,{PKG}", "-o", str(exe)]
    if name in ("cabi_client3", "cabi_client4"):  # the drop-in headers allocate with the CUDA runtime
        if not (CUDA_HOME / "include" / "cuda_runtime.h").exists():
            pytest.skip("CUDA runtime headers not found")
        cmd[-2:-2] = ["-isystem", str(CUDA_HOME / "include"), "-L", str(CUDA_HOME / "lib64"),
                      "-lcudart", f"-Wl,-rpath,{CUDA_HOME / 'lib64'}"]
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


@pytest.mark.parametrize("name", ["cabi_client", "cabi_client2", "cabi_client3", "cabi_client4"])
def test_client_compiles_and_links(tmp_path, name):
    assert build_client(tmp_path, name).exists()


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


def read_run2(path):
    data = path.read_bytes()
    nl, nb, steps = struct.unpack_from("<III", data, 0)
    (dt,) = struct.unpack_from("<f", data, 12)
    off = 16
    cfg = _abi.sph_config2.from_buffer_copy(data, off)
    off += C.sizeof(_abi.sph_config2)

    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(data, dtype, count, off).copy()
        off += 4 * count
        return a

    low = take(np.float32, 3 * nl).reshape(nl, 3)
    boundary = take(np.float32, 3 * nb).reshape(nb, 3)
    stats = dict(zip(STAT_NAMES, map(int, take(np.uint32, 6))))
    pops = []
    for _ in (LOW, HIGH):
        (n,) = struct.unpack_from("<I", data, off)
        off += 4
        pops.append({"ids": take(np.uint32, n), "x": take(np.float32, 3 * n).reshape(n, 3),
                     "v": take(np.float32, 3 * n).reshape(n, 3), "lam": take(np.float32, n),
                     "state": take(np.int32, n), "group": take(np.uint32, n)})
    assert off == len(data)
    return cfg, low, boundary, steps, dt, stats, pops


@pytest.mark.gpu
def test_two_scale_client_run_equals_python_binding(tmp_path):
    exe = build_client(tmp_path, "cabi_client2")
    out = tmp_path / "run2.bin"
    r = subprocess.run([str(exe), str(out), "30"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    cfg, low, boundary, steps, dt, stats, pops = read_run2(out)
    assert low.shape == (4096, 3) and steps == 30 and cfg.refine_axis == 0
    assert pops[HIGH]["ids"].size > 0  # the slab refined part of the block
    with Solver2(low, None, boundary, cfg) as s:
        s.advance(dt, steps)
        assert s.last_stats() == stats
        for pop in (LOW, HIGH):
            st = s.state(pop)
            for k in ("ids", "x", "v", "lam", "state", "group"):
                np.testing.assert_array_equal(st[k], pops[pop][k], err_msg=f"{pop} {k}")
    assert np.isfinite(pops[LOW]["x"]).all() and np.isfinite(pops[HIGH]["x"]).all()


def read_run3(path):
    data = path.read_bytes()
    nf, nb, steps = struct.unpack_from("<III", data, 0)
    (dt,) = struct.unpack_from("<f", data, 12)
    off = 16
    cfg = _abi.sph_config.from_buffer_copy(data, off)
    off += C.sizeof(_abi.sph_config)
    fluid = np.frombuffer(data, np.float32, 3 * nf, off).reshape(nf, 3).copy()
    off += 12 * nf
    boundary = np.frombuffer(data, np.float32, 3 * nb, off).reshape(nb, 3).copy()
    off += 12 * nb
    x = np.frombuffer(data, np.float32, 3 * nf, off).reshape(nf, 3).copy()
    off += 12 * nf
    ids = np.frombuffer(data, np.uint32, nf, off).copy()
    off += 4 * nf
    assert off == len(data)
    return cfg, fluid, boundary, steps, dt, x, ids


@pytest.mark.gpu
def test_reference_host_flow_on_the_drop_in_header(tmp_path):
    """initSim / display through include/sph2s_solver.hpp: the positions the
    Solver writes into the fluid ParticleData's device array every Advance are
    the Python binding's sorted positions, bit for bit."""
    exe = build_client(tmp_path, "cabi_client3")
    out = tmp_path / "run3.bin"
    r = subprocess.run([str(exe), str(out), "20"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    cfg, fluid, boundary, steps, dt, x, ids = read_run3(out)
    assert steps == 20 and fluid.shape[0] > 10000 and boundary.shape[0] > 100000
    with Solver(ParticleData(fluid), ParticleData(boundary), cfg) as s:
        s.advance(dt, steps)
        np.testing.assert_array_equal(s.ids(), ids)
        np.testing.assert_array_equal(s.positions("sorted"), x)
    assert np.abs(x[np.argsort(ids)] - fluid).max() > 0  # the client did step the scene


def read_run4(path):
    data = path.read_bytes()
    nl, nb, steps = struct.unpack_from("<III", data, 0)
    (dt,) = struct.unpack_from("<f", data, 12)
    off = 16
    cfg = _abi.sph_config2.from_buffer_copy(data, off)
    off += C.sizeof(_abi.sph_config2)

    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(data, dtype, count, off).copy()
        off += 4 * count
        return a

    low = take(np.float32, 3 * nl).reshape(nl, 3)
    boundary = take(np.float32, 3 * nb).reshape(nb, 3)
    pops = []
    for _ in (LOW, HIGH):
        (n,) = struct.unpack_from("<I", data, off)
        off += 4
        pops.append({"x": take(np.float32, 3 * n).reshape(n, 3), "state": take(np.int32, n),
                     "ids": take(np.uint32, n)})
    assert off == len(data)
    return cfg, low, boundary, steps, dt, pops


@pytest.mark.gpu
def test_two_scale_reference_host_flow_on_the_drop_in_header(tmp_path):
    """The two-scale initSim / display through include/sph2s_solver2.hpp: after
    every Advance both ParticleData hold the solver's positions, state bits and
    counts; after 25 steps they equal the Python binding's, bit for bit."""
    exe = build_client(tmp_path, "cabi_client4")
    out = tmp_path / "run4.bin"
    r = subprocess.run([str(exe), str(out), "25"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    cfg, low, boundary, steps, dt, pops = read_run4(out)
    assert steps == 25 and low.shape[0] > 10000 and cfg.refine_axis == 0
    assert pops[HIGH]["ids"].size > 0  # the slab refined part of the block
    with Solver2(low, None, boundary, cfg, low.shape[0], 8 * low.shape[0]) as s:
        s.advance(dt, steps)
        for pop in (LOW, HIGH):
            st = s.state(pop)
            for k in ("ids", "x", "state"):
                np.testing.assert_array_equal(pops[pop][k], st[k], err_msg=f"{pop} {k}")
