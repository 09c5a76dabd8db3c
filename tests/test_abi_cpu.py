"""C-ABI checks that need no GPU: the library loads, exports every symbol the
headers declare, and its host-only entry points (grid, configuration, scene
builders, argument validation) behave like the reference's."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from sph2s_final_gb300 import _abi
from sph2s_final_gb300.solver import Grid, ParticleData, SolverConfiguration

ROOT = Path(__file__).resolve().parent.parent


def declared_functions():
    names = []
    for h in sorted((ROOT / "include").glob("*.h")):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(sph\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    lib = _abi.lib()
    names = declared_functions()
    assert len(names) >= 19
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # and the Python binding declares a signature for each
    assert set(names) <= set(_abi.SIGNATURES), set(names) - set(_abi.SIGNATURES)


def test_struct_layouts_match_header():
    assert C.sizeof(_abi.sph_grid) == 28
    assert C.sizeof(_abi.sph_config) == 9 * 4 + 28


def test_make_grid_matches_reference_formula():
    """Grid::MakeGrid: dims = (int)ceil((end - origin)/spacing) in FP32."""
    for o, e, s in [((0, 0, 0), (1, 1, 1), 1 / 32), ((-0.1, -0.1, -0.2), (1.7, 1.6, 0.6), 0.0203),
                    ((0, 0, 0), (1, 1, 1), 1 / 128)]:
        g = Grid.make_grid(o, e, s)
        want = np.ceil((np.float32(e) - np.float32(o)) / np.float32(s)).astype(int)
        assert list(g.dims) == list(want)
        assert g.spacing == np.float32(s)


def test_make_configuration_matches_reference_formula():
    """SolverConfiguration::MakeConfiguration (Solver.h:15-48) for the reference scene."""
    pg = Grid.make_grid((0.04, 0.04, 0.0), (0.35, 0.75, 0.4), 0.0075)
    vol = Grid.compute_volume(pg)
    n = Grid.compute_num_grid_cells(pg)
    c = SolverConfiguration.make_configuration((-0.1, -0.1, -0.2), (1.7, 1.6, 0.6), vol, n, 35,
                                               1000.0, 30.0, 5.0, 88.1472, 0.8, 0.05)
    num = np.float32(np.float32(0.75) * np.float32(vol) * np.float32(35))
    q = float(num) / (np.pi * float(np.float32(n)))
    h = np.float32(np.float32(q) ** np.float32(1.0 / 3.0))
    assert c.effective_radius == pytest.approx(float(h), rel=2e-7)
    m = np.float32(np.float32(1000.0) * np.float32(vol)) / np.float32(n)
    assert c.fluid_particle_mass == np.float32(m)
    assert c.boundary_particle_mass == c.fluid_particle_mass
    assert (c.bulk_modulus, c.viscosity, c.tension_coefficient) == (30.0, 5.0, np.float32(0.8))
    assert n == 215460 or n > 0


def test_particle_box_positions_fp32():
    g = Grid.make_grid((0.04, 0.04, 0.0), (0.35, 0.75, 0.4), 0.0075)
    p = ParticleData.create_particle_box(g).positions
    d = list(g.dims)
    assert p.shape == (d[0] * d[1] * d[2], 3)
    k, j, i = np.meshgrid(np.arange(d[2]), np.arange(d[1]), np.arange(d[0]), indexing="ij")
    o = np.array(g.origin[:], np.float32)
    s = np.float32(g.spacing)
    want = np.stack([o[0] + i.ravel().astype(np.float32) * s, o[1] + j.ravel().astype(np.float32) * s,
                     o[2] + k.ravel().astype(np.float32) * s], 1)
    np.testing.assert_array_equal(p, want)


def test_canvas_is_hollow_shell():
    g = Grid.make_grid((0, 0, 0), (1, 1, 1), 0.25)
    p = ParticleData.create_particle_box_canvas(g, 2).positions
    assert p.shape[0] == 8 ** 3 - 4 ** 3
    idx = np.rint(p / 0.25).astype(int)
    inside = np.all((idx >= 0) & (idx < 4), axis=1)
    assert not inside.any()
    assert len({tuple(r) for r in idx}) == p.shape[0]


def test_union_concatenates():
    a = ParticleData(np.zeros((3, 3), np.float32))
    b = ParticleData(np.ones((2, 3), np.float32))
    u = ParticleData.union(a, b)
    assert u.num_particles == 5 and ParticleData.union(a, None) is None


def test_null_handles_and_bad_arguments_return_status_codes():
    lib = _abi.lib()
    assert lib.sph_advance(None, C.c_float(1e-4), 1) == _abi.SPH_E_INVALID
    assert b"NULL" in lib.sph_last_error()
    assert lib.sph_sync(None) == _abi.SPH_E_INVALID
    assert lib.sph_get_positions(None, None, 0) == _abi.SPH_E_INVALID
    assert lib.sph_destroy(None) == _abi.SPH_OK
    g = _abi.sph_grid()
    o = (C.c_float * 3)(0, 0, 0)
    e = (C.c_float * 3)(1, 1, 1)
    assert lib.sph_make_grid(o, e, C.c_float(0.0), C.byref(g)) == _abi.SPH_E_INVALID
    assert lib.sph_make_grid(o, e, C.c_float(1e-4), C.byref(g)) == _abi.SPH_E_INVALID  # > 1024 cells
    n = C.c_uint32()
    assert lib.sph_particle_box_canvas(C.byref(g), -1, None, 0, C.byref(n)) == _abi.SPH_E_INVALID
    with pytest.raises(_abi.SphError):
        Grid.make_grid((0, 0, 0), (1, 1, 1), -1.0)
    # the coherent sort and the sort-mode hook check their arguments first
    assert lib.sph_sort_keys_coherent(None, None, None, None, 0, 21, None) == _abi.SPH_OK
    assert lib.sph_sort_keys_coherent(None, None, None, None, 9, 21, None) == _abi.SPH_E_INVALID
    assert lib.sph_debug_sort_mode(None, 1) == _abi.SPH_E_INVALID


def test_create_rejects_invalid_config_before_touching_the_device():
    lib = _abi.lib()
    c = _abi.sph_config()
    h = C.c_void_p()
    assert lib.sph_create(C.byref(c), None, 0, None, 0, None, C.byref(h)) == _abi.SPH_E_INVALID
    assert lib.sph_create(None, None, 0, None, 0, None, C.byref(h)) == _abi.SPH_E_INVALID
