"""GB300-native SPH2S particle step (single-scale and two-scale WCSPH).

The solver runs in libsph2s.so (hand-written sm_103a kernels behind the C ABI
declared in include/sph2s.h); this package is the thin host-side mirror of the
reference's Solver / ParticleData surface plus scene builders.
"""
from ._abi import SphError, lib  # noqa: F401
from .solver import Grid, ParticleData, Solver, SolverConfiguration  # noqa: F401

__all__ = ["Grid", "ParticleData", "Solver", "SolverConfiguration", "SphError", "lib"]
