"""GB300-native rebuild of wendy's approximate 1D N-body integrator.

``wendy_gb300.nbody(x, v, m, dt, approx=True, nleap=..., sort='cuda')`` is a
drop-in for ``wendy.nbody``'s approximate path; the work runs in one CUDA
shared library (include/wendy_gb300.h) loaded through ctypes.
"""
from .diagnostics import energy, momentum, potential  # noqa: F401
from .extforce import Harmonic, PulseTanh  # noqa: F401
from .wendy import Simulation, accel, approx_onestep, nbody  # noqa: F401

__all__ = ["nbody", "accel", "approx_onestep", "energy", "momentum", "potential", "Simulation", "Harmonic", "PulseTanh"]
