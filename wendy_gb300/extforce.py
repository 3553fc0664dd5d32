"""Registered external forces.

wendy accepts any Python callable F(x, t) as ``ext_force`` and calls it
through numba or a ctypes callback once per force evaluation
(wendy/wendy.py:389-418).  A GPU kernel cannot call back into Python, so
wendy_gb300 evaluates closed forms inside the fused force kernel instead.
Each class below is one registered form.  Instances are also ordinary
callables with the same formula in numpy, so the same object can be handed
to the reference's ``wendy.nbody`` for comparison.
"""
import numpy

from ._lib import EXT_HARMONIC, EXT_PULSE_TANH


class RegisteredForce:
    kind = None
    params = ()

    def __call__(self, x, t):  # pragma: no cover - overridden
        raise NotImplementedError


class Harmonic(RegisteredForce):
    """F(x, t) = -omega^2 x, the form of wendy's own external-force tests
    (tests/test_approx_external.py:12)."""

    kind = EXT_HARMONIC

    def __init__(self, omega):
        self.omega2 = float(omega) ** 2.
        self.params = (self.omega2,)

    def __call__(self, x, t):
        return -self.omega2 * x


class PulseTanh(RegisteredForce):
    """F(x, t) = A exp(-(t - t0)^2 / (2 tau^2)) tanh(x / h): a transient
    antisymmetric kick that peaks at t0."""

    kind = EXT_PULSE_TANH

    def __init__(self, A, t0, tau, h):
        if tau == 0 or h == 0:
            raise ValueError("tau and h must be non-zero")
        self.A, self.t0, self.tau, self.h = float(A), float(t0), float(tau), float(h)
        self.params = (self.A, self.t0, self.tau, self.h)

    def __call__(self, x, t):
        return self.A * numpy.exp(-(t - self.t0) ** 2 / (2 * self.tau ** 2)) * numpy.tanh(x / self.h)


def evaluate_on_device(ext_force, x, t):
    """F(x, t) of a registered force evaluated on the GPU by the force
    kernels' own code (wg_ext_force_eval): the device counterpart of calling
    the force object itself."""
    from . import _lib
    kind, params = resolve(ext_force)
    x = numpy.ascontiguousarray(x, dtype=numpy.float64)
    out = numpy.empty(len(x))
    _lib.check(_lib.lib().wg_ext_force_eval(len(x), x, float(t), int(kind),
                                            _lib.ext_params(params), len(params), out),
               "wg_ext_force_eval")
    return out


def resolve(ext_force):
    """(kind, params) for the C ABI; rejects anything that is not registered."""
    if ext_force is None:
        return 0, ()
    if isinstance(ext_force, RegisteredForce):
        return ext_force.kind, tuple(ext_force.params)
    raise ValueError("ext_force must be a registered force (wendy_gb300.extforce.Harmonic, "
                     "wendy_gb300.extforce.PulseTanh); arbitrary Python callables cannot run "
                     "inside the GPU kernel")
