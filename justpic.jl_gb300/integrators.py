"""Time integrators of advection!, mirroring src/Advection/types.jl:17-62."""
from __future__ import annotations

from ._native import JP_EULER, JP_RUNGE_KUTTA2, JP_RUNGE_KUTTA4, ArgumentError


class AbstractAdvectionIntegrator:
    code = -1
    alpha = 0.0


class Euler(AbstractAdvectionIntegrator):
    """Forward Euler (src/Advection/types.jl:17-19); any arguments are ignored."""

    code = JP_EULER

    def __init__(self, *args):
        pass


class RungeKutta2(AbstractAdvectionIntegrator):
    """Two-stage Runge-Kutta with stage position alpha, 0 < alpha < 1
    (src/Advection/types.jl:29-40); alpha = 0.5 is the midpoint method."""

    code = JP_RUNGE_KUTTA2

    def __init__(self, alpha: float = 0.5):
        if not (0 < alpha < 1):
            raise ArgumentError("Only 0 < α < 1 is supported")
        self.alpha = float(alpha)

    @property
    def α(self):  # noqa: N802 - the reference's field name
        return self.alpha


class RungeKutta4(AbstractAdvectionIntegrator):
    """Classical fourth-order Runge-Kutta (src/Advection/types.jl:47-49)."""

    code = JP_RUNGE_KUTTA4

    def __init__(self, *args):
        pass
