"""Integrator selectors with the reference's names (torchfsm/integrator).

The enum members select the exponential time-stepping scheme run by the CUDA
library: ``ETDRKIntegrator.ETDRK0/1/2`` (Cox-Matthews, integrator/_etdrk.py)
and ``SETDRKIntegrator.SETDRK1..4`` (Kassam-Trefethen contour coefficients,
integrator/_stable_etdrk/). ``set_integrator(enum, n_integration_points=..,
integration_radius=.., cpu_cached=..)`` accepts the reference's options;
``cpu_cached`` is accepted and ignored (coefficients are always evaluated on
the device in FP64). ``RKIntegrator`` (explicit Runge-Kutta) is listed for
API compatibility; selecting it raises NotImplementedError.
"""

from enum import Enum

from .. import _lib


class ETDRKIntegrator(Enum):
    ETDRK0 = _lib.FSM_ETDRK0
    ETDRK1 = _lib.FSM_ETDRK1
    ETDRK2 = _lib.FSM_ETDRK2


class SETDRKIntegrator(Enum):
    SETDRK1 = _lib.FSM_SETDRK1
    SETDRK2 = _lib.FSM_SETDRK2
    SETDRK3 = _lib.FSM_SETDRK3
    SETDRK4 = _lib.FSM_SETDRK4


class RKIntegrator(Enum):
    Euler = "Euler"
    Midpoint = "Midpoint"
    Heun12 = "Heun12"
    Ralston12 = "Ralston12"
    BogackiShampine23 = "BogackiShampine23"
    RK4 = "RK4"
    RK4_38Rule = "RK4_38Rule"
    Dorpi45 = "Dorpi45"
    Fehlberg45 = "Fehlberg45"
    CashKarp45 = "CashKarp45"


__all__ = ["ETDRKIntegrator", "SETDRKIntegrator", "RKIntegrator"]
