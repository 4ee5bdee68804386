"""Integrator selectors with the reference's names (torchfsm/integrator).

The enum members select the exponential time-stepping scheme run by the CUDA
library: ``ETDRKIntegrator.ETDRK0/1/2`` (Cox-Matthews, integrator/_etdrk.py)
and ``SETDRKIntegrator.SETDRK1..4`` (Kassam-Trefethen contour coefficients,
integrator/_stable_etdrk/). ``set_integrator(enum, n_integration_points=..,
integration_radius=.., cpu_cached=..)`` accepts the reference's options;
``cpu_cached`` is accepted and ignored (coefficients are always evaluated on
the device in FP64). ``RKIntegrator`` members select the explicit Runge-Kutta
schemes of integrator/_rk.py with a fixed step on the full right-hand side
L u + N(u) (operator/_base.py:408-431, 492-502); ``adaptive=True`` (step-size
control, integrator/_rk.py:60-79) raises NotImplementedError, as the reference's own
adaptive step does on spectral states (it takes torch.max of a complex tensor).

Each member's ``value`` is the library's scheme code (an int) and, like the reference's enum
values, builds an integrator object when called: ``SETDRKIntegrator.SETDRK4.value(dt,
linear_coef, nonlinear_func)`` (``.dt``, ``.step(u_hat)``), ``RKIntegrator.RK4.value()``
(``.step(f, x_t, dt)``); see ``_standalone``.
"""

from enum import Enum

from .. import _lib
from ._standalone import SchemeCode


class ETDRKIntegrator(Enum):
    ETDRK0 = SchemeCode(_lib.FSM_ETDRK0)
    ETDRK1 = SchemeCode(_lib.FSM_ETDRK1)
    ETDRK2 = SchemeCode(_lib.FSM_ETDRK2)


class SETDRKIntegrator(Enum):
    SETDRK1 = SchemeCode(_lib.FSM_SETDRK1)
    SETDRK2 = SchemeCode(_lib.FSM_SETDRK2)
    SETDRK3 = SchemeCode(_lib.FSM_SETDRK3)
    SETDRK4 = SchemeCode(_lib.FSM_SETDRK4)


class RKIntegrator(Enum):
    Euler = SchemeCode(_lib.FSM_RK_EULER)
    Midpoint = SchemeCode(_lib.FSM_RK_MIDPOINT)
    Heun12 = SchemeCode(_lib.FSM_RK_HEUN12)
    Ralston12 = SchemeCode(_lib.FSM_RK_RALSTON12)
    BogackiShampine23 = SchemeCode(_lib.FSM_RK_BOGACKI_SHAMPINE23)
    RK4 = SchemeCode(_lib.FSM_RK4)
    RK4_38Rule = SchemeCode(_lib.FSM_RK4_38RULE)
    Dorpi45 = SchemeCode(_lib.FSM_RK_DORPI45)
    Fehlberg45 = SchemeCode(_lib.FSM_RK_FEHLBERG45)
    CashKarp45 = SchemeCode(_lib.FSM_RK_CASHKARP45)


__all__ = ["ETDRKIntegrator", "SETDRKIntegrator", "RKIntegrator"]
