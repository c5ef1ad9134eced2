"""Built-in callback systems.

Each system exposes Python callables F, B, S with the reference's callback
signatures (pypde/solvers.py:80-119): ``F(Q, d)`` (or ``F(Q, DQ, d)`` for
the second-order form), ``B(Q, d)``, ``S(Q)``.  They are plain numpy
functions, usable on their own, and each carries the name of its compiled
device twin (pypde_gb300/csrc/systems.cuh) so that ``pde_solver`` runs the
device code.  Both evaluate the same formulas in the same operation order.

    euler(ndim)     V = ndim+2, Q = (rho, m_0..m_{ndim-1}, E), gamma = 1.4
    cattaneo(ndim)  V = 2 ndim+3: Euler + relaxing heat flux q + passive
                    s = log10(tau); T = p/rho; heat-flux flux kappa_h T with
                    kappa_h = kappa/tau_ref = 1e-2/1e-2; S_q = -q/tau
    ncp(ndim)       V = 3, a non-conservative test system with F, B and S
    burgers2()      V = 1, viscous Burgers F(Q, DQ, d) (second order)
"""
from dataclasses import dataclass
from typing import Callable, Optional

import numpy as np

GAMMA = 1.4
KAPPA_H = 1.0  # kappa / tau_ref = 1e-2 / 1e-2


# 1/k! for k = 0..16, each the double nearest to it
_INV_FACT = (1.0, 1.0, 0.5, 0.16666666666666666, 0.041666666666666664, 0.008333333333333333, 0.001388888888888889, 0.0001984126984126984, 2.48015873015873e-05, 2.7557319223985893e-06, 2.755731922398589e-07, 2.505210838544172e-08, 2.08767569878681e-09, 1.6059043836821613e-10, 1.1470745597729725e-11, 7.647163731819816e-13, 4.779477332387385e-14)


def pow10_portable(x):
    """10^x from +, *, floor and ldexp only, so that host and device agree
    bitwise: 10^x = 2^n e^r with n = round(x log2 10), |r| <= ln2/2, and e^r
    by its Taylor polynomial of degree 16 in Horner form (truncation error
    below 1e-22)."""
    y = x * 3.321928094887362
    n = np.floor(y + 0.5)
    r = (y - n) * 0.6931471805599453
    p = _INV_FACT[16]
    for k in range(15, -1, -1):
        p = p * r + _INV_FACT[k]
    return float(np.ldexp(p, int(n)))


@dataclass
class System:
    name: str
    ndim: int
    V: int
    F: Optional[Callable]
    B: Optional[Callable]
    S: Optional[Callable]
    second_order: bool = False


def _tag(fn, name, ndim, role):
    fn._pypde_builtin = (name, ndim)
    fn._pypde_role = role
    return fn


def euler(ndim):
    def F(Q, d):
        r = Q[0]
        ke = 0.0
        for i in range(ndim):
            ke += Q[1 + i] * Q[1 + i]
        p = (GAMMA - 1.0) * (Q[ndim + 1] - 0.5 * ke / r)
        ud = Q[1 + d] / r
        out = np.zeros(ndim + 2)
        out[0] = Q[1 + d]
        for i in range(ndim):
            out[1 + i] = Q[1 + i] * ud
        out[1 + d] += p
        out[ndim + 1] = (Q[ndim + 1] + p) * ud
        return out

    return System("euler", ndim, ndim + 2, _tag(F, "euler", ndim, "F"), None, None)


def cattaneo(ndim):
    V = 2 * ndim + 3

    def F(Q, d):
        r = Q[0]
        ke = 0.0
        for i in range(ndim):
            ke += Q[1 + i] * Q[1 + i]
        p = (GAMMA - 1.0) * (Q[ndim + 1] - 0.5 * ke / r)
        ud = Q[1 + d] / r
        out = np.zeros(V)
        out[0] = Q[1 + d]
        for i in range(ndim):
            out[1 + i] = Q[1 + i] * ud
        out[1 + d] += p
        out[ndim + 1] = (Q[ndim + 1] + p) * ud
        T = p / Q[0]
        out[ndim + 1] += Q[ndim + 2 + d]
        out[ndim + 2 + d] = KAPPA_H * T
        return out

    def S(Q):
        inv_tau = pow10_portable(-Q[2 * ndim + 2])
        out = np.zeros(V)
        for i in range(ndim):
            out[ndim + 2 + i] = -Q[ndim + 2 + i] * inv_tau
        return out

    return System("cattaneo", ndim, V, _tag(F, "cattaneo", ndim, "F"), None,
                  _tag(S, "cattaneo", ndim, "S"))


_NCP_A = (1.0, 0.5, 0.25)


def ncp(ndim):
    def F(Q, d):
        a = _NCP_A[d]
        return np.array([a * (0.5 * Q[0] * Q[0]), a * (Q[0] * Q[1]), a * (Q[0] * Q[2])])

    def B(Q, d):
        a = _NCP_A[d]
        out = np.zeros((3, 3))
        out[1, 1] = a * Q[0]
        out[1, 2] = a * 0.2
        out[2, 1] = a * 0.2
        out[2, 2] = a * Q[0]
        return out

    def S(Q):
        return np.array([0.0, 0.1 * (Q[2] - Q[1]), -0.1 * (Q[1] + Q[2])])

    return System("ncp", ndim, 3, _tag(F, "ncp", ndim, "F"), _tag(B, "ncp", ndim, "B"),
                  _tag(S, "ncp", ndim, "S"))


def burgers2():
    def F(Q, DQ, d):
        return np.array([_NCP_A[d] * (0.5 * Q[0] * Q[0]) - 0.01 * DQ[d][0]])

    return System("burgers2", 1, 1, _tag(F, "burgers2", 1, "F"), None, None, True)


BUILTINS = {"euler": euler, "cattaneo": cattaneo, "ncp": ncp}
