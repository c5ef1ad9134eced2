"""Single stages of the ADER-WENO step on the GPU (numpy in, numpy out).

Each wraps one C-ABI entry point of include/pypde_gb300.h and mirrors one
stage of the reference (haranjackson/PyPDE):
  boundaries  src/grid/boundaries.cpp:25-53
  weno        src/solvers/weno/weno.cpp:61-121 (= weno_solver)
  timestep    src/solvers/stepper.cpp:35-76
  predictor   src/solvers/dg/dg.cpp:204-224
  fv          src/solvers/fv/fv.cpp:200-207
"""
import ctypes

import numpy as np

from . import _lib
from .callbacks import builtin_system

FLUXES = {"rusanov": 0, "roe": 1, "osher": 2}


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def boundaries(u, N, bt):
    u = _f64(u)
    nX = np.array(u.shape[:-1], dtype=np.int32)
    V = u.shape[-1]
    ub = np.zeros(tuple(nX + 2 * N) + (V,))
    _lib.check(_lib.lib().pypde_boundaries(_lib.c_ptr(u), _lib.c_ptr(nX), len(nX),
                                           _lib.c_ptr(np.array(bt, dtype=np.int32)), N, V,
                                           _lib.c_ptr(ub)))
    return ub


def weno(ub, N):
    ub = _f64(ub)
    nXb = np.array(ub.shape[:-1], dtype=np.int32)
    ndim, V = len(nXb), ub.shape[-1]
    w = np.zeros((int(np.prod(nXb - 2 * (N - 1))) * N ** ndim, V))
    _lib.check(_lib.lib().weno_solver(_lib.c_ptr(w), _lib.c_ptr(ub), _lib.c_ptr(nXb), ndim, N,
                                      V))
    return w


def timestep(system, w, dX, N, cfl, tf, t, count):
    dX = np.asarray(dX, dtype=np.float64)
    s = builtin_system(system, len(dX))
    dt = ctypes.c_double()
    w = _f64(w)
    _lib.check(_lib.lib().pypde_timestep(s.handle, _lib.c_ptr(w), w.shape[0], _lib.c_ptr(dX),
                                         len(dX), N, cfl, tf, t, count, ctypes.byref(dt)))
    return dt.value


def predictor(system, w, dX, N, stiff, dt, tol=1e-12):
    """Returns (qh, stats dict)."""
    dX = np.asarray(dX, dtype=np.float64)
    s = builtin_system(system, len(dX))
    w = _f64(w)
    qh = np.zeros((w.shape[0] * N, w.shape[1]))
    st = _lib.Stats()
    _lib.check(_lib.lib().pypde_predictor(s.handle, _lib.c_ptr(w), w.shape[0], _lib.c_ptr(dX),
                                          len(dX), N, bool(stiff), dt, tol, _lib.c_ptr(qh), st))
    return qh, st.as_dict()


def predictor_guess(system, w, dX, N, dt, guess=None, warm=None, tol=1e-12):
    """Stiff predictor from an initial guess: a host array (N rows per row
    of w) or a WarmStart network.  Returns (qh, stats dict)."""
    dX = np.asarray(dX, dtype=np.float64)
    s = builtin_system(system, len(dX)) if isinstance(system, str) else system
    w = _f64(w)
    qh = np.zeros((w.shape[0] * N, w.shape[1]))
    g = None if guess is None else _f64(np.asarray(guess).reshape(qh.shape))
    st = _lib.Stats()
    _lib.check(_lib.lib().pypde_predictor_guess(
        s.handle, _lib.c_ptr(w), w.shape[0], _lib.c_ptr(dX), len(dX), N, dt, tol,
        _lib.c_ptr(g) if g is not None else None, warm.handle if warm is not None else None,
        _lib.c_ptr(qh), st))
    return qh, st.as_dict()


def fv(system, u, qh, dX, N, dt, flux="rusanov"):
    dX = np.asarray(dX, dtype=np.float64)
    s = builtin_system(system, len(dX))
    u = _f64(u).copy()
    qh = _f64(qh)
    nX = np.array(u.shape[:-1], dtype=np.int32)
    _lib.check(_lib.lib().pypde_fv(s.handle, _lib.c_ptr(u), _lib.c_ptr(qh), _lib.c_ptr(nX),
                                   _lib.c_ptr(dX), len(dX), N, FLUXES.get(flux, flux), dt))
    return u


def tables(N):
    out = np.zeros(4 * N + 8 * N * N)
    _lib.check(_lib.lib().pypde_tables(N, _lib.c_ptr(out)))
    return out
