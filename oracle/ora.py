"""ctypes binding of the CPU checkers.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product (pypde_gb300).

  port()  -> liboracle.so, the plain-C restatement of the reference's step
             (oracle/ader_oracle.c), built on demand with `make port`.
  ref()   -> libref_driver.so, the reference itself compiled from its own
             sources (`make ref`); only where the reference tree exists.
"""
import ctypes
import os
import subprocess
from ctypes import POINTER, c_char_p, c_double, c_int, c_long, c_void_p

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_driver.so")
REF_TIGHT_LIB = os.path.join(HERE, "_ref", "libref_driver_tight.so")
# the reference tree: $PYPDE_REFERENCE, else a directory `reference` beside
# this repository
REF_SRC = os.environ.get("PYPDE_REFERENCE",
                         os.path.abspath(os.path.join(HERE, "..", "..", "reference")))

D = c_double
dp = POINTER(c_double)
ip = POINTER(c_int)

_port = None
_ref = {}


def build_port():
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    return PORT_LIB


def build_ref():
    if not os.path.isdir(os.path.join(REF_SRC, "src")):
        raise FileNotFoundError("reference tree not present")
    subprocess.run(["make", "-s", "-j8", "-C", HERE, "ref", f"REF={REF_SRC}"], check=True)
    return REF_LIB


def ptr(a):
    if a is None:
        return None
    if a.dtype == np.int32:
        return a.ctypes.data_as(ip)
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(dp)


def port():
    global _port
    if _port is None:
        if not os.path.exists(PORT_LIB):
            build_port()
        L = ctypes.CDLL(PORT_LIB)
        L.ora_timestep.restype = D
        L.ora_timestep.argtypes = [c_void_p, c_void_p, dp, c_long, dp, c_int, c_int, c_int, D,
                                   D, D, c_long, c_int]
        L.ora_predictor.restype = c_long
        L.ora_predictor.argtypes = [c_void_p, c_void_p, c_void_p, dp, c_long, dp, c_int, c_int,
                                    c_int, c_int, D, D, dp, ip, c_int]
        L.ora_predictor_guess.restype = c_long
        L.ora_predictor_guess.argtypes = [c_void_p, c_void_p, c_void_p, dp, c_long, dp, c_int,
                                          c_int, c_int, D, D, dp, dp, ip,
                                          POINTER(ctypes.c_long), c_int]
        L.ora_fv.restype = None
        L.ora_fv.argtypes = [c_void_p, c_void_p, c_void_p, dp, dp, ip, dp, c_int, c_int, c_int,
                             c_int, c_int, D]
        L.ora_pde_solver.restype = c_long
        L.ora_pde_solver.argtypes = [c_void_p, c_void_p, c_void_p, dp, D, ip, c_int, dp, D, ip,
                                     c_int, c_int, c_int, c_int, c_int, c_int, dp, c_int, c_long,
                                     D, dp]
        L.ora_boundaries.argtypes = [dp, ip, c_int, ip, c_int, c_int, dp]
        L.ora_weno.argtypes = [dp, ip, c_int, c_int, c_int, dp]
        L.ora_system_lookup.argtypes = [c_char_p, c_int, ip, POINTER(c_void_p),
                                        POINTER(c_void_p), POINTER(c_void_p), ip]
        L.ora_system_lookup32.argtypes = [c_char_p, c_int, POINTER(c_void_p),
                                          POINTER(c_void_p), POINTER(c_void_p)]
        L.ora_predictor_mixed.restype = c_long
        L.ora_predictor_mixed.argtypes = [c_void_p] * 6 + [dp, c_long, dp, c_int, c_int, c_int,
                                                           D, D, dp, ip, POINTER(c_long), c_int]
        L.ora_predictor_guess_mixed.restype = c_long
        L.ora_predictor_guess_mixed.argtypes = [c_void_p] * 6 + [
            dp, c_long, dp, c_int, c_int, c_int, D, D, dp, dp, ip, POINTER(ctypes.c_long),
            POINTER(c_long), c_int]
        L.ora_pde_solver_mixed.restype = c_long
        L.ora_pde_solver_mixed.argtypes = [c_void_p] * 6 + [dp, D, ip, c_int, dp, D, ip, c_int,
                                                            c_int, c_int, c_int, c_int, dp,
                                                            c_int, c_long, D, dp]
        L.ora_max_abs_eig.restype = D
        L.ora_max_abs_eig.argtypes = [dp, c_int]
        L.ora_eig.argtypes = [dp, c_int, dp, dp, dp, dp]
        _port = L
    return _port


def ref(tight=False):
    path = REF_TIGHT_LIB if tight else REF_LIB
    if path not in _ref:
        if not os.path.exists(path):
            build_ref()
        L = ctypes.CDLL(path)
        L.ref_timestep.restype = D
        L.ref_timestep.argtypes = [c_char_p, dp, c_long, dp, c_int, c_int, D, D, D, c_int]
        L.ref_predictor.argtypes = [c_char_p, dp, c_long, dp, c_int, c_int, c_int, D, dp]
        L.ref_fv.argtypes = [c_char_p, dp, dp, ip, dp, c_int, c_int, c_int, D]
        L.ref_pde_solver.argtypes = [c_char_p, dp, D, ip, c_int, dp, D, ip, c_int, c_int, c_int,
                                     c_int, dp, c_int]
        L.ref_step_times.argtypes = [c_char_p, dp, ip, c_int, dp, D, ip, c_int, c_int, c_int, D,
                                     c_int, dp]
        L.ref_tables.argtypes = [c_int, dp, dp, dp, dp]
        L.ref_boundaries.argtypes = [dp, ip, c_int, ip, c_int, c_int, dp]
        L.ref_weno.argtypes = [dp, ip, c_int, c_int, c_int, dp]
        _ref[path] = L
    return _ref[path]


class PortSystem:
    """The C callbacks of one test system (oracle_systems.c)."""

    def __init__(self, name, ndim):
        V = c_int()
        so = c_int()
        self.F, self.B, self.S = c_void_p(), c_void_p(), c_void_p()
        rc = port().ora_system_lookup(name.encode(), ndim, ctypes.byref(V), ctypes.byref(self.F),
                                      ctypes.byref(self.B), ctypes.byref(self.S),
                                      ctypes.byref(so))
        if rc:
            raise ValueError(f"unknown system {name}/{ndim}")
        self.name, self.ndim, self.V, self.second_order = name, ndim, V.value, so.value
        self.F32, self.B32, self.S32 = c_void_p(), c_void_p(), c_void_p()
        port().ora_system_lookup32(name.encode(), ndim, ctypes.byref(self.F32),
                                   ctypes.byref(self.B32), ctypes.byref(self.S32))


# ---------------------------------------------------------------- stages


def boundaries(u, N, bt):
    nX = np.array(u.shape[:-1], dtype=np.int32)
    V = u.shape[-1]
    ub = np.zeros(tuple(nX + 2 * N) + (V,))
    port().ora_boundaries(ptr(np.ascontiguousarray(u)), ptr(nX), len(nX),
                          ptr(np.array(bt, dtype=np.int32)), N, V, ptr(ub))
    return ub


def weno(ub, N):
    nXb = np.array(ub.shape[:-1], dtype=np.int32)
    ndim = len(nXb)
    V = ub.shape[-1]
    nout = int(np.prod(nXb - 2 * (N - 1)))
    w = np.zeros((nout * N ** ndim, V))
    port().ora_weno(ptr(np.ascontiguousarray(ub)), ptr(nXb), ndim, N, V, ptr(w))
    return w


def timestep(sysname, w, dX, N, cfl, tf, t, count):
    dX = np.asarray(dX, dtype=np.float64)
    s = PortSystem(sysname, len(dX))
    return port().ora_timestep(s.F, s.B, ptr(w), w.shape[0], ptr(dX), len(dX), N, s.V, cfl, tf,
                               t, count, s.second_order)


def predictor(sysname, w, dX, N, stiff, dt, tol=1e-12):
    dX = np.asarray(dX, dtype=np.float64)
    s = PortSystem(sysname, len(dX))
    qh = np.zeros((w.shape[0] * N, s.V))
    mi = c_int()
    its = port().ora_predictor(s.F, s.B, s.S, ptr(w), w.shape[0], ptr(dX), len(dX), N, s.V,
                               int(stiff), dt, tol, ptr(qh), ctypes.byref(mi),
                               s.second_order)
    return qh, its, mi.value


def predictor_guess(sysname, w, dX, N, dt, guess, tol=1e-12, mixed=False):
    """Stiff predictor from a warm start; returns (qh, iters, max_iters,
    cells that fell back to the plain guess).  mixed=True: FP32 sweeps from
    the guess first, and a fifth item, the FP32 sweeps."""
    dX = np.asarray(dX, dtype=np.float64)
    s = PortSystem(sysname, len(dX))
    qh = np.zeros((w.shape[0] * N, s.V))
    g = np.ascontiguousarray(guess, dtype=np.float64).reshape(qh.shape)
    mi = c_int()
    fb = ctypes.c_long()
    if mixed:
        sw = ctypes.c_long()
        its = port().ora_predictor_guess_mixed(s.F, s.B, s.S, s.F32, s.B32, s.S32, ptr(w),
                                               w.shape[0], ptr(dX), len(dX), N, s.V, dt, tol,
                                               ptr(g), ptr(qh), ctypes.byref(mi),
                                               ctypes.byref(fb), ctypes.byref(sw),
                                               s.second_order)
        return qh, its, mi.value, fb.value, sw.value
    its = port().ora_predictor_guess(s.F, s.B, s.S, ptr(w), w.shape[0], ptr(dX), len(dX), N,
                                     s.V, dt, tol, ptr(g), ptr(qh), ctypes.byref(mi),
                                     ctypes.byref(fb), s.second_order)
    return qh, its, mi.value, fb.value


def predictor_mixed(sysname, w, dX, N, dt, tol=1e-12):
    """The mixed-precision stiff predictor: FP32 sweeps, then FP64 Newton
    with at least two updates; returns (qh, FP64 iterations, their per-cell
    maximum, FP32 sweeps)."""
    dX = np.asarray(dX, dtype=np.float64)
    s = PortSystem(sysname, len(dX))
    qh = np.zeros((w.shape[0] * N, s.V))
    mi = c_int()
    sw = ctypes.c_long()
    its = port().ora_predictor_mixed(s.F, s.B, s.S, s.F32, s.B32, s.S32, ptr(w), w.shape[0],
                                     ptr(dX), len(dX), N, s.V, dt, tol, ptr(qh),
                                     ctypes.byref(mi), ctypes.byref(sw), s.second_order)
    return qh, its, mi.value, sw.value


def fv(sysname, u, qh, dX, N, dt, flux=0):
    dX = np.asarray(dX, dtype=np.float64)
    s = PortSystem(sysname, len(dX))
    u = np.ascontiguousarray(u).copy()
    nX = np.array(u.shape[:-1], dtype=np.int32)
    port().ora_fv(s.F, s.B, s.S, ptr(u), ptr(qh), ptr(nX), ptr(dX), len(dX), N, s.V, flux,
                  s.second_order, dt)
    return u


def pde_solver(sysname, u0, tf, L, bt, cfl, N, stiff=False, flux=0, ndt=1, nthreads=1,
               max_steps=-1, newton_tol=1e-12, mixed=False):
    """Run the port; returns (u_final, ret, steps, t_final).  mixed=True: the
    mixed-precision stiff predictor (stiff implied)."""
    nX = np.array(u0.shape[:-1], dtype=np.int32)
    ndim = len(nX)
    s = PortSystem(sysname, ndim)
    dX = np.array([L[i] / nX[i] for i in range(ndim)], dtype=np.float64)
    u = np.ascontiguousarray(u0, dtype=np.float64).copy()
    ret = np.zeros((ndt,) + u.shape)
    tout = D()
    if mixed:
        steps = port().ora_pde_solver_mixed(s.F, s.B, s.S, s.F32, s.B32, s.S32, ptr(u), tf,
                                            ptr(nX), ndim, ptr(dX), cfl,
                                            ptr(np.array(bt, dtype=np.int32)), flux, N, s.V, ndt,
                                            s.second_order, ptr(ret), nthreads, max_steps,
                                            newton_tol, ctypes.byref(tout))
        return u, ret, steps, tout.value
    steps = port().ora_pde_solver(s.F, s.B, s.S, ptr(u), tf, ptr(nX), ndim, ptr(dX), cfl,
                                  ptr(np.array(bt, dtype=np.int32)), int(stiff), flux, N, s.V,
                                  ndt, s.second_order, ptr(ret), nthreads, max_steps, newton_tol,
                                  ctypes.byref(tout))
    return u, ret, steps, tout.value


def tables(N):
    """nodes, wghts, dervals, endvals, dgmat, dgmat_inv, weno_inv[4], sig."""

    class Tab(ctypes.Structure):
        _fields_ = [("N", c_int), ("nodes", D * 8), ("wghts", D * 8), ("dervals", D * 64),
                    ("endvals", D * 16), ("dgmat", D * 64), ("dgmat_inv", D * 64),
                    ("weno_inv", D * 256), ("sig", D * 64)]

    T = Tab()
    port().ora_make_tables(N, ctypes.byref(T))
    n2 = N * N
    wi = np.array(T.weno_inv).reshape(4, 64)[:, :n2].ravel()
    return np.concatenate([np.array(T.nodes[:N]), np.array(T.wghts[:N]),
                           np.array(T.dervals[:n2]), np.array(T.endvals[:2 * N]),
                           np.array(T.dgmat[:n2]), np.array(T.dgmat_inv[:n2]), wi,
                           np.array(T.sig[:n2])])
