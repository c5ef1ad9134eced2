"""The reference-signature C entry point, bound exactly as the reference
binds its own library.

pypde/utils.py:9-16 declares ADER_ARGTYPES, and pypde/solvers.py:200-212
calls `solver(_F.ctypes, _B.ctypes, _S.ctypes, useF, useB, useS, c_ptr(ur),
tf, c_ptr(nX), ndim, c_ptr(dX), cfl, c_ptr(boundaryTypes), stiff,
FLUXES[flux], order, V, ndt, secondOrder, c_ptr(ret), nThreads)`.  These
tests make that call against libpypde_gb300.so with the same argument list
and a device callback handle (pypde_system_builtin) in the callback slots,
and compare the in-place final state and the snapshot rows with the CPU
oracle bit for bit.
"""
import os
from ctypes import POINTER, byref, c_bool, c_char_p, c_double, c_int, c_void_p

import numpy as np
import pytest

from oracle import ora
from pypde_gb300 import _lib, workloads

# the reference's argument list, pypde/utils.py:9-16
ADER_ARGTYPES = [
    c_void_p, c_void_p, c_void_p, c_bool, c_bool, c_bool,
    POINTER(c_double), c_double,
    POINTER(c_int), c_int,
    POINTER(c_double), c_double,
    POINTER(c_int), c_bool, c_int, c_int, c_int, c_int, c_bool,
    POINTER(c_double), c_int
]


def c_ptr(arr):  # pypde/utils.py:25-34
    return arr.ctypes.data_as(POINTER(c_int) if arr.dtype == np.int32 else POINTER(c_double))


def solver_and_handle(name, ndim):
    lib = _lib.lib()
    solver = lib.pde_solver
    solver.argtypes = ADER_ARGTYPES
    solver.restype = c_int
    lib.pypde_system_builtin.argtypes = [c_char_p, c_int, POINTER(c_void_p)]
    lib.pypde_system_builtin.restype = c_int
    h = c_void_p()
    assert lib.pypde_system_builtin(name.encode(), ndim, byref(h)) == _lib.PYPDE_OK
    return solver, h


def call(solver, h, use, Q0, tf, L, bt, cfl, stiff, flux, order, ndt):
    """pypde/solvers.py:177-214 with the callbacks replaced by the handle."""
    nX = np.array(Q0.shape[:-1], dtype=np.int32)
    ndim, V = len(nX), Q0.shape[-1]
    dX = np.array([L[i] / nX[i] for i in range(ndim)])
    boundaryTypes = np.array(bt, dtype=np.int32)
    ret = np.zeros(ndt * Q0.size)
    ur = Q0.ravel()
    useF, useB, useS = use
    rc = solver(h if useF else None, h if useB else None, h if useS else None, useF, useB, useS,
                c_ptr(ur), tf, c_ptr(nX), ndim, c_ptr(dX), cfl, c_ptr(boundaryTypes), stiff,
                flux, order, V, ndt, False, c_ptr(ret), -1)
    return rc, ret.reshape((ndt,) + Q0.shape)


def test_reference_signature_checks_arguments_on_host(gpu_lib):
    """A V that does not match the callback system is refused with
    PYPDE_ERR_ARG before any device work (runs without a GPU too)."""
    solver, h = solver_and_handle("euler", 1)
    Q0 = workloads.sod(16)
    nX = np.array([16], dtype=np.int32)
    dX = np.array([1.0 / 16])
    bt = np.array([0], dtype=np.int32)
    ret = np.zeros(Q0.size)
    rc = solver(h, None, None, True, False, False, c_ptr(Q0.ravel()), 0.2, c_ptr(nX), 1,
                c_ptr(dX), 0.9, c_ptr(bt), False, 0, 2, 4, 1, False, c_ptr(ret), -1)
    assert rc == _lib.PYPDE_ERR_ARG


@pytest.mark.gpu
def test_sod400_full_run_through_reference_signature(gpu_lib):
    """Config 1 of the benchmark (1-D Sod + 1e-3 noise, 400 cells,
    transmissive, N=2, Rusanov, CFL 0.9, tf=0.2) with ndt=4 snapshots, as
    pypde/solvers.py calls it: state and every snapshot row equal the CPU
    oracle's bit for bit, and Q0 holds the final state."""
    solver, h = solver_and_handle("euler", 1)
    u0 = workloads.sod(400)
    Q0 = u0.copy()
    rc, ret = call(solver, h, (True, False, False), Q0, 0.2, [1.0], [0], 0.9, False, 0, 2, 4)
    assert rc == _lib.PYPDE_OK
    u_o, ret_o, steps, t_o = ora.pde_solver("euler", u0, 0.2, [1.0], [0], 0.9, 2, ndt=4,
                                            nthreads=os.cpu_count() or 1)
    assert steps == 199 and t_o == 0.2
    assert np.array_equal(Q0, u_o)
    assert np.array_equal(ret, ret_o)
    assert np.array_equal(ret[-1], Q0)


@pytest.mark.gpu
def test_stiff_relaxation_through_reference_signature(gpu_lib):
    """The stiff relaxation system (F and S from one handle, STIFF=True):
    the Newton predictor to 1e-12 through the reference-signature entry
    point equals the CPU oracle bit for bit."""
    solver, h = solver_and_handle("cattaneo", 2)
    u0 = workloads.relaxation(24, 2, seed=5)
    # the end time of the oracle's fifth step, so that both run 5 steps
    _, _, steps, tf = ora.pde_solver("cattaneo", u0, 10.0, [1.0, 1.0], [1, 1], 0.8, 2,
                                     stiff=True, max_steps=5)
    assert steps == 5
    u_o, ret_o, steps_o, t_o = ora.pde_solver("cattaneo", u0, tf, [1.0, 1.0], [1, 1], 0.8, 2,
                                              stiff=True, ndt=2)
    Q0 = u0.copy()
    rc, ret = call(solver, h, (True, False, True), Q0, tf, [1.0, 1.0], [1, 1], 0.8, True, 0, 2,
                   2)
    assert rc == _lib.PYPDE_OK
    assert steps_o == 5 and t_o == tf
    assert np.array_equal(Q0, u_o)
    assert np.array_equal(ret, ret_o)
