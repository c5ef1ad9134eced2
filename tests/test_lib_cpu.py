"""CPU-only checks of the library and the host-side API: the C-ABI library
loads without a GPU and exports every entry point of include/pypde_gb300.h;
the host-side tables are bit-identical to the CPU restatement's; argument
handling follows the reference (pypde/utils.py, pypde/solvers.py)."""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT
from oracle import ora


def header_functions():
    src = open(os.path.join(ROOT, "include", "pypde_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\s*\*?\s*(\w+)\s*\(", src, flags=re.M)))


def test_library_exports_header(gpu_lib):
    names = header_functions()
    assert "pde_solver" in names and "weno_solver" in names
    for n in names:
        assert hasattr(gpu_lib, n), n


def test_library_loads_without_gpu_and_fails_loudly(gpu_lib):
    """No CPU fallback: without a usable GPU the solver reports a CUDA error."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from pypde_gb300 import _lib, systems
    from pypde_gb300.solvers import pde_solver
    s = systems.euler(1)
    with pytest.raises(_lib.PyPDEError) as e:
        pde_solver(np.ones((8, 3)), 0.1, [1.0], F=s.F, stiff=False)
    assert e.value.code == _lib.PYPDE_ERR_CUDA


BUILTINS = [("euler", 1, 3), ("euler", 2, 4), ("euler", 3, 5), ("cattaneo", 2, 7),
            ("cattaneo", 3, 9), ("ncp", 1, 3), ("ncp", 2, 3), ("burgers2", 1, 1)]


@pytest.mark.parametrize("case", BUILTINS, ids=lambda c: f"{c[0]}{c[1]}")
def test_builtin_orders_registered(gpu_lib, case):
    """Each (system, order) pair is compiled in its own unit and the units
    register into one description per system: orders 1-3 pass the host's
    order check and only then meet the missing GPU (a CUDA error); order 4
    is refused as unsupported before any CUDA call."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from pypde_gb300 import _lib, stages
    name, ndim, V = case
    for N in (1, 2, 3, 4):
        w = np.zeros((N ** ndim, V))
        with pytest.raises(_lib.PyPDEError) as e:
            stages.timestep(name, w, [1.0] * ndim, N, 0.9, 1.0, 0.0, 7)
        want = _lib.PYPDE_ERR_CUDA if N <= 3 else _lib.PYPDE_ERR_UNSUPPORTED
        assert e.value.code == want, (N, e.value)


@pytest.mark.parametrize("N", range(1, 7))
def test_tables_bitwise_equal_to_port(gpu_lib, N):
    from pypde_gb300 import stages
    assert np.array_equal(stages.tables(N), ora.tables(N))


def test_boundary_parsing_matches_reference():
    from pypde_gb300.utils import parse_boundary_types
    assert list(parse_boundary_types("periodic", 2)) == [1, 1]
    assert list(parse_boundary_types(["transitive", "periodic"], 2)) == [0, 1]
    for bad in ("wall", ["periodic"], 3):
        with pytest.raises(SystemExit):
            parse_boundary_types(bad, 2)


def test_builtin_python_callbacks_match_c_callbacks():
    """The numpy twins of the built-in systems equal the C callbacks."""
    from pypde_gb300 import systems, workloads
    P = ora.port()
    for name, ndim in (("euler", 1), ("euler", 2), ("euler", 3), ("cattaneo", 2), ("ncp", 2)):
        s = getattr(systems, name)(ndim)
        ps = ora.PortSystem(name, ndim)
        fn = ctypes.CFUNCTYPE(None, ctypes.POINTER(ctypes.c_double),
                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                              ctypes.c_int)(ps.F.value)
        q = workloads.random_state(name, (1,) * ndim, 3).reshape(-1)
        for d in range(ndim):
            out = np.zeros(s.V)
            fn(ora.ptr(out), ora.ptr(q.copy()), ora.ptr(np.zeros(ndim * s.V)), d)
            assert np.array_equal(out, s.F(q, d))


def untranslatable_flux(Q, d):
    return [q * d for q in Q]


def test_untranslatable_callback_is_rejected():
    """Callbacks outside the translatable subset fail with a message naming
    the function and line, before any device work."""
    from pypde_gb300.solvers import pde_solver
    from pypde_gb300.translate import TranslateError
    with pytest.raises(TranslateError, match="untranslatable_flux"):
        pde_solver(np.ones((8, 3)), 0.1, [1.0], F=untranslatable_flux, stiff=False)


def test_batch_arguments_checked_before_device_work():
    """pde_solver_batch validates every problem on the host: a bad order, a
    periodic axis shorter than the order, or mismatched shapes fail with
    PYPDE_ERR_ARG (or a Python error) before any device call."""
    from pypde_gb300 import _lib, systems
    from pypde_gb300.solvers import pde_solver_batch
    s = systems.cattaneo(2)
    good = {"Q0": np.ones((8, 8, 7)), "tf": 0.1, "L": [1.0, 1.0], "order": 2}
    with pytest.raises(_lib.PyPDEError) as e:
        pde_solver_batch([good, dict(good, Q0=np.ones((8, 8, 7)), order=0)], F=s.F, S=s.S)
    assert e.value.code == _lib.PYPDE_ERR_ARG
    with pytest.raises(_lib.PyPDEError) as e:
        pde_solver_batch([dict(good, Q0=np.ones((1, 8, 7)), boundaryTypes="periodic")],
                         F=s.F, S=s.S)
    assert e.value.code == _lib.PYPDE_ERR_ARG
    with pytest.raises(ValueError):
        pde_solver_batch([good, dict(good, Q0=np.ones((8, 8, 4)))], F=s.F, S=s.S)
    with pytest.raises(ValueError):
        pde_solver_batch([], F=s.F, S=s.S)


def test_empty_grid_rejected_before_device_work():
    from pypde_gb300 import _lib, systems
    from pypde_gb300.solvers import pde_solver
    s = systems.euler(1)
    with pytest.raises(_lib.PyPDEError) as e:
        pde_solver(np.ones((0, 3)), 0.1, [1.0], F=s.F, stiff=False)
    assert e.value.code == _lib.PYPDE_ERR_ARG


def test_ader_solver_alias_takes_only_m_none():
    """ader_solver is pde_solver; M is accepted only as None (the
    reference's pde_solver has no M), and refused before any GPU work."""
    from pypde_gb300 import ader_solver, pde_solver, systems
    assert ader_solver is pde_solver
    s = systems.euler(1)
    with pytest.raises(NotImplementedError):
        ader_solver(np.ones((8, 3)), 0.1, [1.0], F=s.F, M=lambda Q: Q, stiff=False)



def test_flux_code_checked_before_device_work(gpu_lib):
    """FLUX outside 0-2 is refused with PYPDE_ERR_ARG on the host for
    built-in and run-time compiled systems alike (a run-time system's
    kernels are compiled on first use, after this check)."""
    import ctypes

    from pypde_gb300 import _lib
    u = np.ones((8, 3))
    nX = np.array([8], dtype=np.int32)
    dX = np.array([1.0 / 8])
    bt = np.array([0], dtype=np.int32)
    ret = np.zeros((1, 8, 3))
    handles = []
    h = ctypes.c_void_p()
    _lib.check(gpu_lib.pypde_system_builtin(b"euler", 1, ctypes.byref(h)))
    handles.append(h)
    h = ctypes.c_void_p()
    src = b"struct UserSystem {};"  # recorded only: compiled on first use
    _lib.check(gpu_lib.pypde_system_compile(src, b"user", 1, 3, 1, 0, 0, 0, ctypes.byref(h)))
    handles.append(h)
    try:
        for h in handles:
            for flux in (-1, 3):
                rc = gpu_lib.pde_solver_ex(h, True, False, False, _lib.c_ptr(u), 0.1,
                                           _lib.c_ptr(nX), 1, _lib.c_ptr(dX), 0.9,
                                           _lib.c_ptr(bt), False, flux, 2, 1, _lib.c_ptr(ret),
                                           None, None)
                assert rc == _lib.PYPDE_ERR_ARG
                assert b"FLUX" in gpu_lib.pypde_last_error()
    finally:
        for h in handles:
            gpu_lib.pypde_system_free(h)


def test_boundary_codes_checked_before_device_work(gpu_lib):
    """The ghost-fill entry point refuses boundary codes other than 0 and 1
    on the host (the kernel would treat them as periodic without the
    periodic axis-length check)."""
    from pypde_gb300 import _lib
    u = np.ones((3, 4, 2))
    nX = np.array([3, 4], dtype=np.int32)
    ub = np.zeros((3 + 4, 4 + 4, 2))
    for bt in ([2, 0], [0, -1]):
        rc = gpu_lib.pypde_boundaries(_lib.c_ptr(u), _lib.c_ptr(nX), 2,
                                      _lib.c_ptr(np.array(bt, dtype=np.int32)), 2, 2,
                                      _lib.c_ptr(ub))
        assert rc == _lib.PYPDE_ERR_ARG
        assert b"boundaryTypes" in gpu_lib.pypde_last_error()


def test_strip_count_checked_before_device_work(gpu_lib):
    """pypde_options.strips outside 0-32 is refused with PYPDE_ERR_ARG on
    the host, before any device work."""
    import ctypes

    from pypde_gb300 import _lib
    u = np.ones((8, 3))
    nX = np.array([8], dtype=np.int32)
    dX = np.array([1.0 / 8])
    bt = np.array([0], dtype=np.int32)
    ret = np.zeros((1, 8, 3))
    h = ctypes.c_void_p()
    _lib.check(gpu_lib.pypde_system_builtin(b"euler", 1, ctypes.byref(h)))
    try:
        for strips in (-1, 33):
            opt = _lib.Options()
            opt.strips = strips
            rc = gpu_lib.pde_solver_ex(h, True, False, False, _lib.c_ptr(u), 0.1,
                                       _lib.c_ptr(nX), 1, _lib.c_ptr(dX), 0.9,
                                       _lib.c_ptr(bt), False, 0, 2, 1, _lib.c_ptr(ret),
                                       ctypes.byref(opt), None)
            assert rc == _lib.PYPDE_ERR_ARG
            assert b"strips" in gpu_lib.pypde_last_error()
    finally:
        gpu_lib.pypde_system_free(h)
