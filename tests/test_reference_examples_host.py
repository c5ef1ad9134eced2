"""The reference's own example callbacks (pypde/tests/: the Sod shock tube,
Navier-Stokes viscous shock and Taylor-Green vortex, the detonation wave
and the GPR viscous shock) through the run-time callback path, on the CPU.

Runs only where the reference tree is present (it is read in place, never
copied); numba, which the examples import for their helpers, is absent here
and is replaced by a stand-in whose njit returns the Python function.

For each example:
1. the translated callbacks (pypde_gb300.translate, compiled as host C++)
   equal the Python functions on sample states to 1e-13 relative: numpy
   evaluates dot and sum through BLAS and pairwise sums, whose order the
   translation does not reproduce;
2. the device step (the kernels compiled as host C++ with the translated
   UserSystem, CUDA blocks as fibers) equals the C restatement running the
   same translated callbacks, bit for bit;
3. against the restatement running the Python callbacks themselves, the
   final states agree to 1e-7 relative L1: the FD Jacobians behind the
   eigenvalues divide callback differences of ~1e-16 relative by the step
   h ~ 1e-8, so the last-bit differences of item 1 reach ~1e-8 in the time
   step and the state."""
import contextlib
import ctypes
import importlib
import os
import sys
import types

import numpy as np
import pytest

from conftest import build_device_host, load_device_host
from oracle import ora
from pypde_gb300 import stages
from pypde_gb300.translate import translate
from pypde_gb300.utils import nargs
from test_device_user_callbacks_host import _port_run, _port_run_ptrs, callback_lib, callback_ptrs

EXAMPLES = os.path.join(ora.REF_SRC, "pypde", "tests")
pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(EXAMPLES, "gpr")),
                                reason="reference tree not present")


@contextlib.contextmanager
def _reference_modules():
    """Import path for the reference's example packages without running
    their __init__ files (which import matplotlib and the numba-compiled
    solver), with a numba stand-in; removed again afterwards."""
    added = []

    def put(name, mod):
        if name not in sys.modules:
            sys.modules[name] = mod
            added.append(name)

    for name, sub in (("pypde", ""), ("pypde.tests", "tests"), ("pypde.tests.gpr", "tests/gpr"),
                      ("pypde.tests.euler", "tests/euler"),
                      ("pypde.tests.navier_stokes", "tests/navier_stokes"),
                      ("pypde.tests.reactive_euler", "tests/reactive_euler")):
        m = types.ModuleType(name)
        m.__path__ = [os.path.join(ora.REF_SRC, "pypde", sub)]
        put(name, m)
    try:
        importlib.import_module("numba")
    except ImportError:
        nb = types.ModuleType("numba")
        nb.njit = nb.jit = lambda *a, **k: a[0] if len(a) == 1 and callable(a[0]) and not k \
            else (lambda f: f)
        put("numba", nb)
    try:
        yield
    finally:
        for name in list(sys.modules):
            if name in added or name.startswith("pypde.tests."):
                sys.modules.pop(name, None)


def _examples():
    """name -> (F, B, S, u0, order, boundary types, cfl, stiff, flux, steps)."""
    with _reference_modules():
        eu = importlib.import_module("pypde.tests.euler.system")
        ns = importlib.import_module("pypde.tests.navier_stokes.system")
        re = importlib.import_module("pypde.tests.reactive_euler.system")
        gs = importlib.import_module("pypde.tests.gpr.system")
        gu = importlib.import_module("pypde.tests.gpr.misc.utils")
    rng = np.random.default_rng(7)
    out = {}

    # Sod shock tube on a 2-D grid with the 1-D flux F(Q) (3 variables)
    n, m = 16, 4
    u = np.zeros((n, m, 3))
    for i in range(n):
        rho, p = (1.0, 1.0) if i < n // 2 else (0.125, 0.1)
        rho *= 1 + 1e-3 * rng.random()
        u[i, :] = rho * np.array([1.0, eu.energy(rho, p, 0.0), 0.0])
    out["sod-2d"] = (eu.F_euler, None, None, u, 2, [0, 1], 0.9, False, 0, 4)

    def ns_state(shape, fn):
        u = np.zeros(tuple(shape) + (5,))
        for idx in np.ndindex(*shape):
            rho, p, v = fn(idx)
            u[idx] = [rho, rho * ns.total_energy(rho, p, v), *(rho * v)]
        return u

    n = 24
    s = 0.5 * (1 + np.tanh(((np.arange(n) + 0.5) / n - 0.5) / 0.1))
    out["ns-viscous-shock-1d"] = (ns.F_navier_stokes, None, None, ns_state(
        (n,), lambda i: (1 + s[i[0]], 1 + 2 * s[i[0]], np.array([0.5 - 0.4 * s[i[0]], 0, 0]))),
        2, [0], 0.9, False, 0, 4)
    n = 8
    x = 2 * np.pi * (np.arange(n) + 0.5) / n

    def taylor_green(i):
        a, b = x[i[0]], x[i[1]]
        return 1.0, 10.0, np.array([np.sin(a) * np.cos(b), -np.cos(a) * np.sin(b), 0.0])

    out["ns-taylor-green-2d"] = (ns.F_navier_stokes, None, None, ns_state((n, n), taylor_green),
                                 2, [1, 1], 0.9, False, 0, 3)

    # detonation: burnt gas behind the front, Roe flux at order 3
    n = 48
    u = np.zeros((n, 6))
    for i in range(n):
        if i < n // 4:
            rho, p, v, lam = 1.4, 1.0, [0.0, 0.0, 0.0], 0.0
        else:
            rho, p, v, lam = 0.887565, 0.191709, [-0.57735, 0.0, 0.0], 1.0
        u[i] = rho * np.array([1.0, re.energy(rho, p, np.array(v), lam)] + v + [lam])
    out["detonation-roe-N3"] = (re.F_reactive_euler, None, re.S_reactive_euler, u, 3, [0], 0.6,
                                False, 1, 3)

    # GPR viscous shock: 17 variables, F, B and a stiff S
    n = 24
    s = 0.5 * (1 + np.tanh(((np.arange(n) + 0.5) / n - 0.5) / 0.1))
    u = np.zeros((n, 17))
    for i in range(n):
        rho = 1 + s[i]
        u[i] = gu.Cvec(rho, 1 + 2 * s[i], np.array([0.5 - 0.4 * s[i], 0, 0]),
                       rho ** (1 / 3) * np.eye(3), np.zeros(3))
    out["gpr-viscous-shock-1d"] = (gs.F_gpr, gs.B_gpr, gs.S_gpr, u, 2, [0], 0.6, True, 0, 3)
    return out


EX = _examples() if os.path.isdir(os.path.join(EXAMPLES, "gpr")) else {}


@pytest.mark.parametrize("name", sorted(EX))
def test_reference_example_through_translation(tmp_path, name):
    F, B, S, u0, N, bt, cfl, stiff, flux, K = EX[name]
    ndim, V = u0.ndim - 1, u0.shape[-1]
    src = translate(F, B, S, ndim, V)
    cb = callback_lib(tmp_path, src)
    dp = ctypes.POINTER(ctypes.c_double)

    # 1. translated callbacks against the Python functions
    rng = np.random.default_rng(3)
    for q0 in u0.reshape(-1, V)[::3]:
        q = q0 * (1 + 1e-3 * rng.standard_normal(V))
        dq = 0.1 * rng.standard_normal((ndim, V))
        for d in range(ndim):
            for fn, c, nout in ((F, cb.cbF, V), (B, cb.cbB, V * V), (S, cb.cbS, V)):
                if fn is None or (fn is S and d > 0):
                    continue
                got = np.zeros(nout)
                qa, dqa = q.copy(), dq.copy()
                if fn is F:
                    c(got.ctypes.data_as(dp), qa.ctypes.data_as(dp), dqa.ctypes.data_as(dp), d)
                    want = {1: lambda: F(q.copy()), 2: lambda: F(q.copy(), d),
                            3: lambda: F(q.copy(), dq.copy(), d)}[nargs(F)]()
                elif fn is B:
                    c(got.ctypes.data_as(dp), qa.ctypes.data_as(dp), d)
                    want = B(q.copy(), d) if nargs(B) == 2 else B(q.copy())
                else:
                    c(got.ctypes.data_as(dp), qa.ctypes.data_as(dp))
                    want = S(q.copy())
                want = np.asarray(want, dtype=np.float64).reshape(-1)
                assert np.abs(got - want).max() <= 1e-13 * max(np.abs(want).max(), 1e-300)

    # 2. the device step with the translated system against the restatement
    #    with the same translated callbacks
    (tmp_path / "user_system.h").write_text(src)
    L = load_device_host(build_device_host(
        tmp_path, [f'HOST_USER_SYSTEM="{tmp_path / "user_system.h"}"', f"HOST_USER_N={N}"]))
    nX = np.array(u0.shape[:-1], dtype=np.int32)
    dX = np.array([1.0 / n for n in nX])
    u_c, steps_c, t_c = _port_run_ptrs(callback_ptrs(cb, F, B, S), nargs(F) == 3, u0, N, bt,
                                       cfl, stiff, flux, K)
    u = u0.copy()
    t, its = ctypes.c_double(), ctypes.c_ulonglong()
    steps = L.host_run(b"user", ndim, N, flux, ora.ptr(u), ora.ptr(nX),
                       ora.ptr(np.array(bt, dtype=np.int32)), ora.ptr(dX),
                       ora.ptr(stages.tables(N)), 10.0, cfl, int(stiff), 1e-12, 0, K,
                       ctypes.byref(t), ctypes.byref(its))
    assert steps == steps_c == K and t.value == t_c
    assert np.all(np.isfinite(u)) and np.abs(u - u0).max() > 0
    assert np.array_equal(u, u_c), np.abs(u - u_c).max()

    # 3. against the restatement running the Python callbacks
    u_p, steps_p, t_p = _port_run(F, B, S, u0, N, bt, cfl, stiff, flux, K)
    # numpy and the translated C round F differently; the second-order
    # time step differentiates F by forward differences in dQ, which enters
    # only through the small viscous term, so dt moves by up to ~1e-7
    assert steps_p == K and abs(t_p - t.value) <= 1e-6 * t_p
    scale = np.abs(u_p).reshape(-1, V).sum(axis=0)
    err = np.abs(u - u_p).reshape(-1, V).sum(axis=0) / np.where(scale > 0, scale, 1.0)
    assert err.max() <= 1e-7, err


@pytest.mark.parametrize("name", [n for n in ("gpr-viscous-shock-1d", "detonation-roe-N3")
                                  if n in EX])
def test_reference_example_compiles_with_nvrtc(name):
    """The translated GPR (17 variables, F, B and stiff S) and detonation
    (Roe flux at order 3) systems compile with the kernel templates for
    sm_103a, as the run-time path compiles them."""
    from test_translate import _nvrtc_compile
    F, B, S, u0, N, bt, cfl, stiff, flux, K = EX[name]
    kernels = [f"k_faces<UserSystem, {N}, {flux}>"] + \
        ([f"k_newton<UserSystem, {N}>"] if stiff else [])
    _nvrtc_compile(translate(F, B, S, u0.ndim - 1, u0.shape[-1]), kernels)
