"""Python callbacks of the kinds the reference's examples use, through the
run-time callback path, on the CPU: pypde_gb300.translate turns them into a
`struct UserSystem`, which instantiates the device kernels compiled as host
C++ (tests/device_step_host.cpp with HOST_USER_SYSTEM, CUDA blocks as
fibers), exactly as the run-time compiled kernels include it.  The C
restatement runs the same Python functions as ctypes callbacks, the way
the reference runs its numba cfuncs (pypde/cfuncs.py:30-75).

The systems restate textbook physics in the style of the reference's
example problems (pypde/tests/): the compressible Navier-Stokes equations
in the second-order form F(Q, DQ, d) in 1-D (viscous shock) and 2-D
(Taylor-Green vortex), reactive Euler with a stiff switch-on reaction and
the Roe flux at order 3 (detonation wave), and shallow water over
topography, a non-conservative B(Q) with a stiff friction source.  The
callbacks use IEEE arithmetic and sqrt only, so both sides give the same
bits: the final states must be identical."""
import ctypes
import os

import numpy as np
import pytest

from conftest import build_device_host, load_device_host
from oracle import ora
from pypde_gb300 import stages
from pypde_gb300.translate import translate
from pypde_gb300.utils import nargs

GAMMA = 1.4
MU = 2e-2       # dynamic viscosity
KAPPA = 3e-2    # heat conductivity (T = p / rho)
Q_HEAT = 1.0    # heat of reaction per unit mass of fuel
K_RATE = 50.0   # reaction rate above ignition
T_IGN = 1.1     # ignition temperature
G = 1.0         # gravity
C_F = 40.0      # friction coefficient


def ns1_flux(Q, DQ, d):
    """1-D Navier-Stokes: Euler flux minus the viscous stress and plus the
    conductive heat flux, from the state gradient DQ[d]."""
    rho = Q[0]
    u = Q[1] / rho
    E = Q[2]
    p = (GAMMA - 1.0) * (E - 0.5 * rho * u * u)
    drho = DQ[d][0]
    du = (DQ[d][1] - u * drho) / rho
    dp = (GAMMA - 1.0) * (DQ[d][2] - 0.5 * u * u * drho - rho * u * du)
    dT = (dp - p / rho * drho) / rho
    tau = 4.0 / 3.0 * MU * du
    F = np.zeros(3)
    F[0] = rho * u
    F[1] = rho * u * u + p - tau
    F[2] = (E + p) * u - tau * u - KAPPA * dT
    return F


def ns2_flux(Q, DQ, d):
    """2-D Navier-Stokes flux in direction d (no heat conduction)."""
    rho = Q[0]
    v = Q[1:3] / rho
    E = Q[3]
    p = (GAMMA - 1.0) * (E - 0.5 * rho * (v[0] * v[0] + v[1] * v[1]))
    grad = np.zeros((2, 2))
    for j in range(2):
        for i in range(2):
            grad[j, i] = (DQ[j][1 + i] - v[i] * DQ[j][0]) / rho
    div = grad[0, 0] + grad[1, 1]
    F = np.zeros(4)
    F[0] = rho * v[d]
    work = 0.0
    for i in range(2):
        tau = MU * (grad[d, i] + grad[i, d])
        if i == d:
            tau = tau - 2.0 / 3.0 * MU * div
        F[1 + i] = rho * v[d] * v[i] - tau
        work = work + tau * v[i]
    F[1 + d] += p
    F[3] = (E + p) * v[d] - work
    return F


def reactive_flux(Q, d):
    """Euler flux of (rho, rho u, E, rho lambda); E includes the chemical
    energy Q_HEAT rho lambda of the unburnt fuel fraction lambda."""
    rho = Q[0]
    u = Q[1] / rho
    p = (GAMMA - 1.0) * (Q[2] - 0.5 * rho * u * u - Q_HEAT * Q[3])
    return np.array([Q[1], Q[1] * u + p, (Q[2] + p) * u, Q[3] * u])


def reactive_source(Q):
    """Fuel burns at rate K_RATE once the temperature passes ignition."""
    rho = Q[0]
    u = Q[1] / rho
    p = (GAMMA - 1.0) * (Q[2] - 0.5 * rho * u * u - Q_HEAT * Q[3])
    S = np.zeros(4)
    if p / rho > T_IGN:
        S[3] = -K_RATE * Q[3]
    return S


def sw_flux(Q, d):
    """Shallow water (h, hu, b): the bed b is carried along unchanged."""
    u = Q[1] / Q[0]
    return np.array([Q[1], Q[1] * u + 0.5 * G * Q[0] * Q[0], 0.0])


def sw_ncp(Q, d):
    """The non-conservative bed-slope term g h db/dx."""
    B = np.zeros((3, 3))
    B[1, 2] = G * Q[0]
    return B


def sw_source(Q):
    """Linear bed friction, stiff for large C_F."""
    S = np.zeros(3)
    S[1] = -C_F * Q[1]
    return S


def _ns1_state(n, seed):
    """A smoothed shock-like profile with noise (viscous shock setting)."""
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    s = 0.5 * (1 + np.tanh((x - 0.5) / 0.08))
    rho = 1.0 + 1.5 * s + 0.01 * rng.standard_normal(n)
    u = 0.8 - 0.5 * s
    p = 1.0 + 2.0 * s
    return np.stack([rho, rho * u, p / (GAMMA - 1) + 0.5 * rho * u * u], axis=-1)


def _tg_state(n, seed):
    """Taylor-Green vortex on the periodic unit square."""
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x, indexing="ij")
    rho = 1.0 + 0.01 * rng.standard_normal((n, n))
    u = np.sin(2 * np.pi * X) * np.cos(2 * np.pi * Y)
    v = -np.cos(2 * np.pi * X) * np.sin(2 * np.pi * Y)
    p = 10.0 + 0.25 * rho * (np.cos(4 * np.pi * X) + np.cos(4 * np.pi * Y))
    return np.stack([rho, rho * u, rho * v, p / (GAMMA - 1) + 0.5 * rho * (u * u + v * v)],
                    axis=-1)


def _det_state(n, seed):
    """A hot burnt region behind a shock, unburnt fuel ahead (detonation)."""
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    burnt = x < 0.3
    rho = np.where(burnt, 1.6, 1.0) * (1 + 0.01 * rng.random(n))
    u = np.where(burnt, 0.5, 0.0)
    p = np.where(burnt, 2.5, 1.0)
    lam = np.where(burnt, 0.0, 1.0)
    E = p / (GAMMA - 1) + 0.5 * rho * u * u + Q_HEAT * rho * lam
    return np.stack([rho, rho * u, E, rho * lam], axis=-1)


def _sw_state(n, seed):
    """A water hump over a sinusoidal bed."""
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    b = 0.2 * np.sin(2 * np.pi * x)
    h = 1.0 - b + 0.1 * np.exp(-((x - 0.5) / 0.1) ** 2) + 0.001 * rng.random(n)
    return np.stack([h, 0.1 * h, b], axis=-1)


# name, F, B, S, initial state, order, boundary types, cfl, stiff, flux, steps
CASES = [
    ("ns1d-viscous-shock", ns1_flux, None, None, _ns1_state(32, 1), 2, [0], 0.8, False, 0, 6),
    ("ns2d-taylor-green", ns2_flux, None, None, _tg_state(10, 2), 2, [1, 1], 0.8, False, 0, 3),
    ("reactive-roe-N3", reactive_flux, None, reactive_source, _det_state(24, 3), 3, [0], 0.8,
     True, 1, 4),
    ("shallow-water-ncp", sw_flux, sw_ncp, sw_source, _sw_state(24, 4), 2, [1], 0.8, True, 0, 4),
]


def _port_callbacks(F, B, S, ndim, V):
    """ctypes callbacks with the reference's C signatures around the Python
    functions (the parts of pypde/cfuncs.py:30-75 that copy Q, DQ and the
    result)."""
    dp = ctypes.POINTER(ctypes.c_double)
    FT = ctypes.CFUNCTYPE(None, dp, dp, dp, ctypes.c_int)
    BT = ctypes.CFUNCTYPE(None, dp, dp, ctypes.c_int)
    ST = ctypes.CFUNCTYPE(None, dp, dp)
    keep = []

    def wrap_f(out, Q, dQ, d):
        q = np.ctypeslib.as_array(Q, (V,)).copy()
        if nargs(F) == 3:
            r = F(q, np.ctypeslib.as_array(dQ, (ndim * V,)).reshape(ndim, V).copy(), d)
        elif nargs(F) == 2:
            r = F(q, d)
        else:
            r = F(q)
        np.ctypeslib.as_array(out, (V,))[:] = r

    def wrap_b(out, Q, d):
        q = np.ctypeslib.as_array(Q, (V,)).copy()
        np.ctypeslib.as_array(out, (V * V,))[:] = \
            np.asarray(B(q, d) if nargs(B) == 2 else B(q)).reshape(-1)

    def wrap_s(out, Q):
        np.ctypeslib.as_array(out, (V,))[:] = S(np.ctypeslib.as_array(Q, (V,)).copy())

    ptrs = []
    for fn, T, w in ((F, FT, wrap_f), (B, BT, wrap_b), (S, ST, wrap_s)):
        if fn is None:
            ptrs.append(None)
        else:
            c = T(w)
            keep.append(c)
            ptrs.append(ctypes.cast(c, ctypes.c_void_p))
    return ptrs, keep


def _port_run_ptrs(ptrs, second_order, u0, N, bt, cfl, stiff, flux, K):
    """K steps of the restatement with the callbacks behind ptrs (F, B, S
    function pointers or None); dX = 1/n.  Returns (u, steps, t)."""
    nX = np.array(u0.shape[:-1], dtype=np.int32)
    ndim, V = len(nX), u0.shape[-1]
    dX = np.array([1.0 / n for n in nX])
    u = u0.copy()
    ret = np.zeros((1,) + u.shape)
    tout = ctypes.c_double()
    steps = ora.port().ora_pde_solver(*ptrs, ora.ptr(u), 10.0, ora.ptr(nX), ndim, ora.ptr(dX),
                                      cfl, ora.ptr(np.array(bt, dtype=np.int32)), int(stiff),
                                      flux, N, V, 1, int(second_order), ora.ptr(ret), 1, K,
                                      1e-12, ctypes.byref(tout))
    return u, steps, tout.value


def _port_run(F, B, S, u0, N, bt, cfl, stiff, flux, K):
    """The restatement running the Python callbacks themselves."""
    ptrs, keep = _port_callbacks(F, B, S, u0.ndim - 1, u0.shape[-1])
    out = _port_run_ptrs(ptrs, F is not None and nargs(F) == 3, u0, N, bt, cfl, stiff, flux, K)
    del keep
    return out


def callback_lib(dirpath, src):
    """The translated callbacks compiled as host C++ into C functions with
    the reference's callback signatures (cbF, cbB, cbS), for the
    restatement; the same source the device kernels include."""
    import subprocess
    cpp = os.path.join(str(dirpath), "callbacks.cpp")
    with open(cpp, "w") as f:
        f.write("#include <cmath>\nusing namespace std;\n#define __device__\n"
                "#define __forceinline__ inline\n" + src +
                "\n#define API extern \"C\" __attribute__((visibility(\"default\")))"
                "\nAPI void cbF(double *o, double *Q, double *dQ, int d) "
                "{ UserSystem::F(o, Q, dQ, d); }"
                "\nAPI void cbB(double *o, double *Q, int d) { UserSystem::B(o, Q, d); }"
                "\nAPI void cbS(double *o, double *Q) { UserSystem::S(o, Q); }\n")
    so = os.path.join(str(dirpath), "libcallbacks.so")
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-fvisibility=hidden",
                    "-fvisibility-inlines-hidden", "-fno-gnu-unique", cpp, "-o", so], check=True)
    return ctypes.CDLL(so)


def callback_ptrs(lib, F, B, S):
    return [ctypes.cast(getattr(lib, f"cb{r}"), ctypes.c_void_p) if fn is not None else None
            for r, fn in (("F", F), ("B", B), ("S", S))]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_translated_callbacks_device_step_equals_port(tmp_path, case):
    name, F, B, S, u0, N, bt, cfl, stiff, flux, K = case
    ndim, V = u0.ndim - 1, u0.shape[-1]
    src = tmp_path / "user_system.h"
    src.write_text(translate(F, B, S, ndim, V))
    L = load_device_host(build_device_host(tmp_path, [f'HOST_USER_SYSTEM="{src}"',
                                                      f"HOST_USER_N={N}"]))
    u_o, steps_o, t_o = _port_run(F, B, S, u0, N, bt, cfl, stiff, flux, K)
    assert steps_o == K and np.all(np.isfinite(u_o))
    nX = np.array(u0.shape[:-1], dtype=np.int32)
    dX = np.array([1.0 / n for n in nX])
    for reverse in (False, True):
        L.host_set_order(int(reverse))
        u = u0.copy()
        t, its = ctypes.c_double(), ctypes.c_ulonglong()
        steps = L.host_run(b"user", ndim, N, flux, ora.ptr(u), ora.ptr(nX),
                           ora.ptr(np.array(bt, dtype=np.int32)), ora.ptr(dX),
                           ora.ptr(stages.tables(N)), 10.0, cfl, int(stiff), 1e-12, 0, K,
                           ctypes.byref(t), ctypes.byref(its))
        assert steps == K and t.value == t_o
        assert np.array_equal(u, u_o), np.abs(u - u_o).max()


# A 13-variable system in the style of the reference's GPR example: density,
# momentum and a distortion matrix A, written with tuple-returning helpers,
# matrix products, transposes, reshape / ravel, trace / eye / det and slice
# updates around d; arithmetic only, so device and host evaluate it to the
# same bits.
CS2 = 1.0
P0 = 1.0
TAU_A = 1e-2


def mat_unpack(Q):
    rho = Q[0]
    v = Q[1:4] / rho
    A = Q[4:13].copy().reshape((3, 3))
    return rho, v, A


def mat_dev(A):
    G = A.T @ A
    return G - np.trace(G) / 3.0 * np.eye(3)


def mat_flux(Q, d):
    ret = np.zeros(13)
    rho, v, A = mat_unpack(Q)
    sig = -rho * CS2 * np.dot(A.T, mat_dev(A))
    ret[0] = rho * v[d]
    ret[1:4] = rho * v[d] * v
    ret[1 + d] += P0 * rho
    ret[1:4] -= sig[d]
    Av = np.dot(A, v)
    ret[4 + d] = Av[0]
    ret[7 + d] = Av[1]
    ret[10 + d] = Av[2]
    return ret


def mat_ncp(Q, d):
    ret = np.zeros((13, 13))
    v = Q[1:4] / Q[0]
    for i in range(4, 13):
        ret[i, i] = v[d]
    ret[4 + d, 4 + d:7 + d] -= v
    ret[7 + d, 7 + d:10 + d] -= v
    ret[10 + d, 10:13] -= v
    return ret


def mat_src(Q):
    ret = np.zeros(13)
    rho, v, A = mat_unpack(Q)
    ret[4:13] = -mat_dev(A).ravel() * (np.linalg.det(A) / (TAU_A * rho))
    return ret


def _mat_state(n, seed):
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    u = np.zeros((n, 13))
    for i in range(n):
        s = 0.5 * (1 + np.tanh((x[i] - 0.5) / 0.1))
        rho = 1.0 + 0.5 * s
        A = rho ** (1 / 3) * np.eye(3) + 0.01 * rng.standard_normal((3, 3))
        u[i] = np.concatenate([[rho], rho * np.array([0.4 - 0.3 * s, 0.1, 0.0]), A.ravel()])
    return u


# name, F, B, S, state, order, boundary types, cfl, stiff, flux, steps
MATRIX_CASE = ("matrix-13var-stiff", mat_flux, mat_ncp, mat_src, _mat_state(20, 9), 2, [0],
               0.6, True, 0, 3)


def test_matrix_system_device_step_equals_port(tmp_path):
    """The matrix-style system: the device step with its translated source
    equals the restatement running the same translated callbacks, bit for
    bit, in both fiber orders."""
    name, F, B, S, u0, N, bt, cfl, stiff, flux, K = MATRIX_CASE
    src = translate(F, B, S, 1, 13)
    (tmp_path / "user_system.h").write_text(src)
    cb = callback_lib(tmp_path, src)
    u_o, steps_o, t_o = _port_run_ptrs(callback_ptrs(cb, F, B, S), False, u0, N, bt, cfl, stiff,
                                       flux, K)
    assert steps_o == K and np.all(np.isfinite(u_o)) and np.abs(u_o - u0).max() > 0
    L = load_device_host(build_device_host(
        tmp_path, [f'HOST_USER_SYSTEM="{tmp_path / "user_system.h"}"', f"HOST_USER_N={N}"]))
    nX = np.array(u0.shape[:-1], dtype=np.int32)
    dX = np.array([1.0 / n for n in nX])
    for reverse in (False, True):
        L.host_set_order(int(reverse))
        u = u0.copy()
        t, its = ctypes.c_double(), ctypes.c_ulonglong()
        steps = L.host_run(b"user", 1, N, flux, ora.ptr(u), ora.ptr(nX),
                           ora.ptr(np.array(bt, dtype=np.int32)), ora.ptr(dX),
                           ora.ptr(stages.tables(N)), 10.0, cfl, int(stiff), 1e-12, 0, K,
                           ctypes.byref(t), ctypes.byref(its))
        assert steps == K and t.value == t_o
        assert np.array_equal(u, u_o), np.abs(u - u_o).max()
