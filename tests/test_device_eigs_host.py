"""Device code compiled as host C++, against the C restatement, bit for bit,
on the CPU: the max|eig| path (tests/device_eigs_host.cpp, with
pypde_gb300/csrc/ader_common.cuh and systems.cuh) and the face fluxes
(tests/device_flux_host.cpp, with kernels.cuh).

The GPU parity tests compare the kernels with the restatement on the GPU;
this test checks the same source's operation order without one.  It covers:
- the FD Jacobian, including the active-column form of systems with passive
  variables;
- the FP32 Hessenberg/QR candidates, the DMW refinement and its fallbacks;
- systems with a B matrix;
- the Rusanov, Roe and Osher fluxes (full complex eigendecompositions) and
  the B path integral, orders 1-3, and the second-order flux form."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from oracle import ora
from pypde_gb300 import workloads


def _host_build(tmp_path_factory, name):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("devhost") / f"lib{name}.so")
    src = os.path.join(ROOT, "tests", name + ".cpp")
    subprocess.run([cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                    "-Wno-unknown-pragmas", "-o", out, src], check=True)
    return ctypes.CDLL(out)


@pytest.fixture(scope="module")
def host_lib(tmp_path_factory):
    L = _host_build(tmp_path_factory, "device_eigs_host")
    L.host_max_abs_eigs.restype = ctypes.c_double
    L.host_max_abs_eigs.argtypes = [ctypes.c_char_p, ctypes.c_int, ora.dp, ora.dp, ctypes.c_int]
    return L


@pytest.fixture(scope="module")
def flux_lib(tmp_path_factory):
    L = _host_build(tmp_path_factory, "device_flux_host")
    L.host_face_flux.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int] + [ora.dp] * 4 + \
        [ctypes.c_int, ctypes.c_int] + [ora.dp] * 4
    return L


CASES = [("euler", 1), ("euler", 2), ("euler", 3), ("cattaneo", 2), ("cattaneo", 3),
         ("ncp", 1), ("ncp", 2)]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}{c[1]}")
def test_device_eigs_equal_port(host_lib, case):
    name, ndim = case
    s = ora.PortSystem(name, ndim)
    P = ora.port()
    P.ora_system_max_abs_eigs.restype = ctypes.c_double
    P.ora_system_max_abs_eigs.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                          ctypes.c_int, ora.dp, ora.dp, ctypes.c_int, ora.dp]
    states = workloads.random_state(name, (40,) + (1,) * (ndim - 1), 3).reshape(-1, s.V)
    if name == "cattaneo":  # stiff and non-stiff tau, and states at rest
        states[::2, -1] = -6.0
        states[::5, 1:ndim + 1] = 0.0
    dq = np.zeros(ndim * s.V)
    for q in states:
        for d in range(ndim):
            M = np.zeros(s.V * s.V)
            want = P.ora_system_max_abs_eigs(s.F, s.B, ndim, s.V, ora.ptr(q.copy()), ora.ptr(dq),
                                             d, ora.ptr(M))
            got = host_lib.host_max_abs_eigs(name.encode(), ndim, ora.ptr(q.copy()),
                                             ora.ptr(dq.copy()), d)
            assert got == want or (np.isnan(got) and np.isnan(want)), (q, d, got, want)


FLUX_CASES = CASES + [("burgers2", 1)]


@pytest.mark.parametrize("case", FLUX_CASES, ids=lambda c: f"{c[0]}{c[1]}")
def test_device_face_fluxes_equal_port(flux_lib, case):
    name, ndim = case
    s = ora.PortSystem(name, ndim)
    P = ora.port()
    P.ora_face_flux.argtypes = [ctypes.c_void_p] * 2 + [ctypes.c_int] * 4 + [ora.dp] * 4 + \
        [ctypes.c_int, ctypes.c_int, ora.dp, ora.dp]
    rng = np.random.default_rng(7)
    states = workloads.random_state(name, (13,) + (1,) * (ndim - 1), 5).reshape(-1, s.V)
    if name == "cattaneo":
        states[::2, -1] = -6.0
    for N in (1, 2, 3):
        tab = ora.tables(N)
        nodes, wghts = tab[:N].copy(), tab[N:2 * N].copy()
        for flux in (0, 1, 2):
            for i in range(len(states) - 1):
                qL, qR = states[i].copy(), states[i + 1].copy()
                d = i % ndim
                if s.second_order:
                    dqL, dqR = 0.1 * rng.standard_normal((2, ndim * s.V))
                else:
                    dqL, dqR = np.zeros((2, ndim * s.V))
                f0, b0 = np.zeros(s.V), np.zeros(s.V)
                P.ora_face_flux(s.F, s.B, ndim, N, s.V, s.second_order, ora.ptr(qL.copy()),
                                ora.ptr(qR.copy()), ora.ptr(dqL.copy()), ora.ptr(dqR.copy()), d,
                                flux, ora.ptr(f0), ora.ptr(b0))
                f1, b1 = np.zeros(s.V), np.zeros(s.V)
                rc = flux_lib.host_face_flux(name.encode(), ndim, N, ora.ptr(qL.copy()),
                                             ora.ptr(qR.copy()), ora.ptr(dqL.copy()),
                                             ora.ptr(dqR.copy()), d, flux, ora.ptr(nodes),
                                             ora.ptr(wghts), ora.ptr(f1), ora.ptr(b1))
                assert rc == 0
                assert np.array_equal(f1, f0), (N, flux, i, f1 - f0)
                assert np.array_equal(b1, b0), (N, flux, i, b1 - b0)



def test_fd_quotient_is_correctly_rounded(host_lib):
    """The kernels form each FD Jacobian entry (v2 - v1) / h from one
    reciprocal of h per column (fd_step, fd_div: a faithful quotient and one
    Markstein correction); it must equal IEEE division bit for bit.  Steps
    h = 2^-26 max(|q|, 1) over the magnitudes states take, and beyond;
    differences v2 - v1 over the range of a flux's finite differences,
    including zeros of both signs, tiny, huge, infinite and NaN values, and
    random mantissas; 4 million pairs plus quotients that lie exactly half
    way between two doubles' neighbours of x / h."""
    host_lib.host_fd_div.argtypes = [ora.dp, ora.dp, ora.dp, ctypes.c_long]
    rng = np.random.default_rng(17)
    n = 1 << 22
    q = rng.uniform(0.5, 2.0, n) * 10.0 ** rng.integers(-12, 13, n)
    q[: n // 8] = 10.0 ** rng.uniform(-300, 300, n // 8)
    h = np.maximum(2.0 ** -26 * np.abs(q), 2.0 ** -26)
    x = rng.standard_normal(n) * 10.0 ** rng.uniform(-30, 10, n)
    x[: n // 16] = (rng.uniform(-1, 1, n // 16) * 10.0 ** rng.uniform(-320, 300, n // 16))
    x[n // 16: n // 16 + 6] = [0.0, -0.0, np.inf, -np.inf, np.nan, 5e-324]
    # near-ties: x = h (m + 1/2 + tiny) for integers m with few bits
    k = n // 4
    m = rng.integers(1, 1 << 20, k).astype(np.float64)
    x[-k:] = h[-k:] * (m + 0.5) * (1.0 + rng.choice([-1, 1], k) * 2.0 ** -52)
    out = np.empty(n)
    host_lib.host_fd_div(ora.ptr(x), ora.ptr(h), ora.ptr(out), n)
    want = x / h
    same = (out == want) | (np.isnan(out) & np.isnan(want))
    assert same.all(), (x[~same][:5], h[~same][:5], out[~same][:5], want[~same][:5])
    assert np.array_equal(np.signbit(out[~np.isnan(out)]), np.signbit(want[~np.isnan(want)]))
