"""The device max|eig| path, compiled as host C++ (tests/device_eigs_host.cpp
includes pypde_gb300/csrc/ader_common.cuh and systems.cuh), against the C
restatement, bit for bit, on the CPU.

The GPU parity tests compare the kernels with the restatement on the GPU;
this test checks the same source's operation order without one.  It covers:
- the FD Jacobian, including the active-column form of systems with passive
  variables;
- the FP32 Hessenberg/QR candidates, the DMW refinement and its fallbacks;
- systems with a B matrix."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT
from oracle import ora
from pypde_gb300 import workloads


@pytest.fixture(scope="module")
def host_lib(tmp_path_factory):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    out = str(tmp_path_factory.mktemp("devhost") / "libdevice_eigs_host.so")
    src = os.path.join(ROOT, "tests", "device_eigs_host.cpp")
    subprocess.run([cxx, "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                    "-Wno-unknown-pragmas", "-o", out, src], check=True)
    L = ctypes.CDLL(out)
    L.host_max_abs_eigs.restype = ctypes.c_double
    L.host_max_abs_eigs.argtypes = [ctypes.c_char_p, ctypes.c_int, ora.dp, ora.dp, ctypes.c_int]
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
