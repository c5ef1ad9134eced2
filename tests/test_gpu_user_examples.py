"""Python callbacks of the kinds the reference's examples use (Navier-Stokes
in the second-order form, reactive Euler with the Roe flux at order 3,
shallow water with a non-conservative B and a stiff source) through the
public pde_solver on the GPU: translated to device code, compiled at run
time with NVRTC, and compared bit for bit with the C restatement running
the same Python functions as ctypes callbacks.  The systems and states are
those of tests/test_device_user_callbacks_host.py, which runs the same
translated source through the kernels compiled as host C++.

The 13-variable matrix-style system (tuple-returning helpers, matrix
products, transposes, reshape / ravel, trace / eye / det, slice updates
around d; B and a stiff S) is compared with the restatement running the
same translated callbacks compiled by the host compiler: numpy's BLAS dot
sums in another order than the translation, so only the translated source
gives the same bits on both sides."""
import os

import numpy as np
import pytest

from pypde_gb300.solvers import pde_solver
from pypde_gb300.translate import translate
from test_device_user_callbacks_host import (CASES, MATRIX_CASE, _port_run, _port_run_ptrs,
                                             callback_lib, callback_ptrs)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def private_cache(tmp_path_factory):
    old = os.environ.get("PYPDE_GB300_CACHE")
    os.environ["PYPDE_GB300_CACHE"] = str(tmp_path_factory.mktemp("jitcache"))
    yield
    if old is None:
        del os.environ["PYPDE_GB300_CACHE"]
    else:
        os.environ["PYPDE_GB300_CACHE"] = old


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_reference_style_callbacks_on_gpu_equal_port(gpu_lib, case):
    name, F, B, S, u0, N, bt, cfl, stiff, flux, K = case
    u_o, steps_o, t_o = _port_run(F, B, S, u0, N, bt, cfl, stiff, flux, K)
    q = u0.copy()
    st = {}
    pde_solver(q, 10.0, [1.0] * (u0.ndim - 1), F=F, B=B, S=S,
               boundaryTypes=[("transitive", "periodic")[b] for b in bt], cfl=cfl, order=N,
               ndt=1, flux=("rusanov", "roe", "osher")[flux], stiff=stiff, max_steps=K,
               stats=st)
    assert st["steps"] == steps_o == K and st["t_final"] == t_o
    assert np.array_equal(q, u_o), np.abs(q - u_o).max()


def test_matrix_style_callbacks_on_gpu_equal_port(gpu_lib, tmp_path):
    name, F, B, S, u0, N, bt, cfl, stiff, flux, K = MATRIX_CASE
    cb = callback_lib(tmp_path, translate(F, B, S, 1, u0.shape[-1]))
    u_o, steps_o, t_o = _port_run_ptrs(callback_ptrs(cb, F, B, S), False, u0, N, bt, cfl, stiff,
                                       flux, K)
    q = u0.copy()
    st = {}
    pde_solver(q, 10.0, [1.0], F=F, B=B, S=S, boundaryTypes="transitive", cfl=cfl, order=N,
               ndt=1, stiff=stiff, max_steps=K, stats=st)
    assert st["steps"] == steps_o == K and st["t_final"] == t_o
    assert np.array_equal(q, u_o), np.abs(q - u_o).max()
