"""Python callbacks of the kinds the reference's examples use (Navier-Stokes
in the second-order form, reactive Euler with the Roe flux at order 3,
shallow water with a non-conservative B and a stiff source) through the
public pde_solver on the GPU: translated to device code, compiled at run
time with NVRTC, and compared bit for bit with the C restatement running
the same Python functions as ctypes callbacks.  The systems and states are
those of tests/test_device_user_callbacks_host.py, which runs the same
translated source through the kernels compiled as host C++."""
import os

import numpy as np
import pytest

from pypde_gb300.solvers import pde_solver
from test_device_user_callbacks_host import CASES, _port_run

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
