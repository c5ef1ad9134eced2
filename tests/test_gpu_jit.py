"""Python callbacks translated to device code and compiled at run time
(pde_solver(..., jit=True)), against the CPU restatement.

The built-in systems' Python callbacks, forced down the run-time path,
must give the same bits as the restatement's C callbacks: the translator
keeps Python's operation order and the kernels are the same templates as
the ahead-of-time build.  A user-written system (not one of the built-in
ones) must run and agree with the built-in system it restates.
"""
import os

import numpy as np
import pytest

from conftest import l1
from oracle import ora
from pypde_gb300 import systems, workloads
from pypde_gb300.solvers import pde_solver

pytestmark = pytest.mark.gpu

RUNS = [("euler", (17,), 3, [1], 0.9, 5), ("euler", (12, 10), 2, [1, 0], 0.9, 5),
        ("euler", (5, 6, 4), 2, [1, 0, 1], 0.5, 3), ("ncp", (9, 8), 2, [1, 1], 0.5, 4),
        ("burgers2", (24,), 2, [1], 0.5, 4)]


@pytest.fixture(scope="module", autouse=True)
def private_cache(tmp_path_factory):
    old = os.environ.get("PYPDE_GB300_CACHE")
    os.environ["PYPDE_GB300_CACHE"] = str(tmp_path_factory.mktemp("jitcache"))
    yield
    if old is None:
        del os.environ["PYPDE_GB300_CACHE"]
    else:
        os.environ["PYPDE_GB300_CACHE"] = old


def _sys(name, ndim):
    return systems.burgers2() if name == "burgers2" else getattr(systems, name)(ndim)


@pytest.mark.parametrize("run", RUNS, ids=[f"{r[0]}-{len(r[1])}d-N{r[2]}" for r in RUNS])
def test_jit_run_matches_port(gpu_lib, run):
    name, shape, N, bt, cfl, K = run
    u0 = workloads.random_state(name, shape, 11)
    L = [1.0] * len(shape)
    u_o, _, steps, t_o = ora.pde_solver(name, u0, 10.0, L, bt, cfl, N, max_steps=K)
    s = _sys(name, len(shape))
    q = u0.copy()
    st = {}
    pde_solver(q, 10.0, L, F=s.F, B=s.B, S=s.S,
               boundaryTypes=[("transitive", "periodic")[b] for b in bt], cfl=cfl, order=N,
               ndt=1, stiff=False, max_steps=K, stats=st, jit=True)
    assert st["steps"] == steps == K and st["t_final"] == t_o
    assert np.array_equal(q, u_o)


def test_jit_stiff_newton_matches_port(gpu_lib):
    u0 = workloads.relaxation(16, 2, seed=5)
    s = systems.cattaneo(2)
    K = 3
    u_o, _, steps, t_o = ora.pde_solver("cattaneo", u0, 10.0, [1.0, 1.0], [1, 1], 0.8, 2,
                                        stiff=True, max_steps=K)
    q = u0.copy()
    st = {}
    pde_solver(q, 10.0, [1.0, 1.0], F=s.F, S=s.S, boundaryTypes="periodic", cfl=0.8, order=2,
               ndt=1, stiff=True, max_steps=K, stats=st, jit=True)
    assert st["steps"] == steps == K and st["pred_fail"] == 0 and st["t_final"] == t_o
    assert np.array_equal(q, u_o)


@pytest.mark.parametrize("flux", ["roe", "osher"])
def test_jit_eigen_fluxes_match_port(gpu_lib, flux):
    u0 = workloads.random_state("euler", (10, 9), 12)
    s = systems.euler(2)
    K = 3
    fl = {"roe": 1, "osher": 2}[flux]
    u_o, _, steps, t_o = ora.pde_solver("euler", u0, 10.0, [1.0, 1.0], [1, 1], 0.9, 2,
                                        flux=fl, max_steps=K)
    q = u0.copy()
    pde_solver(q, 10.0, [1.0, 1.0], F=s.F, boundaryTypes="periodic", cfl=0.9, order=2, ndt=1,
               flux=flux, stiff=False, max_steps=K, jit=True)
    assert np.array_equal(q, u_o)


GAMMA = 1.4


def user_flux(Q, d):
    """Euler flux written the numpy way, independently of pypde_gb300.systems."""
    rho = Q[0]
    v = Q[1:3] / rho
    p = (GAMMA - 1.0) * (Q[3] - 0.5 * rho * (v[0] * v[0] + v[1] * v[1]))
    out = v[d] * Q
    out[1 + d] += p
    out[3] += p * v[d]
    return out


def test_user_written_callback_runs(gpu_lib):
    u0 = workloads.shear(32)
    tf = 0.02
    q_user = u0.copy()
    st = {}
    pde_solver(q_user, tf, [1.0, 1.0], F=user_flux, boundaryTypes="periodic", order=3, ndt=1,
               stiff=False, stats=st)
    q_ref = u0.copy()
    pde_solver(q_ref, tf, [1.0, 1.0], F=systems.euler(2).F, boundaryTypes="periodic", order=3,
               ndt=1, stiff=False)
    assert st["steps"] > 0 and np.isfinite(q_user).all()
    # Same physics, a different order of operations in the pressure: the
    # runs agree to rounding amplified by the WENO weights and the
    # finite-difference Jacobians (measured 2e-7 in the y momentum, whose
    # L1 norm is small next to the others').
    assert np.all(l1(q_user, q_ref) <= 1e-5), l1(q_user, q_ref)


def test_jit_cache_reused(gpu_lib):
    """A second solve with the same callbacks compiles nothing new."""
    cache = os.environ["PYPDE_GB300_CACHE"]
    u0 = workloads.random_state("euler", (8,), 2)
    s = systems.euler(1)
    pde_solver(u0.copy(), 0.01, [1.0], F=s.F, order=2, ndt=1, stiff=False, jit=True)
    before = sorted(os.listdir(cache))
    assert before
    pde_solver(u0.copy(), 0.01, [1.0], F=s.F, order=2, ndt=1, stiff=False, jit=True)
    assert sorted(os.listdir(cache)) == before
