"""Mixed-precision stiff predictor: FP32 Newton sweeps (FP32 callbacks, FP32
FD Jacobian and LU), then at least two FP64 sweeps to the same 1e-12
tolerance.  The answer must stay at the plain FP64 form's error level
against a tolerance-1e-15 oracle (two converged Newton solves differ by the
tolerance's own effect, measured by the plain form at tolerances 1e-12 and
1e-13), and the FP64 sweeps must not increase."""
import pytest

from conftest import l1
from pypde_gb300 import _lib, systems, workloads
from pypde_gb300.solvers import pde_solver

pytestmark = pytest.mark.gpu


def _run(u0, s, tol, K, **kw):
    q, st = u0.copy(), {}
    pde_solver(q, 10.0, [1.0] * (u0.ndim - 1), F=s.F, B=s.B, S=s.S, boundaryTypes="periodic",
               cfl=0.8, order=2, stiff=True, max_steps=K, stats=st, newton_tol=tol, **kw)
    assert st["steps"] == K and st["pred_fail"] == 0
    return q, st


@pytest.mark.parametrize("case", ["cattaneo2d", "cattaneo3d", "ncp2d"])
def test_mixed_precision_matches_plain_error_level(gpu_lib, case):
    if case == "cattaneo2d":
        u0, s, K = workloads.relaxation(48, 2, seed=11, patches=4), systems.cattaneo(2), 20
    elif case == "cattaneo3d":
        u0, s, K = workloads.relaxation(12, 3, seed=4), systems.cattaneo(3), 6
    else:
        u0, s, K = workloads.random_state("ncp", (20, 18), 3), systems.ncp(2), 10
    q_o, _ = _run(u0, s, 1e-15, K)
    q_p, st_p = _run(u0, s, 1e-12, K)
    q_p13, _ = _run(u0, s, 1e-13, K)
    q_m, st_m = _run(u0, s, 1e-12, K, mixed_precision=True)
    floor = max(l1(q_p, q_o).max(), l1(q_p13, q_o).max())
    err = l1(q_m, q_o).max()
    print(f"{case}: L1 vs oracle plain {l1(q_p, q_o).max():.2e} mixed {err:.2e}; FP64 sweeps "
          f"plain {st_p['pred_iters']} mixed {st_m['pred_iters']}; FP32 sweeps "
          f"{st_m['pred_iters32']}")
    assert err <= max(1e-8, 3 * floor), (err, floor)
    assert st_m["pred_iters32"] > 0
    assert st_m["pred_iters"] <= st_p["pred_iters"] * 1.05


def test_mixed_precision_refused_where_it_cannot_run(gpu_lib):
    s = systems.cattaneo(2)
    u0 = workloads.relaxation(8, 2, seed=1)
    with pytest.raises(_lib.PyPDEError):
        pde_solver(u0.copy(), 1.0, [1.0, 1.0], F=s.F, S=s.S, stiff=True, max_steps=1,
                   mixed_precision=True, jit=True)   # run-time callbacks have no FP32 twin


@pytest.mark.parametrize("case", ["cattaneo2d", "cattaneo3d", "ncp2d", "cattaneo2d-N3"])
def test_mixed_precision_run_matches_port(gpu_lib, case):
    """The mixed form against the restatement's mixed form (the same FP32
    sweeps with FP32 twins of the callbacks, then the FP64 iteration with at
    least two updates): bit for bit after K steps."""
    import numpy as np

    from oracle import ora
    N = 3 if case.endswith("N3") else 2
    if case.startswith("cattaneo2d"):
        u0, s, name, K = workloads.relaxation(16, 2, seed=11, patches=4), systems.cattaneo(2), \
            "cattaneo", 6
    elif case == "cattaneo3d":
        u0, s, name, K = workloads.relaxation(6, 3, seed=4), systems.cattaneo(3), "cattaneo", 2
    else:
        u0, s, name, K = workloads.random_state("ncp", (12, 10), 3), systems.ncp(2), "ncp", 4
    ndim = u0.ndim - 1
    u_o, _, steps_o, t_o = ora.pde_solver(name, u0, 10.0, [1.0] * ndim, [1] * ndim, 0.8, N,
                                          stiff=True, max_steps=K, mixed=True)
    q, st = u0.copy(), {}
    pde_solver(q, 10.0, [1.0] * ndim, F=s.F, B=s.B, S=s.S, boundaryTypes="periodic", cfl=0.8,
               order=N, stiff=True, max_steps=K, stats=st, mixed_precision=True)
    assert st["steps"] == steps_o == K and st["t_final"] == t_o
    assert st["pred_iters32"] > 0
    assert np.array_equal(q, u_o), np.abs(q - u_o).max()
