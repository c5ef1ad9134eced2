"""Batched problems (pde_solver_batch): every problem of a mixed batch --
different sizes, orders, boundary types and end times -- gives the same
bits as the same problem solved alone, whatever tile shape the autotuner
or the caller picks."""
import numpy as np
import pytest

from pypde_gb300 import systems, workloads
from pypde_gb300.solvers import pde_solver, pde_solver_batch

pytestmark = pytest.mark.gpu


def _problems(system, seed, stiff):
    rng = np.random.default_rng(seed)
    out = []
    for k, (n, N) in enumerate([(24, 2), (9, 1), (40, 3), (17, 2), (12, 3), (31, 1), (8, 2)]):
        m = int(n + rng.integers(0, 4))
        shape = (m, n)
        if system == "cattaneo":
            u = workloads.relaxation(n, 2, seed=seed + k, patches=4)[:, :n].copy()
            u = u[:m] if m <= n else np.concatenate([u, u[:m - n]], 0).copy()
        else:
            u = workloads.random_state("euler", shape, seed + k)
        bt = ["periodic", "transitive"][k % 2]
        if bt == "periodic" and min(shape) < N:
            bt = "transitive"
        out.append({"Q0": np.ascontiguousarray(u), "tf": float(rng.uniform(0.002, 0.02)),
                    "L": [1.0, float(m) / n], "order": N, "boundaryTypes": bt,
                    "cfl": 0.8 if stiff else 0.9})
    return out


@pytest.mark.parametrize("system,stiff", [("euler", False), ("cattaneo", True)])
@pytest.mark.parametrize("mode", ["autotune", "per_pop3", "direct"])
def test_batch_matches_single_problems(gpu_lib, system, stiff, mode):
    s = systems.euler(2) if system == "euler" else systems.cattaneo(2)
    probs = _problems(system, 3, stiff)
    singles = []
    for p in probs:
        q = p["Q0"].copy()
        st = {}
        pde_solver(q, p["tf"], p["L"], F=s.F, S=s.S, boundaryTypes=p["boundaryTypes"],
                   cfl=p["cfl"], order=p["order"], ndt=1, stiff=stiff, stats=st)
        singles.append((q, st))
    batch = [dict(p, Q0=p["Q0"].copy()) for p in probs]
    stats = {}
    pde_solver_batch(batch, F=s.F, S=s.S, stiff=stiff, autotune=(mode == "autotune"),
                     per_pop=0 if mode == "direct" else 3, stats=stats)
    for p, (q, st), k, t in zip(batch, singles, stats["steps_per_problem"], stats["t_final"]):
        assert k == st["steps"] and t == st["t_final"]
        assert np.array_equal(p["Q0"], q)
    assert stats["steps"] == sum(st["steps"] for _, st in singles)
    assert stats["nan_found"] == 0
    if mode == "autotune":
        assert all(v in (0, 1, 2, 4, 8) for v in stats["per_pop"].values())


def test_batch_max_steps_and_jit(gpu_lib):
    """A step cap per problem, and a batch of run-time compiled callbacks."""
    s = systems.euler(2)
    probs = _problems("euler", 9, False)[:4]
    singles = []
    for p in probs:
        q = p["Q0"].copy()
        pde_solver(q, p["tf"], p["L"], F=s.F, boundaryTypes=p["boundaryTypes"], cfl=p["cfl"],
                   order=p["order"], ndt=1, stiff=False, max_steps=3)
        singles.append(q)
    batch = [dict(p, Q0=p["Q0"].copy()) for p in probs]
    stats = {}
    pde_solver_batch(batch, F=s.F, stiff=False, max_steps=3, stats=stats, jit=True)
    assert stats["steps_per_problem"] == [3] * 4
    for p, q in zip(batch, singles):
        assert np.array_equal(p["Q0"], q)


def test_batch_learned_and_mixed_forms_match_single_problems(gpu_lib):
    """The learned warm start (one network per order, its guess computed by
    one batched launch per order) and the FP32 Newton sweeps through the
    batch: every problem gives the bits pde_solver gives it alone with the
    same warm start and precision, for each of the three forms."""
    from pypde_gb300 import warmstart
    s = systems.cattaneo(2)
    probs = _problems("cattaneo", 5, True)
    nets = {}
    for N in (1, 2, 3):
        u0 = workloads.relaxation(16, 2, seed=20 + N, patches=4)
        ws = warmstart.train_warm_start(u0, 10.0, [1.0, 1.0], F=s.F, S=s.S, cfl=0.8,
                                        order=N, tau_var=6, steps=4, per_step=128, iters=100,
                                        seed=N)
        ws.active = True  # use the network whatever its validation found
        nets[N] = ws
    for opts in ({"warm_start": nets}, {"mixed_precision": True},
                 {"warm_start": nets, "mixed_precision": True}):
        singles = []
        for p in probs:
            q = p["Q0"].copy()
            st = {}
            pde_solver(q, p["tf"], p["L"], F=s.F, S=s.S, boundaryTypes=p["boundaryTypes"],
                       cfl=p["cfl"], order=p["order"], ndt=1, stiff=True, stats=st,
                       warm_start=nets[p["order"]] if "warm_start" in opts else None,
                       mixed_precision=opts.get("mixed_precision", False))
            singles.append((q, st))
        batch = [dict(p, Q0=p["Q0"].copy()) for p in probs]
        stats = {}
        pde_solver_batch(batch, F=s.F, S=s.S, stiff=True, stats=stats, **opts)
        for p, (q, st), k in zip(batch, singles, stats["steps_per_problem"]):
            assert k == st["steps"]
            assert np.array_equal(p["Q0"], q), opts.keys()
        assert stats["pred_iters"] == sum(st["pred_iters"] for _, st in singles)
        if "warm_start" in opts:
            assert stats["per_pop"]["guess"] in (0, 1, 2, 4, 8)
