"""Learned warm start on the GPU: the training kernels against the CPU
oracle of the network (oracle/mlp_oracle.py), the fused inference kernel
against the training forward pass, the Newton iteration from a guess
against the restatement (bit for bit, fallbacks included), harvesting, and
a trained network end to end: same answer as the plain form within 1e-8
relative L1, fewer Newton iterations."""
import numpy as np
import pytest

from conftest import l1
from oracle import mlp_oracle as mo
from oracle import ora
from pypde_gb300 import stages, systems, warmstart, workloads
from pypde_gb300.callbacks import builtin_system
from pypde_gb300.solvers import pde_solver

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _rel(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def _net(k1=48, no=56, seed=0):
    net = warmstart.WarmStartNet(37, k1, no, 56, 7, seed=seed)
    return net, [p.detach().cpu().numpy().astype(np.float64) for p in net.params]


@pytest.mark.parametrize("shape", [(1, 48, 128), (77, 48, 128), (4096, 128, 128),
                                   (300, 128, 56), (5, 16, 8)])
def test_gemm_against_oracle(gpu_lib, shape):
    """C = x W^T + b: BF16 operands, FP32 accumulation (tolerance: FP32
    accumulation order, 1e-5 of max |C|)."""
    M, K, Nn = shape
    rng = np.random.default_rng(M)
    x = rng.standard_normal((M, K)).astype(np.float32)
    W = (rng.standard_normal((Nn, K)) * 0.2).astype(np.float32)
    b = rng.standard_normal(Nn).astype(np.float32)
    X, Wt, bt = (torch.from_numpy(a).cuda() for a in (x, W, b))
    C, A = warmstart.gemm(X, Wt, M, Nn, K, K, 1, 1, K, bias=bt, act=True)
    want = mo.linear(x, W, b)
    tol = 1e-5 * np.abs(want).max()
    assert np.abs(C.cpu().numpy() - want).max() <= tol
    assert np.abs(A.cpu().numpy() - mo.silu(want)).max() <= 2 * tol + 1e-6


def test_gemm_split_k_transposed(gpu_lib):
    """dW = dZ^T X with the batch as the split reduction dimension."""
    rng = np.random.default_rng(3)
    M, n_out, n_in = 5000, 56, 128
    dZ = rng.standard_normal((M, n_out)).astype(np.float32)
    X = rng.standard_normal((M, n_in)).astype(np.float32)
    for splits in (1, 7, 64):
        C, _ = warmstart.gemm(torch.from_numpy(dZ).cuda(), torch.from_numpy(X).cuda(), n_out,
                              n_in, M, 1, n_out, n_in, 1, splits=splits)
        want = mo.bf16(dZ).T @ mo.bf16(X)
        assert np.abs(C.cpu().numpy() - want).max() <= 1e-5 * np.abs(want).max()


def test_autograd_function_against_oracle(gpu_lib):
    """Forward output and every parameter gradient of the autograd.Function
    against the oracle (relative Frobenius error <= 2e-3: FP32 accumulation
    plus activations that round to the other BF16 neighbour)."""
    net, P = _net()
    rng = np.random.default_rng(7)
    x = rng.standard_normal((2048, 48)).astype(np.float32)
    dy = rng.standard_normal((2048, 56)).astype(np.float32)
    X = torch.from_numpy(x).cuda()
    y = net.forward(X)
    y.backward(torch.from_numpy(dy).cuda())
    y_o, cache = mo.forward(x, P)
    assert _rel(y.detach().cpu().numpy(), y_o) <= 2e-3
    grads = mo.backward(dy, P, cache)
    for p, g in zip(net.params, grads):
        assert _rel(p.grad.cpu().numpy(), g) <= 2e-3


def _stiff_case(n=12, seed=5):
    u = workloads.relaxation(n, 2, seed=seed)
    N, dX = 2, [1 / n, 1 / n]
    w = ora.weno(ora.boundaries(u, N, [1, 1]), N)
    dt = ora.timestep("cattaneo", w, dX, N, 0.8, 10.0, 0.0, 0)
    qh, its, mx = ora.predictor("cattaneo", w, dX, N, True, dt)
    return w, dX, N, dt, qh, its


@pytest.mark.parametrize("kind", ["exact", "close", "rough", "nan", "huge"])
def test_newton_from_guess_bitwise(gpu_lib, kind):
    w, dX, N, dt, qh, its = _stiff_case()
    wb = np.repeat(w.reshape(-1, 1, 4, 7), N, axis=1).reshape(qh.shape)
    rng = np.random.default_rng(1)
    g = {"exact": qh, "close": qh + 1e-7 * (qh - wb) * rng.standard_normal(qh.shape),
         "rough": qh + 0.3 * (qh - wb) * rng.standard_normal(qh.shape),
         "nan": np.where(rng.random(qh.shape) < 0.01, np.nan, qh),
         "huge": qh * 1e30}[kind]
    q_o, it_o, mx_o, fb_o = ora.predictor_guess("cattaneo", w, dX, N, dt, g)
    q_g, st = stages.predictor_guess("cattaneo", w, dX, N, dt, guess=g)
    assert np.array_equal(q_g, q_o)
    assert st["pred_iters"] == it_o and st["pred_max_iters"] == mx_o
    assert st["pred_fallbacks"] == fb_o
    if kind == "nan":
        assert fb_o > 0
    assert np.abs(q_o - qh).max() <= 1e-9 * np.abs(qh).max()


def test_harvest_matches_stages(gpu_lib):
    """One harvested step of every cell equals the stage-by-stage pass."""
    n, N = 10, 2
    u0 = workloads.relaxation(n, 2, seed=2)
    s = systems.cattaneo(2)
    hw, hq, hdt = warmstart.harvest(u0, 10.0, [1.0, 1.0], F=s.F, S=s.S, cfl=0.8, order=N,
                                    steps=1, per_step=(n + 2) ** 2)
    w = ora.weno(ora.boundaries(u0, N, [1, 1]), N)
    dt = ora.timestep("cattaneo", w, [1 / n, 1 / n], N, 0.8, 10.0, 0.0, 0)
    qh, _, _ = ora.predictor("cattaneo", w, [1 / n, 1 / n], N, True, dt)
    assert np.all(hdt == dt)
    assert np.array_equal(hw.reshape(w.shape), w)
    assert np.array_equal(hq.reshape(qh.shape), qh)


def test_fused_inference_matches_training_forward(gpu_lib):
    """k_mlp_guess (through a Newton call whose tolerance accepts the guess
    as it is) against features -> autograd forward -> de-normalisation."""
    w, dX, N, dt, qh, its = _stiff_case()
    sysobj = builtin_system("cattaneo", 2)
    feat, k1, no = warmstart.shape(sysobj, N)
    net = warmstart.WarmStartNet(feat, k1, no, N * 4 * 7, 7, seed=3)
    f = warmstart.features(w, dt, N, 2, 7, tau_var=6)
    d = warmstart.targets(w, qh, N, 2, 7)
    net.fit_normalisation(f, d)
    ws = warmstart.WarmStart(sysobj, N, net, tau_var=6)
    q_g, st = stages.predictor_guess("cattaneo", w, dX, N, dt, warm=ws, tol=1e300)
    assert st["pred_iters"] == 0
    x, r = net.inputs(f)
    with torch.no_grad():
        y = net.forward(torch.from_numpy(x).cuda()).cpu().numpy()
    corr = net.correction(y, r)
    want = np.repeat(w.reshape(-1, 1, 4, 7), N, axis=1).reshape(-1, N * 28) + \
        corr.astype(np.float64)
    got = q_g.reshape(-1, N * 28)
    assert np.abs(got - want).max() <= 1e-6 * np.abs(corr).max() + 1e-15


def test_trained_warm_start_end_to_end(gpu_lib):
    """Train on 20 harvested steps of a 48x48 relaxation problem, then run
    30 steps plain and learned, both with Newton tolerance 1e-12, and
    compare each with an oracle run at tolerance 1e-15.  Two Newton solves
    stopped at the same residual tolerance from different guesses differ
    by that tolerance's effect, which grows with the steps taken: the bound
    is the stiff form's 1e-8 relative L1 per 10 steps, 3e-8 here (the plain
    form's own distance from the converged run, printed, is of that order).
    Newton iterations are measured against the plain run and written to
    the test output.  Perturbing the converged corrections at random shows
    what a guess must achieve on this iteration: a 10% relative error per
    entry costs iterations, 1% saves none, 0.1% saves about 13%; the
    network's per-cell error is tens of percent, so it saves none, and the
    bound checked is that it costs at most 10% more."""
    n, N, K = 48, 2, 30
    u0 = workloads.relaxation(n, 2, seed=11, patches=4)
    s = systems.cattaneo(2)
    ws = warmstart.train_warm_start(u0, 10.0, [1.0, 1.0], F=s.F, S=s.S, cfl=0.8, order=N,
                                    tau_var=6, steps=20, per_step=1024, iters=3000, seed=0)

    def run(tol, warm=None):
        q, st = u0.copy(), {}
        pde_solver(q, 10.0, [1.0, 1.0], F=s.F, S=s.S, boundaryTypes="periodic", cfl=0.8,
                   order=N, stiff=True, max_steps=K, stats=st, newton_tol=tol,
                   warm_start=warm)
        assert st["steps"] == K and st["pred_fail"] == 0
        return q, st

    q_o, _ = run(1e-15)
    q_p, st_p = run(1e-12)
    q_p13, _ = run(1e-13)
    # the validation gate: the network is used only if it saved iterations
    # on the held-out harvested cells; otherwise pde_solver keeps the plain
    # guess and gives the plain form's bits
    v = ws.validation
    assert ws.active == (v["iters_learned"] < v["iters_plain"]), v
    print(f"validation on {v['cells']} held-out cells: Newton iterations plain "
          f"{v['iters_plain']}, learned {v['iters_learned']}")
    if not ws.active:
        q_g, st_g = run(1e-12, ws)
        assert np.array_equal(q_g, q_p) and st_g["pred_iters"] == st_p["pred_iters"]
    ws.active = True  # the network's own guess from here on
    q_l, st_l = run(1e-12, ws)
    floor = max(l1(q_p, q_o).max(), l1(q_p13, q_o).max())
    err = l1(q_l, q_o).max()
    saved = 1 - st_l["pred_iters"] / st_p["pred_iters"]
    print(f"warm start: train rms {ws.train_rms:.3g}; L1 vs tol-1e-15 oracle: plain "
          f"{l1(q_p, q_o).max():.2e}, learned {err:.2e} (floor {floor:.2e}); Newton "
          f"iterations plain {st_p['pred_iters']} learned {st_l['pred_iters']} "
          f"(saved {100 * saved:.1f}%), fallbacks {st_l['pred_fallbacks']}")
    assert err <= 1e-8 * K / 10, (err, floor)
    assert st_l["pred_iters"] <= 1.1 * st_p["pred_iters"]
