"""Learned warm start, CPU side: the network oracle pinned against finite
differences, BF16 rounding known answers, the feature recipe, and the
restatement's Newton-from-a-guess with its fallback rule."""
import numpy as np
import pytest

from oracle import mlp_oracle as mo
from oracle import ora
from pypde_gb300 import warmstart, workloads


def test_bf16_rounding_known_answers():
    big = float(np.finfo(np.float32).max)
    x = np.array([1.0, 1 + 2 ** -8, 1 + 3 * 2 ** -8, 1 + 2 ** -8 + 2 ** -20, -2.5, 0.0,
                  3.3895313892515355e38, big])
    want = [1.0, 1.0, 1 + 2 ** -6, 1 + 2 ** -7, -2.5, 0.0, 3.3895313892515355e38]
    got = mo.bf16(x)
    assert got[:7].tolist() == want              # ties to even; largest BF16 kept
    assert np.isinf(got[7])                      # the FP32 maximum rounds past it
    assert np.isnan(mo.bf16(np.array([np.nan]))[0])


def _params(rng, k1=16, h=12, no=8):
    return [rng.standard_normal((h, k1)) * 0.3, rng.standard_normal(h) * 0.1,
            rng.standard_normal((h, h)) * 0.3, rng.standard_normal(h) * 0.1,
            rng.standard_normal((no, h)) * 0.3, rng.standard_normal(no) * 0.1]


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    P = _params(rng)
    x = rng.standard_normal((5, 16))
    dy = rng.standard_normal((5, 8))
    y, cache = mo.forward(x, P, rounding=False)
    grads = mo.backward(dy, P, cache, rounding=False)
    h = 1e-6
    for pi, (p, g) in enumerate(zip(P, grads)):
        flat = p.reshape(-1)
        for j in rng.choice(flat.size, size=min(6, flat.size), replace=False):
            old = flat[j]
            flat[j] = old + h
            yp = mo.forward(x, P, rounding=False)[0]
            flat[j] = old - h
            ym = mo.forward(x, P, rounding=False)[0]
            flat[j] = old
            fd = ((yp - ym) * dy).sum() / (2 * h)
            assert abs(fd - g.reshape(-1)[j]) <= 1e-6 * max(1.0, abs(fd)), (pi, j)


def test_features_recipe():
    rng = np.random.default_rng(1)
    N, ndim, V = 2, 2, 7
    Nd = N ** ndim
    w = rng.standard_normal((9, Nd, V)) + 3
    dt = 1e-3
    f = warmstart.features(w, dt, N, ndim, V, tau_var=6)
    assert f.dtype == np.float32 and f.shape == (9, V + Nd * V + 1)
    for c in range(9):
        for v in range(V):
            s = w[c, 0, v]
            for i in range(1, Nd):
                s += w[c, i, v]
            m = s * (1.0 / Nd)
            assert f[c, v] == np.float32(m)
            for i in range(Nd):
                assert f[c, V + i * V + v] == np.float32(w[c, i, v] - m)
        m6 = sum(w[c, i, 6] for i in range(Nd)) * (1.0 / Nd)
        assert abs(f[c, -1] - np.float32(np.log10(dt) - m6)) <= 1e-6 * abs(f[c, -1])
    d = warmstart.targets(w, np.repeat(w[:, None], N, 1) + 0.5, N, ndim, V)
    assert d.shape == (9, N * Nd * V) and np.allclose(d, 0.5, rtol=0, atol=1e-14)


def _stiff_case(n=12, seed=5):
    u = workloads.relaxation(n, 2, seed=seed)
    N, dX = 2, [1 / n, 1 / n]
    w = ora.weno(ora.boundaries(u, N, [1, 1]), N)
    dt = ora.timestep("cattaneo", w, dX, N, 0.8, 10.0, 0.0, 0)
    qh, its, _ = ora.predictor("cattaneo", w, dX, N, True, dt)
    return w, dX, N, dt, qh, its


def test_port_newton_from_guess():
    w, dX, N, dt, qh, its = _stiff_case()
    # the converged answer is already converged: no iteration
    q0, it0, _, fb0 = ora.predictor_guess("cattaneo", w, dX, N, dt, qh)
    assert it0 == 0 and fb0 == 0 and np.array_equal(q0, qh)
    # a close guess converges in fewer iterations, to the same tolerance
    wb = np.repeat(w.reshape(-1, 1, 4, 7), N, axis=1).reshape(qh.shape)
    g = qh + 1e-6 * (qh - wb)
    q1, it1, _, fb1 = ora.predictor_guess("cattaneo", w, dX, N, dt, g)
    assert fb1 == 0 and it1 < its
    assert np.abs(q1 - qh).max() <= 1e-10 * np.abs(qh).max()


def test_guess_accuracy_needed_to_save_iterations():
    """How accurate a warm start must be before Newton saves sweeps, on the
    restatement (24^2 relaxation state after 10 steps, the step-9 dt): a
    guess that carries the converged correction with a relative error eps
    per entry.  The plain guess (w at every time node) needs ~5.8 sweeps per
    cell; eps = 1e-4 saves more than one, eps = 1e-2 less than half a sweep,
    and eps = 0.1, the accuracy class of a BF16 network, costs sweeps."""
    n, N = 24, 2
    u0 = workloads.relaxation(n, 2, seed=0)
    u = ora.pde_solver("cattaneo", u0, 1.0, [1.0, 1.0], [1, 1], 0.8, N, stiff=True,
                       max_steps=10, nthreads=2)[0]
    dX = [1.0 / n] * 2
    w = ora.weno(ora.boundaries(u, N, [1, 1]), N)
    dt = ora.timestep("cattaneo", w, dX, N, 0.8, 1.0, 0.0, 9)
    qh, its, _ = ora.predictor("cattaneo", w, dX, N, True, dt)
    cells = w.shape[0] // N ** 2
    wq = np.repeat(w.reshape(cells, 1, N * N, 7), N, axis=1).reshape(qh.shape)
    corr = qh - wq
    rng = np.random.default_rng(0)
    plain = its / cells
    sweeps = {}
    for eps in (1e-8, 1e-4, 1e-2, 0.1):
        g = wq + corr * (1 + eps * rng.standard_normal(corr.shape))
        _, it, _, fb = ora.predictor_guess("cattaneo", w, dX, N, dt, g)
        assert fb == 0
        sweeps[eps] = it / cells
    assert sweeps[1e-8] < sweeps[1e-4] < sweeps[1e-2] < sweeps[0.1]
    assert sweeps[1e-4] < plain - 1.0
    assert sweeps[1e-2] > plain - 0.5
    assert sweeps[0.1] > plain


def test_port_fallback_to_plain_guess():
    """A non-finite guess falls back at iteration 0; the cell then runs the
    plain iteration and gives the plain result bit for bit."""
    w, dX, N, dt, qh, its = _stiff_case()
    g = np.full_like(qh, np.nan)
    q, it, _, fb = ora.predictor_guess("cattaneo", w, dX, N, dt, g)
    ncell = qh.shape[0] // (N * 4)
    assert fb == ncell
    assert it == its + ncell                      # one spent iteration per cell
    assert np.array_equal(q, qh)


def test_normalisation_is_homogeneous():
    """Scaling a cell's deviations by lambda leaves the network's deviation
    inputs unchanged and scales r (and so the correction) by lambda."""
    pytest.importorskip("torch")
    rng = np.random.default_rng(4)
    N, ndim, V = 2, 2, 7
    w = 1 + 0.01 * rng.standard_normal((50, 4, V))
    f = warmstart.features(w, 1e-3, N, ndim, V, tau_var=-1)
    net = warmstart.WarmStartNet(V + 4 * V + 2, 48, 56, 56, V, device="cpu")
    net.fit_normalisation(f, rng.standard_normal((50, 56)) * 1e-4)
    x1, r1 = net.inputs(f)
    f2 = f.copy()
    f2[:, V:V + 4 * V] *= 8.0                    # a power of two: exact in float32
    x2, r2 = net.inputs(f2)
    assert np.array_equal(x1[:, V:V + 4 * V], x2[:, V:V + 4 * V])
    assert np.allclose(r2, 8 * r1, rtol=1e-6)
