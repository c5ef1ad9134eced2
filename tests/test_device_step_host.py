"""The whole device step on the CPU: the kernels of pypde_gb300/csrc compiled
as host C++ (tests/device_step_host.cpp) and run with every CUDA thread of a
block as a fiber, against the C restatement, bit for bit.

The GPU parity tests compare the kernels with the restatement on the GPU.
This test checks the same source, with the runtime's launch shapes and stage
order, without one:
- ghost fill, the WENO passes, the CFL reduction (warp shuffles and
  atomics), the Picard and Newton predictors (shared memory, block barriers
  with AND reductions), face fluxes, centres and the gather;
- full runs of every built-in system, orders 1-3, 1-D to 3-D, periodic and
  transmissive axes, Rusanov/Roe/Osher fluxes, B terms, the second-order
  form and the stiff Newton predictor: final state, t and step count equal;
- the predictor stage alone with its iteration counts, and the Newton
  predictor started from a given guess with its fallbacks;
- batched steps (batch.cuh) of problems of mixed sizes, boundary types and
  end times: each problem equals the restatement run on it alone;
- the mixed-precision stiff predictor (FP32 sweeps, then FP64) against the
  restatement's mixed form, FP32 sweep counts included;
- the fibers of a block run in thread order and in reverse order, and the
  results must agree: a read of shared memory that no barrier orders after
  its write would change with the order.

The only edit to the device headers is the one the host compiler needs:
`extern __shared__ double smem[];` becomes a pointer to a host buffer."""
import ctypes

import numpy as np
import pytest

from conftest import build_device_host, l1, load_device_host
from oracle import ora
from pypde_gb300 import stages, workloads


@pytest.fixture(scope="module")
def step_lib(tmp_path_factory):
    return load_device_host(build_device_host(tmp_path_factory.mktemp("devstep")))


def _run(L, name, u0, N, bt, cfl, K, stiff=False, flux=0, tol=1e-12, mixed=0, reverse=False,
         strips=1):
    nX = np.array(u0.shape[:-1], dtype=np.int32)
    dX = np.array([1.0 / n for n in nX])
    u = np.ascontiguousarray(u0, dtype=np.float64).copy()
    t, its = ctypes.c_double(), ctypes.c_ulonglong()
    L.host_set_order(int(reverse))
    L.host_set_strips(int(strips))
    steps = L.host_run(name.encode(), len(nX), N, flux, ora.ptr(u), ora.ptr(nX),
                       ora.ptr(np.array(bt, dtype=np.int32)), ora.ptr(dX),
                       ora.ptr(stages.tables(N)), 10.0, cfl, int(stiff), tol, mixed, K,
                       ctypes.byref(t), ctypes.byref(its))
    assert steps >= 0, "combination not instantiated" if steps == -1 else "barrier deadlock"
    return u, steps, t.value, its.value


def _state(system, shape, seed, log10_tau=(-4.0, -2.0)):
    u = workloads.random_state(system, shape, seed)
    if system == "cattaneo":
        u[..., -1] = np.random.default_rng(seed).uniform(*log10_tau, shape)
    return u


RUNS = [
    ("euler", workloads.sod(40), 2, [0], 0.9, 10, False, 0, "sod40-N2"),
    ("euler", _state("euler", (17,), 1), 1, [1], 0.9, 6, False, 0, "euler17-N1"),
    ("euler", _state("euler", (24,), 2), 3, [1], 0.9, 6, False, 0, "euler24-N3"),
    ("euler", workloads.shear(16), 2, [1, 0], 0.8, 10, False, 0, "shear16-N2"),
    ("euler", _state("euler", (12, 10), 3), 3, [1, 1], 0.5, 4, False, 0, "euler12x10-N3"),
    ("euler", _state("euler", (6, 5, 7), 6), 2, [1, 1, 0], 0.5, 4, False, 0, "euler3d-N2"),
    ("euler", workloads.sod(16), 2, [0], 0.9, 6, False, 1, "sod16-roe"),
    ("euler", workloads.sod(16), 2, [0], 0.9, 6, False, 2, "sod16-osher"),
    ("euler", _state("euler", (7, 6), 5), 2, [1, 0], 0.6, 3, False, 1, "euler2d-roe"),
    ("euler", _state("euler", (6, 7), 6), 2, [0, 1], 0.6, 3, False, 2, "euler2d-osher"),
    ("ncp", _state("ncp", (7, 6), 7), 2, [1, 1], 0.5, 3, False, 2, "ncp2d-osher"),
    ("cattaneo", workloads.relaxation(8, 2, seed=9), 2, [1, 1], 0.8, 2, True, 1,
     "relax8-stiff-roe"),
    ("ncp", _state("ncp", (16,), 4), 2, [0], 0.5, 6, False, 0, "ncp16-N2"),
    ("ncp", _state("ncp", (12, 10), 4), 2, [1, 1], 0.5, 6, False, 0, "ncp12x10-N2"),
    ("burgers2", _state("burgers2", (32,), 5), 3, [1], 0.5, 6, False, 0, "burgers32-N3"),
    ("cattaneo", workloads.relaxation(24, 2, seed=3), 2, [1, 1], 0.8, 4, True, 0,
     "relax24-stiff-N2"),
    ("cattaneo", workloads.relaxation(12, 2, seed=5), 1, [1, 1], 0.8, 4, True, 0,
     "relax12-stiff-N1"),
    ("cattaneo", workloads.relaxation(12, 2, seed=6), 3, [1, 1], 0.8, 3, True, 0,
     "relax12-stiff-N3"),
    ("cattaneo", _state("cattaneo", (6, 5, 4), 7), 2, [1, 1, 1], 0.8, 2, True, 0,
     "cattaneo3d-stiff-N2"),
    ("cattaneo", _state("cattaneo", (10, 8), 8, (-1.0, 0.0)), 2, [1, 0], 0.8, 4, False, 0,
     "cattaneo10x8-picard"),
]


@pytest.mark.parametrize("run", RUNS, ids=[r[-1] for r in RUNS])
def test_device_step_equals_port(step_lib, run):
    name, u0, N, bt, cfl, K, stiff, flux, _ = run
    u_o, _, steps_o, t_o = ora.pde_solver(name, u0, 10.0, [1.0] * (u0.ndim - 1), bt, cfl, N,
                                          stiff=stiff, flux=flux, max_steps=K)
    u_f, steps_f, t_f, its_f = _run(step_lib, name, u0, N, bt, cfl, K, stiff, flux)
    u_r, steps_r, t_r, its_r = _run(step_lib, name, u0, N, bt, cfl, K, stiff, flux,
                                    reverse=True)
    assert steps_f == steps_o == K
    assert t_f == t_o
    assert np.array_equal(u_f, u_o), np.abs(u_f - u_o).max()
    assert (steps_r, t_r, its_r) == (steps_f, t_f, its_f)
    assert np.array_equal(u_r, u_f)


STRIP_RUNS = [r for r in RUNS if r[-1] in (
    "sod40-N2", "euler24-N3", "shear16-N2", "euler12x10-N3", "euler3d-N2", "euler2d-osher",
    "ncp12x10-N2", "relax24-stiff-N2", "relax12-stiff-N3", "cattaneo3d-stiff-N2",
    "cattaneo10x8-picard")]


@pytest.mark.parametrize("strips", [2, 5, 32])
@pytest.mark.parametrize("run", STRIP_RUNS, ids=[r[-1] for r in STRIP_RUNS])
def test_device_step_in_strips_equals_port(step_lib, run, strips):
    """The predictor in strips with each strip's faces run before the next
    strip is predicted (the order the second stream may take on the GPU):
    a face that read a cell of a later strip would read the last step's qh
    and miss the restatement."""
    name, u0, N, bt, cfl, K, stiff, flux, _ = run
    u_o, _, steps_o, t_o = ora.pde_solver(name, u0, 10.0, [1.0] * (u0.ndim - 1), bt, cfl, N,
                                          stiff=stiff, flux=flux, max_steps=K)
    u, steps, t, _ = _run(step_lib, name, u0, N, bt, cfl, K, stiff, flux, strips=strips)
    assert steps == steps_o == K and t == t_o
    assert np.array_equal(u, u_o), np.abs(u - u_o).max()


def _face_cells(nX, N, d, p_local):
    """Low- and high-side w-cells of face point p_local of direction d (the
    numbering of k_faces: face, time node, transverse node)."""
    ndim = len(nX)
    face = p_local // (N * N ** (ndim - 1))
    ext = [n + 1 if e == d else n for e, n in enumerate(nX)]
    O = list(np.unravel_index(face, ext))
    O = [o if e == d else o + 1 for e, o in enumerate(O)]
    nXw = [n + 2 for n in nX]
    lo = np.ravel_multi_index(O, nXw)
    O[d] += 1
    return lo, np.ravel_multi_index(O, nXw)


@pytest.mark.parametrize("shape,N,cpb,S", [((40,), 2, 12, 4), ((13, 9), 2, 12, 8),
                                           ((9, 13), 3, 5, 32), ((5, 6, 7), 2, 12, 6),
                                           ((64, 3), 1, 7, 32), ((2, 50), 2, 12, 8),
                                           ((4, 4, 4), 3, 1, 32), ((1, 1), 2, 12, 3)])
def test_strip_plan_partitions_faces_after_their_cells(step_lib, shape, N, cpb, S):
    """Every face point is released by exactly one strip, in its own
    direction's range, and only once the strips so far have predicted both
    of its cells."""
    L = step_lib
    nX = np.array(shape, dtype=np.int32)
    blk = np.zeros(33, dtype=np.int64)
    lo = np.zeros(96, dtype=np.int64)
    n = np.zeros(96, dtype=np.int64)
    i64 = ctypes.POINTER(ctypes.c_longlong)
    S_ = L.host_plan_strips(S, len(shape), ora.ptr(nX), N, cpb, blk.ctypes.data_as(i64),
                            lo.ctypes.data_as(i64), n.ctypes.data_as(i64))
    Cw = int(np.prod(nX + 2))
    nblocks = -(-Cw // cpb)
    assert 1 <= S_ <= min(S, nblocks)
    assert blk[0] == 0 and blk[S_] == nblocks and np.all(np.diff(blk[:S_ + 1]) >= 0)
    nodes = N * N ** (len(shape) - 1)
    nface = [np.prod([m + 1 if e == d else m for e, m in enumerate(shape)]) * nodes
             for d in range(len(shape))]
    off = np.concatenate([[0], np.cumsum(nface)])
    seen = np.zeros(off[-1], dtype=np.int32)
    for s in range(S_):
        done = Cw if s == S_ - 1 else min(blk[s + 1] * cpb, Cw)
        for d in range(3):
            lo_, n_ = lo[s * 3 + d], n[s * 3 + d]
            if d >= len(shape):
                assert n_ == 0
                continue
            assert n_ >= 0 and off[d] <= lo_ and lo_ + n_ <= off[d + 1]
            seen[lo_:lo_ + n_] += 1
            for p in range(lo_, lo_ + n_, max(1, n_ // 50)):
                c0, c1 = _face_cells(shape, N, d, p - off[d])
                assert c0 < done and c1 < done, (s, d, p)
    assert np.all(seen == 1)


PRED_CASES = [("cattaneo", (10, 8), 2, True), ("cattaneo", (6, 5, 4), 2, True),
              ("cattaneo", (9, 7), 3, True), ("cattaneo", (8, 7), 1, True),
              ("ncp", (12,), 2, True), ("euler", (8, 6), 2, True), ("euler", (8, 6), 2, False),
              ("euler", (9,), 3, False), ("ncp", (7, 6), 2, False)]


@pytest.mark.parametrize("case", PRED_CASES,
                         ids=[f"{c[0]}-{len(c[1])}d-N{c[2]}-{'newton' if c[3] else 'picard'}"
                              for c in PRED_CASES])
def test_device_predictor_equals_port(step_lib, case):
    """The predictor stage on the same w and dt: qh and the iteration counts
    (sum over cells and maximum) equal the restatement's."""
    system, shape, N, stiff = case
    u = workloads.random_state(system, shape, 2)
    dX = np.array([1.0 / n for n in shape])
    bt = [1] * len(shape)
    w = ora.weno(ora.boundaries(u, N, bt), N)
    dt = ora.timestep(system, w, dX, N, 0.9, 1.0, 0.0, 9)
    qh_o, its_o, mx_o = ora.predictor(system, w, dX, N, stiff, dt, 1e-12)
    for reverse in (False, True):
        step_lib.host_set_order(int(reverse))
        qh = np.zeros_like(qh_o)
        its, mx, fail = ctypes.c_ulonglong(), ctypes.c_int(), ctypes.c_int()
        rc = step_lib.host_predictor(system.encode(), len(shape), N, int(stiff), ora.ptr(w),
                                     w.shape[0], ora.ptr(dX), dt, 1e-12,
                                     ora.ptr(stages.tables(N)), ora.ptr(qh), ctypes.byref(its),
                                     ctypes.byref(mx), ctypes.byref(fail))
        assert rc == 0
        assert np.array_equal(qh, qh_o), np.abs(qh - qh_o).max()
        assert its.value == its_o and mx.value == mx_o and fail.value == 0


@pytest.mark.parametrize("mixed", [False, True], ids=["fp64", "mixed"])
@pytest.mark.parametrize("kind", ["exact", "close", "rough", "nan", "huge"])
def test_device_newton_from_guess_equals_port(step_lib, kind, mixed):
    """The Newton predictor started from a given guess (the warm start's
    entry), in FP64 or with FP32 sweeps from the guess first (the learned
    and mixed form): qh, iteration counts, FP32 sweeps and the cells reset
    to the plain guess (non-finite or non-decreasing residual) equal the
    restatement's."""
    n, N = 12, 2
    u = workloads.relaxation(n, 2, seed=5)
    dX = np.array([1 / n, 1 / n])
    w = ora.weno(ora.boundaries(u, N, [1, 1]), N)
    dt = ora.timestep("cattaneo", w, dX, N, 0.8, 10.0, 0.0, 0)
    qh, _, _ = ora.predictor("cattaneo", w, dX, N, True, dt)
    wb = np.repeat(w.reshape(-1, 1, 4, 7), N, axis=1).reshape(qh.shape)
    rng = np.random.default_rng(1)
    g = {"exact": qh, "close": qh + 1e-7 * (qh - wb) * rng.standard_normal(qh.shape),
         "rough": qh + 0.3 * (qh - wb) * rng.standard_normal(qh.shape),
         "nan": np.where(rng.random(qh.shape) < 0.01, np.nan, qh),
         "huge": qh * 1e30}[kind]
    out = ora.predictor_guess("cattaneo", w, dX, N, dt, g, mixed=mixed)
    q_o, it_o, mx_o, fb_o = out[:4]
    sw_o = out[4] if mixed else 0
    for reverse in (False, True):
        step_lib.host_set_order(int(reverse))
        q = np.zeros_like(qh)
        its, mx, fb = ctypes.c_ulonglong(), ctypes.c_int(), ctypes.c_ulonglong()
        sw = ctypes.c_ulonglong()
        rc = step_lib.host_predictor_guess(b"cattaneo", 2, N, ora.ptr(w), w.shape[0],
                                           ora.ptr(dX), dt, 1e-12, ora.ptr(stages.tables(N)),
                                           ora.ptr(np.ascontiguousarray(g)), ora.ptr(q),
                                           ctypes.byref(its), ctypes.byref(mx), ctypes.byref(fb),
                                           int(mixed), ctypes.byref(sw))
        assert rc == 0
        assert np.array_equal(q, q_o)
        assert (its.value, mx.value, fb.value, sw.value) == (it_o, mx_o, fb_o, sw_o)
    if kind == "nan":
        assert fb_o > 0


MIXED_RUNS = [("cattaneo", workloads.relaxation(16, 2, seed=11, patches=4), 2, [1, 1], 6),
              ("ncp", workloads.random_state("ncp", (12, 10), 3), 2, [1, 0], 4),
              ("cattaneo", workloads.relaxation(6, 3, seed=4), 2, [1, 1, 1], 2),
              ("cattaneo", workloads.relaxation(10, 2, seed=2), 3, [1, 1], 3)]


@pytest.mark.parametrize("run", MIXED_RUNS,
                         ids=[f"{r[0]}-{r[1].ndim - 1}d-N{r[2]}" for r in MIXED_RUNS])
def test_device_mixed_precision_step_equals_port(step_lib, run):
    """The mixed-precision stiff predictor (FP32 sweeps with the FP32
    callbacks, then at least two FP64 updates to the same 1e-12): equal to
    the restatement's mixed form bit for bit, in both fiber orders, and at
    the plain form's error level against a tolerance-1e-15 run."""
    name, u0, N, bt, K = run
    L = [1.0] * (u0.ndim - 1)
    u_o, _, steps_o, t_o = ora.pde_solver(name, u0, 10.0, L, bt, 0.8, N, stiff=True,
                                          max_steps=K, mixed=True)
    for reverse in (False, True):
        u_m, steps, t, _ = _run(step_lib, name, u0, N, bt, 0.8, K, stiff=True, mixed=1,
                                reverse=reverse)
        assert steps == steps_o == K and t == t_o
        assert np.array_equal(u_m, u_o), np.abs(u_m - u_o).max()
    u_ref, _, _, _ = ora.pde_solver(name, u0, 10.0, L, bt, 0.8, N, stiff=True, max_steps=K,
                                    newton_tol=1e-15)
    u_p, _, _, _ = ora.pde_solver(name, u0, 10.0, L, bt, 0.8, N, stiff=True, max_steps=K)
    floor = l1(u_p, u_ref).max()
    assert not np.array_equal(u_o, u_p)          # the FP32 sweeps change the iterate
    assert l1(u_o, u_ref).max() <= max(1e-8, 3 * floor), (l1(u_o, u_ref).max(), floor)


@pytest.mark.parametrize("case", [("cattaneo", (10, 8), 2), ("cattaneo", (9, 7), 3),
                                  ("cattaneo", (6, 5, 4), 2), ("ncp", (12,), 2),
                                  ("ncp", (7, 6), 2)],
                         ids=lambda c: f"{c[0]}-{len(c[1])}d-N{c[2]}")
def test_device_mixed_predictor_equals_port(step_lib, case):
    """The mixed predictor stage on the same w and dt: qh, the FP64
    iterations (sum and per-cell maximum) and the FP32 sweeps equal the
    restatement's."""
    system, shape, N = case
    u = workloads.random_state(system, shape, 2)
    dX = np.array([1.0 / n for n in shape])
    w = ora.weno(ora.boundaries(u, N, [1] * len(shape)), N)
    dt = ora.timestep(system, w, dX, N, 0.9, 1.0, 0.0, 9)
    qh_o, its_o, mx_o, sw_o = ora.predictor_mixed(system, w, dX, N, dt, 1e-12)
    assert sw_o > 0
    for reverse in (False, True):
        step_lib.host_set_order(int(reverse))
        qh = np.zeros_like(qh_o)
        its, mx, sw = ctypes.c_ulonglong(), ctypes.c_int(), ctypes.c_ulonglong()
        rc = step_lib.host_predictor_mixed(system.encode(), len(shape), N, ora.ptr(w),
                                           w.shape[0], ora.ptr(dX), dt, 1e-12,
                                           ora.ptr(stages.tables(N)), ora.ptr(qh),
                                           ctypes.byref(its), ctypes.byref(mx), ctypes.byref(sw))
        assert rc == 0
        assert np.array_equal(qh, qh_o), np.abs(qh - qh_o).max()
        assert (its.value, mx.value, sw.value) == (its_o, mx_o, sw_o)


BATCHES = [
    ("cattaneo", [workloads.relaxation(n, 2, seed=n) for n in (20, 12, 7)], 2,
     [[1, 1], [0, 1], [1, 0]], [0.8, 0.7, 0.9], [10.0, 10.0, 0.004], 4, True, "relax-stiff-N2"),
    ("euler", [workloads.shear(16), _state("euler", (12, 10), 3), _state("euler", (5, 7), 4)], 3,
     [[1, 0], [1, 1], [0, 0]], [0.8, 0.5, 0.5], [10.0, 10.0, 10.0], 3, False, "euler2d-N3"),
    ("ncp", [_state("ncp", (9, 8), 1), _state("ncp", (6, 11), 2)], 2, [[1, 0], [1, 1]],
     [0.5, 0.5], [10.0, 10.0], 4, False, "ncp2d-N2"),
]


@pytest.mark.parametrize("per_pop", [0, 1, 3])
@pytest.mark.parametrize("batch", BATCHES, ids=[b[-1] for b in BATCHES])
def test_device_batch_equals_port(step_lib, batch, per_pop):
    """Problems of mixed sizes, boundary types and end times stepped as one
    batch (batch.cuh: one launch per stage, tiles drained from a queue by
    persistent blocks, or one block per tile for per_pop = 0): each equals
    the restatement run on it alone, bit for bit, in both fiber orders."""
    name, us, N, bts, cfls, tfs, K, stiff, _ = batch
    nX = np.array([u.shape[:-1] for u in us], dtype=np.int32).ravel()
    dX = np.array([[1.0 / n for n in u.shape[:-1]] for u in us]).ravel()
    results = []
    for reverse in (False, True):
        step_lib.host_set_order(int(reverse))
        u_all = np.concatenate([u.ravel() for u in us])
        steps = (ctypes.c_longlong * len(us))()
        t = np.zeros(len(us))
        rc = step_lib.host_run_batch(name.encode(), us[0].ndim - 1, N, 0, len(us),
                                     ora.ptr(u_all), ora.ptr(nX),
                                     ora.ptr(np.array(bts, dtype=np.int32).ravel()),
                                     ora.ptr(dX), ora.ptr(np.array(tfs)), ora.ptr(np.array(cfls)),
                                     ora.ptr(stages.tables(N)), int(stiff), 1e-12, per_pop, 3, K,
                                     steps, ora.ptr(t))
        assert rc == 0
        results.append((u_all, list(steps), t))
    (u_f, steps_f, t_f), (u_r, steps_r, t_r) = results
    assert np.array_equal(u_f, u_r) and steps_f == steps_r and np.array_equal(t_f, t_r)
    o = 0
    for p, u0 in enumerate(us):
        u_o, _, steps_o, t_o = ora.pde_solver(name, u0, tfs[p], [1.0] * (u0.ndim - 1), bts[p],
                                              cfls[p], N, stiff=stiff, max_steps=K)
        assert steps_f[p] == steps_o and t_f[p] == t_o
        assert np.array_equal(u_f[o:o + u0.size].reshape(u0.shape), u_o)
        o += u0.size


# (system, ndim, order, flux, stiff) combinations the host unit instantiates
FUZZ_COMBOS = [("euler", 1, 1, 0, False), ("euler", 1, 2, 0, False), ("euler", 1, 3, 0, False),
               ("euler", 1, 2, 1, False), ("euler", 1, 2, 2, False), ("euler", 2, 2, 0, False),
               ("euler", 2, 3, 0, False), ("euler", 2, 2, 1, False), ("euler", 2, 2, 2, False),
               ("euler", 3, 2, 0, False), ("cattaneo", 2, 2, 1, True), ("ncp", 2, 2, 2, False),
               ("cattaneo", 2, 1, 0, True), ("cattaneo", 2, 2, 0, True),
               ("cattaneo", 2, 3, 0, True), ("cattaneo", 3, 2, 0, True),
               ("ncp", 1, 2, 0, False), ("ncp", 2, 2, 0, False), ("burgers2", 1, 3, 0, False)]


def test_device_step_fuzzed_small_grids(step_lib):
    """Hypothesis-drawn small grids (1-7 cells per axis), boundary types,
    states and step counts for every instantiated (system, ndim, order,
    flux): the device step equals the restatement bit for bit."""
    hyp = pytest.importorskip("hypothesis")
    st = hyp.strategies

    @st.composite
    def problems(draw):
        name, ndim, N, flux, stiff = draw(st.sampled_from(FUZZ_COMBOS))
        shape = tuple(draw(st.integers(1, 7)) for _ in range(ndim))
        # a periodic axis needs at least N cells (the reference's wrap rule)
        bt = [draw(st.integers(0, 1)) if n >= N else 0 for n in shape]
        return name, shape, N, flux, stiff, bt, draw(st.integers(0, 2 ** 16)), \
            draw(st.integers(1, 3)), draw(st.sampled_from([0.5, 0.8, 0.9])), \
            draw(st.sampled_from([1, 2, 3, 8]))

    @hyp.settings(max_examples=40, deadline=None, derandomize=True,
                  suppress_health_check=list(hyp.HealthCheck))
    @hyp.given(problems())
    def check(prob):
        name, shape, N, flux, stiff, bt, seed, K, cfl, strips = prob
        u0 = _state(name, shape, seed)
        u_o, _, steps_o, t_o = ora.pde_solver(name, u0, 10.0, [1.0] * len(shape), bt, cfl, N,
                                              stiff=stiff, flux=flux, max_steps=K)
        u, steps, t, _ = _run(step_lib, name, u0, N, bt, cfl, K, stiff, flux, strips=strips)
        assert steps == steps_o == K and t == t_o
        assert np.array_equal(u, u_o, equal_nan=True), (prob, np.abs(u - u_o).max())

    check()
