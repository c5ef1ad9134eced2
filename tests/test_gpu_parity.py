"""GPU kernels against the CPU restatement (oracle/) and the reference's
golden vectors, through the C ABI.

The plain FP64 form is built to be bit-identical to the restatement: same
algorithms, same summation orders, the same explicit fma() calls and no
implicit contraction on either side.  So every
stage is compared for exact equality, and full runs must agree to well
inside the 1e-10 relative L1 bar (they are expected to agree exactly),
including the benchmark's own workloads at full size.
"""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN, l1, load
from oracle import ora
from pypde_gb300 import stages, systems, workloads
from pypde_gb300.solvers import pde_solver

pytestmark = pytest.mark.gpu

CASES = [("euler", (40,), 2, [0]), ("euler", (40,), 3, [1]), ("euler", (17,), 1, [1]),
         ("euler", (12, 10), 2, [1, 0]), ("euler", (12, 10), 3, [1, 1]),
         ("euler", (5, 6, 4), 2, [1, 0, 1]), ("euler", (4, 3, 5), 3, [0, 1, 1]),
         ("cattaneo", (10, 8), 2, [1, 1]), ("ncp", (16,), 3, [0]), ("ncp", (9, 8), 2, [1, 0]),
         ("burgers2", (24,), 2, [1]), ("euler", (1,), 2, [0]), ("euler", (2, 1), 2, [1, 0]),
         ("euler", (2, 3), 2, [1, 1])]


def _ids(c):
    return f"{c[0]}-{'x'.join(map(str, c[1]))}-N{c[2]}"


def _state(system, shape, seed=1):
    u = workloads.random_state(system, shape, seed)
    if system == "cattaneo":
        u[..., -1] = np.random.default_rng(seed).uniform(-1, 0, shape)
    return u


@pytest.mark.parametrize("case", CASES, ids=_ids)
def test_stages_bitwise(gpu_lib, case):
    system, shape, N, bt = case
    u = _state(system, shape)
    dX = [1.0 / n for n in shape]
    ub_o = ora.boundaries(u, N, bt)
    ub_g = stages.boundaries(u, N, bt)
    assert np.array_equal(ub_g, ub_o)
    w_o = ora.weno(ub_o, N)
    w_g = stages.weno(ub_o, N)
    assert np.array_equal(w_g, w_o)
    for count in (0, 9):
        dt_o = ora.timestep(system, w_o, dX, N, 0.9, 1.0, 0.0, count)
        dt_g = stages.timestep(system, w_o, dX, N, 0.9, 1.0, 0.0, count)
        assert dt_g == dt_o
    qh_o, its_o, mx_o = ora.predictor(system, w_o, dX, N, False, dt_o)
    qh_g, st = stages.predictor(system, w_o, dX, N, False, dt_o)
    assert np.array_equal(qh_g, qh_o)
    assert st["pred_iters"] == its_o and st["pred_max_iters"] == mx_o
    u_o = ora.fv(system, u, qh_o, dX, N, dt_o)
    u_g = stages.fv(system, u, qh_o, dX, N, dt_o)
    assert np.array_equal(u_g, u_o)


def test_periodic_axis_shorter_than_order_is_rejected(gpu_lib):
    """The periodic ghost fill wraps once (boundaries.cpp:7-23): an axis
    with fewer than N cells cannot be padded and is refused before any
    device work."""
    from pypde_gb300 import _lib
    with pytest.raises(_lib.PyPDEError) as e:
        stages.boundaries(np.ones((1, 4)), 2, [1])
    assert e.value.code == _lib.PYPDE_ERR_ARG
    s = systems.euler(1)
    with pytest.raises(_lib.PyPDEError):
        pde_solver(np.ones((2, 3)), 0.1, [1.0], F=s.F, boundaryTypes="periodic", order=3,
                   stiff=False)


def test_dt_clipped_to_tf(gpu_lib):
    u = _state("euler", (12, 10))
    w = ora.weno(ora.boundaries(u, 2, [1, 1]), 2)
    dt_full = stages.timestep("euler", w, [0.1, 0.1], 2, 0.9, 1.0, 0.0, 9)
    t = 1.0 - 0.25 * dt_full
    assert stages.timestep("euler", w, [0.1, 0.1], 2, 0.9, 1.0, t, 9) == 1.0 - t


@pytest.mark.parametrize("fixture", sorted(os.path.basename(f) for f in
                                           glob.glob(os.path.join(GOLDEN, "stages_*.npz"))))
def test_weno_against_reference_golden(gpu_lib, fixture):
    z = load(fixture)
    w = stages.weno(z["ub"], int(z["N"]))
    assert np.abs(w - z["w"]).max() <= 1e-10 * np.abs(z["w"]).max()
    assert np.array_equal(stages.boundaries(z["u"], int(z["N"]), z["bt"]).ravel(),
                          z["ub"].ravel())


RUNS = [("euler", workloads.sod(400), 2, [0], 0.9, 30, "sod400"),
        ("euler", workloads.shear(32), 3, [1, 1], 0.8, 10, "shear32"),
        ("euler", workloads.shear(16), 2, [1, 0], 0.8, 10, "shear16"),
        ("ncp", workloads.random_state("ncp", (12, 10), 4), 2, [1, 1], 0.5, 6, "ncp12x10"),
        ("burgers2", workloads.random_state("burgers2", (32,), 5), 3, [1], 0.5, 6, "burgers32"),
        ("euler", workloads.random_state("euler", (6, 5, 7), 6), 2, [1, 1, 0], 0.5, 4, "euler3d")]


@pytest.mark.parametrize("run", RUNS, ids=[r[-1] for r in RUNS])
def test_full_run_matches_port(gpu_lib, run):
    system, u0, N, bt, cfl, K, _ = run
    ndim = u0.ndim - 1
    L = [1.0] * ndim
    u_o, ret_o, steps_o, t_o = ora.pde_solver(system, u0, 10.0, L, bt, cfl, N, ndt=4,
                                              max_steps=K)
    sysobj = {"euler": systems.euler, "ncp": systems.ncp}.get(system)
    s = sysobj(ndim) if sysobj else systems.burgers2()
    q = u0.copy()
    st = {}
    ret = pde_solver(q, 10.0, L, F=s.F, B=s.B, S=s.S,
                     boundaryTypes=[("transitive", "periodic")[b] for b in bt], cfl=cfl,
                     order=N, ndt=4, stiff=False, max_steps=K, stats=st)
    assert st["steps"] == steps_o == K
    assert st["t_final"] == t_o
    err = l1(q, u_o)
    assert np.all(err <= 1e-10), err
    assert np.array_equal(q, u_o)               # expected bit-identical
    assert np.array_equal(ret[-1], q)


@pytest.mark.parametrize("fixture", sorted(os.path.basename(f) for f in
                                           glob.glob(os.path.join(GOLDEN, "run_*.npz"))))
def test_full_run_within_reference_band(gpu_lib, fixture):
    z = load(fixture)
    ndim = z["u0"].ndim - 1
    s = systems.euler(ndim)
    q = z["u0"].copy()
    st = {}
    bt = [("transitive", "periodic")[b] for b in z["bt"]]
    pde_solver(q, float(z["tf"]), [float(z["L"])] * ndim, F=s.F, boundaryTypes=bt,
               cfl=float(z["cfl"]), order=int(z["N"]), ndt=1, stiff=False,
               max_steps=int(z["K"]), stats=st)
    assert st["steps"] == int(z["K"])
    err = l1(q, z["uK"])
    # within twice the reference's own spread under +-1 ulp changes of its input
    assert np.all(err <= np.maximum(2 * z["band"], 1e-13)), (err, z["band"])


def test_snapshots_follow_reference_rule(gpu_lib):
    """ret[k] is the state when t first reaches (k+1) tf / ndt
    (iterator.cpp:136-139); ret[ndt-1] the final state."""
    u0 = workloads.sod(200)
    s = systems.euler(1)
    tf, ndt = 0.05, 5
    u_o, ret_o, steps, t = ora.pde_solver("euler", u0, tf, [1.0], [0], 0.9, 2, ndt=ndt)
    q = u0.copy()
    ret = pde_solver(q, tf, [1.0], F=s.F, cfl=0.9, order=2, ndt=ndt, stiff=False)
    assert np.array_equal(ret, ret_o)
    assert np.array_equal(q, u_o)
    assert abs(t - tf) <= 1e-15


def test_in_place_final_state(gpu_lib):
    u0 = workloads.sod(64)
    q = u0.copy()
    s = systems.euler(1)
    ret = pde_solver(q, 0.01, [1.0], F=s.F, order=2, ndt=2, stiff=False)
    assert not np.array_equal(q, u0)
    assert np.array_equal(q, ret[-1])


def test_nan_stops_with_reference_rows(gpu_lib):
    u0 = workloads.sod(32)
    u0[5, 0] = np.nan
    q = u0.copy()
    s = systems.euler(1)
    st = {}
    ret = pde_solver(q, 0.05, [1.0], F=s.F, order=2, ndt=3, stiff=False, stats=st)
    assert st["nan_found"] == 1
    assert np.isnan(ret[-1]).any()


def test_weno_solver_api_shape(gpu_lib):
    from pypde_gb300 import weno_solver
    u = workloads.random_state("euler", (9, 8))
    r = weno_solver(u, order=3)
    assert r.shape == (5, 4, 3, 3, 4)
    assert np.array_equal(r.reshape(-1, 4), ora.weno(u, 3))


STIFF_CASES = [("cattaneo", (10, 8), 2), ("cattaneo", (6, 5, 4), 2), ("cattaneo", (9, 7), 3),
               ("ncp", (12,), 2), ("euler", (8, 6), 2)]


@pytest.mark.parametrize("case", STIFF_CASES, ids=[f"{c[0]}-{len(c[1])}d-N{c[2]}"
                                                   for c in STIFF_CASES])
def test_newton_predictor_bitwise(gpu_lib, case):
    """The locally implicit Newton predictor equals the restatement's bit for
    bit, iteration counts included; stiff relaxation times 1e-4..1e-2."""
    system, shape, N = case
    u = workloads.random_state(system, shape, 2)
    dX = [1.0 / n for n in shape]
    bt = [1] * len(shape)
    w = ora.weno(ora.boundaries(u, N, bt), N)
    dt = ora.timestep(system, w, dX, N, 0.9, 1.0, 0.0, 9)
    qh_o, its_o, mx_o = ora.predictor(system, w, dX, N, True, dt, 1e-12)
    qh_g, st = stages.predictor(system, w, dX, N, True, dt, 1e-12)
    assert np.array_equal(qh_g, qh_o)
    assert st["pred_iters"] == its_o and st["pred_max_iters"] == mx_o
    assert st["pred_fail"] == 0


def test_newton_against_tight_reference(gpu_lib):
    """Same fixed point as the reference's Newton-Krylov predictor built with
    DG_TOL = 1e-12 (tests/golden/make_golden.py)."""
    z = load("stiff_cattaneo_6x5_N2.npz")
    qh, st = stages.predictor("cattaneo", z["w"], z["dX"], int(z["N"]), True, float(z["dt"]),
                              1e-12)
    assert np.abs(qh - z["qh"]).max() <= 1e-10 * np.abs(z["qh"]).max()


def test_stiff_run_matches_port(gpu_lib):
    """The stiff relaxation workload (tau down to 1e-7, dt/tau >> 1): GPU and
    restatement bit-identical after K steps."""
    u0 = workloads.relaxation(24, 2, seed=3)
    s = systems.cattaneo(2)
    K = 4
    u_o, _, steps, t_o = ora.pde_solver("cattaneo", u0, 10.0, [1.0, 1.0], [1, 1], 0.8, 2,
                                        stiff=True, max_steps=K)
    q = u0.copy()
    st = {}
    pde_solver(q, 10.0, [1.0, 1.0], F=s.F, S=s.S, boundaryTypes="periodic", cfl=0.8, order=2,
               ndt=1, stiff=True, max_steps=K, stats=st)
    assert st["steps"] == steps == K and st["pred_fail"] == 0
    assert st["t_final"] == t_o
    assert np.array_equal(q, u_o)


EIG_FLUX_CASES = [("euler", (16,), 2), ("euler", (6, 5), 3), ("euler", (4, 3, 5), 2),
                  ("ncp", (7, 6), 2), ("cattaneo", (6, 5), 2)]


@pytest.mark.parametrize("flux", ["roe", "osher"])
@pytest.mark.parametrize("case", EIG_FLUX_CASES, ids=[f"{c[0]}-{len(c[1])}d-N{c[2]}"
                                                              for c in EIG_FLUX_CASES])
def test_roe_osher_faces_bitwise(gpu_lib, case, flux):
    """Roe and Osher face fluxes (full eigen-decomposition per face point,
    fluxes.cpp:20-70) equal the restatement's bit for bit."""
    system, shape, N = case
    u = _state(system, shape, 3)
    dX = [1.0 / n for n in shape]
    bt = [1] * len(shape)
    w = ora.weno(ora.boundaries(u, N, bt), N)
    dt = ora.timestep(system, w, dX, N, 0.5, 1.0, 0.0, 9)
    qh, _, _ = ora.predictor(system, w, dX, N, False, dt)
    fl = {"roe": 1, "osher": 2}[flux]
    u_o = ora.fv(system, u, qh, dX, N, dt, flux=fl)
    u_g = stages.fv(system, u, qh, dX, N, dt, flux=flux)
    assert np.array_equal(u_g, u_o)


@pytest.mark.parametrize("flux", ["roe", "osher"])
def test_roe_osher_full_run_matches_port(gpu_lib, flux):
    u0 = workloads.sod(120)
    s = systems.euler(1)
    fl = {"roe": 1, "osher": 2}[flux]
    u_o, _, steps, t_o = ora.pde_solver("euler", u0, 10.0, [1.0], [0], 0.9, 2, flux=fl,
                                        max_steps=8)
    q = u0.copy()
    st = {}
    pde_solver(q, 10.0, [1.0], F=s.F, cfl=0.9, order=2, ndt=1, flux=flux, stiff=False,
               max_steps=8, stats=st)
    assert st["steps"] == steps == 8
    assert np.array_equal(q, u_o)


def test_shear512_N3_full_size_matches_port():
    """The shear-layer workload at its benchmark size (512x512 periodic,
    N=3, CFL 0.8, Picard predictor), 10 steps: GPU and the CPU oracle
    (all host cores) bit-identical, t included."""
    u0 = workloads.shear(512)
    K = 10
    u_o, _, steps, t_o = ora.pde_solver("euler", u0, 10.0, [1.0, 1.0], [1, 1], 0.8, 3,
                                        max_steps=K, nthreads=os.cpu_count() or 1)
    s = systems.euler(2)
    q = u0.copy()
    st = {}
    pde_solver(q, 10.0, [1.0, 1.0], F=s.F, boundaryTypes="periodic", cfl=0.8, order=3, ndt=1,
               stiff=False, max_steps=K, stats=st)
    assert st["steps"] == steps == K and st["t_final"] == t_o
    assert np.array_equal(q, u_o)


def test_stiff128_matches_port_and_tight_reference():
    """The stiff relaxation workload at 128x128 (N=2, CFL 0.8, Newton to
    1e-12), 10 steps to the reference's own t_10: GPU and CPU oracle
    bit-identical, and both within 1e-8 relative L1 per variable of the
    tolerance-tightened reference (Newton-Krylov to 1e-12; two solvers
    stopped at one tolerance differ by its effect)."""
    from test_oracle_golden import _stiff128_u0
    z, u0 = _stiff128_u0()
    tf = float(z["tf"])
    u_o, _, steps, t_o = ora.pde_solver("cattaneo", u0, tf, [1.0, 1.0], [1, 1],
                                        float(z["cfl"]), 2, stiff=True,
                                        nthreads=os.cpu_count() or 1)
    s = systems.cattaneo(2)
    q = u0.copy()
    st = {}
    pde_solver(q, tf, [1.0, 1.0], F=s.F, S=s.S, boundaryTypes="periodic", cfl=float(z["cfl"]),
               order=2, ndt=1, stiff=True, stats=st)
    assert st["steps"] == steps == int(z["K"]) and st["t_final"] == t_o == tf
    assert st["pred_fail"] == 0
    assert np.array_equal(q, u_o)
    assert np.all(l1(q, z["uK"]) <= 1e-8), l1(q, z["uK"])


@pytest.mark.parametrize("case", [("cattaneo", (192, 160), 2, True, [0, 0]),
                                  ("euler", (24, 20, 16), 2, False, [1, 0, 1]),
                                  ("euler", (3000,), 3, False, [0])],
                         ids=["stiff-192x160-N2", "euler-3d-N2", "euler-1d-N3"])
def test_predictor_strips_equal_port(case):
    """The predictor in strips with the faces of finished strips on a second
    stream (the overlapped step the large workloads take by default): every
    strip count gives the restatement's state bit for bit."""
    name, shape, N, stiff, bt = case
    u0 = _state(name, shape, 3)
    if name == "cattaneo":
        u0 = workloads.relaxation(shape[0], 2, seed=3)[:, :shape[1]].copy()
    K = 4
    u_o, _, steps, t_o = ora.pde_solver(name, u0, 10.0, [1.0] * len(shape), bt, 0.8, N,
                                        stiff=stiff, max_steps=K, nthreads=os.cpu_count() or 1)
    s = getattr(systems, name)(len(shape))
    for strips in (1, 2, 8, 32, 0):
        q = u0.copy()
        st = {}
        pde_solver(q, 10.0, [1.0] * len(shape), F=s.F, S=s.S if stiff else None,
                   boundaryTypes=[["transitive", "periodic"][b] for b in bt],
                   cfl=0.8, order=N, ndt=1, stiff=stiff, max_steps=K, stats=st, strips=strips)
        assert st["steps"] == steps == K and st["t_final"] == t_o, strips
        assert np.array_equal(q, u_o), (strips, np.abs(q - u_o).max())
