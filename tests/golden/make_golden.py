"""Generate the golden vectors of tests/golden from the reference itself.

Runs haranjackson/PyPDE's C++ core, compiled from its own sources by
`make -C oracle ref` (oracle/_ref/libref_driver.so, a C shim over the
reference's exported stages, with the C test callbacks of
oracle/oracle_systems.c), on seeded inputs and stores inputs and outputs as
.npz fixtures.  Needs the reference tree ($PYPDE_REFERENCE, by default a directory
`reference` beside this repository); the fixtures are self-contained.

    python tests/golden/make_golden.py

Fixtures:
  tables.npz        nodes, weights, DERVALS, ENDVALS for N = 1..6
  stages_*.npz      one seeded state through boundaries, WENO, CFL dt,
                    predictor (Picard) and FV update, per system/shape/order
  cfl_ncp_*.npz     CFL dt of the non-conservative system (F + B)
  run_*.npz         K full steps through the reference's pde_solver, with
                    the reference's own sensitivity to last-bit changes
                    (set by its finite-difference Jacobian): `band`, the
                    largest L1 change over 8 draws of a +-1 ulp perturbation
                    of the initial state (`band1`: the first draw alone),
                    and `band_dt`, the largest over 8 draws of a +-1 ulp
                    change of every step's dt
  stiff_*.npz       the stiff predictor of the tolerance-tightened
                    reference build (Newton-Krylov to 1e-12)
  tightrun_*.npz    K full steps of the stiff relaxation workload through
                    that build's pde_solver
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), "..", ".."))
sys.path.insert(0, ROOT)

from oracle import ora  # noqa: E402
from pypde_gb300 import workloads  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
D = ctypes.c_double


def l1(a, b):
    ax = tuple(range(a.ndim - 1))
    return np.abs(a - b).sum(axis=ax) / np.abs(b).sum(axis=ax)


def ref_tables():
    R = ora.ref()
    out = {}
    for N in range(1, 7):
        x, w, dv, ev = np.zeros(N), np.zeros(N), np.zeros(N * N), np.zeros(2 * N)
        R.ref_tables(N, ora.ptr(x), ora.ptr(w), ora.ptr(dv), ora.ptr(ev))
        out.update({f"nodes{N}": x, f"wghts{N}": w, f"dervals{N}": dv, f"endvals{N}": ev})
    np.savez_compressed(os.path.join(OUT, "tables.npz"), **out)


def ref_stages(system, shape, N, bt, seed, full=True):
    """full=False stops after WENO: the reference's 3-D derivs/endpts index
    node blocks with zero_index (src/poly/evaluations.cpp:4-21), which for
    ndim=3, d=1 returns i0*N^3+i1 instead of i0*N^2+i1 and reads and writes
    past the block (AddressSanitizer: heap-buffer-overflow in derivs,
    evaluations.cpp:42), so its 3-D CFL, predictor and FV are undefined."""
    R = ora.ref()
    u = workloads.random_state(system, shape, seed)
    ndim = len(shape)
    V = u.shape[-1]
    if system == "cattaneo":  # non-stiff tau: the Picard predictor converges
        u[..., 2 * ndim + 2] = np.random.default_rng(seed).uniform(-1, 0, shape)
    nX = np.array(shape, dtype=np.int32)
    dX = np.array([1.0 / n for n in shape])
    bta = np.array(bt, dtype=np.int32)
    ub = np.zeros(tuple(nX + 2 * N) + (V,))
    R.ref_boundaries(ora.ptr(u), ora.ptr(nX), ndim, ora.ptr(bta), N, V, ora.ptr(ub))
    nXb = (nX + 2 * N).astype(np.int32)
    nw = int(np.prod(nX + 2))
    Nd = N ** ndim
    w = np.zeros((nw * Nd, V))
    R.ref_weno(ora.ptr(ub), ora.ptr(nXb), ndim, N, V, ora.ptr(w))
    tag = f"stages_{system}_{'x'.join(map(str, shape))}_N{N}"
    if not full:
        np.savez_compressed(os.path.join(OUT, tag + ".npz"), u=u, bt=bta, N=N, dX=dX, ub=ub, w=w)
        return tag
    sysb = system.encode()
    dt3 = R.ref_timestep(sysb, ora.ptr(w), nw * Nd, ora.ptr(dX), ndim, N, 0.9, 1.0, 0.0, 3)
    dt = R.ref_timestep(sysb, ora.ptr(w), nw * Nd, ora.ptr(dX), ndim, N, 0.9, 1.0, 0.0, 7)
    qh = np.zeros((nw * Nd * N, V))
    R.ref_predictor(sysb, ora.ptr(w), nw * Nd, ora.ptr(dX), ndim, N, 0, dt, ora.ptr(qh))
    u1 = u.copy()
    R.ref_fv(sysb, ora.ptr(u1), ora.ptr(qh), ora.ptr(nX), ora.ptr(dX), ndim, N, 0, dt)
    np.savez_compressed(os.path.join(OUT, tag + ".npz"), u=u, bt=bta, N=N, dX=dX, ub=ub, w=w,
                        dt_count3=dt3, dt=dt, qh=qh, u_fv=u1)
    return tag


def ref_cfl_ncp(shape, N, seed):
    R = ora.ref()
    ndim = len(shape)
    nw = int(np.prod(np.array(shape) + 2))
    rng = np.random.default_rng(seed)
    w = 0.5 + 0.3 * rng.standard_normal((nw * N ** ndim, 3))
    dX = np.array([1.0 / n for n in shape])
    dt = R.ref_timestep(b"ncp", ora.ptr(w), w.shape[0], ora.ptr(dX), ndim, N, 0.9, 1.0, 0.0, 7)
    tag = f"cfl_ncp_{'x'.join(map(str, shape))}_N{N}"
    np.savez_compressed(os.path.join(OUT, tag + ".npz"), w=w, dX=dX, N=N, dt=dt)
    return tag


def ref_stage_loop(system, u0, N, bt, cfl, K, tf, L=1.0, dt_sign=None):
    """K steps of the reference's step loop (iterator.cpp:99-132, one slab)
    made of its exported stages: boundaries, WENO, CFL dt, predictor, FV.
    dt_sign (K signs or None): each step's dt, but the last, is moved by
    one ulp up or down, as a timestep whose max|eig| differs from Eigen's
    in the last bit would move it."""
    R = ora.ref()
    sysb = system.encode()
    nX = np.array(u0.shape[:-1], dtype=np.int32)
    ndim = len(nX)
    V = u0.shape[-1]
    dX = np.array([L / n for n in nX])
    bta = np.array(bt, dtype=np.int32)
    nXb = (nX + 2 * N).astype(np.int32)
    nw, Nd = int(np.prod(nX + 2)), N ** ndim
    u = u0.copy()
    t, count = 0.0, 0
    while t < tf and count < K:
        ub = np.zeros(tuple(nXb) + (V,))
        R.ref_boundaries(ora.ptr(u), ora.ptr(nX), ndim, ora.ptr(bta), N, V, ora.ptr(ub))
        w = np.zeros((nw * Nd, V))
        R.ref_weno(ora.ptr(ub), ora.ptr(nXb), ndim, N, V, ora.ptr(w))
        dt = R.ref_timestep(sysb, ora.ptr(w), nw * Nd, ora.ptr(dX), ndim, N, cfl, tf, t, count)
        if dt_sign is not None and t + dt < tf:
            dt = float(np.nextafter(dt, np.inf if dt_sign[count] > 0 else -np.inf))
        qh = np.zeros((nw * Nd * N, V))
        R.ref_predictor(sysb, ora.ptr(w), nw * Nd, ora.ptr(dX), ndim, N, 0, dt, ora.ptr(qh))
        R.ref_fv(sysb, ora.ptr(u), ora.ptr(qh), ora.ptr(nX), ora.ptr(dX), ndim, N, 0, dt)
        t += dt
        count += 1
    return u


def ref_run(tag, system, u0, N, bt, cfl, K, L=1.0, stiff=False, tight=False, draws=8):
    """K steps of the reference's pde_solver (tf = t_K of its own loop), with
    the reference's own sensitivity to last-bit differences:
      band1    L1 change when the initial state is perturbed by +-1 ulp
               (one seeded draw);
      band     the largest such change over `draws` seeded draws;
      band_dt  the largest L1 change over `draws` seeded draws when every
               step's dt is moved by +-1 ulp (ref_stage_loop), the effect
               of an eigenvalue solver that rounds differently from Eigen's.
    """
    R = ora.ref(tight)
    nX = np.array(u0.shape[:-1], dtype=np.int32)
    ndim = len(nX)
    dX = np.array([L / n for n in nX])
    bta = np.array(bt, dtype=np.int32)
    times = np.zeros(K)
    R.ref_step_times(system.encode(), ora.ptr(u0), ora.ptr(nX), ndim, ora.ptr(dX), cfl,
                     ora.ptr(bta), int(stiff), 0, N, 1e9, K, ora.ptr(times))
    tf = float(times[-1])

    def run(u_init):
        u = u_init.copy()
        ret = np.zeros((1,) + u.shape)
        R.ref_pde_solver(system.encode(), ora.ptr(u), tf, ora.ptr(nX), ndim, ora.ptr(dX), cfl,
                         ora.ptr(bta), int(stiff), 0, N, 1, ora.ptr(ret), 1)
        return u

    uK = run(u0)
    bands = []
    for k in range(draws):
        rng = np.random.default_rng(12345 + k)
        pert = u0 + np.spacing(u0) * rng.choice([-1.0, 0.0, 1.0], size=u0.shape)
        bands.append(l1(run(pert), uK))
    band_dt = None
    if not stiff:
        # the stage loop is the reference's pde_solver, bit for bit
        assert np.array_equal(ref_stage_loop(system, u0, N, bt, cfl, K, tf, L), uK)
        bdt = []
        for k in range(draws):
            sign = np.random.default_rng(777 + k).choice([-1, 1], size=K)
            bdt.append(l1(ref_stage_loop(system, u0, N, bt, cfl, K, tf, L, sign), uK))
        band_dt = np.max(bdt, axis=0)
    extra = {} if band_dt is None else {"band_dt": band_dt}
    np.savez_compressed(os.path.join(OUT, tag + ".npz"), u0=u0, uK=uK, tf=tf, times=times, K=K,
                        N=N, bt=bta, cfl=cfl, L=L, band1=bands[0], band=np.max(bands, axis=0),
                        system=system, stiff=stiff, **extra)
    print(tag, "band1", bands[0], "band", np.max(bands, axis=0), "band_dt", band_dt)
    return tag


def ref_stiff_run(n, K, cfl=0.8, seed=0):
    """K steps of the stiff relaxation workload (2-D Euler + relaxing heat
    flux, 16x16 tau patches with log10 tau ~ U(-7, -2), periodic, N=2)
    through the tolerance-tightened reference's pde_solver (Newton-Krylov
    to 1e-12, the tolerance of the GPU forms).  The initial state is
    workloads.relaxation(n, 2, seed); its SHA-256 is stored so that a test
    can tell if that generator has changed."""
    import hashlib
    R = ora.ref(True)
    u0 = workloads.relaxation(n, 2, seed=seed)
    nX = np.array(u0.shape[:-1], dtype=np.int32)
    dX = np.array([1.0 / n] * 2)
    bta = np.array([1, 1], dtype=np.int32)
    times = np.zeros(K)
    R.ref_step_times(b"cattaneo", ora.ptr(u0), ora.ptr(nX), 2, ora.ptr(dX), cfl, ora.ptr(bta), 1,
                     0, 2, 1e9, K, ora.ptr(times))
    tf = float(times[-1])
    u = u0.copy()
    ret = np.zeros((1,) + u.shape)
    R.ref_pde_solver(b"cattaneo", ora.ptr(u), tf, ora.ptr(nX), 2, ora.ptr(dX), cfl, ora.ptr(bta),
                     1, 0, 2, 1, ora.ptr(ret), 1)
    tag = f"tightrun_stiff{n}_N2_K{K}"
    np.savez_compressed(os.path.join(OUT, tag + ".npz"), uK=u, tf=tf, times=times, K=K, N=2,
                        n=n, seed=seed, cfl=cfl,
                        u0_sha256=hashlib.sha256(u0.tobytes()).hexdigest())
    return tag


def ref_stiff_predictor(shape, N, seed, dt):
    R = ora.ref(tight=True)
    ndim = len(shape)
    nw = int(np.prod(np.array(shape)))
    u = workloads.random_state("cattaneo", shape, seed).reshape(nw, -1)
    # one node value per cell and node: smooth cell states repeated per node
    Nd = N ** ndim
    rng = np.random.default_rng(seed + 1)
    w = np.repeat(u, Nd, axis=0) * (1 + 1e-3 * rng.standard_normal((nw * Nd, u.shape[-1])))
    w[:, 2 * ndim + 2] = np.repeat(u[:, 2 * ndim + 2], Nd)
    dX = np.array([1.0 / n for n in shape])
    qh = np.zeros((nw * Nd * N, w.shape[-1]))
    R.ref_predictor(b"cattaneo", ora.ptr(w), w.shape[0], ora.ptr(dX), ndim, N, 1, dt,
                    ora.ptr(qh))
    tag = f"stiff_cattaneo_{'x'.join(map(str, shape))}_N{N}"
    np.savez_compressed(os.path.join(OUT, tag + ".npz"), w=w, dX=dX, N=N, dt=dt, qh=qh)
    return tag


def ref_flux_points():
    """D(qL,qR) + F(qL) + F(qR) and the B path integral at single face
    points through the reference's FluxGenerator (fluxes.cpp:80-117), for
    Rusanov (0), Roe (1) and Osher (2)."""
    R = ora.ref()
    R.ref_flux.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int] + [ora.dp] * 4 + \
        [ctypes.c_int, ctypes.c_int, ora.dp, ora.dp]
    out = {}
    for name, ndim, N in (("euler", 1, 2), ("euler", 2, 3), ("ncp", 2, 2), ("cattaneo", 2, 2),
                          ("cattaneo", 3, 2)):
        u = workloads.random_state(name, (6,) * ndim, 11).reshape(-1, workloads.random_state(
            name, (1,) * ndim, 0).shape[-1])
        if name == "cattaneo":
            u[:, -1] = -3.0
        V = u.shape[1]
        qL, qR = u[:-1].copy(), u[1:].copy()
        for flux in (0, 1, 2):
            f = np.zeros_like(qL)
            b = np.zeros_like(qL)
            for i in range(len(qL)):
                dq = np.zeros(ndim * V)
                fi, bi = np.zeros(V), np.zeros(V)
                R.ref_flux(name.encode(), ndim, N, ora.ptr(qL[i].copy()), ora.ptr(qR[i].copy()),
                           ora.ptr(dq), ora.ptr(dq.copy()), i % ndim, flux, ora.ptr(fi),
                           ora.ptr(bi))
                f[i], b[i] = fi, bi
            out[f"{name}{ndim}_N{N}_flux{flux}_f"] = f
            out[f"{name}{ndim}_N{N}_flux{flux}_b"] = b
        out[f"{name}{ndim}_N{N}_qL"] = qL
        out[f"{name}{ndim}_N{N}_qR"] = qR
    np.savez_compressed(os.path.join(OUT, "flux_points.npz"), **out)


def main():
    if "--runs" in sys.argv:  # only the full-run fixtures
        return main_runs()
    if "--stiff-run" in sys.argv:  # only the stiff run (about 5 minutes)
        return print(ref_stiff_run(128, 10))
    ref_tables()
    ref_flux_points()
    for system, shape, N, bt in [("euler", (40,), 2, [0]), ("euler", (40,), 3, [1]),
                                 ("euler", (12, 10), 2, [1, 0]), ("euler", (12, 10), 3, [1, 1]),
                                 ("cattaneo", (10, 8), 2, [1, 1])]:
        print(ref_stages(system, shape, N, bt, seed=1))
    print(ref_stages("euler", (6, 5, 4), 2, [1, 0, 1], seed=1, full=False))
    print(ref_stages("euler", (5, 6, 7), 3, [0, 1, 1], seed=2, full=False))
    print(ref_cfl_ncp((16,), 3, 2), ref_cfl_ncp((9, 8), 2, 3))
    main_runs()
    print(ref_stiff_run(128, 10))
    print(ref_stiff_predictor((6, 5), 2, 7, 2e-3))
    print(ref_stiff_predictor((6, 5), 1, 7, 2e-3))
    print(ref_stiff_predictor((5, 4), 3, 8, 2e-3))


def main_runs():
    ref_run("run_sod400_N2_K10", "euler", workloads.sod(400), 2, [0], 0.9, 10)
    ref_run("run_sod400_N2_K199", "euler", workloads.sod(400), 2, [0], 0.9, 199)
    ref_run("run_shear32_N3_K10", "euler", workloads.shear(32), 3, [1, 1], 0.8, 10)
    ref_run("run_shear16_N2_K10", "euler", workloads.shear(16), 2, [1, 0], 0.8, 10)


if __name__ == "__main__":
    main()
