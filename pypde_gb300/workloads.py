"""Seeded synthetic initial states of the benchmark workloads.

The reference publishes no benchmark suite; these are the workloads its
headline metric is defined on, generated from numpy default_rng(seed):

  sod(n)          1-D Euler (rho, rho u, E), gamma 1.4, Sod data
                  (rho, u, p) = (1, 0, 1) for x < 0.5 else (0.125, 0, 0.1),
                  plus 1e-3 U(-1, 1) on rho.  Transmissive, N=2, CFL 0.9.
  shear(n)        2-D Euler on [0,1]^2 periodic: s = tanh((|y-0.5|-0.25)/0.01),
                  u = 0.5 s, rho = 1 + 0.5 s, p = 2.5, and
                  v = sum_{k=1..8} a_k sin(2 pi k x + phi_k), a_k ~ N(0, 1e-2),
                  phi_k ~ U(0, 2 pi).  N=3, CFL 0.8.
  relaxation(n, ndim)
                  Euler + Cattaneo heat flux + passive log10(tau) (the
                  "cattaneo" system): rho = 1 + 0.1 * (sum of 6 seeded Fourier
                  modes, 12 in 3-D), u = 0, p = 1, q = 0; log10(tau) constant
                  on a 16x16 patch layout (per octant in 3-D) drawn from
                  U(lo, hi).  Periodic, N=2.
"""
import numpy as np

GAMMA = 1.4


def _energy(rho, p, vel2):
    return p / (GAMMA - 1.0) + 0.5 * rho * vel2


def sod(n=400, seed=0):
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    rho = np.where(x < 0.5, 1.0, 0.125) + 1e-3 * rng.uniform(-1, 1, n)
    p = np.where(x < 0.5, 1.0, 0.1)
    u = np.zeros((n, 3))
    u[:, 0] = rho
    u[:, 2] = _energy(rho, p, 0.0)
    return u


def shear(n=512, seed=0):
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    X, Y = np.meshgrid(x, x, indexing="ij")
    s = np.tanh((np.abs(Y - 0.5) - 0.25) / 0.01)
    ux = 0.5 * s
    rho = 1 + 0.5 * s
    a = rng.normal(0, 1e-2, 8)
    ph = rng.uniform(0, 2 * np.pi, 8)
    uy = sum(a[k] * np.sin(2 * np.pi * (k + 1) * X + ph[k]) for k in range(8))
    u = np.zeros((n, n, 4))
    u[..., 0] = rho
    u[..., 1] = rho * ux
    u[..., 2] = rho * uy
    u[..., 3] = _energy(rho, 2.5, ux ** 2 + uy ** 2)
    return u


def relaxation(n=1024, ndim=2, seed=0, log10_tau=(-7.0, -2.0), patches=16, amp=0.1):
    rng = np.random.default_rng(seed)
    x = (np.arange(n) + 0.5) / n
    grids = np.meshgrid(*([x] * ndim), indexing="ij")
    nmodes = 6 if ndim == 2 else 12
    pert = np.zeros((n,) * ndim)
    for _ in range(nmodes):
        k = rng.integers(1, 5, ndim)
        a_k = rng.uniform(-1, 1) / np.sqrt(nmodes)
        ph = rng.uniform(0, 2 * np.pi)
        pert += a_k * np.sin(2 * np.pi * sum(k[i] * grids[i] for i in range(ndim)) + ph)
    rho = 1 + amp * pert
    V = 2 * ndim + 3
    u = np.zeros((n,) * ndim + (V,))
    u[..., 0] = rho
    u[..., ndim + 1] = _energy(rho, 1.0, 0.0)
    npatch = patches if ndim == 2 else 2
    taus = rng.uniform(log10_tau[0], log10_tau[1], (npatch,) * ndim)
    idx = [np.minimum((g * npatch).astype(int), npatch - 1) for g in grids]
    u[..., 2 * ndim + 2] = taus[tuple(idx)]
    return u


def random_state(system, shape, seed=0):
    """Smooth-plus-noise states for the unit tests of each stage."""
    rng = np.random.default_rng(seed)
    ndim = len(shape)
    if system in ("euler", "cattaneo"):
        V = ndim + 2 if system == "euler" else 2 * ndim + 3
        u = np.zeros(tuple(shape) + (V,))
        u[..., 0] = 1 + 0.2 * rng.random(shape)
        for i in range(ndim):
            u[..., 1 + i] = 0.3 * rng.standard_normal(shape)
        ke = sum(u[..., 1 + i] ** 2 for i in range(ndim))
        u[..., ndim + 1] = 2.5 * (1 + 0.3 * rng.random(shape)) + 0.5 * ke / u[..., 0]
        if system == "cattaneo":
            u[..., ndim + 2:2 * ndim + 2] = 0.01 * rng.standard_normal(tuple(shape) + (ndim,))
            u[..., 2 * ndim + 2] = rng.uniform(-4, -2, shape)
        return u
    if system == "ncp":
        return 0.5 + 0.3 * rng.standard_normal(tuple(shape) + (3,))
    if system == "burgers2":
        return 0.5 + 0.3 * rng.standard_normal(tuple(shape) + (1,))
    raise ValueError(system)


def batched(nprob=256, seed=0, side=(64, 512), orders=(1, 2, 3), log10_tau=(-6.0, -2.0),
            tf=0.1, cfl=0.8):
    """Uneven batch of 2-D Euler + relaxing heat flux problems (7 vars):
    side floor(64 8^U) (log-uniform in [64, 512]), order N from `orders`,
    one log10 tau ~ U(-6, -2) per problem, rho = 1 + 0.1 f, p = 1 + 0.1 g
    with f, g sums of 4 seeded Fourier modes, zero velocity and heat flux,
    periodic, each to its own tf.  Returns pde_solver_batch problem dicts."""
    rng = np.random.default_rng(seed)
    lo, hi = side
    out = []
    for _ in range(nprob):
        n = int(lo * (hi / lo) ** rng.uniform())
        N = int(rng.choice(orders))
        x = (np.arange(n) + 0.5) / n
        X, Y = np.meshgrid(x, x, indexing="ij")
        f = np.zeros((n, n))
        g = np.zeros((n, n))
        for acc in (f, g):
            for _ in range(4):
                kx, ky = rng.integers(1, 5, 2)
                acc += rng.uniform(-0.5, 0.5) * np.sin(2 * np.pi * (kx * X + ky * Y)
                                                        + rng.uniform(0, 2 * np.pi))
        rho = 1 + 0.1 * f
        p = 1 + 0.1 * g
        u = np.zeros((n, n, 7))
        u[..., 0] = rho
        u[..., 3] = _energy(rho, p, 0.0)
        u[..., 6] = rng.uniform(*log10_tau)
        out.append({"Q0": u, "tf": tf, "L": [1.0, 1.0], "order": N,
                    "boundaryTypes": "periodic", "cfl": cfl})
    return out
