"""pde_solver and weno_solver with the reference's Python API
(haranjackson/PyPDE pypde/solvers.py:13-244), run on the GPU.

Differences from the reference, all at the callback boundary:
  * F, B and S run on the GPU: the built-in systems of pypde_gb300.systems
    use kernels compiled ahead of time; other Python callbacks are
    translated to device code (pypde_gb300.translate) and compiled at run
    time with NVRTC (the reference compiles them with numba into host
    cfuncs, pypde/cfuncs.py:30-75).  jit=True forces the run-time path.
  * ``nThreads`` is accepted and ignored (one GPU does the work of the
    reference's CPU thread pool).
  * Extensions (keyword-only): ``max_steps``, ``newton_tol``, ``device``,
    ``stats`` (a dict filled with step and iteration counts), ``jit``,
    ``warm_start`` (a pypde_gb300.warmstart.WarmStart: learned initial guess
    of the stiff predictor's Newton iteration; one whose validation showed
    no saving, ``active`` False, leaves the plain guess), ``mixed_precision`` (Newton
    sweeps in FP32 first, then at least two FP64 sweeps to the same
    tolerance; built-in systems).
"""
import ctypes

import numpy as np

from . import _lib
from .callbacks import resolve_system
from .utils import nargs, parse_boundary_types

FLUXES = {"rusanov": 0, "roe": 1, "osher": 2}


def pde_solver(Q0, tf, L, F=None, B=None, S=None, boundaryTypes="transitive", cfl=0.9,
               order=2, ndt=100, flux="rusanov", stiff=True, nThreads=-1, *, M=None,
               max_steps=None, newton_tol=None, device=0, stats=None, jit=False,
               warm_start=None, mixed_precision=False, strips=0):
    """Solve dQ/dt + div F(Q, grad Q) + B(Q) . grad Q = S(Q) on [0, L] (see
    pypde/solvers.py:28-175 for the full description of the arguments).

    Returns an array of shape (ndt,) + Q0.shape: row k holds the state when t
    first reaches (k+1) tf / ndt, row ndt-1 the state at tf.  Like the
    reference, the final state is also written into Q0 when Q0 is a
    contiguous float64 array.

    strips: the predictor runs in this many strips of cells while the faces
    of finished strips run on a second CUDA stream (0: the library's choice,
    1: no overlap); the results do not depend on it.
    """
    if M is not None:
        # the reference's pde_solver (pypde/solvers.py:13-25) has no M
        raise NotImplementedError("M has no counterpart in the reference's pde_solver; "
                                  "only M=None is accepted")
    nX = np.array(Q0.shape[:-1], dtype="int32")
    ndim = len(nX)
    V = Q0.shape[-1]
    dX = np.array([L[i] / nX[i] for i in range(len(L))], dtype="float64")

    bt = parse_boundary_types(boundaryTypes, ndim)

    useF, useB, useS = F is not None, B is not None, S is not None
    secondOrder = useF and nargs(F) == 3
    system = resolve_system(F, B, S, ndim, V, secondOrder, jit=jit)

    ret = np.zeros(ndt * Q0.size)
    ur = Q0.ravel()
    if ur.dtype != np.float64:
        print("invalid array type")
        raise TypeError("Q0 must be a float64 array")

    opt = _lib.Options()
    opt.max_steps = int(max_steps) if max_steps else -1
    opt.newton_tol = float(newton_tol) if newton_tol else 0.0
    opt.device = int(device)
    if warm_start is not None:
        if not stiff:
            raise ValueError("warm_start applies to the stiff (Newton) predictor")
        if getattr(warm_start, "active", True):  # validated to save iterations
            opt.warm_start = warm_start.handle
    opt.mixed_precision = int(bool(mixed_precision))
    opt.strips = int(strips)
    st = _lib.Stats()
    lib = _lib.lib()
    code = lib.pde_solver_ex(system.handle, useF, useB, useS, _lib.c_ptr(ur), float(tf),
                             _lib.c_ptr(nX), ndim, _lib.c_ptr(dX), float(cfl), _lib.c_ptr(bt),
                             bool(stiff), FLUXES[flux], int(order), int(ndt), _lib.c_ptr(ret),
                             opt, st)
    _lib.check(code)
    if code == _lib.PYPDE_NAN_FOUND:
        print("NaNs found")
    if stats is not None:
        stats.update(st.as_dict())
    return ret.reshape((ndt,) + Q0.shape)


# Another name for pde_solver (same function, same arguments, M=None).
ader_solver = pde_solver


def pde_solver_batch(problems, F=None, B=None, S=None, stiff=True, flux="rusanov", *,
                     max_steps=None, newton_tol=None, device=0, autotune=True, per_pop=1,
                     stats=None, jit=False, warm_start=None, mixed_precision=False):
    """Step many independent problems of one system together (one persistent
    launch per stage and order, see include/pypde_gb300.h).

    problems: a list of dicts with keys Q0 (float64 array (n_1..n_d, V),
    overwritten with the final state, like pde_solver), tf, L, and optional
    order (2), boundaryTypes ('transitive'), cfl (0.9).  All problems share
    F, B, S; sizes, orders, boundary types and end times may differ.
    Returns the list of final states (the Q0 arrays).  stats (a dict) gets
    the batch statistics plus per-problem 'steps' and 't_final' lists.
    warm_start: a WarmStart, or a dict {order: WarmStart}, the learned warm
    start of the stiff predictor for the problems of that order (one whose
    validation found no saving, ``active`` False, is not used);
    mixed_precision: FP32 Newton sweeps first (built-in systems).  Each
    problem gives the bits pde_solver gives it alone with the same
    options."""
    if not problems:
        raise ValueError("no problems")
    Q0s = [p["Q0"] for p in problems]
    ndim = Q0s[0].ndim - 1
    V = Q0s[0].shape[-1]
    for q in Q0s:
        if q.dtype != np.float64 or not q.flags.c_contiguous:
            raise TypeError("Q0 must be a C-contiguous float64 array")
        if q.ndim - 1 != ndim or q.shape[-1] != V:
            raise ValueError("all problems need the same ndim and V")
    secondOrder = F is not None and nargs(F) == 3
    system = resolve_system(F, B, S, ndim, V, secondOrder, jit=jit)
    arr = (_lib.BatchProblem * len(problems))()
    for i, p in enumerate(problems):
        q = Q0s[i]
        nX = q.shape[:-1]
        L = p["L"]
        bt = parse_boundary_types(p.get("boundaryTypes", "transitive"), ndim)
        arr[i].u = _lib.c_ptr(q.reshape(-1))
        arr[i].tf = float(p["tf"])
        arr[i].N = int(p.get("order", 2))
        arr[i].cfl = float(p.get("cfl", 0.9))
        for d in range(ndim):
            arr[i].nX[d] = int(nX[d])
            arr[i].dX[d] = float(L[d]) / nX[d]
            arr[i].boundaryTypes[d] = int(bt[d])
    opt = _lib.BatchOptions()
    opt.max_steps = int(max_steps) if max_steps else -1
    opt.newton_tol = float(newton_tol) if newton_tol else 0.0
    opt.device = int(device)
    opt.autotune = int(bool(autotune))
    opt.per_pop = int(per_pop)
    opt.mixed_precision = int(bool(mixed_precision))
    if warm_start is not None:
        if not stiff:
            raise ValueError("warm_start applies to the stiff (Newton) predictor")
        ws = warm_start if isinstance(warm_start, dict) else {warm_start.N: warm_start}
        for n, w in ws.items():
            if w.N != n or not 1 <= n <= 3:
                raise ValueError(f"warm start for order {w.N} given for order {n}")
            if getattr(w, "active", True):
                opt.warm_start[n] = w.handle.value
    st = _lib.BatchStats()
    steps = (ctypes.c_longlong * len(problems))()
    tout = np.zeros(len(problems))
    code = _lib.lib().pde_solver_batch(system.handle, bool(stiff), FLUXES[flux], len(problems),
                                       arr, opt, st, steps, _lib.c_ptr(tout))
    _lib.check(code)
    if stats is not None:
        stats.update(st.as_dict())
        stats["steps_per_problem"] = list(steps)
        stats["t_final"] = tout.tolist()
    return Q0s


def weno_solver(u, order=2):
    """WENO reconstruction of an already padded array u of shape
    (n_1..n_d, V) (pypde/solvers.py:217-244).  Returns shape
    (n_1-2(order-1), ..., order, ..., order, V)."""
    nX = np.array(u.shape[:-1], dtype=np.int32)
    ndim = len(nX)
    V = u.shape[-1]
    nXret = nX - 2 * (order - 1)
    ret = np.zeros(int(nXret.prod()) * order ** ndim * V)
    ur = np.ascontiguousarray(u, dtype=np.float64).ravel()
    _lib.check(_lib.lib().weno_solver(_lib.c_ptr(ret), _lib.c_ptr(ur), _lib.c_ptr(nX), ndim,
                                      order, V))
    return ret.reshape(np.concatenate([nXret, [order] * ndim, [V]]))
