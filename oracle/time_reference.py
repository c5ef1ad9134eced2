"""Times the reference's own CPU path against the CPU restatement.

TEST INFRASTRUCTURE ONLY: a measurement recipe, not part of the product.
It needs the reference built from its sources (`make -C oracle ref`, the
tolerance-tightened `libref_driver_tight.so`).  That build exists only
where the reference tree is, so this does not run on the GPU host.

Stiff relaxation workload (2-D, N=2, periodic): the reference's
pde_solver with its Newton-Krylov tightened to 1e-12 runs exactly K steps
(`ref_step_times` gives t_K), next to the restatement on 1 thread and on
every core.  The reference runs one thread whatever nThreads is
(src/solvers/iterator.cpp:50-51).

    python oracle/time_reference.py [n] [K]
"""
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.abspath(os.path.join(os.path.dirname(__file__), "..")))

from oracle import ora  # noqa: E402
from pypde_gb300 import workloads  # noqa: E402


def main(n=96, K=8):
    u0 = workloads.relaxation(n, 2, seed=0)
    nX = np.array([n, n], dtype=np.int32)
    dX = np.array([1.0 / n] * 2)
    bt = np.array([1, 1], dtype=np.int32)
    R = ora.ref(tight=True)
    times = np.zeros(K)
    R.ref_step_times(b"cattaneo", ora.ptr(u0.copy()), ora.ptr(nX), 2, ora.ptr(dX), 0.8,
                     ora.ptr(bt), 1, 0, 2, 1e9, K, ora.ptr(times))
    tf = float(times[-1])
    u = u0.copy()
    ret = np.zeros((1,) + u.shape)
    t0 = time.perf_counter()
    R.ref_pde_solver(b"cattaneo", ora.ptr(u), tf, ora.ptr(nX), 2, ora.ptr(dX), 0.8,
                     ora.ptr(bt), 1, 0, 2, 1, ora.ptr(ret), os.cpu_count() or 1)
    t_ref = time.perf_counter() - t0
    upd = n * n * K
    print(f"stiff {n}^2, N=2, {K} steps")
    print(f"  reference (Newton-Krylov to 1e-12, 1 thread): {upd / t_ref:10.0f} cell-updates/s")
    for th in (1, os.cpu_count() or 1):
        t0 = time.perf_counter()
        up = ora.pde_solver("cattaneo", u0, 1.0, [1.0, 1.0], [1, 1], 0.8, 2, stiff=True,
                            max_steps=K, nthreads=th)[0]
        el = time.perf_counter() - t0
        print(f"  restatement, {th:2d} thread(s):                  {upd / el:10.0f} cell-updates/s")
    l1 = np.abs(up - u).sum(axis=(0, 1)) / np.abs(u).sum(axis=(0, 1))
    print(f"  largest relative L1 between the two: {l1.max():.1e}")


if __name__ == "__main__":
    main(*(int(a) for a in sys.argv[1:3]))
