"""weno_solver_noalloc: WENO reconstruction for callers that cannot allocate
device memory (they run inside another framework's device-memory budget or
on paths where cudaMalloc's device synchronisation is not allowed).  The
caller owns the input and output device buffers; the entry point keeps its
pass-to-pass scratch in a fixed 32 MiB __device__ array.

Checked through the C ABI against the existing weno_solver entry point (bit
for bit, the tolerance of the other WENO tests), on two calls in a row so
that the second call runs over the scratch contents the first one left.
Collected last: if it fails, a run that stops at the first failure has
already run every other test.
"""
import ctypes

import numpy as np
import pytest

from pypde_gb300 import _lib, stages, workloads

pytestmark = pytest.mark.gpu


def _call(lib, out, u, N):
    nX = np.array(u.shape[:-1], dtype=np.int32)
    return lib.weno_solver_noalloc(ctypes.c_void_p(out.data_ptr()),
                                   ctypes.c_void_p(u.data_ptr()), _lib.c_ptr(nX), len(nX), N,
                                   u.shape[-1], None)


@pytest.mark.parametrize("shape,N", [((20, 18), 3), ((9, 8, 7), 2), ((33,), 2)])
def test_noalloc_matches_weno_solver_twice(gpu_lib, shape, N):
    torch = pytest.importorskip("torch")
    u = workloads.random_state("euler", shape, 5)
    expect = stages.weno(u, N)  # the existing entry point, host buffers
    du = torch.from_numpy(u).cuda()
    for call in range(2):
        out = torch.full(expect.shape, float("nan"), dtype=torch.float64, device="cuda")
        assert _call(gpu_lib, out, du, N) == _lib.PYPDE_OK
        torch.cuda.synchronize()
        assert np.array_equal(out.cpu().numpy(), expect), f"call {call}"


def test_noalloc_rejects_grids_beyond_its_scratch(gpu_lib):
    torch = pytest.importorskip("torch")
    # a 2-D N=3 grid whose first-pass output needs more than 4 Mi doubles
    shape, N, V = (700, 700), 3, 4
    du = torch.zeros(shape + (V,), dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    nX = np.array(shape, dtype=np.int32)
    rc = gpu_lib.weno_solver_noalloc(ctypes.c_void_p(out.data_ptr()),
                                     ctypes.c_void_p(du.data_ptr()), _lib.c_ptr(nX), 2, N, V, None)
    assert rc == _lib.PYPDE_ERR_ARG
    assert b"limit" in gpu_lib.pypde_last_error()
