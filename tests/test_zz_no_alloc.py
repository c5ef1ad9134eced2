"""weno_solver_noalloc: WENO reconstruction for callers that cannot allocate
device memory (they run inside another framework's device-memory budget or
on paths where cudaMalloc's device synchronisation is not allowed).  The
caller owns the input and output device buffers; the entry point keeps its
pass-to-pass scratch in a fixed 32 MiB __device__ array.

Checked through the C ABI against the existing weno_solver entry point (bit
for bit, the tolerance of the other WENO tests), on two calls in a row so
that the second call runs over the scratch contents the first one left;
the device memory the driver reports free is the same before and after the
second call, and a grid whose intermediate pass fills the scratch exactly
is accepted while one row more is refused.
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


# (779, 451) at N=3 with 4 variables: the one intermediate pass holds
# 3 x 4 x 775 x 451 = 4,194,300 doubles, which rounds up to exactly the
# 4 Mi-double scratch; one more row of cells does not fit
AT_LIMIT = (779, 451)


@pytest.mark.parametrize("shape,N", [((20, 18), 3), ((9, 8, 7), 2), ((33,), 2),
                                     (AT_LIMIT, 3)])
def test_noalloc_matches_weno_solver_twice(gpu_lib, shape, N):
    torch = pytest.importorskip("torch")
    u = workloads.random_state("euler", shape, 5)
    expect = stages.weno(u, N)  # the existing entry point, host buffers
    du = torch.from_numpy(u).cuda()
    outs = [torch.full(expect.shape, float("nan"), dtype=torch.float64, device="cuda")
            for _ in range(2)]
    torch.cuda.synchronize()
    for call in range(2):
        if call == 1:  # the first call loaded the module and its scratch
            free0 = torch.cuda.mem_get_info()[0]
        assert _call(gpu_lib, outs[call], du, N) == _lib.PYPDE_OK
        torch.cuda.synchronize()
        if call == 1:  # the entry point's contract: it allocates nothing
            assert torch.cuda.mem_get_info()[0] == free0
        assert np.array_equal(outs[call].cpu().numpy(), expect), f"call {call}"


@pytest.mark.parametrize("shape", [(700, 700), (AT_LIMIT[0] + 1, AT_LIMIT[1])])
def test_noalloc_rejects_grids_beyond_its_scratch(gpu_lib, shape):
    torch = pytest.importorskip("torch")
    # 2-D N=3 grids whose first-pass output needs more than 4 Mi doubles
    N, V = 3, 4
    du = torch.zeros(shape + (V,), dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    nX = np.array(shape, dtype=np.int32)
    rc = gpu_lib.weno_solver_noalloc(ctypes.c_void_p(out.data_ptr()),
                                     ctypes.c_void_p(du.data_ptr()), _lib.c_ptr(nX), 2, N, V, None)
    assert rc == _lib.PYPDE_ERR_ARG
    assert b"limit" in gpu_lib.pypde_last_error()
