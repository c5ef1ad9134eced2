import glob
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run with -m gpu)")


def l1(a, b):
    """Relative L1 error per variable: sum|a-b| / sum|b| over all cells."""
    ax = tuple(range(a.ndim - 1))
    return np.abs(a - b).sum(axis=ax) / np.abs(b).sum(axis=ax)


def load(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built in place; fails loudly when it is missing."""
    from pypde_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        from pypde_gb300 import build
        build.build()
    return _lib.lib()


DYN_SMEM = "extern __shared__ double smem[];"


def build_device_host(out_dir, defines=()):
    """Compile tests/device_step_host.cpp (the device kernels as host C++,
    CUDA blocks emulated by fibers) into out_dir; returns the library path.
    The headers of pypde_gb300/csrc are copied there first, and the two
    `extern __shared__ double smem[];` declarations (a static array of unknown
    size, which a host compiler refuses) become pointers to a host buffer."""
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    csrc = os.path.join(ROOT, "pypde_gb300", "csrc")
    for f in glob.glob(os.path.join(csrc, "*.cuh")) + glob.glob(os.path.join(csrc, "*.h")):
        shutil.copy(f, out_dir)
    k = os.path.join(out_dir, "kernels.cuh")
    text = open(k).read()
    assert text.count(DYN_SMEM) == 2
    open(k, "w").write(text.replace(DYN_SMEM, "double *smem = host_dynamic_smem();"))
    out = os.path.join(out_dir, "libdevice_step_host.so")
    # PYPDE_HOST_ASAN=1 builds with AddressSanitizer, a bounds check of the
    # kernel source on the CPU (run with LD_PRELOAD=$(g++
    # -print-file-name=libasan.so) and ASAN_OPTIONS=detect_leaks=0:
    # detect_stack_use_after_return=0, the fibers switch stacks)
    opt = ["-O1", "-g", "-fsanitize=address", "-fno-omit-frame-pointer"] \
        if os.environ.get("PYPDE_HOST_ASAN") == "1" else ["-O2"]
    # hidden visibility and no GNU unique symbols: the shared-memory statics
    # of kernel templates over different UserSystem structs in two of these
    # libraries would otherwise be merged by the dynamic linker
    subprocess.run([cxx] + opt + ["-std=c++17", "-fPIC", "-shared", "-ffp-contract=off",
                    "-fvisibility=hidden", "-fvisibility-inlines-hidden", "-fno-gnu-unique",
                    "-Wno-unknown-pragmas", "-I", str(out_dir)] + [f"-D{d}" for d in defines] +
                   ["-o", out, os.path.join(ROOT, "tests", "device_step_host.cpp")], check=True)
    return out


def load_device_host(path):
    """Load a library built by build_device_host with its entry points typed."""
    import ctypes

    from oracle import ora
    L = ctypes.CDLL(path)
    c_int, c_ll, c_d = ctypes.c_int, ctypes.c_longlong, ctypes.c_double
    u64p = ctypes.POINTER(ctypes.c_ulonglong)
    L.host_run.restype = c_ll
    L.host_run.argtypes = [ctypes.c_char_p, c_int, c_int, c_int, ora.dp, ora.ip, ora.ip, ora.dp,
                           ora.dp, c_d, c_d, c_int, c_d, c_int, c_ll, ctypes.POINTER(c_d), u64p]
    L.host_predictor.restype = c_int
    L.host_predictor.argtypes = [ctypes.c_char_p, c_int, c_int, c_int, ora.dp, c_ll, ora.dp,
                                 c_d, c_d, ora.dp, ora.dp, u64p, ctypes.POINTER(c_int),
                                 ctypes.POINTER(c_int)]
    L.host_set_order.argtypes = [c_int]
    L.host_predictor_guess.restype = c_int
    L.host_predictor_guess.argtypes = [ctypes.c_char_p, c_int, c_int, ora.dp, c_ll, ora.dp, c_d,
                                       c_d, ora.dp, ora.dp, ora.dp, u64p, ctypes.POINTER(c_int),
                                       u64p, c_int, u64p]
    L.host_predictor_mixed.restype = c_int
    L.host_predictor_mixed.argtypes = [ctypes.c_char_p, c_int, c_int, ora.dp, c_ll, ora.dp, c_d,
                                       c_d, ora.dp, ora.dp, u64p, ctypes.POINTER(c_int), u64p]
    L.host_run_batch.restype = c_int
    L.host_run_batch.argtypes = [ctypes.c_char_p, c_int, c_int, c_int, c_int, ora.dp, ora.ip,
                                 ora.ip, ora.dp, ora.dp, ora.dp, ora.dp, c_int, c_d, c_int, c_int,
                                 c_ll, ctypes.POINTER(c_ll), ora.dp]
    return L
