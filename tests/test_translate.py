"""The Python -> CUDA C++ callback translator (pypde_gb300/translate.py).

Each translated callback is compiled as host C++ (the device qualifiers
defined away, no FMA contraction) and evaluated on random states against
the Python function itself: same operation order, so the same bits (a few
ulp where a libm function and numpy's differ).  A second test compiles the
full kernel templates for a translated system with NVRTC, which needs no
GPU.
"""
import ctypes
import math
import os
import subprocess
import tempfile

import numpy as np
import pytest

from pypde_gb300 import systems, workloads
from pypde_gb300.translate import TranslateError, translate

GAMMA = 1.4
RHO_FLOOR = 1e-12
COEF = (0.3, 0.7, 1.1)


def helper_pressure(Q, n):
    ke = 0.0
    for i in range(n):
        ke += Q[1 + i] * Q[1 + i]
    return (GAMMA - 1.0) * (Q[n + 1] - 0.5 * ke / Q[0])


def user_euler2(Q, d):
    """numpy style: slices, array arithmetic, a helper, a conditional."""
    r = max(Q[0], RHO_FLOOR)
    v = Q[1:3] / r
    p = helper_pressure(Q, 2)
    ret = v[d] * Q
    ret[1 + d] += p
    ret[3] += p * v[d]
    return ret


def user_src(Q):
    out = np.zeros(4)
    e = Q[3] / Q[0]
    out[3] = -0.5 * e if e > 2.0 else 0.25 * e ** 2
    out[1] = COEF[0] * Q[1] + COEF[1] * Q[2]
    return out


def user_ncp(Q, d):
    B = np.zeros((4, 4))
    for i in range(4):
        B[i, i] = Q[0] * COEF[d]
    B[1, 2] = 0.1
    B[2][1] = 0.1
    return B


def user_second_order(Q, DQ, d):
    a, b = 0.5, 0.01
    return np.array([a * Q[0] * Q[0] - b * DQ[d][0] + b * DQ[d, 0] * 0.0])


CASES = [
    ("F", user_euler2, 2, 4), ("S", user_src, 2, 4), ("B", user_ncp, 2, 4),
    ("F", user_second_order, 1, 1),
    ("F", systems.euler(1).F, 1, 3), ("F", systems.euler(2).F, 2, 4),
    ("F", systems.euler(3).F, 3, 5), ("F", systems.cattaneo(2).F, 2, 7),
    ("S", systems.cattaneo(2).S, 2, 7), ("F", systems.ncp(2).F, 2, 3),
    ("B", systems.ncp(2).B, 2, 3), ("S", systems.ncp(2).S, 2, 3),
    ("F", systems.burgers2().F, 1, 1),
]


def _host_lib(src, role):
    d = tempfile.mkdtemp()
    cpp = os.path.join(d, "cb.cpp")
    so = os.path.join(d, "cb.so")
    call = {"F": "UserSystem::F(out, Q, dQ, d);", "B": "UserSystem::B(out, Q, d);",
            "S": "UserSystem::S(out, Q);"}[role]
    with open(cpp, "w") as f:
        f.write("#include <cmath>\nusing namespace std;\n#define __device__\n"
                "#define __forceinline__ inline\n" + src +
                "\nextern \"C\" void call(double *out, const double *Q, const double *dQ, int d)"
                " { (void)dQ; (void)d; " + call + " }\n")
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-fPIC", "-shared", cpp, "-o", so],
                   check=True)
    lib = ctypes.CDLL(so)
    lib.call.argtypes = [ctypes.POINTER(ctypes.c_double)] * 3 + [ctypes.c_int]
    return lib


def _p(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{c[1].__name__}-{c[2]}d-V{c[3]}"
                                             for c in CASES])
def test_translated_callback_matches_python(case):
    role, fn, ndim, V = case
    src = translate(fn if role == "F" else None, fn if role == "B" else None,
                    fn if role == "S" else None, ndim, V)
    lib = _host_lib(src, role)
    rng = np.random.default_rng(0)
    nout = V * V if role == "B" else V
    for k in range(50):
        name = "cattaneo" if V == 7 else ("euler" if V == ndim + 2 else "ncp")
        Q = workloads.random_state(name, (1,) * ndim, k).reshape(-1)[:V].copy() \
            if name != "ncp" or V == 3 else 0.5 + rng.random(V)
        if Q.shape[0] != V:
            Q = 0.5 + rng.random(V)
        dQ = rng.standard_normal(ndim * V)
        for d in range(ndim if role != "S" else 1):
            out = np.zeros(nout)
            lib.call(_p(out), _p(Q), _p(dQ), d)
            if role == "S":
                want = fn(Q)
            elif fn.__code__.co_argcount == 3:
                want = fn(Q, dQ.reshape(ndim, V), d)
            elif fn.__code__.co_argcount == 2:
                want = fn(Q, d)
            else:
                want = fn(Q)
            want = np.asarray(want, dtype=np.float64).reshape(-1)
            assert np.array_equal(out, want), (k, d, out, want)


def test_unsupported_constructs_are_reported():
    def bad(Q, d):
        return [q for q in Q]
    with pytest.raises(TranslateError):
        translate(bad, None, None, 1, 3)


def _nvrtc_compile(src, kernels):
    """Compile the translated source with the kernel templates for sm_103a
    by NVRTC (no GPU needed); asserts success with the log."""
    try:
        nv = ctypes.CDLL("libnvrtc.so")
    except OSError:
        try:
            nv = ctypes.CDLL("/usr/local/cuda/lib64/libnvrtc.so")
        except OSError:
            pytest.skip("NVRTC not available")
    here = os.path.join(os.path.dirname(__file__), "..", "pypde_gb300", "csrc")
    names = ["kernels.cuh", "ader_common.cuh", "eig_full.cuh", "mlp.cuh", "batch.cuh"]
    hdrs = [open(os.path.join(here, n)).read().encode() for n in names]
    src = ('#include "mlp.cuh"\n' + src).encode()
    prog = ctypes.c_void_p()
    arr = ctypes.c_char_p * len(names)
    assert nv.nvrtcCreateProgram(ctypes.byref(prog), src, b"u.cu", len(names), arr(*hdrs),
                                 arr(*[n.encode() for n in names])) == 0
    for e in kernels:
        nv.nvrtcAddNameExpression(prog, f"&pypde::{e}".encode())
    opts = [b"--gpu-architecture=sm_103a", b"-std=c++17", b"--fmad=false"]
    rc = nv.nvrtcCompileProgram(prog, len(opts), (ctypes.c_char_p * len(opts))(*opts))
    n = ctypes.c_size_t()
    nv.nvrtcGetProgramLogSize(prog, ctypes.byref(n))
    log = ctypes.create_string_buffer(n.value)
    nv.nvrtcGetProgramLog(prog, log)
    assert rc == 0, log.value.decode()[:4000]


def test_nvrtc_compiles_the_kernels_for_a_translated_system():
    _nvrtc_compile(translate(user_euler2, user_ncp, user_src, 2, 4),
                   ["k_faces<UserSystem, 2, 0>", "k_newton<UserSystem, 2>",
                    "k_mlp_guess<UserSystem, 2>", "kb_mlp_guess<UserSystem, 2>",
                    "kb_newton<UserSystem, 2>"])


def test_lambda_callback_translates():
    src = translate(lambda Q, d: Q * 2.0, None, None, 1, 3)
    assert "Q[i_] * 2.0" in src


# Constructs of the reference's larger examples (GPR, Navier-Stokes): slice
# assignment, bounds around d, tuple-returning helpers, matrix products,
# transposes, reshape / ravel, eye / det / trace, branches on module flags,
# and Greek names.
LINEAR_EOS = True
τ_INF = math.inf


def unpack(Q):
    ρ = Q[0]
    v = Q[1:4] / ρ
    A = Q[4:13].copy().reshape((3, 3))
    return ρ, v, A


def gram_dev(A):
    G = A.T @ A
    return G - np.trace(G) / 3 * np.eye(3)


def relax_rate(ρ, A):
    if τ_INF == math.inf:
        if LINEAR_EOS:
            return 2.0 * np.linalg.det(A) ** (5 / 3) / ρ
        return None + 1.0   # dead code: never translated
    return 0.0


def flux_matrix_style(Q, d):
    ret = np.zeros(13)
    ρ, v, A = unpack(Q)
    σ = -ρ * np.dot(A.T, gram_dev(A))
    ret[0] = ρ * v[d]
    ret[1:4] = ρ * v[d] * v
    ret[1:4] -= σ[d]
    ret[1 + d] += np.dot(v, v)
    Av = np.dot(A, v)
    ret[4 + 3 * d:7 + 3 * d] = Av
    return ret


def ncp_matrix_style(Q, d):
    ret = np.zeros((13, 13))
    v = Q[1:4] / Q[0]
    for i in range(4, 13):
        ret[i, i] = v[d]
    ret[4 + d, 4 + d:7 + d] -= v
    ret[2, 0:3] = ret[4, 4:7] * 0.5
    return ret


def src_matrix_style(Q):
    ret = np.zeros(13)
    ρ, v, A = unpack(Q)
    ψ = gram_dev(A)
    ret[4:13] = -ψ.ravel() * relax_rate(ρ, A)
    return ret


def _matrix_style_state(rng):
    A = np.eye(3) + 0.1 * rng.standard_normal((3, 3))
    return np.concatenate([[1 + rng.random()], 0.3 * rng.standard_normal(3), A.ravel()])


@pytest.mark.parametrize("role,fn", [("F", flux_matrix_style), ("B", ncp_matrix_style),
                                     ("S", src_matrix_style)])
def test_matrix_style_callbacks_translate(role, fn):
    """Translated against the Python function on random states.  The
    translation sums each dot product in index order, numpy through BLAS, so
    they agree to a few ulp rather than bit for bit."""
    src = translate(fn if role == "F" else None, fn if role == "B" else None,
                    fn if role == "S" else None, 1, 13)
    lib = _host_lib(src, role)
    rng = np.random.default_rng(5)
    for k in range(40):
        Q = _matrix_style_state(rng)
        for d in range(3 if role != "S" else 1):
            out = np.zeros(169 if role == "B" else 13)
            lib.call(_p(out), _p(Q), _p(np.zeros(13)), d)
            want = np.asarray(fn(Q) if role == "S" else fn(Q, d)).reshape(-1)
            assert np.abs(out - want).max() <= 1e-13 * np.abs(want).max(), (k, d)


def test_slice_assignment_writes_the_array():
    """ret[a:b] = x and ret[a:b] += x write into ret (a numpy slice is a
    view), also for bounds around d and for part of a matrix row."""
    def f(Q, d):
        ret = np.zeros(6)
        ret[0:3] = Q[3:6] * 2.0
        ret[3 + d:5 + d] += Q[0:2]
        ret[1:4] += ret[0:3]            # overlapping operands, as numpy
        return ret

    def b(Q, d):
        m = np.zeros((6, 6))
        m[1, 2 + d:4 + d] = Q[0:2]
        m[d, :] -= Q
        return m

    for role, fn in (("F", f), ("B", b)):
        src = translate(fn if role == "F" else None, fn if role == "B" else None, None, 1, 6)
        lib = _host_lib(src, role)
        Q = np.arange(1.0, 7.0)
        for d in range(2):
            out = np.zeros(36 if role == "B" else 6)
            lib.call(_p(out), _p(Q), _p(np.zeros(6)), d)
            assert np.array_equal(out, np.asarray(fn(Q, d)).reshape(-1)), (role, d, out)


def numpy_helpers_flux(Q, d):
    """ones / full, one-argument max / min, elementwise maximum / minimum,
    sign, square, clip, prod, norm, outer, cross, concatenate / hstack."""
    v = Q[0:3]
    w = Q[3:6]
    ret = np.full(6, 0.25) + np.ones(6)
    ret[0] = max(v) - np.min(w) + np.amax(Q)
    ret[1:4] = np.maximum(v, 0.5) + np.minimum(w, v) + np.sign(v - 0.6)
    ret[4] = np.square(Q[0]) + np.prod(v) + np.linalg.norm(w) + np.clip(Q[1], 0.2, 0.7)
    ret[5] = np.trace(np.outer(v, w)) + np.cross(v, w)[d]
    ret += np.concatenate((v, w)) * 0.5 + np.hstack([w, v]) * np.square(w[0])
    return ret


def test_numpy_helpers_translate():
    """The added numpy functions, translated, against the Python function on
    random states (norm sums in index order, numpy through BLAS: a few ulp)."""
    src = translate(numpy_helpers_flux, None, None, 1, 6)
    lib = _host_lib(src, "F")
    rng = np.random.default_rng(9)
    for k in range(60):
        Q = rng.random(6)
        for d in range(3):
            out = np.zeros(6)
            lib.call(_p(out), _p(Q), _p(np.zeros(6)), d)
            want = numpy_helpers_flux(Q, d)
            assert np.abs(out - want).max() <= 1e-14 * np.abs(want).max(), (k, d, out, want)


def comprehension_flux(Q, d):
    scale = np.array([1.0 + 0.5 * i for i in range(4)])
    return np.array([Q[i] * scale[i] + Q[(i + d) % 4] for i in range(4)])


def test_list_comprehension_translates():
    """[expr for i in range(n)] becomes a loop filling an array; the loop
    variable may index and take part in integer arithmetic."""
    src = translate(comprehension_flux, None, None, 1, 4)
    lib = _host_lib(src, "F")
    Q = np.array([0.3, 1.7, -2.2, 4.1])
    for d in range(3):
        out = np.zeros(4)
        lib.call(_p(out), _p(Q), _p(np.zeros(4)), d)
        assert np.array_equal(out, comprehension_flux(Q, d)), (d, out)


def where_atan2_flux(Q, d):
    v = Q[0:3]
    ret = np.zeros(5)
    ret[0:3] = np.where(v > 0.5, v * 2.0, -v) + np.arctan2(v, 0.3)
    ret[3] = np.where(Q[3] > Q[4], Q[3], 0.0) + math.hypot(Q[3], Q[4]) + math.atan2(Q[d], 1.5)
    ret[4] = math.copysign(Q[4], -1.0) + math.fmod(Q[3] * 7.0, 1.3)
    return ret


def test_where_and_two_argument_functions_translate():
    src = translate(where_atan2_flux, None, None, 1, 5)
    lib = _host_lib(src, "F")
    rng = np.random.default_rng(11)
    for k in range(40):
        Q = rng.random(5)
        for d in range(3):
            out = np.zeros(5)
            lib.call(_p(out), _p(Q), _p(np.zeros(5)), d)
            want = where_atan2_flux(Q, d)
            assert np.abs(out - want).max() <= 4e-16 * np.abs(want).max(), (k, d, out, want)



@pytest.mark.parametrize("case", ["matrix", "numpy_helpers", "comprehension", "where"])
def test_nvrtc_compiles_the_newer_constructs(case):
    """The translations that use tuple-returning helpers, matrix products,
    det, slices around d, list comprehensions, where and the added numpy
    functions compile with the kernel templates for sm_103a."""
    if case == "matrix":
        src, ks = translate(flux_matrix_style, ncp_matrix_style, src_matrix_style, 1, 13), \
            ["k_faces<UserSystem, 2, 1>", "k_newton<UserSystem, 2>"]
    else:
        fn = {"numpy_helpers": numpy_helpers_flux, "comprehension": comprehension_flux,
              "where": where_atan2_flux}[case]
        V = {"numpy_helpers": 6, "comprehension": 4, "where": 5}[case]
        src, ks = translate(fn, None, None, 1, V), ["k_faces<UserSystem, 2, 0>"]
    _nvrtc_compile(src, ks)


def array_power_flux(Q, d):
    v = Q[0:3]
    return np.array([np.sum(v ** 2), np.sum(v ** 0.5), np.sum(v ** 3) + Q[3] ** 2, Q[3]])


def test_array_power_translates():
    """x**2 of an array squares each item, x**0.5 takes square roots and
    other constant exponents call pow, as numpy does item by item."""
    src = translate(array_power_flux, None, None, 1, 4)
    lib = _host_lib(src, "F")
    Q = np.array([0.3, 1.7, 2.2, 4.1])
    out = np.zeros(4)
    lib.call(_p(out), _p(Q), _p(np.zeros(4)), 0)
    want = array_power_flux(Q, 0)
    assert np.abs(out - want).max() <= 4e-16 * np.abs(want).max(), (out, want)


def floor_mod_flux(Q, d):
    ret = np.zeros(6)
    for i in range(-3, 3):
        ret[i + 3] = Q[(i - d) % 6] * 10.0 + float((i - 2 * d) // 4) + float(i % -4)
    return ret


def test_integer_floor_division_and_modulo_follow_python():
    """// and % of integers floor as Python does (a periodic index (i - d) % n
    stays in range), also for negative operands."""
    src = translate(floor_mod_flux, None, None, 1, 6)
    lib = _host_lib(src, "F")
    Q = np.arange(1.0, 7.0)
    for d in range(3):
        out = np.zeros(6)
        lib.call(_p(out), _p(Q), _p(np.zeros(6)), d)
        assert np.array_equal(out, floor_mod_flux(Q, d)), (d, out, floor_mod_flux(Q, d))


def negative_index_flux(Q, d):
    ret = np.zeros(4)
    ret[-1] = Q[-1] * 2.0
    ret[0] = Q[-2] + Q[-4]
    m = np.zeros((2, 2))
    m[-1, -2] = Q[1]
    m[-2] = Q[2:4]
    ret[1] = m[1, 0] + m[-2, -1]
    return ret


def out_of_range_flux(Q, d):
    return np.array([Q[4], Q[0], Q[1], Q[2]])


def test_constant_indices_follow_python():
    """A constant negative index counts from the end, as in Python; a
    constant index outside the dimension is refused at translation time."""
    src = translate(negative_index_flux, None, None, 1, 4)
    lib = _host_lib(src, "F")
    Q = np.array([0.3, 1.7, -2.2, 4.1])
    out = np.zeros(4)
    lib.call(_p(out), _p(Q), _p(np.zeros(4)), 0)
    assert np.array_equal(out, negative_index_flux(Q, 0)), out
    with pytest.raises(TranslateError, match="out of range"):
        translate(out_of_range_flux, None, None, 1, 4)


def computed_negative_index_flux(Q, d):
    ret = np.zeros(4)
    for i in range(4):
        ret[i] = Q[i - 1] * 10.0 + Q[-1 - i] + Q[1 + d]
    return ret


def test_computed_negative_indices_follow_python():
    """Q[i - 1] at i = 0 is the last element, as in Python."""
    src = translate(computed_negative_index_flux, None, None, 1, 4)
    lib = _host_lib(src, "F")
    Q = np.array([0.3, 1.7, -2.2, 4.1])
    for d in range(2):
        out = np.zeros(4)
        lib.call(_p(out), _p(Q), _p(np.zeros(4)), d)
        assert np.array_equal(out, computed_negative_index_flux(Q, d)), (d, out)


def array_truth_if(Q, d):
    ret = np.zeros(3)
    if Q[0:2] > 0.5:
        ret[0] = 1.0
    return ret


def array_truth_and(Q, d):
    return Q * (1.0 if (Q > 0.0) and Q[0] > 1.0 else 2.0)


def test_array_truth_values_are_refused():
    """An array where Python needs one truth value (if, and/or, not, a
    conditional expression) raises in Python; the translation refuses it
    instead of testing a pointer."""
    for fn in (array_truth_if, array_truth_and):
        with pytest.raises(TranslateError, match="ambiguous"):
            translate(fn, None, None, 1, 3)


def writes_input_flux(Q, d):
    Q[0] = 2.0
    return Q


def writes_copy_flux(Q, d):
    q = Q.copy()
    q[0] = 2.0
    return q


def test_assignment_into_the_input_is_refused():
    """The callback's Q is the solver's state: writing into it is refused
    with a message naming the fix, and writing into a copy translates."""
    with pytest.raises(TranslateError, match="copy it first"):
        translate(writes_input_flux, None, None, 1, 3)
    lib = _host_lib(translate(writes_copy_flux, None, None, 1, 3), "F")
    Q = np.array([0.5, 1.5, 2.5])
    out = np.zeros(3)
    lib.call(_p(out), _p(Q), _p(np.zeros(3)), 0)
    assert np.array_equal(out, [2.0, 1.5, 2.5]) and Q[0] == 0.5


def float_floor_mod_flux(Q, d):
    a = Q // 0.7
    b = Q % -0.7
    c = Q[0] // Q[1]
    e = Q[1] % Q[2]
    return np.array([a[0], a[1], a[2], b[0], b[1], b[2], c, e, 1.0 // 0.1, -7.5 % 2.0])


def test_float_floor_division_and_modulo_follow_numpy():
    """// and % of floats and of arrays floor as numpy and Python do (the
    remainder takes the sign of the divisor); they were C's truncating
    quotient, or refused."""
    src = translate(float_floor_mod_flux, None, None, 1, 10)
    lib = _host_lib(src, "F")
    rng = np.random.default_rng(4)
    for Q in [np.array([2.5, -1.3, 0.4] + [0.0] * 7), rng.standard_normal(10) * 5,
              np.array([-0.7, 0.7, -1.4] + [1.0] * 7), np.array([0.0, -2.0, 3.0] + [0.0] * 7)]:
        out = np.zeros(10)
        lib.call(_p(out), _p(Q), _p(np.zeros(10)), 0)
        want = float_floor_mod_flux(Q, 0)
        assert np.array_equal(out, want), (Q, out, want)
        assert np.array_equal(np.signbit(out), np.signbit(want))


def name_negative_index_flux(Q, d):
    ret = np.zeros(4)
    k = -1
    ret[0] = Q[k]
    for i in range(-3, 0):
        ret[i] = Q[i] * 2.0
    j = d - 2
    ret[0] += Q[j]
    return ret


def test_negative_index_in_a_name_follows_python():
    """A negative index held in a name or a loop variable counts from the
    end, as in Python (it used to read before the array)."""
    src = translate(name_negative_index_flux, None, None, 1, 4)
    lib = _host_lib(src, "F")
    Q = np.array([0.3, 1.7, -2.2, 4.1])
    for d in range(2):
        out = np.zeros(4)
        lib.call(_p(out), _p(Q), _p(np.zeros(4)), d)
        assert np.array_equal(out, name_negative_index_flux(Q, d)), (d, out)


def rebinds_input_flux(Q, d):
    Q = Q * 2.0
    Q = Q + 1.0
    return Q


def test_rebinding_the_input_makes_a_new_array():
    """Q = Q * 2 rebinds the name to a new array, as in Python; the solver's
    state is not written (it was emitted as a copy into the const input)."""
    lib = _host_lib(translate(rebinds_input_flux, None, None, 1, 3), "F")
    Q = np.array([0.5, 1.5, 2.5])
    out = np.zeros(3)
    lib.call(_p(out), _p(Q), _p(np.zeros(3)), 0)
    assert np.array_equal(out, rebinds_input_flux(Q.copy(), 0))
    assert np.array_equal(Q, [0.5, 1.5, 2.5])
