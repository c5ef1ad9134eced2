"""CPU oracle of the warm-start network's arithmetic -- test
infrastructure only, never on the product path.

The GPU kernels (pypde_gb300/csrc/mlp.cuh, mlp_train.cu) round every GEMM
operand to BF16 (round to nearest even) and accumulate in FP32.  This
restatement rounds the same operands the same way and accumulates in
float64, so the two differ only by FP32 accumulation order (and, rarely,
an activation that lands on the other side of a BF16 rounding boundary).

The network is not in the reference (its predictor has no learned guess);
the oracle is pinned against finite differences of its own float64 form
in tests/test_warmstart_cpu.py.
"""
import numpy as np


def bf16(a):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    a32 = np.ascontiguousarray(a, dtype=np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    nan = (u & 0x7FFFFFFF) > 0x7F800000
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    r = np.where(nan, (u | 0x400000) & 0xFFFF0000, r)
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def linear(x, W, b, rounding=True):
    """x W^T + b with BF16 operands (float64 accumulation)."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    return r(x) @ r(W).T + np.asarray(b, np.float64)


def forward(x, params, rounding=True):
    """Returns (y, cache) for params (W1, b1, W2, b2, W3, b3)."""
    W1, b1, W2, b2, W3, b3 = params
    z1 = linear(x, W1, b1, rounding)
    a1 = silu(z1)
    z2 = linear(a1, W2, b2, rounding)
    a2 = silu(z2)
    y = linear(a2, W3, b3, rounding)
    return y, (x, z1, a1, z2, a2)


def backward(dy, params, cache, rounding=True):
    """Gradients (dW1, db1, dW2, db2, dW3, db3) of sum(dy * y), with the
    operands of every GEMM rounded to BF16 as the GPU backward pass does."""
    r = bf16 if rounding else (lambda a: np.asarray(a, np.float64))
    W1, b1, W2, b2, W3, b3 = params
    x, z1, a1, z2, a2 = cache
    dy = np.asarray(dy, np.float64)
    dW3 = r(dy).T @ r(a2)
    db3 = dy.sum(0)
    da2 = r(dy) @ r(W3)
    dz2 = da2 * silu_grad(z2)
    dW2 = r(dz2).T @ r(a1)
    db2 = dz2.sum(0)
    da1 = r(dz2) @ r(W2)
    dz1 = da1 * silu_grad(z1)
    dW1 = r(dz1).T @ r(x)
    db1 = dz1.sum(0)
    return dW1, db1, dW2, db2, dW3, db3
