"""CPU: the learned locator's network oracle (oracle/mlp_oracle.py) checked on its own.

The analytic FP64 gradient must agree with central finite differences, and the
bfloat16 rounding helper must round to nearest even with at most 2^-9 relative error;
the GPU gradient tests then compare the tensor-core kernels with this oracle.
"""
import numpy as np

from fdf_gb300 import workloads as W
from oracle import mlp_oracle as M


def _batch(n, dims, seed=1):
    rng = np.random.default_rng(seed)
    xhat = rng.uniform(-1.0, 1.0, size=(n, 3))
    cells = np.stack([rng.integers(0, d, size=n) for d in dims], axis=1)
    return xhat, M.targets(cells, dims)


def test_finite_difference_gradient():
    dims = (16, 16, 64)
    params = M.init_params(seed=3)
    # non-zero biases so their gradients are exercised too
    rng = np.random.default_rng(7)
    params = [(W_, (0.1 * rng.standard_normal(b.shape)).astype(np.float32)) for W_, b in params]
    xhat, t = _batch(24, dims)
    worst = M.finite_difference_check(params, xhat, t, dims, n_probe=40, eps=1e-6)
    assert worst < 1e-5, worst


def test_bf16_rounding():
    x = np.array([1.0, -2.5, 0.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -9, 3.14159265, -1e-20, 6.5e4])
    r = M.bf16(x)
    assert r[0] == 1.0 and r[1] == -2.5 and r[2] == 0.0
    assert r[3] == 1.0                         # tie -> even
    assert r[4] == 1.0 + 2.0 ** -7             # tie -> even (upwards)
    nz = x != 0
    assert np.all(np.abs(r[nz] - x[nz]) <= 2.0 ** -8 * np.abs(x[nz]) * (1 + 1e-7))
    # idempotent, and representable in 8 mantissa bits
    assert np.array_equal(M.bf16(r), r)
    u = r.astype(np.float32).view(np.uint32)
    assert np.all(u & 0xFFFF == 0)


def test_init_params_deterministic_and_scaled():
    a, b = M.init_params(seed=5), M.init_params(seed=5)
    for (Wa, ba), (Wb, bb) in zip(a, b):
        assert np.array_equal(Wa, Wb) and np.array_equal(ba, bb)
    for L, (Wl, bl) in enumerate(a):
        fin = M.SIZES[L]
        assert Wl.shape == (M.SIZES[L + 1], fin) and Wl.dtype == np.float32
        assert np.abs(Wl).max() <= 1.0 / np.sqrt(fin) and not bl.any()
    u = W.uniform01(5, 100, 4)
    assert Wl.dtype == np.float32 and np.isclose(a[0][0].ravel()[0], (2 * u[0] - 1) / np.sqrt(3), rtol=1e-7)


def test_bf16_backward_close_to_exact():
    """The GPU's rounding points change the gradient only at the bfloat16 level."""
    dims = (16, 16, 64)
    params = M.init_params(seed=2)
    xhat, t = _batch(64, dims, seed=4)
    p64 = [(W_.astype(np.float64), b.astype(np.float64)) for W_, b in params]
    y, cache = M.forward(p64, xhat, use_bf16=False)
    _, gy = M.loss_and_grad_y(y, t, dims)
    exact = M.backward(p64, cache, gy, use_bf16=False)
    yb, cb = M.forward(params, xhat, use_bf16=True)
    _, gyb = M.loss_and_grad_y(yb, t, dims)
    rounded = M.backward(params, cb, gyb, use_bf16=True)
    for (dWe, dbe), (dWr, dbr) in zip(exact, rounded):
        assert np.linalg.norm(dWr - dWe) <= 0.05 * np.linalg.norm(dWe)
        assert np.linalg.norm(dbr - dbe) <= 0.05 * np.linalg.norm(dbe) + 1e-12


def test_input_pair_and_half_rounding():
    """The bfloat16 input pair carries 16 significant bits; f16 rounds to half precision."""
    rng = np.random.default_rng(8)
    x = rng.uniform(-1, 1, 10000).astype(np.float32)
    pair = M.split_bf16(x)
    rel = np.abs(pair - x.astype(np.float64)) / np.abs(x.astype(np.float64))
    assert rel.max() <= 2.0 ** -16
    alone = np.abs(M.bf16(x) - x) / np.abs(x.astype(np.float64))
    assert alone.max() > 2.0 ** -10                              # bfloat16 alone: 8 significant bits
    assert np.array_equal(M.f16(x), x.astype(np.float16).astype(np.float64))
    assert np.abs(M.f16(x) - x).max() <= 2.0 ** -12
