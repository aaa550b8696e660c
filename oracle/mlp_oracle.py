"""TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.

CPU reference of the learned start-cell locator's network (the checker for the
tensor-core kernels in fdf_gb300/csrc/fdf_mlp.cu).  There is no reference
counterpart -- PICurv locates particles only by the walking search -- so the
network is defined by this build:

    xhat = (p - centre) / half_extent                       (3)
    h1 = SiLU(W1 xhat + b1)   h2 = SiLU(W2 h1 + b2)          (128, 128)
    h3 = SiLU(W3 h2 + b3)     y = W4 h3 + b4                 (128, 3)
    target t_d = 2 (idx_d + 0.5) / N_d - 1  for (i, j, k), N = (IM, JM, KM)
    loss = mean over samples of sum_d (s_d (y_d - t_d))^2 / 3,  s_d = N_d / 2   (cell units)

The GPU rounds GEMM operands to bfloat16 and accumulates in FP32; `forward` and
`backward` here round at the same points (use_bf16=True) so the two can be compared
closely, and without rounding (use_bf16=False, FP64) for the finite-difference check.
A bfloat16 input coordinate enters as the pair hi = bf16(x), lo = bf16(x - hi) (its value
hi + lo has 16 significant bits); `forward(..., f16=True)` rounds inputs, weights and
activations to half precision instead (the locator's half-precision inference).
"""
from __future__ import annotations

import numpy as np

SIZES = (3, 128, 128, 128, 3)


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (nearest even) and return as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    nan = np.isnan(a)
    out = r.astype(np.uint32).view(np.float32).astype(np.float64)
    out[nan] = np.nan
    return out


def f16(x: np.ndarray) -> np.ndarray:
    """Round to IEEE half precision (nearest even) and return as float64."""
    return np.asarray(x, dtype=np.float64).astype(np.float16).astype(np.float64)


def split_bf16(x: np.ndarray) -> np.ndarray:
    """hi + lo with hi = bf16(x), lo = bf16(x - hi), x taken as float32 (the network's input pair)."""
    x32 = np.asarray(x, dtype=np.float32).astype(np.float64)
    hi = bf16(x32)
    return hi + bf16(x32 - hi)


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def init_params(seed: int = 0):
    """Uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights, zero biases (float32)."""
    from fdf_gb300.workloads import uniform01
    params = []
    for L in range(4):
        fin, fout = SIZES[L], SIZES[L + 1]
        u = uniform01(seed, 100 + L, fout * fin).reshape(fout, fin)
        W = ((2.0 * u - 1.0) / np.sqrt(fin)).astype(np.float32)
        params.append((W, np.zeros(fout, dtype=np.float32)))
    return params


def normalise(pos, centre, half):
    return (np.asarray(pos, dtype=np.float64) - centre) / half


def targets(cells, dims):
    N = np.asarray(dims, dtype=np.float64)
    return 2.0 * (np.asarray(cells, dtype=np.float64) + 0.5) / N - 1.0


def forward(params, xhat, use_bf16: bool = True, f16: bool = False):
    if f16:
        r, r_in = globals()["f16"], globals()["f16"]
    elif use_bf16:
        r, r_in = bf16, split_bf16
    else:
        r = r_in = (lambda a: np.asarray(a, dtype=np.float64))
    cache = {"h0": r_in(xhat)}
    h = cache["h0"]
    for L in range(3):
        W, b = params[L]
        z = h @ r(W).T + np.asarray(b, dtype=np.float64)
        cache[f"z{L + 1}"] = z
        h = r(silu(z))
        cache[f"h{L + 1}"] = h
    W, b = params[3]
    y = h @ r(W).T + np.asarray(b, dtype=np.float64)
    cache["y"] = y
    return y, cache


def loss_and_grad_y(y, t, dims):
    s = np.asarray(dims, dtype=np.float64) / 2.0
    d = (y - t) * s
    B = y.shape[0]
    loss = float((d * d).sum() / (3.0 * B))
    gy = 2.0 * d * s / (3.0 * B)
    return loss, gy


def backward(params, cache, gy, use_bf16: bool = True):
    """Gradients (dW, db) per layer, rounding like the GPU when use_bf16."""
    r = bf16 if use_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    grads = [None] * 4
    g = gy
    for L in range(3, -1, -1):
        W, _ = params[L]
        gb = r(g)
        db = g.sum(axis=0)
        dW = gb.T @ cache[f"h{L}"]
        grads[L] = (dW, db)
        if L > 0:
            dh = gb @ r(W)
            g = dh * silu_grad(cache[f"z{L}"])
    return grads


def adam_step(params, grads, state, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One Adam update in FP32 (state: list of (mW, vW, mb, vb), t)."""
    t = state["t"] + 1
    state["t"] = t
    out = []
    for L in range(4):
        (W, b), (dW, db) = params[L], grads[L]
        mW, vW, mb, vb = state["m"][L]
        mW = beta1 * mW + (1 - beta1) * dW
        vW = beta2 * vW + (1 - beta2) * dW * dW
        mb = beta1 * mb + (1 - beta1) * db
        vb = beta2 * vb + (1 - beta2) * db * db
        state["m"][L] = (mW, vW, mb, vb)
        c1, c2 = 1 - beta1 ** t, 1 - beta2 ** t
        W = (W - lr * (mW / c1) / (np.sqrt(vW / c2) + eps)).astype(np.float32)
        b = (b - lr * (mb / c1) / (np.sqrt(vb / c2) + eps)).astype(np.float32)
        out.append((W, b))
    return out


def finite_difference_check(params, xhat, t, dims, n_probe: int = 20, eps: float = 1e-6, seed: int = 0):
    """Max relative error of the analytic FP64 gradient against central differences."""
    rng = np.random.default_rng(seed)
    p64 = [(W.astype(np.float64), b.astype(np.float64)) for W, b in params]
    y, cache = forward(p64, xhat, use_bf16=False)
    _, gy = loss_and_grad_y(y, t, dims)
    grads = backward(p64, cache, gy, use_bf16=False)
    worst = 0.0
    for _ in range(n_probe):
        L = int(rng.integers(0, 4))
        which = int(rng.integers(0, 2))
        arr = p64[L][which]
        idx = tuple(int(rng.integers(0, s)) for s in arr.shape)
        orig = arr[idx]
        arr[idx] = orig + eps
        lp, _ = loss_and_grad_y(forward(p64, xhat, use_bf16=False)[0], t, dims)
        arr[idx] = orig - eps
        lm, _ = loss_and_grad_y(forward(p64, xhat, use_bf16=False)[0], t, dims)
        arr[idx] = orig
        fd = (lp - lm) / (2 * eps)
        an = grads[L][which][idx]
        worst = max(worst, abs(fd - an) / max(abs(fd), abs(an), 1e-8))
    return worst
