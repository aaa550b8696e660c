"""GPU: the learned start-cell locator (tensor-core MLP) and the learned form.

* Initial weights equal the oracle's (oracle/mlp_oracle.py init_params), bit for bit.
* Gradients of the tensor-core forward/backward kernels match the oracle's backward
  with the same bfloat16 rounding points (relative L2 error per block <= 5e-3), and
  match it far more closely than they match the unrounded FP64 gradient.
* Inference (fused kernel, SiLU by tanh.approx) matches the oracle's forward with the same
  operand type (bfloat16 by default, half precision on request) to a few units in the last
  place of the type, and its cells are floor((y + 1) N / 2) of its outputs.
* Training on walk-produced pairs is deterministic and reduces the loss.
* The learned form gives the FP32 form's swarm, fields and deposits bit for bit, with a
  trained and with an untrained network, with either guess policy, and the trained network
  reduces the walk.
"""
import numpy as np
import pytest

from fdf_gb300 import workloads as W
from fdf_gb300.context import FORM_FP32, FORM_LEARNED_FP32, LOCATOR_BF16, LOCATOR_F16, LOCATOR_NPARAM, PicContext
from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu

OFFS = [(0, 384), (384, 512), (512, 16896), (16896, 17024), (17024, 33408), (33408, 33536), (33536, 33920),
        (33920, 33923)]
NAMES = ["W1", "b1", "W2", "b2", "W3", "b3", "W4", "b4"]
# (max, mean) |y - y_oracle| of inference by operand type, outputs |y| <= 0.44 here; measured
# on GB300: bfloat16 7.4e-4 / 1.5e-4, half 9.6e-5 / 1.9e-5
PREDICT_TOL = {"bf16": (3e-3, 6e-4), "f16": (5e-4, 1e-4)}


def flat(params):
    return np.concatenate([np.concatenate([W_.ravel(), b.ravel()]) for W_, b in params]).astype(np.float32)


def unflat(v):
    out = []
    for L in range(4):
        (a, b), (c, d) = OFFS[2 * L], OFFS[2 * L + 1]
        out.append((v[a:b].reshape(M.SIZES[L + 1], M.SIZES[L]), v[c:d]))
    return out


@pytest.fixture(scope="module")
def small(require_gpu):
    c = PicContext(0)
    wl = W.config_bent_pipe(12, 12, 48, n=1000, cfl=2.0, materialize=False)
    c.set_grid(wl.coor)
    yield c, wl
    c.close()


def test_init_matches_oracle(small):
    ctx, _ = small
    ctx.locator_init(seed=3)
    assert np.array_equal(ctx.locator_get_params(), flat(M.init_params(seed=3)))


@pytest.mark.parametrize("B", [512, 300])   # whole 128-sample tiles, and a last tile partly empty
def test_gradients_match_oracle(small, B):
    ctx, wl = small
    dims = wl.dims
    rng = np.random.default_rng(11)
    params = [(W_, (0.2 * rng.standard_normal(b.shape)).astype(np.float32)) for W_, b in M.init_params(seed=4)]
    ctx.locator_set_params(flat(params))
    xhat = rng.uniform(-1, 1, size=(B, 3)).astype(np.float32)
    cells = np.stack([rng.integers(0, d, size=B) for d in dims], axis=1)
    t = M.targets(cells, dims).astype(np.float32)
    g_gpu, loss_gpu = ctx.locator_gradients(xhat, t)

    y, cache = M.forward(params, xhat.astype(np.float64), use_bf16=True)
    loss, gy = M.loss_and_grad_y(y, t.astype(np.float64), dims)
    ref = flat([(dW, db) for dW, db in M.backward(params, cache, gy, use_bf16=True)])
    p64 = [(W_.astype(np.float64), b.astype(np.float64)) for W_, b in params]
    y6, c6 = M.forward(p64, xhat.astype(np.float64), use_bf16=False)
    _, gy6 = M.loss_and_grad_y(y6, t.astype(np.float64), dims)
    exact = flat([(dW, db) for dW, db in M.backward(p64, c6, gy6, use_bf16=False)])

    assert abs(loss_gpu - loss) <= 1e-3 * loss
    for name, (a, b) in zip(NAMES, OFFS):
        e_ref = np.linalg.norm(g_gpu[a:b] - ref[a:b]) / np.linalg.norm(ref[a:b])
        e_exact = np.linalg.norm(g_gpu[a:b] - exact[a:b]) / np.linalg.norm(exact[a:b])
        print(f"[grad {name}] vs bf16 oracle {e_ref:.2e}  vs FP64 {e_exact:.2e}")
        assert e_ref <= 5e-3, (name, e_ref)
        if name in ("W1", "W2", "W3", "b1", "b2", "b3"):
            assert e_ref <= 0.3 * e_exact, (name, e_ref, e_exact)


@pytest.mark.parametrize("kind", ["bf16", "f16"])
def test_predict_matches_oracle_forward(small, kind):
    """Inference against the oracle's forward with the kernel's operand type (bfloat16: input
    pairs, bfloat16 weights and activations; half: all in half precision).  The kernel rounds
    the SiLU's intermediate values to the operand type as well (h = z/2 + b/2, tanh.approx,
    h + h tanh(h)), so it differs from the oracle's single rounding per activation by a few
    units in the last place of the type: bfloat16 keeps 8 significant bits, half 11."""
    ctx, wl = small
    rng = np.random.default_rng(5)
    params = [(W_, (0.2 * rng.standard_normal(b.shape)).astype(np.float32)) for W_, b in M.init_params(seed=6)]
    ctx.locator_set_params(flat(params))
    ctx.locator_inference_type(LOCATOR_BF16 if kind == "bf16" else LOCATOR_F16)
    try:
        pos, _ = W.volumetric_particles(wl.coor, 5000, seed=9)
        cells, y = ctx.locator_predict(pos)
    finally:
        ctx.locator_inference_type(LOCATOR_BF16)
    c, ih = ctx.locator_normalization()
    xhat = (pos.astype(np.float32) - c) * ih
    y_ref, _ = M.forward(params, xhat.astype(np.float64), use_bf16=True, f16=(kind == "f16"))
    err = np.abs(y.astype(np.float64) - y_ref)
    print(f"[predict {kind}] max |dy| {err.max():.3e} mean {err.mean():.3e} (|y| max {np.abs(y_ref).max():.2f})")
    tol_max, tol_mean = PREDICT_TOL[kind]
    assert err.max() <= tol_max and err.mean() <= tol_mean
    N = np.array(wl.dims, dtype=np.float32)
    want = np.clip(np.floor((y + np.float32(1.0)) * np.float32(0.5) * N), 0, N - 1).astype(np.int64)
    assert np.array_equal(cells, want)


def test_training_deterministic_and_learns(small):
    ctx, wl = small
    ctx.locator_init(seed=1)
    h1 = ctx.locator_train(200_000, seed=2, steps=600, batch=4096, lr=3e-3)
    p1 = ctx.locator_get_params()
    ctx.locator_init(seed=1)
    h2 = ctx.locator_train(200_000, seed=2, steps=600, batch=4096, lr=3e-3)
    assert np.array_equal(p1, ctx.locator_get_params()) and np.array_equal(h1, h2)
    print(f"[train] loss {h1[:20].mean():.3f} -> {h1[-50:].mean():.4f}")
    assert np.all(np.isfinite(h1)) and h1[-50:].mean() < 0.1 * h1[:20].mean()
    pos, cell = W.volumetric_particles(wl.coor, 20000, seed=13)
    pred, _ = ctx.locator_predict(pos)
    cheb = np.abs(pred - cell).max(axis=1)
    print(f"[train] held-out: exact {np.mean(cheb == 0):.3f}, within 1 cell {np.mean(cheb <= 1):.3f}")
    assert np.mean(cheb <= 1) >= 0.6


def _run(form, wl, steps, params=None, train=None, min_cells=None):
    """Initial setup + steps in one form; the learned form gets trained (train), given (params)
    or untrained (neither) weights.  Returns (swarm, faces, fields, psteps, evals, stats, params)."""
    ctx = PicContext(0)
    try:
        ctx.load_workload(wl, form=form)
        p = None
        if form == FORM_LEARNED_FP32:   # the locator belongs to the grid set by load_workload
            if train is not None:
                ctx.locator_train(**train)
            elif params is not None:
                ctx.locator_set_params(params)
            else:
                ctx.locator_init(seed=0)
            if min_cells is not None:
                ctx.locator_min_distance(min_cells)
            p = ctx.locator_get_params()
        ctx.initial_setup()
        for _ in range(steps):
            ctx.step(info=False)
        ctx.synchronize()
        s = ctx.get_swarm()
        faces = ctx.get_faces()
        sc = ctx.get_scattered()
        psteps, evals, _ = ctx.counters()
        stats = ctx.locator_stats() if form == FORM_LEARNED_FP32 else None
        return s, faces, sc, psteps, evals, stats, p
    finally:
        ctx.close()


@pytest.fixture(scope="module")
def pipe_runs(require_gpu):
    wl = W.config_bent_pipe(24, 24, 192, n=300_000, cfl=4.0, materialize=False)
    train = dict(n_samples=1_000_000, seed=7, steps=3000, batch=8192, lr=2e-3)
    learned = _run(FORM_LEARNED_FP32, wl, 4, train=train)
    return wl, {
        "fp32": _run(FORM_FP32, wl, 4),
        "learned": learned,                                                         # default policy
        "learned_all": _run(FORM_LEARNED_FP32, wl, 4, params=learned[6], min_cells=0.0),   # every mover
        "untrained": _run(FORM_LEARNED_FP32, wl, 4, min_cells=0.0),
    }


def _same(a, b):
    sa, fa, ca = a[:3]
    sb, fb, cb = b[:3]
    for f in ("position", "velocity", "weight", "P", "cell", "pid", "status"):
        assert np.array_equal(getattr(sa, f), getattr(sb, f)), f
    for x, y in zip(fa + ca, fb + cb):
        assert np.array_equal(x, y)


def test_learned_form_identical_to_fp32_form(pipe_runs):
    _, r = pipe_runs
    for key in ("learned", "learned_all", "untrained"):
        _same(r["fp32"], r[key])


def test_trained_locator_predicts_the_walk(pipe_runs):
    """The learned form's walk is the reference's, so every form makes the FP32 form's walk
    evaluations whatever the network; what the network gains is the path of the walk from P1 known
    ahead, its rows fetched before the walk reaches them.  With the trained network far more of
    those walks' evaluations lie on the predicted path than with an untrained one."""
    _, r = pipe_runs
    ev = {k: r[k][4] for k in ("fp32", "learned", "learned_all", "untrained")}
    assert len(set(ev.values())) == 1, ev
    frac = {}
    for k in ("learned", "learned_all", "untrained"):
        asked, on_path, walk_evals, unused = r[k][5]
        frac[k] = on_path / max(walk_evals - asked, 1)   # evaluations after P1's
        print(f"[gain] {k}: walks from P1 {asked}, evaluations {walk_evals}, on the predicted path {on_path} "
              f"({frac[k]:.3f} of those after P1)")
        assert unused == 0
    assert frac["learned_all"] > 0.3 and frac["learned_all"] > 2.0 * frac["untrained"]
    assert r["learned"][5][0] < r["learned_all"][5][0]   # the default policy asks fewer particles
