"""GPU: the precision form (FP32 interpolation/advection/deposition, exact walk decisions).

* Cells and statuses: every step, the oracle's FP64 walk is run on the form's own
  positions from the previous cells; cells, statuses and the removed set must match
  exactly.  The form holds a position as a float pair (hi, lo) and advects it by
  double-float addition of fl32(u * dt); the host replays those FP32 operations with
  numpy float32 (IEEE-identical), starting each step from a fresh upload so that both
  sides split the same FP64 values the same way.
* Values: against the plain FP64 oracle run from the same initial state, the relative
  velocity error must stay <= 1e-5 (max over particles present in both), positions
  <= 1e-9 absolute, face deposits <= 1e-5 relative to the face's absolute sum.
"""
import numpy as np
import pytest

from fdf_gb300 import workloads as W
from fdf_gb300.context import FORM_FP32, FORM_PLAIN_FP64, PicContext, SwarmArrays
from oracle import oracle as O
from tests.parity_util import to_oracle_swarm

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(require_gpu):
    c = PicContext(0)
    yield c
    c.close()


def _split(v: np.ndarray):
    h = v.astype(np.float32)
    return h, (v - h.astype(np.float64)).astype(np.float32)


def advect_like_device(s: SwarmArrays, dt: float) -> np.ndarray:
    """(hi, lo) + fl32(u * dt) by the device's double-float addition, returned as hi + lo."""
    f = np.float32
    h, l = _split(s.position)
    v = s.velocity.astype(np.float32) * f(dt)
    sh = h + v
    bv = sh - h
    e = (h - (sh - bv)) + (v - bv)
    t = l + e
    hh = sh + t
    ll = t - (hh - sh)
    return hh.astype(np.float64) + ll.astype(np.float64)


def check_cells_exact(g: O.Grid, pre: SwarmArrays, post: SwarmArrays, dt: float, bbox):
    """Oracle FP64 walk on the form's positions from the previous cells."""
    pos = advect_like_device(pre, dt)
    os_ = O.Swarm.create(pos, cell=pre.cell, pid=pre.pid, status=O.NEEDS_LOCATION)
    err, _ = O.locate_all(g, os_)
    assert err == 0
    bmin, bmax = bbox
    v = os_.view()
    kept = (v["status"] == O.ACTIVE_AND_LOCATED) & np.all((pos >= bmin) & (pos <= bmax), axis=1)
    ref_pid = v["pid"][kept]
    a = post.sorted_by_pid()
    order = np.argsort(ref_pid)
    assert np.array_equal(a.pid, ref_pid[order]), "kept particle sets differ"
    assert np.array_equal(a.cell, v["cell"][kept][order]), "cells differ from the FP64 walk"
    assert np.array_equal(a.position, pos[kept][order]), "positions differ from the FP32-displacement advection"


@pytest.mark.parametrize("wl_args", [
    dict(IM=16, JM=12, KM=40, n=20_000, cfl=0.5, steps=6),
    dict(IM=20, JM=20, KM=48, n=30_000, cfl=4.0, steps=4),
])
def test_fp32_cells_exact_sinusoidal(ctx, wl_args):
    wl = W.config_sinusoidal(**wl_args)
    g = O.Grid(wl.coor)
    bbox = O.bounding_box(g)
    ctx.load_workload(wl, form=FORM_FP32)
    ctx.initial_setup()
    fallbacks = 0
    for _ in range(wl.steps):
        pre = ctx.get_swarm()
        ctx.set_swarm(pre)     # fresh split of the FP64 values, replayed identically on the host
        info = ctx.step()
        fallbacks += info.fp64_fallbacks
        check_cells_exact(g, pre, ctx.get_swarm(), wl.dt, bbox)


def test_fp32_cells_exact_bent_pipe(ctx):
    wl = W.config_bent_pipe(IM=12, JM=12, KM=48, n=20_000, cfl=2.0, steps=4)
    g = O.Grid(wl.coor)
    bbox = O.bounding_box(g)
    ctx.load_workload(wl, form=FORM_FP32)
    ctx.initial_setup()
    for _ in range(wl.steps):
        pre = ctx.get_swarm()
        ctx.set_swarm(pre)
        ctx.step()
        check_cells_exact(g, pre, ctx.get_swarm(), wl.dt, bbox)


def test_fp32_errors_against_fp64_oracle(ctx, capsys):
    wl = W.config_sinusoidal(IM=24, JM=24, KM=96, n=40_000, cfl=0.5, steps=10)
    ctx.load_workload(wl, form=FORM_FP32)
    ctx.set_momentum_deposit(True)
    ctx.initial_setup()
    ctx.steps(wl.steps)
    gpu = ctx.get_swarm().sorted_by_pid()
    gfi, gfj, gfk = ctx.get_faces()
    # plain FP64 oracle from the same initial state
    g = O.Grid(wl.coor)
    os_ = to_oracle_swarm(SwarmArrays.create(wl.pos, cell=wl.cell0))
    sim = O.Simulation(g, wl.ucat_node_sized(), os_, wl.dt)
    sim.initial_setup()
    for _ in range(wl.steps):
        sim.step()
    ref = os_.sorted_by_pid()
    common, ia, ib = np.intersect1d(gpu.pid, ref["pid"], return_indices=True)
    assert len(common) >= 0.99 * max(gpu.n, len(ref["pid"]))
    du = gpu.velocity[ia] - ref["vel"][ib]
    umag = np.linalg.norm(ref["vel"][ib], axis=1, keepdims=True)
    rel_u = np.abs(du) / np.maximum(umag, 1e-30)
    dx = np.abs(gpu.position[ia] - ref["pos"][ib])
    same_cell = np.all(gpu.cell[ia] == ref["cell"][ib], axis=1)
    with capsys.disabled():
        print(f"\n[fp32 form vs FP64 oracle, {len(common)} particles, {wl.steps} steps] "
              f"velocity rel err max {rel_u.max():.3e} rms {np.sqrt((rel_u ** 2).mean()):.3e}; "
              f"position abs err max {dx.max():.3e} rms {np.sqrt((dx ** 2).mean()):.3e}; "
              f"same cell {same_cell.mean():.6f}")
    assert rel_u.max() <= 1e-5
    umax = float(np.sqrt((wl.ucat ** 2).sum(-1)).max())
    assert dx.max() <= 1e-6 * wl.steps * wl.dt * umax
    f = O.deposit_faces(g, os_, volume=wl.volume, momentum=True)
    for gf, key, akey in zip((gfi, gfj, gfk), ("fi", "fj", "fk"), ("abs_i", "abs_j", "abs_k")):
        err = np.abs(gf - f[key])
        assert np.all(err <= 1e-5 * f[akey] + 1e-6), key
    # momentum: the volume bound scaled by max |u| (err <= 1e-5 |V| umax + 1e-6 umax per face)
    worst = 0.0
    for gm, key, akey in zip(ctx.get_face_momentum(), ("mom_i", "mom_j", "mom_k"), ("abs_i", "abs_j", "abs_k")):
        err = np.abs(gm - f[key]).max(axis=-1)
        worst = max(worst, float((err / (umax * (f[akey] + 0.1))).max()))
    with capsys.disabled():
        print(f"[fp32 form momentum deposit] max err / (umax (|V| + 0.1)) {worst:.3e}")
    assert worst <= 1e-5
    ctx.set_momentum_deposit(False)


def test_fp32_conservation_and_determinism(ctx):
    wl = W.config_sinusoidal(IM=16, JM=16, KM=32, n=50_000, cfl=1.0, steps=3)
    outs = []
    for _ in range(2):
        ctx.load_workload(wl, form=FORM_FP32)
        ctx.initial_setup()
        ctx.steps(wl.steps)
        s = ctx.get_swarm()
        outs.append((s, ctx.get_faces(), ctx.get_scattered()))
    (s1, f1, c1), (s2, f2, c2) = outs
    for name in ("position", "velocity", "weight", "cell", "pid"):
        assert np.array_equal(getattr(s1, name), getattr(s2, name)), name
    for a, b in zip(f1 + c1, f2 + c2):
        assert np.array_equal(a, b)
    tot = sum(x.sum() for x in f1)
    assert abs(tot - s1.n) <= 1e-4 * s1.n
    assert c1[0].sum() == s1.n
    ctx.set_form(FORM_PLAIN_FP64)


def _ksum(vals):
    """Neumaier-compensated float32 sum in the given order (the deposit kernel's KSum)."""
    f = np.float32
    s, c = f(0.0), f(0.0)
    for v in vals:
        t = f(s + v)
        c = f(c + (f(f(s - t) + v) if abs(s) >= abs(v) else f(f(v - t) + s)))
        s = t
    return f(s + c)


def test_fp32_deposit_matches_host_restatement(ctx):
    """The FP32 deposit (warp-staged kernel) against the same float32 arithmetic on the host:
    particles in the swarm's held order (by cell; within a cell, the precision form keeps the
    previous order), each face summing its lower cell's a V/3 then
    its own cell's (1 - a) V/3 with Neumaier compensation; count and P average per cell.  Every
    value must be bit-identical."""
    wl = W.config_sinusoidal(IM=32, JM=6, KM=12, n=20_000, cfl=1.0, steps=3)   # 33 nodes per row: a warp starts at i = IM
    ctx.load_workload(wl, form=FORM_FP32)
    ctx.initial_setup()
    ctx.steps(wl.steps)
    s = ctx.get_swarm()
    fi, fj, fk = ctx.get_faces()
    cnt, avg = ctx.get_scattered()
    IM, JM, KM = wl.dims
    lin = (s.cell[:, 2] * JM + s.cell[:, 1]) * IM + s.cell[:, 0]
    assert np.all(np.diff(lin) >= 0), "the swarm is held in cell order"
    seg = {}
    for c in np.unique(lin):
        idx = np.nonzero(lin == c)[0]
        seg[int(c)] = idx
    a = s.weight.astype(np.float32)
    P = s.P.astype(np.float32)
    third = np.float32(wl.volume / 3.0)
    cid = lambda i, j, k: (k * JM + j) * IM + i
    empty = np.zeros(0, dtype=np.int64)

    def face(d, lower, upper):
        vals = [np.float32(a[p, d] * third) for p in (seg.get(lower, empty) if lower is not None else empty)]
        vals += [np.float32(np.float32(1.0 - a[p, d]) * third) for p in (seg.get(upper, empty) if upper is not None else empty)]
        return _ksum(vals)

    for k in range(KM):
        for j in range(JM):
            for i in range(IM + 1):
                want = face(0, cid(i - 1, j, k) if i > 0 else None, cid(i, j, k) if i < IM else None)
                assert np.float32(fi[k, j, i]) == want, ("fi", i, j, k)
    for k in range(KM):
        for j in range(JM + 1):
            for i in range(IM):
                want = face(1, cid(i, j - 1, k) if j > 0 else None, cid(i, j, k) if j < JM else None)
                assert np.float32(fj[k, j, i]) == want, ("fj", i, j, k)
    for k in range(KM + 1):
        for j in range(JM):
            for i in range(IM):
                want = face(2, cid(i, j, k - 1) if k > 0 else None, cid(i, j, k) if k < KM else None)
                assert np.float32(fk[k, j, i]) == want, ("fk", i, j, k)
    for c, idx in seg.items():
        i, j, k = c % IM, (c // IM) % JM, c // (IM * JM)
        assert cnt[k, j, i] == len(idx)
        assert np.float32(avg[k, j, i]) == np.float32(_ksum([P[p] for p in idx]) / np.float32(len(idx)))
