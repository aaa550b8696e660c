"""CPU: the error bound behind the walk's FP32 face decisions (fdf_walk.cuh), restated in numpy.

The kernel keeps per cell a 128-B row -- the first vertex c0 as a float pair, thr32, an
absolute slack of 32 eps sigma, and per face n32 = fl32(n), e32 = fl32(n . (fc - c0)) -- and
decides a face from d32 = e32 - n32 . pr when |d32| exceeds M = 4u S32 + thr32 + slack.  This
test builds those rows for cells of curved grids, emulates the kernel's FP32 arithmetic (each
operation rounded to float32; a fused multiply-add as the float64 result rounded once more,
which can differ from the hardware's by one unit in rare cases, hence 1.5 below where the
analysis has 1) and compares d32 with the reference's FP64 distance d64 = (fc - p) . n in the
reference's operation order, for points around the cell and points put within a few ulps of a
face plane:

* |d32 - d64| <= 1.5 u S32 + 23 eps sigma (the analysis gives u S (1 + 12u) + 23 eps sigma),
  also next to the first vertex, where E and P vanish for three faces and the slack carries
  the FP64 roundings, and
* every class the FP32 rule decides is d64's class: d32 > M -> d64 >= thr, d32 < -M -> d64 <= -thr.
"""
import numpy as np
import pytest

from fdf_gb300 import workloads as W

F = np.float32
U = 2.0 ** -24
EPS = 2.0 ** -53
# vertex order of a cell (offsets in i, j, k) and the four vertices of each face LEFT..BACK
OFF = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 1, 1], [1, 1, 1], [1, 0, 1], [0, 0, 1]])
FACES = [(0, 7, 4, 3), (1, 2, 5, 6), (0, 1, 6, 7), (3, 4, 5, 2), (4, 7, 6, 5), (0, 3, 2, 1)]


def f32(x):
    return np.asarray(x, dtype=np.float64).astype(F)


def fma32(a, b, c):
    return f32(a.astype(np.float64) * b.astype(np.float64) + c.astype(np.float64))


def planes_of(v):
    """Face centres and unit normals (pointing into the cell) of cells v [n][8][3]."""
    cc = v.mean(axis=1)
    fcs, ns = [], []
    for f in FACES:
        a, b, c, d = (v[:, q] for q in f)
        fc = 0.25 * (a + b + c + d)
        n = np.cross(c - a, d - b)
        n /= np.linalg.norm(n, axis=1, keepdims=True)
        n = np.where((np.einsum("ij,ij->i", n, cc - fc) < 0)[:, None], -n, n)
        fcs.append(fc)
        ns.append(n)
    return np.stack(fcs, 1), np.stack(ns, 1)


def rows_of(v, fc, n, thr):
    """The kernel's row fields (k_build_table32)."""
    v0 = v[:, 0]
    c0h = f32(v0)
    c0l = f32(v0 - c0h.astype(np.float64))
    c0 = c0h.astype(np.float64) + c0l.astype(np.float64)
    dd = fc - c0[:, None, :]
    e = (dd[..., 0] * n[..., 0] + dd[..., 1] * n[..., 1]) + dd[..., 2] * n[..., 2]
    sigma = np.max(np.sum(np.abs(dd) * np.abs(n), axis=2), axis=1)
    thr32 = np.nextafter(f32(thr * (1.0 + 2.0 ** -22)), F(np.inf))   # rounded up
    slack = np.nextafter(f32(sigma * 2.0 ** -48), F(np.inf))
    return c0h, c0l, thr32, slack, f32(n), f32(e), sigma


def kernel_d32(p, c0h, c0l, thr32, slack, n32, e32):
    """d32, S32, M of every face for positions p [n][3] (FP64), as eval_cell32 computes them."""
    ph = f32(p)
    pl = f32(p - ph.astype(np.float64))
    pr = f32(f32(ph - c0h) + f32(pl - c0l))
    a = fma32(f32(np.abs(ph) + np.abs(c0h)), np.full_like(ph, F(U)), np.abs(pr))
    base = f32(thr32 + slack)
    pr_, a_ = pr[:, None, :], a[:, None, :]
    dot = fma32(n32[..., 2], pr_[..., 2], fma32(n32[..., 1], pr_[..., 1], f32(n32[..., 0] * pr_[..., 0])))
    d32 = f32(e32 - dot)
    inner = fma32(np.abs(n32[..., 2]), a_[..., 2],
                  fma32(np.abs(n32[..., 1]), a_[..., 1], f32(np.abs(n32[..., 0]) * a_[..., 0])))
    S = fma32(np.full_like(inner, F(7.0)), inner, f32(np.abs(e32) + np.abs(e32)))
    M = fma32(S, np.full_like(S, F(4 * U)), np.broadcast_to(base[:, None], S.shape))
    return d32, S, M, ph.astype(np.float64) + pl.astype(np.float64)


def reference_d64(x, fc, n):
    """(fc - x) . n in the reference's operation order (FP64)."""
    x_ = x[:, None, :]
    return ((fc[..., 0] - x_[..., 0]) * n[..., 0] + (fc[..., 1] - x_[..., 1]) * n[..., 1]) \
        + (fc[..., 2] - x_[..., 2]) * n[..., 2]


@pytest.mark.parametrize("grid", ["sinusoidal", "bent_pipe"])
def test_fp32_face_bound(grid):
    coor = W.sinusoidal_grid(24, 20, 64, amp=0.08) if grid == "sinusoidal" else W.bent_pipe_grid(16, 16, 96)
    KM, JM, IM = (s - 1 for s in coor.shape[:3])
    rng = np.random.default_rng(17)
    ncell = 4000
    ijk = np.stack([rng.integers(0, IM, ncell), rng.integers(0, JM, ncell), rng.integers(0, KM, ncell)], 1)
    v = np.stack([coor[ijk[:, 2] + o[2], ijk[:, 1] + o[1], ijk[:, 0] + o[0]] for o in OFF], 1)
    fc, n = planes_of(v)
    h = np.linalg.norm(v[:, 6] - v[:, 0], axis=1)
    thr = 1e-11 * h
    c0h, c0l, thr32, slack, n32, e32, sigma = rows_of(v, fc, n, thr)
    worst, decided, total = 0.0, 0, 0
    for trial in range(10):
        if trial < 4:   # anywhere within about two cells of the cell
            lo, hi = v.min(1), v.max(1)
            p = lo + rng.uniform(-1.0, 2.0, lo.shape) * (hi - lo)
        elif trial < 6:  # next to the first vertex: E and P near zero for its three faces, the slack's case
            p = v[:, 0] + rng.standard_normal((ncell, 3)) * (1e-9 * h)[:, None]
        else:           # within a few ulps of a face plane (the decisions the bound must leave open)
            f = rng.integers(0, 6, ncell)
            nf, fcf = n[np.arange(ncell), f], fc[np.arange(ncell), f]
            t = rng.standard_normal((ncell, 3))
            t -= np.einsum("ij,ij->i", t, nf)[:, None] * nf
            p = fcf + 0.3 * h[:, None] * t + (rng.integers(-40, 41, ncell) * 2.0 ** -50 * h)[:, None] * nf
        d32, S, M, x = kernel_d32(p, c0h, c0l, thr32, slack, n32, e32)
        d64 = reference_d64(x, fc, n)
        err = np.abs(d32.astype(np.float64) - d64)
        bound = 1.5 * U * S.astype(np.float64) + 23 * EPS * sigma[:, None]
        assert np.all(err <= bound), float(np.max(err / bound))
        worst = max(worst, float(np.max(err / (U * S.astype(np.float64) + 23 * EPS * sigma[:, None]))))
        pos, neg = d32 > M, d32 < -M
        assert np.all(d64[pos] >= thr[:, None].repeat(6, 1)[pos])
        assert np.all(d64[neg] <= -thr[:, None].repeat(6, 1)[neg])
        decided += int(pos.sum() + neg.sum())
        total += d32.size
    print(f"[bound {grid}] worst |d32 - d64| / (u S32 + 23 eps sigma) = {worst:.3f}; "
          f"FP32-decided faces {decided / total:.6f}")
    assert worst <= 1.5
    assert decided / total > 0.4   # the near-plane and near-vertex points are meant to be undecidable
