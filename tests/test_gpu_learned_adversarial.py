"""GPU: the learned form against the oracle on inputs built to separate a walk that starts at a
learned guess from the reference's own walk.

* On-face acceptance along the path: the reference accepts a cell whenever the point lies within
  1e-11 h of the *extended* plane of one of its faces, even though another face says outside
  (walkingsearch.c:427-459).  Points are moved onto the extended plane of a face of a cell the
  reference walk evaluates after P1 (its third evaluation or later), so that the reference stops
  there, away from the cell that contains the point.
* k-face gaps: on a curved grid the k-lower face of cell k and the k-upper face of cell k-1 are
  different planes (walkingsearch.c:303-325); a point between them makes the reference walk
  alternate until MAX_TRAVERSAL and end LOST.

Every particle ends in the oracle's cell with the oracle's status (the oracle walks the same
float-pair positions the precision forms hold), and the FP32 form agrees, whatever the network
guessed."""
import numpy as np
import pytest

from fdf_gb300 import workloads as W
from fdf_gb300.context import FORM_FP32, FORM_LEARNED_FP32, PicContext, SwarmArrays
from oracle import oracle as O

pytestmark = pytest.mark.gpu

FACES = {0: (0, 7, 4, 3), 1: (1, 2, 5, 6), 2: (0, 1, 6, 7), 3: (3, 4, 5, 2), 4: (4, 7, 6, 5), 5: (0, 3, 2, 1)}
OFF = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 1, 1], [1, 1, 1], [1, 0, 1], [0, 0, 1]])


def _verts(coor, i, j, k):
    return np.array([coor[k + o[2], j + o[1], i + o[0]] for o in OFF])


def _pair(x):
    """The precision forms' position: the float pair (hi, lo) of x, as a double."""
    hi = np.float32(x)
    lo = np.float32(x - np.float64(hi))
    return np.float64(hi) + np.float64(lo)


def _walk(g, coor, p, start, limit=1000):
    """The reference walk with the oracle's per-cell functions: (evaluated cells, last position code)."""
    L = O.lib()
    KM, JM, IM = (s - 1 for s in coor.shape[:3])
    i, j, k = start
    path, pos = [], -1
    d = np.zeros(6)
    code = np.zeros(1, dtype=np.int64)
    for _ in range(limit):
        if not (0 <= i < IM and 0 <= j < JM and 0 <= k < KM):
            break
        path.append((i, j, k))
        L.o_EvaluateParticlePosition(O.cell_from_vertices(_verts(coor, i, j, k)), O._dp(d), O.cmp(p), O._ip(code),
                                     1e-11)
        pos = int(code[0])
        if pos >= 0:
            break
        ii, jj, kk = (np.array([x], dtype=np.int64) for x in (i, j, k))
        L.o_UpdateCellIndicesBasedOnDistancesTEST(O._dp(d), O._ip(ii), O._ip(jj), O._ip(kk))
        i, j, k = int(ii[0]), int(jj[0]), int(kk[0])
    return path, pos


def _on_face_cases(coor, rng, want):
    """Points on the extended plane of a face of the reference path's third-or-later cell, where
    the reference then stops (accepted on the face while outside another face)."""
    g = O.Grid(coor)
    KM, JM, IM = (s - 1 for s in coor.shape[:3])
    pts, starts = [], []
    tries = 0
    while len(pts) < want and tries < 200 * want:
        tries += 1
        c0 = np.array([rng.integers(1, IM - 1), rng.integers(1, JM - 1), rng.integers(2, KM - 6)])
        c1 = c0 + np.array([rng.integers(-1, 2), rng.integers(-1, 2), rng.integers(3, 6)])
        lo, hi = _verts(coor, *c1).min(0), _verts(coor, *c1).max(0)
        p = rng.uniform(lo, hi)
        path, pos = _walk(g, coor, p, tuple(c0))
        if pos != 0 or len(path) < 4:
            continue
        X = path[rng.integers(2, len(path) - 1)]          # evaluated after P1, before the last cell
        v = _verts(coor, *X)
        cc = v.mean(0)
        f = int(rng.integers(0, 6))
        a, b, c, e = (v[q] for q in FACES[f])
        n = np.cross(b - a, e - a)
        fc = 0.25 * (a + b + c + e)
        if np.dot(n, cc - fc) > 1e-9:
            n = -n
        n /= np.linalg.norm(n)
        q = np.array([_pair(x) for x in p + np.dot(fc - p, n) * n])
        qpath, qpos = _walk(g, coor, q, tuple(c0))
        if qpos >= 1 and len(qpath) >= 3:                 # the reference stops on a face
            pts.append(q)
            starts.append(c0)
    return np.array(pts), np.array(starts)


def _k_gap_cases(coor, rng, want):
    """Points between the k-lower face plane of cell k and the k-upper face plane of cell k-1."""
    L = O.lib()
    KM, JM, IM = (s - 1 for s in coor.shape[:3])
    pts, starts = [], []
    d_up, d_lo = np.zeros(6), np.zeros(6)
    for _ in range(400 * want):
        if len(pts) >= want:
            break
        i, j, k = rng.integers(0, IM), rng.integers(0, JM), rng.integers(1, KM)
        vu, vl = _verts(coor, i, j, k), _verts(coor, i, j, k - 1)
        fc = vu[[0, 3, 2, 1]].mean(0) + rng.uniform(-0.3, 0.3, 3) * (vu[1] - vu[0] + vu[3] - vu[0])
        nz = vu[7] - vu[0]
        nz /= np.linalg.norm(nz)
        h = np.linalg.norm(vu[7] - vu[0])
        for t in np.linspace(-2e-3, 2e-3, 41) * h:
            p = np.array([_pair(x) for x in fc + t * nz])
            L.o_CalculateDistancesToCellFaces(O.cmp(p), O.cell_from_vertices(vu), O._dp(d_up), 1e-15)
            L.o_CalculateDistancesToCellFaces(O.cmp(p), O.cell_from_vertices(vl), O._dp(d_lo), 1e-15)
            if d_up[5] < 0 and d_lo[4] < 0:                # outside both: in the gap
                pts.append(p)
                starts.append((i, j, max(k - 4, 0)))
                break
    return np.array(pts), np.array(starts)


def _locate(form, coor, pts, starts, params=None):
    wl = W.config_sinusoidal(IM=coor.shape[2] - 1, JM=coor.shape[1] - 1, KM=coor.shape[0] - 1, n=10, cfl=1.0,
                             steps=1)
    with PicContext(0) as ctx:
        ctx.set_form(form)
        ctx.set_grid(coor)
        ctx.set_ucat(wl.ucat)
        ctx.set_dt(0.0)
        if form == FORM_LEARNED_FP32:
            if params is None:
                ctx.locator_train(100_000, seed=3, steps=3000, batch=4096, lr=3e-3)
                params = ctx.locator_get_params()
            else:
                ctx.locator_set_params(params)
            ctx.locator_min_distance(0.0)                 # every particle that leaves its cell asks
        s = SwarmArrays.create(pts, cell=starts, status=0)
        ctx.set_swarm(s)
        ctx.locate()
        out = ctx.get_swarm().sorted_by_pid()
        asked = ctx.locator_stats()[0] if form == FORM_LEARNED_FP32 else 0
    return out, params, asked


def test_learned_form_matches_the_oracle_on_adversarial_points(require_gpu):
    coor = W.sinusoidal_grid(16, 12, 48, amp=0.08)
    g = O.Grid(coor)
    rng = np.random.default_rng(31)
    on_face, s1 = _on_face_cases(coor, rng, 60)
    gaps, s2 = _k_gap_cases(coor, rng, 40)
    assert len(on_face) >= 30 and len(gaps) >= 20, (len(on_face), len(gaps))
    pts = np.concatenate([on_face, gaps])
    starts = np.concatenate([s1, s2]).astype(np.int64)
    learned, params, asked = _locate(FORM_LEARNED_FP32, coor, pts, starts)
    fp32, _, _ = _locate(FORM_FP32, coor, pts, starts)
    assert asked > 0
    mism = []
    for p in range(len(pts)):
        r = O.locate_particle(g, pts[p], starts[p])
        if not (np.array_equal(learned.cell[p], r["cell"]) and learned.status[p] == r["status"]):
            mism.append((p, learned.cell[p].tolist(), r["cell"].tolist()))
        assert np.array_equal(fp32.cell[p], r["cell"]) and fp32.status[p] == r["status"], p
    assert not mism, f"{len(mism)} of {len(pts)} differ from the reference walk: {mism[:5]}"
    # the cases do what they are built for: the reference stops on a face, or ends LOST in a gap
    assert (learned.status[len(on_face):] == 3).sum() >= len(gaps) // 2
