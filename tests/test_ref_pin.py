"""The CPU restatement (oracle/picurv_oracle.c) against the reference's own code.

oracle/_ref/libpicurv_ref.so is the reference's walkingsearch.c, ParticleSwarm.c,
interpolation.c, ParticleMotion.c, grid.c and setup.c compiled unmodified (oracle/ref_build.py)
against a one-rank PETSc stand-in (tests/petsc_stub).  Every comparison is bit for bit: the
per-cell functions on random and degenerate cells, single-point walks from every kind of start
cell, and whole runs (initial setup, then steps of reset, advection, location, removals,
interpolation and scatter) on each grid family.  Skipped where the reference's sources are
not present; tests/golden/ carries vectors written by the same library for those machines.
"""
import numpy as np
import pytest

from fdf_gb300 import workloads as W
from fdf_gb300.context import SwarmArrays
from oracle import oracle as O
from oracle import ref as R

pytestmark = pytest.mark.skipif(not R.available(), reason="the reference's sources are not present")


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.int64)


def _random_cells(rng, n, amp):
    """Unit cubes with every vertex moved by up to amp (some nearly degenerate)."""
    base = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 1, 1], [1, 1, 1], [1, 0, 1], [0, 0, 1]], float)
    cells = base[None] + rng.uniform(-amp, amp, size=(n, 8, 3))
    scale = 10.0 ** rng.uniform(-6, 3, size=(n, 1, 1))
    return cells * scale + rng.uniform(-5, 5, size=(n, 1, 3))


def test_per_cell_functions_match_the_reference():
    rng = np.random.default_rng(7)
    L = O.lib()
    cells = _random_cells(rng, 4000, 0.35)
    for q, v in enumerate(cells):
        lo, hi = v.min(0), v.max(0)
        p = rng.uniform(lo - 0.2 * (hi - lo), hi + 0.2 * (hi - lo))
        if q % 5 == 0:   # a point on a face: the mean of one face's vertices
            f = [(0, 3, 2, 1), (4, 7, 6, 5), (0, 1, 6, 7), (3, 4, 5, 2), (0, 7, 4, 3), (1, 2, 5, 6)][q % 6]
            p = v[list(f)].mean(0)
        h_ref = R.characteristic_size(v)
        h = np.zeros(1)
        assert L.o_GetCellCharacteristicSize(O.cell_from_vertices(v), O._dp(h)) == 0
        assert _bits(h[0]) == _bits(h_ref), q
        thr = 1e-11 * h_ref
        rc_ref, d_ref, pos_ref = R.evaluate_position(v, p, thr)
        d = np.zeros(6)
        pos = np.zeros(1, dtype=np.int64)
        rc = L.o_EvaluateParticlePosition(O.cell_from_vertices(v), O._dp(d), O.cmp(p), O._ip(pos), thr)
        assert rc == rc_ref, q
        if rc:
            continue
        assert np.array_equal(_bits(d), _bits(d_ref)) and pos[0] == pos_ref, q
        # index update and weights from these distances
        ijk = rng.integers(-3, 50, 3)
        i, j, k = (np.array([x], dtype=np.int64) for x in ijk)
        dd = d.copy()
        L.o_UpdateCellIndicesBasedOnDistancesTEST(O._dp(dd), O._ip(i), O._ip(j), O._ip(k))
        assert [i[0], j[0], k[0]] == list(R.update_indices(d, ijk)), q
        w_ref, dmut_ref = R.update_weights(d)
        w, dmut = np.zeros(3), d.copy()
        L.o_UpdateParticleWeights(O._dp(dmut), O._dp(w))
        assert np.array_equal(_bits(w), _bits(w_ref)) and np.array_equal(_bits(dmut), _bits(dmut_ref)), q
        # one face through ComputeSignedDistanceToPlane
        cc = v.mean(0)
        rc_ref, dp_ref = R.signed_distance(v[0], v[3], v[2], v[1], cc, p, thr)
        dp = np.zeros(1)
        rc = L.o_ComputeSignedDistanceToPlane(*[O.cmp(x) for x in (v[0], v[3], v[2], v[1], cc, p)], O._dp(dp), thr)
        assert rc == rc_ref and (rc or _bits(dp[0]) == _bits(dp_ref)), q


def test_degenerate_cells_fail_like_the_reference():
    L = O.lib()
    for v in (np.zeros((8, 3)), np.tile([[1.0, 2.0, 3.0]], (8, 1))):
        rc_ref, _, _ = R.evaluate_position(v, [0.5, 0.5, 0.5], 1e-14)
        d = np.zeros(6)
        pos = np.zeros(1, dtype=np.int64)
        rc = L.o_EvaluateParticlePosition(O.cell_from_vertices(v), O._dp(d), O.cmp([0.5, 0.5, 0.5]), O._ip(pos),
                                          1e-14)
        assert rc == rc_ref == O.ERR_USER


def test_determine_point_position_on_random_distance_sets():
    rng = np.random.default_rng(3)
    L = O.lib()
    res = np.zeros(1, dtype=np.int64)
    for _ in range(3000):
        d = rng.choice([-1.0, 0.0, 1.0, -1e-300, 1e-300], size=6)
        L.o_DeterminePointPosition(O._dp(d.copy()), O._ip(res))
        assert res[0] == R.point_position(d), d


GRIDS = {
    "sinusoidal": lambda: W.sinusoidal_grid(10, 8, 24),
    "bent_pipe": lambda: W.bent_pipe_grid(8, 6, 20),
    "curved_pipe": lambda: W.curved_pipe_grid(8, 8, 24),
    "uniform": lambda: W.uniform_grid(5, 4, 12),
}


@pytest.mark.parametrize("family", sorted(GRIDS))
def test_single_point_walks_match_the_reference(family):
    coor = GRIDS[family]()
    KM, JM, IM = (s - 1 for s in coor.shape[:3])
    g = O.Grid(coor)
    sim = R.RefSim(coor)
    rng = np.random.default_rng(11)
    lo, hi = coor.reshape(-1, 3).min(0), coor.reshape(-1, 3).max(0)
    pts = rng.uniform(lo - 0.05 * (hi - lo), hi + 0.05 * (hi - lo), size=(700, 3))
    pts[:100] = coor.reshape(-1, 3)[rng.integers(0, coor.reshape(-1, 3).shape[0], 100)]   # grid nodes
    starts = np.stack([rng.integers(-2, IM + 2, 700), rng.integers(-2, JM + 2, 700), rng.integers(-2, KM + 2, 700)], 1)
    starts[::7] = -1
    starts[3::11] = [1 << 33, 0, 0]
    for p in range(len(pts)):
        a = sim.locate_point(pts[p], starts[p])
        b = O.locate_particle(g, pts[p], starts[p])
        assert a["err"] == b["err"], p
        assert np.array_equal(a["cell"], b["cell"]) and a["status"] == b["status"], p
        assert np.array_equal(_bits(a["weights"]), _bits(b["weights"])), p


def test_max_traversal_from_the_corner_matches_the_reference():
    """walkingsearch.c:10,1123: from the corner cell a walk makes at most 1000 evaluations."""
    coor = W.uniform_grid(1, 1, 1100)
    g = O.Grid(coor)
    sim = R.RefSim(coor)
    for k in (998, 999, 1000, 1050):
        p = [0.5, 0.5, (k + 0.5) / 1100]
        a, b = sim.locate_point(p), O.locate_particle(g, p)
        assert np.array_equal(a["cell"], b["cell"]) and a["status"] == b["status"], k
    assert sim.locate_point([0.5, 0.5, 999.5 / 1100])["status"] == O.ACTIVE_AND_LOCATED
    assert sim.locate_point([0.5, 0.5, 1000.5 / 1100])["status"] == O.LOST


def _run_both(wl, steps):
    s0 = SwarmArrays.create(wl.pos, cell=wl.cell0)
    sim = R.RefSim(wl.coor, wl.ucat_node_sized(), wl.dt)
    sim.set_swarm(s0.position, s0.velocity, s0.weight, s0.P, s0.cell, s0.pid, s0.status)
    os_ = O.Swarm(pos=s0.position.copy(), vel=s0.velocity.copy(), weight=s0.weight.copy(), P=s0.P.copy(),
                  cell=s0.cell.copy(), pid=s0.pid.copy(), status=s0.status.copy(), n=s0.n)
    osim = O.Simulation(O.Grid(wl.coor), wl.ucat_node_sized(), os_, wl.dt, nthreads=1)
    sim.initial_setup()
    osim.initial_setup()
    yield "initial setup", sim, osim, os_, None
    for k in range(steps):
        removed = sim.step()
        info = osim.step()
        yield f"step {k + 1}", sim, osim, os_, (removed, (info.removed_lost, info.removed_oob))


WORKLOADS = {
    "sinusoidal_cfl1": lambda: W.config_sinusoidal(IM=10, JM=8, KM=24, n=3000, cfl=1.0, steps=4),
    "sinusoidal_cfl4": lambda: W.config_sinusoidal(IM=12, JM=10, KM=20, n=2000, cfl=4.0, steps=4),
    "bent_pipe_cfl4": lambda: W.config_bent_pipe(8, 6, 20, n=2000, cfl=4.0),
    "curved_pipe": lambda: W.config_curved_pipe(8, 8, 24, n=2000, cfl=1.0),
    "uniform_corner_start": lambda: W.config1(n=800, IM=5, JM=4, KM=40, steps=4),
}


@pytest.mark.parametrize("name", sorted(WORKLOADS))
def test_runs_match_the_reference(name):
    wl = WORKLOADS[name]()
    for what, sim, osim, os_, removed in _run_both(wl, 4):
        a, b = sim.swarm().sorted_by_pid(), os_.sorted_by_pid()
        assert a.n == len(b["pid"]), what
        if removed is not None:
            assert removed[0] == removed[1], what
        for f in ("cell", "pid", "status"):
            assert np.array_equal(getattr(a, f), b[f]), (what, f)
        for f in ("pos", "vel", "weight", "P"):
            assert np.array_equal(_bits(getattr(a, f)), _bits(b[f])), (what, f)
        c, p = sim.scattered()
        assert np.array_equal(_bits(c), _bits(osim.count)), what
        assert np.array_equal(_bits(p), _bits(osim.avg)), what


def test_bounding_box_matches_the_reference():
    for family, make in GRIDS.items():
        coor = make()
        lo, hi = O.bounding_box(O.Grid(coor))
        bb = R.RefSim(coor).bbox()
        assert np.array_equal(_bits(bb), _bits(np.concatenate([lo, hi]))), family
