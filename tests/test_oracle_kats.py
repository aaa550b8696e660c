"""Known-answer tests pinning the CPU oracle (oracle/picurv_oracle.c).

The reference ships no test vectors for this path; these cases are derived
from its logic (file:line in each docstring) and from the two scenarios of its
old walking-search harness (old/test_walkingsearch.c:69-121).
"""
import numpy as np
import pytest

from fdf_gb300 import workloads as W
from oracle import oracle as O
from tests import pyref


def unit_grid(IM=1, JM=1, KM=1):
    return O.Grid(W.uniform_grid(IM, JM, KM))


def test_unit_cube_centre():
    """Centre of the unit cube: cell (0,0,0), weights 0.5 (ParticleSwarm.c:1039-1041)."""
    g = unit_grid()
    r = O.locate_particle(g, [0.5, 0.5, 0.5])
    assert r["err"] == 0 and r["status"] == O.ACTIVE_AND_LOCATED
    assert list(r["cell"]) == [0, 0, 0]
    assert np.array_equal(r["weights"], [0.5, 0.5, 0.5])
    assert r["steps"] == 1


def test_old_harness_boundary_toggle():
    """old/test_walkingsearch.c:99-121: x = 0.9999999999999 on a 1x1x1 grid is located in cell 0."""
    g = unit_grid()
    r = O.locate_particle(g, [0.9999999999999, 0.5, 0.5])
    assert r["status"] == O.ACTIVE_AND_LOCATED and list(r["cell"]) == [0, 0, 0]


def test_old_harness_degenerate_plane():
    """old/test_walkingsearch.c:69-95 and walkingsearch.c:147-155: all vertices equal -> PETSC_ERR_USER."""
    L = O.lib()
    cell = O.cell_from_vertices(np.zeros((8, 3)))
    d = np.zeros(6)
    err = L.o_CalculateDistancesToCellFaces(O.cmp([0, 0, 0]), cell, O._dp(d), 1e-14)
    assert err == O.ERR_USER


def test_degenerate_cell_aborts_walk():
    """A walk that evaluates a degenerate cell returns PETSC_ERR_USER (CHKERRQ at walkingsearch.c:1193)."""
    coor = W.uniform_grid(2, 1, 1)
    coor[:, :, 0, :] = coor[:, :, 1, :]     # collapse the i=0 cell
    g = O.Grid(coor)
    r = O.locate_particle(g, [0.75, 0.5, 0.5])
    assert r["err"] == O.ERR_USER


def test_determine_point_position_quirk():
    """walkingsearch.c:427-459: on one face but outside another is still accepted (result 1)."""
    L = O.lib()
    res = np.zeros(1, dtype=np.int64)
    for d, want in [([-1.0, 0.0, 1, 1, 1, 1], 1), ([1, 1, 1, 1, 1, 1], 0), ([-1, 1, 1, 1, 1, 1], -1),
                    ([0.0, 0.0, 1, 1, 1, -1], 2), ([0.0, 0.0, 0.0, 1, 1, -1], 3), ([0.0] * 6, 0)]:
        L.o_DeterminePointPosition(O._dp(np.array(d, dtype=np.float64)), O._ip(res))
        assert res[0] == want, d


def test_update_cell_indices_priority():
    """walkingsearch.c:919-946: k then i then j, 'else if' priority, no clamping."""
    L = O.lib()
    i, j, k = (np.array([5], dtype=np.int64) for _ in range(3))
    d = np.array([-1.0, -1.0, -1.0, -1.0, -1.0, -1.0])   # LEFT, BOTTOM, FRONT win their pairs
    L.o_UpdateCellIndicesBasedOnDistancesTEST(O._dp(d), O._ip(i), O._ip(j), O._ip(k))
    assert (i[0], j[0], k[0]) == (4, 4, 6)


def test_weights_clamp_mutates_distances():
    """ParticleSwarm.c:1020-1027: every d <= 1e-14 becomes 1e-14 before the ratios."""
    L = O.lib()
    d = np.array([0.0, 2.0, -3.0, 1.0, 1e-15, 4.0])
    w = np.zeros(3)
    L.o_UpdateParticleWeights(O._dp(d), O._dp(w))
    assert d[0] == 1e-14 and d[2] == 1e-14 and d[4] == 1e-14
    assert w[0] == 1e-14 / (1e-14 + 2.0)
    assert w[2] == 4.0 / (1e-14 + 4.0)


@pytest.mark.parametrize("kt,found", [(998, True), (999, True), (1000, False)])
def test_max_traversal_from_corner(kt, found):
    """walkingsearch.c:10,1123: from the corner cell the walk reaches k = 999 (1000 evaluations)
    but not k = 1000 -> LOST with cell (-1,-1,-1)."""
    g = unit_grid(1, 1, 1100)
    r = O.locate_particle(g, [0.5, 0.5, (kt + 0.5) / 1100])
    if found:
        assert r["status"] == O.ACTIVE_AND_LOCATED and list(r["cell"]) == [0, 0, kt]
        assert r["steps"] == kt + 1
    else:
        assert r["status"] == O.LOST and list(r["cell"]) == [-1, -1, -1]
        assert r["steps"] == 1000


def test_point_on_interior_face_first_cell_wins():
    """A point exactly on the plane between cells 0 and 1 (|d| < thr -> 0) is accepted by the
    first cell the walk evaluates (walkingsearch.c:218-221, :1197-1199)."""
    g = unit_grid(2, 1, 1)
    r0 = O.locate_particle(g, [0.5, 0.5, 0.5])               # from the corner: cell 0 first
    assert list(r0["cell"]) == [0, 0, 0]
    r1 = O.locate_particle(g, [0.5, 0.5, 0.5], cell=[1, 0, 0])   # previous cell 1: cell 1 first
    assert list(r1["cell"]) == [1, 0, 0]
    # the on-face distance was clamped to 1e-14 before the ratio
    assert r0["weights"][0] == 0.5 / (0.5 + 1e-14)


def test_k_face_gap_oscillates_to_lost():
    """On a grid whose k-faces are not planar the lower cell's FRONT plane and the upper cell's
    BACK plane differ (walkingsearch.c:303-325 use different v1); a point in the gap between
    them makes the walk alternate k, k+1 until MAX_TRAVERSAL, then LOST."""
    coor = W.uniform_grid(1, 1, 2)
    coor[1, 1, 1, 2] += 0.2        # lift one node of the middle k-plane: that k-face is warped
    g = O.Grid(coor)
    # search points near the middle plane for one that is in neither cell
    hits = []
    for z in np.linspace(0.45, 0.62, 341):
        for xy in [(0.9, 0.9), (0.8, 0.95), (0.95, 0.8), (0.1, 0.1), (0.5, 0.5)]:
            r = O.locate_particle(g, [xy[0], xy[1], z], cell=[0, 0, 0])
            if r["status"] == O.LOST:
                hits.append(r)
    assert hits, "no gap point found"
    assert all(h["steps"] == 1000 for h in hits)


def test_pyref_agrees_bitwise_on_random_curvilinear():
    """Two independent restatements (C and Python) agree bit for bit on 300 walks."""
    coor = W.sinusoidal_grid(6, 5, 7, amp=0.04)
    g = O.Grid(coor)
    rng = np.random.default_rng(1)
    pts = rng.uniform(-0.05, 1.05, size=(300, 3))
    starts = rng.integers(-1, 6, size=(300, 3))
    for p, st in zip(pts, starts):
        c = O.locate_particle(g, p, cell=st)
        py_cell, py_w, py_st, py_steps = pyref.locate(coor.tolist(), tuple(p), tuple(int(x) for x in st))
        assert c["status"] == py_st and tuple(c["cell"]) == py_cell and c["steps"] == py_steps
        if py_w is not None:
            assert tuple(c["weights"]) == py_w


def test_linear_field_interpolated_exactly_on_uniform_grid():
    """interpolation.c:957-1042: on a uniform grid the node average of a linear cell field is the
    linear field at the nodes (interior), and trilinear weights reproduce it at the particle."""
    IM, JM, KM = 6, 5, 4
    coor = W.uniform_grid(IM, JM, KM)
    g = O.Grid(coor)
    cent = W.cell_centroids(coor)
    lin = lambda x: np.stack([0.5 + 2 * x[..., 0] - x[..., 1], 3 * x[..., 2], x[..., 0] + x[..., 1] + x[..., 2]], -1)
    corner = O.center_to_corner(g, W.node_sized(lin(cent)))
    interior = corner[1:-1, 1:-1, 1:-1]
    assert np.allclose(interior, lin(coor[1:-1, 1:-1, 1:-1]), rtol=0, atol=1e-13)
    s = O.Swarm.create(np.array([[0.52, 0.47, 0.43], [0.41, 0.33, 0.62]]))
    O.locate_all(g, s)
    O.interpolate(g, corner, s)
    assert np.allclose(s.vel[:2], lin(s.pos[:2]), atol=1e-13)


def test_on_extended_face_plane_accepts_wrong_cell():
    """DeterminePointPosition quirk seen through the walk: a point exactly on the extended plane
    of one face (|d| < thr -> 0) is accepted (walkingsearch.c:445-456, :1197) even though another
    face says it is outside; the clamp then gives weights of 1.  From the corner, (0.5,0.5,0.5) on
    a 6x5x4 uniform grid stops in cell (1,1,1), whose FRONT plane is z = 0.5."""
    g = O.Grid(W.uniform_grid(6, 5, 4))
    r = O.locate_particle(g, [0.5, 0.5, 0.5])
    assert r["status"] == O.ACTIVE_AND_LOCATED
    assert list(r["cell"]) == [1, 1, 1]
    assert r["weights"][0] == (0.5 - 1 / 6) / ((0.5 - 1 / 6) + 1e-14)
    py_cell, py_w, _, _ = pyref.locate(W.uniform_grid(6, 5, 4).tolist(), (0.5, 0.5, 0.5))
    assert py_cell == (1, 1, 1) and tuple(r["weights"]) == py_w


def test_center_to_corner_counts():
    """interpolation.c:625-677: corner/edge/face/interior nodes average 1/2/4/8 cells."""
    IM, JM, KM = 3, 3, 3
    g = O.Grid(W.uniform_grid(IM, JM, KM))
    u = np.zeros((KM + 1, JM + 1, IM + 1, 3))
    u[:KM, :JM, :IM, 0] = 1.0               # count probe: every valid cell contributes 1
    u[:KM, :JM, :IM, 1] = np.arange(IM * JM * KM).reshape(KM, JM, IM)
    c = O.center_to_corner(g, u)
    assert np.all(c[..., 0] == 1.0)
    assert c[0, 0, 0, 1] == 0.0                                   # corner node: cell (0,0,0) only
    assert c[0, 0, 1, 1] == (0.0 + 1.0) / 2                        # edge node: 2 cells
    assert c[0, 1, 1, 1] == (0.0 + 1.0 + 3.0 + 4.0) / 4            # face node: 4 cells
    cells = [(k, j, i) for k in (0, 1) for j in (0, 1) for i in (0, 1)]
    want = 0.0
    for (k, j, i) in cells:
        want += u[k, j, i, 1]
    assert c[1, 1, 1, 1] == want / 8                               # interior: 8 cells, (dk, dj, di) order


def test_cell_scatter_sum_count_avg():
    """interpolation.c:1838-2036: sum/count per cell, average where count > 0.5, else 0."""
    IM, JM, KM = 2, 2, 2
    g = O.Grid(W.uniform_grid(IM, JM, KM))
    pos = np.array([[0.2, 0.2, 0.2], [0.3, 0.1, 0.4], [0.7, 0.7, 0.7]])
    s = O.Swarm.create(pos)
    s.P[:] = [1.0, 2.0, 10.0]
    O.locate_all(g, s)
    count, avg = O.scatter_P(g, s)
    assert count[0, 0, 0] == 2 and avg[0, 0, 0] == 1.5
    assert count[1, 1, 1] == 1 and avg[1, 1, 1] == 10.0
    assert count.sum() == 3 and np.count_nonzero(avg) == 2
    assert np.all(count[KM] == 0) and np.all(count[:, JM] == 0) and np.all(count[:, :, IM] == 0)


def test_face_deposit_conservation():
    """Face deposit (defined by this build): the faces receive exactly sum V_p (to rounding)."""
    wl = W.config_sinusoidal(8, 7, 9, n=2000, steps=1)
    g = O.Grid(wl.coor)
    s = O.Swarm.create(wl.pos, cell=wl.cell0)
    O.locate_all(g, s)
    live = int(np.sum(s.status[: s.n] == O.ACTIVE_AND_LOCATED))
    f = O.deposit_faces(g, s, volume=1.0)
    tot = f["fi"].sum() + f["fj"].sum() + f["fk"].sum()
    assert abs(tot - live) < 1e-9 * live
    assert np.all(f["fi"] >= 0) and np.all(f["fj"] >= 0) and np.all(f["fk"] >= 0)


def test_remove_lost_swap_with_last_order():
    """ParticleMotion.c:532-625 + DMSwarmRemovePointAtIndex: a backward loop where each removed
    slot receives the current last particle."""
    s = O.Swarm.create(np.zeros((5, 3)))
    s.status[:] = [O.ACTIVE_AND_LOCATED, O.LOST, O.ACTIVE_AND_LOCATED, O.ACTIVE_AND_LOCATED, O.LOST]
    assert O.remove_lost(s) == 2
    assert list(s.pid[: s.n]) == [0, 3, 2]
    s = O.Swarm.create(np.zeros((5, 3)))
    s.status[:] = [O.LOST, O.LOST, O.ACTIVE_AND_LOCATED, O.ACTIVE_AND_LOCATED, O.ACTIVE_AND_LOCATED]
    O.remove_lost(s)
    assert list(s.pid[: s.n]) == [3, 4, 2]


def test_out_of_bounds_uses_widened_node_bbox():
    """grid.c:851-858 and ParticleMotion.c:106-110: inclusive bbox widened by 1e-6."""
    g = unit_grid(2, 2, 2)
    bmin, bmax = O.bounding_box(g)
    assert np.all(bmin == -1e-6) and np.all(bmax == 1.0 + 1e-6)
    pos = np.array([[0.5, 0.5, 0.5], [1.0 + 5e-7, 0.5, 0.5], [1.0 + 2e-6, 0.5, 0.5], [-1e-6, 0.0, 0.0]])
    s = O.Swarm.create(pos)
    assert O.remove_oob(g, s) == 1
    assert sorted(s.pid[: s.n]) == [0, 1, 3]


def test_reference_step_sequence_config1_small():
    """A few reference steps on a reduced config-1 case keep every particle located and the
    locate/remove/interpolate sequence consistent (simulation.c:240-311)."""
    wl = W.config1(n=500, IM=5, JM=5, KM=20, steps=3)
    g = O.Grid(wl.coor)
    s = O.Swarm.create(wl.pos, cell=wl.cell0)
    sim = O.Simulation(g, wl.ucat_node_sized(), s, wl.dt)
    info0 = sim.initial_setup()
    assert info0.evals > 0
    for _ in range(wl.steps):
        info = sim.step()
        assert info.removed_lost + info.removed_oob <= info.n_start
    v = s.view()
    assert np.all(v["status"] == O.ACTIVE_AND_LOCATED)
    assert np.all(v["cell"] >= 0)
