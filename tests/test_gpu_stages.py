"""The reference's stages one C-ABI call at a time (fdf_ResetAllParticleStatuses,
fdf_UpdateAllParticlePositions, fdf_LocateAllParticlesInGrid, fdf_CheckAndRemoveLostParticles,
fdf_CheckAndRemoveOutOfBoundsParticles, fdf_InterpolateAllFieldsToSwarm,
fdf_ScatterAllParticleFieldsToEulerFields): in the reference's order they give the oracle's
stage-by-stage results and fdf_AdvanceStep's, bit for bit, in every form."""
import ctypes

import numpy as np
import pytest

from fdf_gb300 import workloads as W
from fdf_gb300.context import FORM_FP32, FORM_LEARNED_FP32, FORM_PLAIN_FP64, PicContext
from oracle import oracle as O
from tests.parity_util import assert_faces_bitwise, assert_swarm_bitwise, from_oracle_swarm, to_oracle_swarm

pytestmark = pytest.mark.gpu


def _stage_step(ctx):
    ctx.reset_statuses()
    ctx.update_positions()
    ctx.locate()
    lost = ctx.remove_lost()
    oob = ctx.remove_out_of_bounds()
    ctx.interpolate()
    ctx.scatter()
    return lost, oob


def _oracle_stage_step(g, os_, ucat, dt):
    L = O.lib()
    cs = os_.c()
    L.o_ResetAllParticleStatuses(ctypes.byref(cs))
    L.o_UpdateAllParticlePositions(ctypes.byref(cs), float(dt), O.nthreads_default())
    os_.sync(cs)
    err, _ = O.locate_all(g, os_)
    assert err == 0
    lost = O.remove_lost(os_)
    oob = O.remove_oob(g, os_)
    O.interpolate(g, O.center_to_corner(g, ucat), os_)
    count, avg = O.scatter_P(g, os_)
    return lost, oob, count, avg


def test_stages_match_the_oracle_stage_by_stage(require_gpu):
    wl = W.config_sinusoidal(IM=12, JM=10, KM=24, n=4000, cfl=4.0, steps=3)
    g = O.Grid(wl.coor)
    ucat = wl.ucat_node_sized()
    with PicContext(0) as ctx:
        ctx.load_workload(wl, form=FORM_PLAIN_FP64)
        s0 = ctx.get_swarm()
        os_ = to_oracle_swarm(s0)
        ctx.initial_setup()
        O.Simulation(g, ucat, os_, wl.dt).initial_setup()
        removed = 0
        for st in range(wl.steps):
            lost, oob = _stage_step(ctx)
            olost, ooob, count, avg = _oracle_stage_step(g, os_, ucat, wl.dt)
            assert (lost, oob) == (olost, ooob), f"step {st} removals"
            removed += lost + oob
            assert_swarm_bitwise(ctx.get_swarm(), from_oracle_swarm(os_), f"stages, step {st}")
            cnt, av = ctx.get_scattered()
            assert np.array_equal(cnt, count) and np.array_equal(av, avg), f"step {st} scatter"
            assert_faces_bitwise(ctx.get_faces(), O.deposit_faces(g, os_, volume=wl.volume), what=f"step {st}")
        assert removed > 0   # CFL 4 on a closed box: particles leave through its walls


@pytest.mark.parametrize("form", [FORM_PLAIN_FP64, FORM_FP32, FORM_LEARNED_FP32])
def test_stages_equal_the_fused_step(require_gpu, form):
    wl = W.config_bent_pipe(12, 12, 48, n=20000, cfl=4.0, materialize=True)
    outs = []
    for staged in (True, False):
        with PicContext(0) as ctx:
            ctx.load_workload(wl, form=form)
            if form == FORM_LEARNED_FP32:
                ctx.locator_init(seed=3)          # an untrained network: the cells may not change
                ctx.locator_min_distance(0.0)
            ctx.initial_setup()
            for _ in range(3):
                if staged:
                    _stage_step(ctx)
                else:
                    ctx.step()
            outs.append((ctx.get_swarm(), ctx.get_faces(), ctx.get_scattered(), ctx.counters()[0]))
    (sa, fa, ca, pa), (sb, fb, cb, pb) = outs
    for f in ("position", "velocity", "weight", "P", "cell", "pid", "status"):
        assert np.array_equal(getattr(sa, f), getattr(sb, f)), f
    for x, y in zip(fa + ca, fb + cb):
        assert np.array_equal(x, y)
    assert pa == pb   # particle-steps counted the same way


def test_stage_calls_sort_an_unsorted_swarm(require_gpu):
    """Interpolate and scatter right after fdf_SetSwarm (particles in the caller's order): the
    library sorts them by (cell, PID) first and gives the initial setup's values."""
    wl = W.config_sinusoidal(IM=10, JM=8, KM=16, n=3000, cfl=1.0, steps=1)
    with PicContext(0) as ctx:
        ctx.load_workload(wl, form=FORM_PLAIN_FP64)
        ctx.initial_setup()
        ref = ctx.get_swarm()
        ref_faces, ref_sc = ctx.get_faces(), ctx.get_scattered()
        order = np.random.default_rng(5).permutation(ref.n)
        shuffled = type(ref)(*[np.ascontiguousarray(a[order]) for a in (ref.position, ref.velocity, ref.weight,
                                                                         ref.P, ref.cell, ref.pid, ref.status)])
        shuffled.velocity[:] = 0.0
        ctx.set_swarm(shuffled)
        ctx.interpolate()
        ctx.scatter()
        got = ctx.get_swarm()
        for f in ("position", "velocity", "weight", "P", "cell", "pid", "status"):
            assert np.array_equal(getattr(got, f), getattr(ref, f)), f
        for x, y in zip(ctx.get_faces() + ctx.get_scattered(), ref_faces + ref_sc):
            assert np.array_equal(x, y)


def test_locate_points_matches_the_reference_walk(require_gpu):
    """fdf_LocatePoints: the reference walk for arbitrary points (inside, outside, on the grid's
    boundary), from given cells or from cell (0,0,0), bit for bit against the oracle's
    LocateParticleOrFindMigrationTarget."""
    wl = W.config_sinusoidal(IM=10, JM=8, KM=20, n=10, cfl=1.0, steps=1)
    coor = wl.coor - 0.5   # the origin inside the grid
    g = O.Grid(coor)
    rng = np.random.default_rng(9)
    pts = rng.uniform(-0.6, 0.6, size=(3000, 3))
    pts[:200] = coor.reshape(-1, 3)[rng.integers(0, coor.reshape(-1, 3).shape[0], 200)]   # grid nodes
    # one coordinate at a value the FP32 split cannot carry (tiny, subnormal, signed zero, beyond
    # FP32's range, non-finite), the others inside the grid: the walk's faces then take the FP64
    # route
    special = [0.0, -0.0, 1e-200, -3e-310, 5e-324, 2.0 ** -121, 1e30, -1e39, 1e300, np.inf, -np.inf, np.nan]
    for q, v in enumerate(special * 5):
        pts[200 + q] = (0.01 * (q % 7), -0.02, 0.03)
        pts[200 + q, q % 3] = v
    cells = np.full((3000, 3), -1, dtype=np.int64)
    cells[1000:] = np.stack([rng.integers(0, 10, 2000), rng.integers(0, 8, 2000), rng.integers(0, 20, 2000)], 1)
    with PicContext(0) as ctx:
        ctx.set_grid(coor)
        cout, w, st = ctx.locate_points(pts, cells)
        cout0, w0, st0 = ctx.locate_points(pts[:500])          # no start cells: (0,0,0)
    for p in range(len(pts)):
        r = O.locate_particle(g, pts[p], cells[p])
        assert r["err"] == 0
        assert np.array_equal(cout[p], r["cell"]) and st[p] == r["status"], p
        assert np.array_equal(w[p].view(np.int64), r["weights"].view(np.int64)), p
    for p in range(500):
        r = O.locate_particle(g, pts[p])
        assert np.array_equal(cout0[p], r["cell"]) and st0[p] == r["status"]
    assert (st == 3).any() and (st == 1).any()   # both LOST and located points
