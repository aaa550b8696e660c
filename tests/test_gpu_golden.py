"""GPU: the CUDA path against golden vectors written by the reference's own code
(tests/golden/ref_golden.npz: the reference's C sources compiled unmodified into
oracle/_ref and run on small seeded inputs).  Through the C ABI, bit for bit:

* the plain FP64 form's initial setup and 3 steps (fused fdf_AdvanceStep, the graph-replayed
  fdf_AdvanceSteps, and the stage-by-stage calls) on four grid families: swarm, removal
  counts, ParticleCount and the P average;
* fdf_LocatePoints on 600 single-point walks from start cells of every kind.
"""
import numpy as np
import pytest

from fdf_gb300.context import PicContext, SwarmArrays
from tests import golden_util as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def golden():
    return G.load()


def _load(ctx, golden, name):
    coor, ucat, dt, pos0, cell0, P0 = G.run_inputs(golden, name)
    ctx.set_grid(coor)
    ctx.set_ucat(ucat)
    ctx.set_dt(dt)
    ctx.set_swarm(SwarmArrays.create(pos0, cell=cell0, P=P0))


def _check(ctx, golden, name, k, what):
    s = ctx.get_swarm()
    c, a = ctx.get_scattered()
    G.check_state(golden, name, k, s.position, s.velocity, s.weight, s.P, s.cell, s.pid, s.status, c, a,
                  what=f"{name} {what} snapshot {k}")


@pytest.mark.parametrize("name", G.RUNS)
def test_fused_steps_match_the_reference(require_gpu, golden, name):
    removed = golden[f"run_{name}/removed"]
    with PicContext(0) as ctx:
        _load(ctx, golden, name)
        ctx.initial_setup()
        _check(ctx, golden, name, 0, "fused")
        for k in range(1, G.STEPS + 1):
            info = ctx.step()
            assert (info.removed_lost, info.removed_oob) == tuple(removed[k - 1]), (name, k)
            _check(ctx, golden, name, k, "fused")


@pytest.mark.parametrize("name", G.RUNS)
def test_graph_replayed_steps_match_the_reference(require_gpu, golden, name):
    with PicContext(0) as ctx:
        _load(ctx, golden, name)
        ctx.initial_setup()
        ctx.steps(G.STEPS)
        _check(ctx, golden, name, G.STEPS, "graph")


@pytest.mark.parametrize("name", G.RUNS)
def test_stage_calls_match_the_reference(require_gpu, golden, name):
    removed = golden[f"run_{name}/removed"]
    with PicContext(0) as ctx:
        _load(ctx, golden, name)
        ctx.locate()
        ctx.interpolate()
        ctx.scatter()
        _check(ctx, golden, name, 0, "stages")
        for k in range(1, G.STEPS + 1):
            ctx.reset_statuses()
            ctx.update_positions()
            ctx.locate()
            lost = ctx.remove_lost()
            oob = ctx.remove_out_of_bounds()
            ctx.interpolate()
            ctx.scatter()
            assert (lost, oob) == tuple(removed[k - 1]), (name, k)
            _check(ctx, golden, name, k, "stages")


def test_locate_points_match_the_reference(require_gpu, golden):
    with PicContext(0) as ctx:
        ctx.set_grid(golden["walks/coor"])
        cell, w, st = ctx.locate_points(golden["walks/points"], golden["walks/start"])
    assert np.array_equal(cell, golden["walks/cell"])
    assert np.array_equal(st, golden["walks/status"])
    assert np.array_equal(G.bits(w), G.bits(golden["walks/weights"]))
