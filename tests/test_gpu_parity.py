"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

Bar: bit-exact for cell indices, statuses, PIDs, positions, velocities, weights,
the cell count and P average, and the face deposits (plain FP64 path, no FMA,
same operation order; the face sums run in (cell, PID) order on both sides).
"""
import numpy as np
import pytest

from fdf_gb300 import workloads as W
from fdf_gb300.context import PicContext, SwarmArrays, PetscError, LOST, ACTIVE_AND_LOCATED
from oracle import oracle as O
from tests.parity_util import (assert_faces_bitwise, assert_faces_close, assert_swarm_bitwise, from_oracle_swarm,
                               to_oracle_swarm)

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(require_gpu):
    c = PicContext(0)
    yield c
    c.close()


def oracle_state(wl, s: SwarmArrays):
    g = O.Grid(wl.coor)
    os_ = to_oracle_swarm(s)
    sim = O.Simulation(g, wl.ucat_node_sized(), os_, wl.dt)
    return g, os_, sim


def run_parity(ctx, wl, steps, check_every=1, faces=True):
    ctx.load_workload(wl)
    s0 = ctx.get_swarm()
    g, os_, sim = oracle_state(wl, s0)
    ig = ctx.initial_setup()
    io = sim.initial_setup()
    assert ig.walk_evals == io.evals
    assert_swarm_bitwise(ctx.get_swarm(), from_oracle_swarm(os_), "initial setup")
    assert np.array_equal(ctx.get_corner().view(np.int64), sim.corner.view(np.int64)), "corner field"
    cnt, avg = ctx.get_scattered()
    assert np.array_equal(cnt, sim.count) and np.array_equal(avg, sim.avg), "initial scatter"
    for st in range(steps):
        info = ctx.step()
        oi = sim.step()
        assert (info.removed_lost, info.removed_oob) == (oi.removed_lost, oi.removed_oob), f"step {st} removal"
        assert info.walk_evals == oi.evals, f"step {st} walk evaluations"
        if (st + 1) % check_every == 0 or st == steps - 1:
            gs = ctx.get_swarm()
            assert_swarm_bitwise(gs, from_oracle_swarm(os_), f"step {st}")
            cnt, avg = ctx.get_scattered()
            assert np.array_equal(cnt, sim.count), f"step {st} ParticleCount"
            assert np.array_equal(avg, sim.avg), f"step {st} P average"
            if faces:
                ref = O.deposit_faces(g, os_, volume=wl.volume)
                assert_faces_bitwise(ctx.get_faces(), ref, what=f"step {st}")
                assert_faces_close(ctx.get_faces(), ref, what=f"step {st}")
    return ctx.get_swarm()


def test_config1_full_size_parity(ctx):
    """The uniform configuration at its full size: 20x20x280 grid, 10,000 particles
    located from the corner cell like the reference, 10 steps."""
    wl = W.config1()
    out = run_parity(ctx, wl, wl.steps)
    assert out.n > 9000


def test_sinusoidal_reduced_parity(ctx):
    """The curvilinear family at reduced size (CFL 0.5), corner start, 12 steps."""
    wl = W.config_sinusoidal(IM=16, JM=12, KM=40, n=20_000, cfl=0.5, steps=12, corner_start=True)
    run_parity(ctx, wl, wl.steps, check_every=3)


def test_sinusoidal_high_cfl_parity(ctx):
    """CFL 4: particles cross several cells per step (multi-evaluation walks)."""
    wl = W.config_sinusoidal(IM=20, JM=20, KM=48, n=30_000, cfl=4.0, steps=6)
    run_parity(ctx, wl, wl.steps, check_every=2)


def test_bent_pipe_reduced_parity(ctx):
    wl = W.config_bent_pipe(IM=12, JM=12, KM=48, n=20_000, cfl=2.0, steps=5)
    run_parity(ctx, wl, wl.steps, check_every=1)


def test_curved_pipe_reduced_parity(ctx):
    wl = W.config_curved_pipe(IM=12, JM=12, KM=64, n=20_000, cfl=1.0, steps=5)
    run_parity(ctx, wl, wl.steps, check_every=1)


def test_momentum_deposit_parity(ctx):
    """The curved-pipe family (Poiseuille + swirl) with the momentum face deposit: every
    component bit-identical to the oracle's (same products, same order), and its total equal
    to the sum of V u over the particles."""
    wl = W.config_curved_pipe(IM=12, JM=12, KM=64, n=20_000, cfl=1.0, steps=3)
    ctx.load_workload(wl)
    ctx.set_momentum_deposit(True)
    g, os_, sim = oracle_state(wl, ctx.get_swarm())
    ctx.initial_setup()
    sim.initial_setup()
    for st in range(wl.steps):
        ctx.step()
        sim.step()
        ref = O.deposit_faces(g, os_, volume=wl.volume, momentum=True)
        got = ctx.get_face_momentum()
        for gm, key in zip(got, ("mom_i", "mom_j", "mom_k")):
            assert np.array_equal(gm.view(np.int64), ref[key].view(np.int64)), f"step {st} {key}"
        s = ctx.get_swarm()
        tot = sum(m.reshape(-1, 3).sum(axis=0) for m in got)
        want = wl.volume * s.velocity.sum(axis=0)   # each particle deposits V u over 3 families x (a + 1 - a) / 3
        assert np.allclose(tot, want, rtol=1e-9, atol=1e-9 * np.abs(s.velocity).sum())
    ctx.set_momentum_deposit(False)


@pytest.mark.parametrize("form", [0, 1])
def test_graph_steps_match_eager_steps(ctx, form):
    """fdf_AdvanceSteps replays a captured CUDA graph of the step (per swarm buffer parity):
    the result is bit-identical to the same steps issued one by one."""
    wl = W.config1(n=5000, steps=7)
    outs = []
    for graph in (False, True):
        ctx.load_workload(wl, form=form)
        ctx.initial_setup()
        if graph:
            ctx.steps(wl.steps)
        else:
            for _ in range(wl.steps):
                ctx.step(info=False)
        ctx.synchronize()
        outs.append((ctx.get_swarm(), ctx.get_faces(), ctx.get_scattered(), ctx.counters()[:2]))
    (sa, fa, ca, na), (sb, fb, cb, nb) = outs
    for f in ("position", "velocity", "weight", "P", "cell", "pid", "status"):
        assert np.array_equal(getattr(sa, f), getattr(sb, f)), f
    for x, y in zip(fa + ca, fb + cb):
        assert np.array_equal(x, y)
    assert na == nb
    ctx.set_form(0)


def test_lost_beyond_max_traversal_and_out_of_bounds(ctx):
    """Corner-start walks that need more than 1000 evaluations are LOST at set-up, kept with
    velocity 0, and removed in step 1; particles pushed out of the domain are removed as
    out-of-bounds (walkingsearch.c:1206-1213, ParticleMotion.c:283-383, 532-625)."""
    coor = W.uniform_grid(1, 1, 1100)
    KM = 1100
    z = (np.array([10, 500, 998, 999, 1000, 1050, 1099]) + 0.5) / KM
    pos = np.stack([np.full(7, 0.5), np.full(7, 0.5), z], -1)
    wl = W.Workload("lost_case", coor, np.tile([0.0, 0.0, 1.0], (KM, 1, 1, 1)).reshape(KM, 1, 1, 3), pos,
                    np.full((7, 3), -1, dtype=np.int64), dt=0.5 / KM, steps=3)
    out = run_parity(ctx, wl, 3, faces=True)
    assert sorted(out.pid) == [0, 1, 2, 3]
    # out of bounds: a velocity that leaves the box through the top
    wl2 = W.Workload("oob_case", W.uniform_grid(2, 2, 4), np.tile([0.0, 0.0, 3.0], (4, 2, 2, 1)),
                     np.array([[0.5, 0.5, 0.1], [0.3, 0.6, 0.95], [0.7, 0.2, 0.5]]),
                     np.full((3, 3), -1, dtype=np.int64), dt=0.05, steps=3)
    run_parity(ctx, wl2, 3)


def test_empty_swarm(ctx):
    wl = W.config1(n=0, IM=4, JM=4, KM=4)
    ctx.load_workload(wl)
    info = ctx.initial_setup()
    assert info.n_end == 0
    info = ctx.step()
    assert info.n_end == 0 and ctx.size() == 0
    fi, fj, fk = ctx.get_faces()
    assert fi.sum() == 0 and fj.sum() == 0 and fk.sum() == 0


def test_degenerate_cell_raises_petsc_err_user(ctx):
    coor = W.uniform_grid(2, 1, 1)
    coor[:, :, 0, :] = coor[:, :, 1, :]
    wl = W.Workload("degenerate", coor, np.zeros((1, 1, 2, 3)), np.array([[0.75, 0.5, 0.5]]),
                    np.full((1, 3), -1, dtype=np.int64), dt=0.1, steps=1)
    ctx.load_workload(wl)
    with pytest.raises(PetscError) as e:
        ctx.initial_setup()
    assert e.value.code == 83


def test_nan_and_far_positions(ctx):
    """A NaN position compares false everywhere, so the reference accepts the start cell with
    NaN weights; a position far outside the grid walks out of bounds and is LOST."""
    wl = W.config1(n=4, IM=3, JM=3, KM=3)
    wl.pos[0] = [np.nan, 0.5, 0.5]
    wl.pos[1] = [5.0, 0.5, 0.5]
    run_parity(ctx, wl, 2)


def test_deterministic_repeat(ctx):
    wl = W.config_sinusoidal(IM=16, JM=16, KM=32, n=50_000, cfl=1.0, steps=4)
    outs = []
    for _ in range(2):
        ctx.load_workload(wl)
        ctx.initial_setup()
        ctx.steps(wl.steps)
        s = ctx.get_swarm()
        outs.append((s, ctx.get_faces(), ctx.get_scattered()))
    (s1, f1, c1), (s2, f2, c2) = outs
    for name in ("position", "velocity", "weight", "cell", "pid"):
        assert np.array_equal(getattr(s1, name), getattr(s2, name)), name   # same order too
    # the swarm is held sorted by (cell, PID)
    lin = (s1.cell[:, 2] * 16 + s1.cell[:, 1]) * 16 + s1.cell[:, 0]
    order = np.lexsort((s1.pid, lin))
    assert np.array_equal(order, np.arange(s1.n))
    for a, b in zip(f1 + c1, f2 + c2):
        assert np.array_equal(a.view(np.int64), b.view(np.int64))


def test_full_size_properties_sinusoidal(ctx):
    """The full 64x64x1024 / 1M-particle workload: one step checked against the oracle on the
    whole swarm, plus size-independent properties (face deposits sum to the live count, counts
    sum to the live count, every live particle has a cell)."""
    wl = W.config_sinusoidal()
    ctx.load_workload(wl)
    ctx.initial_setup()
    ctx.steps(2)
    before = ctx.get_swarm()
    g, os_, sim = oracle_state(wl, before)
    info = ctx.step()
    oi = sim.step(scatter=True)
    assert info.walk_evals == oi.evals
    after = ctx.get_swarm()
    assert_swarm_bitwise(after, from_oracle_swarm(os_), "full-size step")
    cnt, avg = ctx.get_scattered()
    assert np.array_equal(cnt, sim.count) and np.array_equal(avg, sim.avg)
    fi, fj, fk = ctx.get_faces()
    assert_faces_bitwise((fi, fj, fk), O.deposit_faces(g, os_, volume=wl.volume), "full-size step")
    tot = fi.sum() + fj.sum() + fk.sum()
    assert abs(tot - after.n * wl.volume) <= 1e-9 * after.n
    assert cnt.sum() == after.n
    assert np.all(after.cell >= 0) and np.all(after.status == ACTIVE_AND_LOCATED)


def test_device_seeding_matches_host_generator(ctx):
    """fdf_SeedParticles reproduces workloads.volumetric_particles bit for bit."""
    wl = W.config_bent_pipe(IM=16, JM=12, KM=40, n=50_000, cfl=2.0, steps=1)
    ctx.set_grid(wl.coor)
    ctx.set_ucat(wl.ucat)
    ctx.seed_particles(wl.n, seed=0, start_in_generating_cell=True)
    s = ctx.get_swarm()
    assert np.array_equal(s.pid, np.arange(wl.n))
    assert np.array_equal(s.position.view(np.int64), wl.pos.view(np.int64))
    assert np.array_equal(s.cell, wl.cell0)
    assert np.all(s.status == 4) and np.all(s.P == 101325.0)
    ctx.seed_particles(1000, seed=0, start_in_generating_cell=False)
    assert np.all(ctx.get_swarm().cell == -1)
