"""The k-slab decomposition (fdf_gb300/slabs.py) over 2 and 3 ranks on the CPU (gloo process
group, each rank's stages by the oracle through the same methods the GPU context has): after
the initial setup and 3 steps, the ranks' swarms together, their removal counts, ParticleCount,
the P average and the face volume and momentum deposits equal the one-rank oracle run bit for bit,
on a curvilinear grid and on a bent pipe at CFL 4 (many particles cross slab boundaries)."""
import os
import socket

import numpy as np
import pytest

from fdf_gb300 import workloads as W
from fdf_gb300.context import SwarmArrays
from oracle import oracle as O

STEPS = 3

WORKLOADS = {
    "sinusoidal": lambda: W.config_sinusoidal(IM=10, JM=8, KM=30, n=4000, cfl=2.0, steps=STEPS),
    "bent_pipe": lambda: W.config_bent_pipe(8, 6, 24, n=3000, cfl=4.0),
}


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, name, momentum, out, gpu=False):
    import torch.distributed as dist
    from fdf_gb300.slabs import SlabRun
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    wl = WORKLOADS[name]()
    if gpu:
        from fdf_gb300.context import PicContext
        ctx = PicContext(0)
        ctx.set_grid(wl.coor)
        ctx.set_ucat(wl.ucat)
        ctx.set_dt(wl.dt)
        ctx.set_volume(wl.volume)
        if momentum:
            ctx.set_momentum_deposit(True)
    else:
        from tests.slab_oracle_ctx import OracleRankCtx
        ctx = OracleRankCtx(wl, momentum)
    run = SlabRun(ctx, dist, momentum=momentum)
    run.set_swarm(SwarmArrays.create(wl.pos, cell=wl.cell0))
    run.initial_setup()
    removed = [run.step() for _ in range(STEPS)]
    migrated = run._sum([run.migrated])[0]
    res = run.gather()
    if rank == 0:
        s = res.pop("swarm")
        np.savez(out, removed=np.array(removed), migrated=migrated, **{f"s_{f}": getattr(s, f) for f in (
                 "position", "velocity", "weight", "P", "cell", "pid", "status")}, **res)
    dist.barrier()
    dist.destroy_process_group()
    if gpu:
        ctx.close()


def run_slabs(tmp_path, name, ranks, gpu=False):
    """Runs the ranks (spawned processes, gloo) and checks their union against the one-rank oracle."""
    import torch.multiprocessing as mp
    O.build()
    momentum = name == "bent_pipe"
    out = str(tmp_path / "slabs.npz")
    mp.spawn(_rank, args=(ranks, _free_port(), name, momentum, out, gpu), nprocs=ranks, join=True)
    got = np.load(out)
    # one rank: the oracle's own loop
    wl = WORKLOADS[name]()
    s0 = SwarmArrays.create(wl.pos, cell=wl.cell0)
    os_ = O.Swarm(pos=s0.position, vel=s0.velocity, weight=s0.weight, P=s0.P, cell=s0.cell, pid=s0.pid,
                  status=s0.status, n=s0.n)
    g = O.Grid(wl.coor)
    sim = O.Simulation(g, wl.ucat_node_sized(), os_, wl.dt, nthreads=1)
    sim.initial_setup()
    removed = [tuple((lambda i: (i.removed_lost, i.removed_oob))(sim.step())) for _ in range(STEPS)]
    assert [tuple(r) for r in got["removed"]] == removed
    ref = os_.sorted_by_pid()
    o = np.argsort(got["s_pid"], kind="stable")
    assert np.array_equal(got["s_pid"][o], ref["pid"])
    for f, k in (("position", "pos"), ("velocity", "vel"), ("weight", "weight"), ("P", "P")):
        assert np.array_equal(got[f"s_{f}"][o].view(np.int64), ref[k].view(np.int64)), f
    for f in ("cell", "status"):
        assert np.array_equal(got[f"s_{f}"][o], ref[f]), f
    assert np.array_equal(got["count"].view(np.int64), sim.count.view(np.int64))
    assert np.array_equal(got["avg"].view(np.int64), sim.avg.view(np.int64))
    f = O.deposit_faces(g, os_, volume=wl.volume, momentum=momentum)
    for key, fk in (("fi", "fi"), ("fj", "fj"), ("fk", "fk")) + ((("mi", "mom_i"), ("mj", "mom_j"),
                                                                ("mk", "mom_k")) if momentum else ()):
        assert np.array_equal(got[key].view(np.int64), f[fk].view(np.int64)), key
    # particles did cross the slab boundaries
    assert int(got["migrated"]) > 50


@pytest.mark.parametrize("ranks", [2, 3])
@pytest.mark.parametrize("name", sorted(WORKLOADS))
def test_slab_ranks_equal_one_rank(tmp_path, name, ranks):
    run_slabs(tmp_path, name, ranks)
