"""GPU: PICurv's step driven through the reference-signature shim (fdf_gb300/shim/picurv_shim.c:
LocateAllParticlesInGrid_TEST, InterpolateAllFieldsToSwarm, ScatterAllParticleFieldsToEulerFields
and the host-side calls, on a DMSwarm and DMDA vectors of the PETSc stand-in), against the golden
vectors written by the reference's own code, bit for bit: initial setup and 3 steps on four grid
families, plus LocateParticleOrFindMigrationTarget_TEST for single points."""
import numpy as np
import pytest

from fdf_gb300.context import SwarmArrays
from tests import golden_util as G
from tests import shim_util as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def golden():
    return G.load()


@pytest.mark.parametrize("name", G.RUNS)
def test_steps_through_the_shim_match_the_reference(require_gpu, golden, name):
    coor, ucat, dt, pos0, cell0, P0 = G.run_inputs(golden, name)
    sim = S.ShimSim(coor, ucat, dt, device=0)
    sim.set_swarm(SwarmArrays.create(pos0, cell=cell0, P=P0))
    removed = golden[f"run_{name}/removed"]
    for k in range(G.STEPS + 1):
        if k == 0:
            sim.initial_setup()
        else:
            assert sim.step() == tuple(removed[k - 1]), (name, k)
        pos, vel, w, P, cell, pid, st = sim.swarm()
        c, a = sim.scattered()
        G.check_state(golden, name, k, pos, vel, w, P, cell, pid, st, c, a, what=f"shim {name} snapshot {k}")
    sim.close()


def test_single_point_locate_through_the_shim(require_gpu, golden):
    sim = S.ShimSim(golden["walks/coor"], device=0)
    for p in range(0, len(golden["walks/status"]), 3):
        r = sim.locate_point(golden["walks/points"][p], golden["walks/start"][p])
        assert r["err"] == 0
        assert np.array_equal(r["cell"], golden["walks/cell"][p]) and r["status"] == golden["walks/status"][p], p
        if r["status"] == 1:
            assert np.array_equal(G.bits(r["weights"]), G.bits(golden["walks/weights"][p])), p
    # a LOST particle keeps the weights it came with, as in the reference
    r = sim.locate_point([50.0, 50.0, 50.0], [2, 2, 2], w_in=[0.25, 0.5, 0.75])
    assert r["status"] == 3 and list(r["cell"]) == [-1, -1, -1] and list(r["weights"]) == [0.25, 0.5, 0.75]
    sim.close()
