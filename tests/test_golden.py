"""The CPU restatement (oracle/picurv_oracle.c) against golden vectors written by the
reference's own code (tests/golden/ref_golden.npz, from oracle/_ref): per-cell functions,
single-point walks, and whole runs (initial setup and 3 steps) on four grid families, bit for
bit.  Runs on every machine; tests/test_ref_pin.py makes the same comparisons against the
compiled reference directly where its sources are present."""
import numpy as np
import pytest

from fdf_gb300.context import SwarmArrays
from oracle import oracle as O
from tests import golden_util as G


@pytest.fixture(scope="module")
def golden():
    return G.load()


def test_per_cell_functions(golden):
    L = O.lib()
    for q in range(len(golden["cells/h"])):
        v, p = golden["cells/verts"][q], golden["cells/points"][q]
        h = np.zeros(1)
        L.o_GetCellCharacteristicSize(O.cell_from_vertices(v), O._dp(h))
        assert G.bits(h[0]) == G.bits(golden["cells/h"][q]), q
        d = np.zeros(6)
        pos = np.zeros(1, dtype=np.int64)
        assert L.o_EvaluateParticlePosition(O.cell_from_vertices(v), O._dp(d), O.cmp(p), O._ip(pos), 1e-11 * h[0]) == 0
        assert np.array_equal(G.bits(d), G.bits(golden["cells/d"][q])) and pos[0] == golden["cells/position"][q], q
        w = np.zeros(3)
        L.o_UpdateParticleWeights(O._dp(d), O._dp(w))
        assert np.array_equal(G.bits(w), G.bits(golden["cells/weights"][q])), q


def test_single_point_walks(golden):
    g = O.Grid(golden["walks/coor"])
    for p in range(len(golden["walks/status"])):
        r = O.locate_particle(g, golden["walks/points"][p], golden["walks/start"][p])
        assert r["err"] == 0
        assert np.array_equal(r["cell"], golden["walks/cell"][p]) and r["status"] == golden["walks/status"][p], p
        assert np.array_equal(G.bits(r["weights"]), G.bits(golden["walks/weights"][p])), p


@pytest.mark.parametrize("name", G.RUNS)
def test_runs(golden, name):
    coor, ucat, dt, pos0, cell0, P0 = G.run_inputs(golden, name)
    s0 = SwarmArrays.create(pos0, cell=cell0, P=P0)
    os_ = O.Swarm(pos=s0.position.copy(), vel=s0.velocity.copy(), weight=s0.weight.copy(), P=s0.P.copy(),
                  cell=s0.cell.copy(), pid=s0.pid.copy(), status=s0.status.copy(), n=s0.n)
    sim = O.Simulation(O.Grid(coor), ucat, os_, dt, nthreads=1)
    removed = golden[f"run_{name}/removed"]
    for k in range(G.STEPS + 1):
        if k == 0:
            sim.initial_setup()
        else:
            info = sim.step()
            assert (info.removed_lost, info.removed_oob) == tuple(removed[k - 1]), (name, k)
        v = os_.view()
        G.check_state(golden, name, k, v["pos"], v["vel"], v["weight"], v["P"], v["cell"], v["pid"], v["status"],
                      sim.count, sim.avg, what=f"{name} snapshot {k}")
