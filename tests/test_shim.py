"""The reference-signature shim (fdf_gb300/shim/picurv_shim.c) on the CPU: it compiles against
the reference's own headers (so every function it defines has the reference's prototype) and
against the stand-in headers used where the reference is absent; its host-side per-cell
arithmetic equals the reference's bit for bit (the golden vectors everywhere, and the reference's
own compiled code where its sources are present); its host loops (status reset, position update,
the two removals) leave the DMSwarm as the reference's do.  The GPU-backed calls are in
tests/test_gpu_shim.py."""
import numpy as np
import pytest

from fdf_gb300 import workloads as W
from fdf_gb300.context import SwarmArrays
from oracle import ref as R
from tests import golden_util as G
from tests import shim_util as S

HEADERS = ["compat"] + (["reference"] if R.available() else [])


def test_shim_compiles_cleanly_against_the_stand_in_headers():
    assert S.compile_warnings("compat").strip() == ""


@pytest.mark.skipif(not R.available(), reason="the reference's sources are not present")
def test_shim_has_the_reference_prototypes():
    """Built against the reference's own include/: a definition whose signature differed from
    the reference's declaration would not compile."""
    assert S.build("reference")


@pytest.mark.parametrize("headers", HEADERS)
def test_per_cell_functions_equal_the_golden_vectors(headers):
    L = S.lib(headers)
    g = G.load()
    for q in range(len(g["cells/h"])):
        v, p = np.ascontiguousarray(g["cells/verts"][q]), np.ascontiguousarray(g["cells/points"][q])
        h = np.zeros(1)
        assert L.shim_characteristic_size(S._d(v), S._d(h)) == 0
        assert G.bits(h[0]) == G.bits(g["cells/h"][q]), q
        d, pos = np.zeros(6), np.zeros(1, np.int64)
        assert L.shim_evaluate_position(S._d(v), S._d(p), 1e-11 * h[0], S._d(d), S._i(pos)) == 0
        assert np.array_equal(G.bits(d), G.bits(g["cells/d"][q])) and pos[0] == g["cells/position"][q], q
        w = np.zeros(3)
        assert L.shim_update_weights(S._d(d), S._d(w)) == 0
        assert np.array_equal(G.bits(w), G.bits(g["cells/weights"][q])), q


@pytest.mark.skipif(not R.available(), reason="the reference's sources are not present")
def test_per_cell_functions_equal_the_reference():
    L = S.lib("compat")
    rng = np.random.default_rng(5)
    base = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 1, 1], [1, 1, 1], [1, 0, 1], [0, 0, 1]], float)
    for q in range(2000):
        v = np.ascontiguousarray((base + rng.uniform(-0.35, 0.35, (8, 3))) * 10.0 ** rng.uniform(-4, 3))
        lo, hi = v.min(0), v.max(0)
        p = np.ascontiguousarray(rng.uniform(lo - 0.2 * (hi - lo), hi + 0.2 * (hi - lo)))
        thr = 1e-11 * R.characteristic_size(v)
        rc_ref, d_ref, pos_ref = R.evaluate_position(v, p, thr)
        d, pos = np.zeros(6), np.zeros(1, np.int64)
        assert L.shim_evaluate_position(S._d(v), S._d(p), thr, S._d(d), S._i(pos)) == rc_ref
        if rc_ref:
            continue
        assert np.array_equal(G.bits(d), G.bits(d_ref)) and pos[0] == pos_ref, q
        ijk = np.ascontiguousarray(rng.integers(-2, 40, 3))
        want = R.update_indices(d, ijk)
        assert L.shim_update_indices(S._d(d.copy()), S._i(ijk)) == 0 and np.array_equal(ijk, want), q
        cc = np.ascontiguousarray(v.mean(0))
        rc_ref, dp_ref = R.signed_distance(v[0], v[3], v[2], v[1], cc, p, thr)
        dp = np.zeros(1)
        a = [np.ascontiguousarray(x) for x in (v[0], v[3], v[2], v[1], cc, p)]
        assert L.shim_signed_distance(*[S._d(x) for x in a], thr, S._d(dp)) == rc_ref
        assert rc_ref or G.bits(dp[0]) == G.bits(dp_ref), q
    for d in np.random.default_rng(1).choice([-1.0, 0.0, 1.0], size=(500, 6)):
        r = np.zeros(1, np.int64)
        L.shim_point_position(S._d(d.copy()), S._i(r))
        assert r[0] == R.point_position(d)


def test_degenerate_face_is_petsc_err_user():
    L = S.lib("compat")
    v = np.zeros((8, 3))
    d, pos = np.zeros(6), np.zeros(1, np.int64)
    p = np.array([0.5, 0.5, 0.5])
    assert L.shim_evaluate_position(S._d(v), S._d(p), 1e-14, S._d(d), S._i(pos)) == 83
    L.shim_clear_error()


@pytest.mark.skipif(not R.available(), reason="the reference's sources are not present")
@pytest.mark.parametrize("headers", HEADERS)
def test_host_loops_leave_the_swarm_as_the_reference_does(headers):
    """Reset, position update and the two removals run on the host over the DMSwarm; after
    them the swarm holds the reference's particles in the reference's order."""
    wl = W.config_bent_pipe(8, 6, 20, n=1500, cfl=4.0)
    rng = np.random.default_rng(4)
    s = SwarmArrays.create(wl.pos, cell=wl.cell0)
    s.velocity[...] = rng.normal(scale=0.3 / wl.dt, size=s.velocity.shape)   # some leave the box
    s.status[...] = rng.choice([0, 1, 3, 4], size=s.n, p=[0.2, 0.5, 0.2, 0.1])   # some LOST
    ref = R.RefSim(wl.coor, wl.ucat_node_sized(), wl.dt)
    ref.set_swarm(s.position, s.velocity, s.weight, s.P, s.cell, s.pid, s.status)
    sh = S.ShimSim(wl.coor, wl.ucat_node_sized(), wl.dt, device=-1, headers=headers)
    sh.set_swarm(s)
    for st in ("reset", "update_positions", "remove_lost", "remove_out_of_bounds"):
        assert sh.stage(st) == ref.stage(st), st
        a, b = sh.swarm(), ref.swarm()
        for x, y in zip(a, (b.pos, b.vel, b.weight, b.P, b.cell, b.pid, b.status)):
            assert np.array_equal(np.asarray(x).view(np.int64), np.asarray(y).view(np.int64)), st
    assert 0 < len(sh.swarm()[5]) < s.n
