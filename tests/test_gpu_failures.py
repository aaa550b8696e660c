"""GPU: error paths, with every failure made on the host or by a bounded wait that runs out.

* A device allocation that fails inside fdf_SetGrid, fdf_ReserveParticles or
  fdf_SetMomentumDeposit (made to fail by fdf_TestFailDeviceAllocations, a host-side hook)
  leaves the context refusing the calls that need the lost buffers (PETSC_ERR_ARG_WRONGSTATE),
  the captured step graphs included, and a later successful set-up works as a fresh one.
* The learned locator's tensor-core kernel, run with no MMA issued, runs out of its bounded
  mbarrier wait: the call returns PETSC_ERR_GPU and the next call works.
* fdf_LocatePoints treats a start cell outside the grid (any index out of range, up to 2^62)
  as no cell: the walk starts in cell (0,0,0), as the reference's InitializeTraversalParameters
  does for a cell outside the rank's ghosted range (walkingsearch.c:571-629).
"""
import ctypes

import numpy as np
import pytest

from fdf_gb300 import workloads as W
from fdf_gb300.context import FORM_FP32, FORM_PLAIN_FP64, PetscError, PicContext
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ERR_MEM, ERR_WRONGSTATE, ERR_GPU = 55, 73, 97


def _fail_allocations(lib, after):
    assert lib.fdf_TestFailDeviceAllocations(int(after)) == 0


def _reference_run(wl, form, steps):
    with PicContext(0) as ctx:
        ctx.load_workload(wl, form=form)
        ctx.initial_setup()
        ctx.steps(steps)
        return ctx.get_swarm(), ctx.get_faces()


def _same(a, b):
    (sa, fa), (sb, fb) = a, b
    for f in ("position", "velocity", "weight", "P", "cell", "pid", "status"):
        assert np.array_equal(getattr(sa, f), getattr(sb, f)), f
    for x, y in zip(fa, fb):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("form", [FORM_PLAIN_FP64, FORM_FP32])
@pytest.mark.parametrize("after", [0, 3, 9])
def test_failed_set_grid_refuses_work(require_gpu, form, after):
    wl = W.config_sinusoidal(IM=10, JM=8, KM=24, n=3000, cfl=1.0, steps=4)
    want = _reference_run(wl, form, 4)
    with PicContext(0) as ctx:
        lib, h = ctx.lib, ctx.h
        ctx.load_workload(wl, form=form)
        ctx.initial_setup()
        ctx.steps(3)                 # eager step, then a captured step graph replayed
        ctx.synchronize()
        coor = np.ascontiguousarray(wl.coor)
        IM, JM, KM = wl.dims
        try:
            _fail_allocations(lib, after)
            rc = lib.fdf_SetGrid(h, IM, JM, KM, ctypes.c_void_p(coor.ctypes.data))
        finally:
            _fail_allocations(lib, -1)
        assert rc == ERR_MEM
        assert lib.fdf_AdvanceStep(h, None) == ERR_WRONGSTATE
        assert lib.fdf_AdvanceSteps(h, 2) == ERR_WRONGSTATE        # no replay of the old graph
        assert lib.fdf_PerformInitialSetup(h, None) == ERR_WRONGSTATE
        assert lib.fdf_InterpolateAllFieldsToSwarm(h) == ERR_WRONGSTATE
        n = np.zeros(3)
        assert lib.fdf_GetScatteredFields(h, ctypes.c_void_p(n.ctypes.data), ctypes.c_void_p(n.ctypes.data)) \
            == ERR_WRONGSTATE
        with pytest.raises(PetscError) as e:
            ctx.seed_particles(10)
        assert e.value.code == ERR_WRONGSTATE
        # a successful set-up afterwards runs as a fresh context does
        ctx.load_workload(wl, form=form)
        ctx.initial_setup()
        ctx.steps(4)
        got = (ctx.get_swarm(), ctx.get_faces())
    _same(got, want)


@pytest.mark.parametrize("after", [0, 1, 4])
def test_failed_reserve_refuses_work(require_gpu, after):
    wl = W.config_sinusoidal(IM=10, JM=8, KM=24, n=3000, cfl=1.0, steps=3)
    want = _reference_run(wl, FORM_PLAIN_FP64, 3)
    with PicContext(0) as ctx:
        lib, h = ctx.lib, ctx.h
        ctx.load_workload(wl)
        ctx.initial_setup()
        ctx.steps(3)
        ctx.synchronize()
        try:
            _fail_allocations(lib, after)
            rc = lib.fdf_ReserveParticles(h, 1_000_000)
        finally:
            _fail_allocations(lib, -1)
        assert rc == ERR_MEM
        assert lib.fdf_AdvanceStep(h, None) == ERR_WRONGSTATE
        assert lib.fdf_AdvanceSteps(h, 2) == ERR_WRONGSTATE
        assert lib.fdf_ResetAllParticleStatuses(h) == ERR_WRONGSTATE
        assert lib.fdf_ScatterAllParticleFieldsToEulerFields(h) == ERR_WRONGSTATE
        ctx.load_workload(wl)
        ctx.initial_setup()
        ctx.steps(3)
        got = (ctx.get_swarm(), ctx.get_faces())
    _same(got, want)


def test_failed_momentum_allocation(require_gpu):
    wl = W.config_sinusoidal(IM=10, JM=8, KM=24, n=3000, cfl=1.0, steps=2)
    with PicContext(0) as ctx:
        lib, h = ctx.lib, ctx.h
        ctx.load_workload(wl, form=FORM_FP32)
        try:
            _fail_allocations(lib, 1)   # the FP64 array is made, the FP32 one fails
            rc = lib.fdf_SetMomentumDeposit(h, 1)
        finally:
            _fail_allocations(lib, -1)
        assert rc == ERR_MEM
        ctx.initial_setup()
        ctx.steps(2)                    # runs without the momentum deposit
        z = np.zeros(1)
        p = ctypes.c_void_p(z.ctypes.data)
        assert lib.fdf_GetFaceMomentum(h, p, p, p) == ERR_WRONGSTATE
        ctx.set_momentum_deposit(True)  # both arrays made again
        ctx.steps(1)
        mi, mj, mk = ctx.get_face_momentum()
        assert np.isfinite(mi).all() and np.abs(mk).sum() > 0


def test_tensor_core_wait_runs_out(require_gpu):
    wl = W.config_bent_pipe(8, 6, 16, n=2000, cfl=1.0)
    pts = np.random.default_rng(2).uniform(-0.2, 0.2, size=(5000, 3)) + wl.coor.reshape(-1, 3).mean(0)
    with PicContext(0) as ctx:
        ctx.set_grid(wl.coor)
        ctx.locator_init(seed=3)
        cells0, y0 = ctx.locator_predict(pts)
        rc = ctx.lib.fdf_TestLocatorWaitTimeout(ctx.h, ctypes.c_void_p(np.ascontiguousarray(pts).ctypes.data),
                                                len(pts))
        assert rc == ERR_GPU
        assert b"timed out" in ctx.lib.fdf_GetLastError(ctx.h)
        cells1, y1 = ctx.locator_predict(pts)   # nothing left in flight: the next call works
        ctx.synchronize()
    assert np.array_equal(cells0, cells1) and np.array_equal(y0, y1)


def test_training_tensor_core_wait_runs_out(require_gpu):
    """The fused training kernel's bounded wait, made to run out with no MMA in flight: the call
    reports the time-out, the weights are untouched, and the next gradient call equals the one
    before it."""
    wl = W.config_bent_pipe(8, 6, 16, n=2000, cfl=1.0)
    rng = np.random.default_rng(5)
    B = 300
    xhat = np.ascontiguousarray(rng.uniform(-1, 1, size=(B, 3)).astype(np.float32))
    tgt = np.ascontiguousarray(rng.uniform(-1, 1, size=(B, 3)).astype(np.float32))
    with PicContext(0) as ctx:
        ctx.set_grid(wl.coor)
        ctx.locator_init(seed=3)
        p0 = ctx.locator_get_params()
        g0, l0 = ctx.locator_gradients(xhat, tgt)
        rc = ctx.lib.fdf_TestLocatorTrainTimeout(ctx.h, ctypes.c_void_p(xhat.ctypes.data),
                                                 ctypes.c_void_p(tgt.ctypes.data), B)
        assert rc == ERR_GPU
        assert b"timed out" in ctx.lib.fdf_GetLastError(ctx.h)
        g1, l1 = ctx.locator_gradients(xhat, tgt)   # nothing left in flight: the next call works
        assert np.array_equal(p0, ctx.locator_get_params())
    assert np.array_equal(g0, g1) and l0 == l1


def test_locate_points_out_of_range_start_cells(require_gpu):
    wl = W.config_sinusoidal(IM=10, JM=8, KM=20, n=10, cfl=1.0, steps=1)
    g = O.Grid(wl.coor)
    rng = np.random.default_rng(11)
    pts = rng.uniform(0.02, 0.98, size=(400, 3))
    bad = np.array([[1 << 32, 0, 0], [0, (1 << 32) + 3, 0], [0, 0, 1 << 62], [10, 0, 0], [0, 8, 0], [0, 0, 20],
                    [-5, 3, 3], [3, -1, 3], [(1 << 32) - 1, 1, 1], [2, 3, -(1 << 40)]], dtype=np.int64)
    cells = bad[np.arange(400) % len(bad)]
    with PicContext(0) as ctx:
        ctx.set_grid(wl.coor)
        cout, w, st = ctx.locate_points(pts, cells)
        cout0, w0, st0 = ctx.locate_points(pts)          # no start cells: (0,0,0)
    assert np.array_equal(cout, cout0) and np.array_equal(st, st0)
    assert np.array_equal(w.view(np.int64), w0.view(np.int64))
    for p in range(0, 400, 7):
        r = O.locate_particle(g, pts[p], cells[p])
        assert np.array_equal(cout[p], r["cell"]) and st[p] == r["status"], p
