"""GPU: swarm fields written and read in the reference's PETSc binary Vec format through the
context (WriteSwarmField / ReadSwarmField), and a run started from an FDFGRID grid file."""
import numpy as np
import pytest

from fdf_gb300 import formats as F
from fdf_gb300 import workloads as W
from fdf_gb300.context import FORM_FP32, FORM_PLAIN_FP64, PicContext
from tests.test_formats import np_read_vec, np_write_vec

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(require_gpu):
    c = PicContext(0)
    yield c
    c.close()


def _run(ctx, wl, coor, steps, form):
    ctx.set_form(form)
    ctx.set_grid(coor)
    ctx.set_ucat(wl.ucat)
    ctx.set_dt(wl.dt)
    from fdf_gb300.context import SwarmArrays
    ctx.set_swarm(SwarmArrays.create(wl.pos, cell=wl.cell0))
    ctx.initial_setup()
    ctx.steps(steps)
    return ctx.get_swarm(), ctx.get_faces()


def test_run_from_grid_file_is_identical(ctx, tmp_path):
    wl = W.config_sinusoidal(IM=12, JM=10, KM=32, n=5000, cfl=1.0, steps=3)
    p = str(tmp_path / "grid.dat")
    F.write_grid_file(p, wl.coor)
    coor = F.read_grid_file(p)
    a = _run(ctx, wl, wl.coor, wl.steps, FORM_PLAIN_FP64)
    b = _run(ctx, wl, coor, wl.steps, FORM_PLAIN_FP64)
    for f in ("position", "velocity", "cell", "pid"):
        assert np.array_equal(getattr(a[0], f), getattr(b[0], f)), f
    for x, y in zip(a[1], b[1]):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("form", [FORM_PLAIN_FP64, FORM_FP32])
def test_swarm_fields_round_trip(ctx, tmp_path, form):
    wl = W.config_sinusoidal(IM=12, JM=10, KM=32, n=5000, cfl=1.0, steps=2)
    s, _ = _run(ctx, wl, wl.coor, wl.steps, form)
    for field, bs in (("position", 3), ("velocity", 3), ("weight", 3), ("P", 1)):
        p = str(tmp_path / f"{field}00002_0.dat")
        ctx.write_swarm_field(field, p)
        vals, n = np_read_vec(p)
        want = getattr(s, field).ravel()
        assert n == want.size and np.array_equal(vals.view(np.int64), want.view(np.int64)), field
        if bs > 1:
            assert open(p + ".info").read() == f"-vecload_block_size {bs}\n"
    # a restart replaces the velocity field from a file the reference's VecLoad would read
    newv = np.arange(s.velocity.size, dtype=np.float64).reshape(-1, 3) * 1e-3
    q = str(tmp_path / "velocity00003_0.dat")
    np_write_vec(q, newv.ravel())
    ctx.read_swarm_field("velocity", q)
    t = ctx.get_swarm()
    want = newv if form == FORM_PLAIN_FP64 else newv.astype(np.float32).astype(np.float64)
    assert np.array_equal(t.velocity, want)
    assert np.array_equal(t.position, s.position) and np.array_equal(t.pid, s.pid)
    ctx.set_form(FORM_PLAIN_FP64)
