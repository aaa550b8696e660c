"""GPU parity of the Eulerian input (fdf_eulerian.cu through the C ABI) against the oracle:
face metrics, Jacobian inverse and orientation fix (Metric.c), Contra2Cart (setup.c:1294-1420)
bit for bit, its errors, the particle path run on the converted field, and the full-size grid
of the 64M-particle bent-pipe workload (96x96x1536)."""
import dataclasses

import numpy as np
import pytest

from fdf_gb300 import workloads as W
from fdf_gb300.context import FORM_FP32, FORM_PLAIN_FP64, PetscError, PicContext
from oracle import oracle as O
from tests import pyref_metrics as R
from tests.parity_util import assert_swarm_bitwise, from_oracle_swarm, to_oracle_swarm
from tests.test_eulerian_oracle import collapsed_grid, folded_grid

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx(require_gpu):
    c = PicContext(0)
    yield c
    c.close()


GRIDS = {
    "sinusoidal": lambda: W.sinusoidal_grid(12, 10, 24),
    "bent_pipe": lambda: W.bent_pipe_grid(10, 10, 20),
    "curved_pipe": lambda: W.curved_pipe_grid(9, 7, 13),
    "thin": lambda: W.sinusoidal_grid(1, 3, 2),
    "left_handed": lambda: np.ascontiguousarray(W.sinusoidal_grid(7, 6, 9)[::-1]),
}


def assert_bitwise(a, b, what):
    """Bit for bit, except that any two NaNs match (their payloads are the machine's)."""
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape, what
    bad = (a.view(np.int64) != b.view(np.int64)) & ~(np.isnan(a) & np.isnan(b))
    assert not bad.any(), f"{what}: {int(bad.sum())} values differ, first at {np.argwhere(bad)[0]}"


@pytest.mark.parametrize("name", list(GRIDS))
def test_grid_metrics_bitwise(ctx, name):
    coor = GRIDS[name]()
    ctx.set_grid(coor)
    got = ctx.grid_metrics()
    ref = O.grid_metrics(O.Grid(coor))
    for a, b, what in zip(got[:4], ref[:4], ("csi", "eta", "zet", "aj")):
        assert_bitwise(a, b, f"{name} {what}")
    assert got[4] == ref[4] == (name == "left_handed")


def _ucat_cells(ctx):
    IM, JM, KM = ctx.dims
    return ctx.get_ucat(node_sized=True)[:KM, :JM, :IM]


@pytest.mark.parametrize("name", list(GRIDS))
def test_contra2cart_bitwise(ctx, name):
    coor = GRIDS[name]()
    KM, JM, IM = (s - 1 for s in coor.shape[:3])
    rng = np.random.default_rng(11)
    ucont = rng.uniform(-2.0, 2.0, size=coor.shape)
    ucat0 = np.zeros(coor.shape)
    ucat0[:KM, :JM, :IM] = rng.uniform(-1.0, 1.0, size=(KM, JM, IM, 3))
    ctx.set_grid(coor)
    ctx.set_ucat(ucat0)
    ctx.set_ucont(ucont)
    ctx.contra2cart()
    g = O.Grid(coor)
    csi, eta, zet, _, _ = O.grid_metrics(g)
    ref = O.contra2cart(g, ucont, csi, eta, zet, ucat0)
    assert_bitwise(_ucat_cells(ctx), ref[:KM, :JM, :IM], f"{name} ucat")
    # a second call with new face velocities reuses the table
    ucont2 = rng.uniform(-2.0, 2.0, size=coor.shape)
    ctx.set_ucont(ucont2)
    ctx.contra2cart()
    ref2 = O.contra2cart(g, ucont2, csi, eta, zet, ucat0)
    assert_bitwise(_ucat_cells(ctx), ref2[:KM, :JM, :IM], f"{name} ucat, second call")


def _check_c2c(ctx, coor, ucont, what):
    KM, JM, IM = (s - 1 for s in coor.shape[:3])
    ctx.set_grid(coor)
    ctx.set_ucont(ucont)
    ctx.contra2cart()
    g = O.Grid(coor)
    csi, eta, zet, _, _ = O.grid_metrics(g)
    ref = O.contra2cart(g, ucont, csi, eta, zet)
    assert_bitwise(_ucat_cells(ctx)[1:, 1:, 1:], ref[1:KM, 1:JM, 1:IM], what)


def test_contra2cart_extreme_face_velocities(ctx):
    """Face sums outside [2^-400, 2^400] (zeros of both signs, subnormals, huge values, inf)
    take the literal sequence; the rest the halved one: both bit for bit."""
    coor = W.sinusoidal_grid(10, 9, 12)
    rng = np.random.default_rng(21)
    ucont = rng.uniform(-1.0, 1.0, size=coor.shape)
    pick = rng.integers(0, 8, size=coor.shape)
    specials = [0.0, -0.0, 5e-324, -3e-310, 1e-300, -2e280, 1e300, np.inf]
    for q, v in enumerate(specials):
        ucont[pick == q] = np.where(rng.uniform(size=coor.shape) < 0.3, v, ucont)[pick == q]
    _check_c2c(ctx, coor, ucont, "extreme face velocities")


def test_contra2cart_wide_table(ctx):
    """A grid scaled by 2^110: tabled minors above 2^400 and 1/det below 2^-400, so the whole
    grid takes the literal sequence."""
    coor = W.sinusoidal_grid(6, 5, 7) * 2.0 ** 110
    ucont = np.random.default_rng(22).uniform(-1.0, 1.0, size=coor.shape) * 2.0 ** 216
    _check_c2c(ctx, coor, ucont, "wide table")


def test_errors(ctx):
    coor = W.sinusoidal_grid(4, 4, 4)
    ctx.set_grid(coor)
    with pytest.raises(PetscError) as e:       # setup.c:1311-1313: no face velocity yet
        ctx.contra2cart()
    assert e.value.code == 73
    for grid, code in ((collapsed_grid(), 90), (folded_grid(), 83)):
        ctx.set_grid(grid)
        with pytest.raises(PetscError) as e:
            ctx.grid_metrics()
        assert e.value.code == code
        ctx.set_ucont(np.zeros(grid.shape))
        with pytest.raises(PetscError) as e:
            ctx.contra2cart()
        assert e.value.code == code
    tiny = W.uniform_grid(3, 3, 3) * 5e-4      # Jacobian passes, the determinant does not
    ctx.set_grid(tiny)
    u0 = np.random.default_rng(3).uniform(size=(3, 3, 3, 3))
    ctx.set_ucat(u0)
    ctx.set_ucont(np.ones(tiny.shape))
    for _ in range(2):                          # the error is sticky for the grid
        with pytest.raises(PetscError) as e:
            ctx.contra2cart()
        assert e.value.code == 90
    assert np.array_equal(ctx.get_ucat(node_sized=False), u0)
    ctx.set_grid(coor)                          # a new grid forgets the face velocity
    with pytest.raises(PetscError) as e:
        ctx.contra2cart()
    assert e.value.code == 73


def _node_field_fluxes(coor, field):
    """Face fluxes of a node-evaluated velocity field through the oracle's metrics."""
    csi, eta, zet, _, _ = O.grid_metrics(O.Grid(coor))
    u = field(coor)
    out = np.empty(coor.shape)
    out[..., 0] = (csi * u).sum(-1)
    out[..., 1] = (eta * u).sum(-1)
    out[..., 2] = (zet * u).sum(-1)
    return out, (csi, eta, zet)


def _converted_workload(wl):
    ucont, (csi, eta, zet) = _node_field_fluxes(wl.coor, W.field_taylor_green)
    IM, JM, KM = wl.dims
    ucat = O.contra2cart(O.Grid(wl.coor), ucont, csi, eta, zet, wl.ucat_node_sized())
    return ucont, dataclasses.replace(wl, ucat=np.ascontiguousarray(ucat[:KM, :JM, :IM]))


def test_particle_path_on_converted_field_matches_oracle(ctx):
    wl = W.config_sinusoidal(IM=12, JM=10, KM=24, n=3000, cfl=1.0, steps=3)
    ucont, wl2 = _converted_workload(wl)
    ctx.load_workload(wl, form=FORM_PLAIN_FP64)
    ctx.set_ucont(ucont)
    ctx.contra2cart()
    s0 = ctx.get_swarm()
    g = O.Grid(wl.coor)
    os_ = to_oracle_swarm(s0)
    sim = O.Simulation(g, wl2.ucat_node_sized(), os_, wl.dt)
    ctx.initial_setup()
    sim.initial_setup()
    for st in range(wl.steps):
        ctx.step()
        sim.step()
    assert_swarm_bitwise(ctx.get_swarm(), from_oracle_swarm(os_), "steps on the converted field")
    assert np.array_equal(ctx.get_corner().view(np.int64), sim.corner.view(np.int64))


def test_fp32_form_reads_the_converted_field(ctx):
    wl = W.config_sinusoidal(IM=12, JM=10, KM=24, n=3000, cfl=1.0, steps=3)
    ucont, wl2 = _converted_workload(wl)
    outs = []
    for convert in (True, False):
        ctx.load_workload(wl if convert else wl2, form=FORM_FP32)
        if convert:
            ctx.set_ucont(ucont)
            ctx.contra2cart()
        ctx.initial_setup()
        for _ in range(wl.steps):
            ctx.step()
        outs.append(ctx.get_swarm())
    assert_swarm_bitwise(outs[0], outs[1], "FP32 form: Contra2Cart vs the same ucat set directly")


def test_full_size_grid_bitwise_and_uniform_flow(ctx):
    """The grid of the 64M-particle workload (96x96x1536 bent pipe, 14.2M cells): metrics and
    Contra2Cart bit for bit against the oracle, and a uniform flow recovered to 1e-12."""
    coor = W.bent_pipe_grid(96, 96, 1536)
    KM, JM, IM = (s - 1 for s in coor.shape[:3])
    ctx.set_grid(coor)
    csi, eta, zet, aj, flipped = ctx.grid_metrics()
    ref = O.grid_metrics(O.Grid(coor))
    for a, b, what in zip((csi, eta, zet, aj), ref[:4], ("csi", "eta", "zet", "aj")):
        assert_bitwise(a, b, f"full-size {what}")
    assert flipped == ref[4]
    u = np.array([0.3, -0.2, 1.1])
    ucont = R.ucont_of_uniform_flow(u, csi, eta, zet)
    ctx.set_ucont(ucont)
    ctx.contra2cart()
    got = _ucat_cells(ctx)
    want = O.contra2cart(O.Grid(coor), ucont, *ref[:3])
    assert_bitwise(got, want[:KM, :JM, :IM], "full-size ucat")
    err = np.abs(got[1:, 1:, 1:] - u).max()
    assert err < 1e-12 * np.abs(u).max(), err


def test_contra2cart_before_every_step(ctx):
    """The coupled pattern: new face velocities converted before every step.  Steps replayed
    from the captured step graph (fdf_AdvanceSteps) and eager steps (fdf_AdvanceStep) both read
    that step's converted ucat, bit for bit like the oracle fed the oracle's Contra2Cart."""
    wl = W.config_sinusoidal(IM=12, JM=10, KM=24, n=3000, cfl=1.0, steps=4)
    base, _ = _node_field_fluxes(wl.coor, W.field_taylor_green)
    fluxes = [base * (1.0 + 0.25 * t) for t in range(wl.steps)]
    g = O.Grid(wl.coor)
    csi, eta, zet, _, _ = O.grid_metrics(g)
    IM, JM, KM = wl.dims
    outs = []
    for replay in (True, False):
        ctx.load_workload(wl, form=FORM_PLAIN_FP64)
        s0 = ctx.get_swarm()
        ctx.initial_setup()
        os_ = to_oracle_swarm(s0)
        sim = O.Simulation(g, wl.ucat_node_sized(), os_, wl.dt)
        sim.initial_setup()
        for t in range(wl.steps):
            ctx.set_ucont(fluxes[t])
            ctx.contra2cart()
            if replay:
                ctx.steps(1)
            else:
                ctx.step()
            sim.ucat = np.ascontiguousarray(O.contra2cart(g, fluxes[t], csi, eta, zet, sim.ucat))
            sim.step()
        got = ctx.get_swarm()
        assert_swarm_bitwise(got, from_oracle_swarm(os_), f"coupled steps (replay={replay})")
        outs.append(got)
    assert_swarm_bitwise(outs[0], outs[1], "graph replay against eager steps")


def test_contra2cart_from_device_memory(ctx):
    """fdf_Contra2CartDevice reads a face velocity that is already on the GPU (a CUDA tensor)
    in place: the same bits as the host upload; host memory is refused (62)."""
    import torch
    coor = GRIDS["bent_pipe"]()
    KM, JM, IM = (s - 1 for s in coor.shape[:3])
    ucont = np.random.default_rng(31).uniform(-1.0, 1.0, size=coor.shape)
    ctx.set_grid(coor)
    ctx.contra2cart_device(torch.from_numpy(ucont).cuda())
    got = _ucat_cells(ctx)
    g = O.Grid(coor)
    csi, eta, zet, _, _ = O.grid_metrics(g)
    want = O.contra2cart(g, ucont, csi, eta, zet)
    assert_bitwise(got[1:, 1:, 1:], want[1:KM, 1:JM, 1:IM], "device-resident face velocity")
    with pytest.raises(PetscError) as e:
        ctx._check(ctx.lib.fdf_Contra2CartDevice(ctx.h, ucont.ctypes.data))
    assert e.value.code == 62
