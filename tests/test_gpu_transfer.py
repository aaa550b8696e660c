"""GPU: fdf_SetSwarm / fdf_GetSwarm move the swarm in chunks of particles on two streams.  A
swarm spanning several chunks round-trips unchanged in the plain form, and in the precision form
every particle converts as it does in a one-chunk transfer of its own tail of the swarm."""
import numpy as np
import pytest

from fdf_gb300 import workloads as W
from fdf_gb300.context import FORM_FP32, FORM_PLAIN_FP64, PicContext, SwarmArrays

pytestmark = pytest.mark.gpu

FIELDS = ("position", "velocity", "weight", "P", "cell", "pid", "status")
N = 5_000_000          # two chunks of at most 4M particles: 4M + 1M


def _swarm(n, dims, rng):
    IM, JM, KM = dims
    s = SwarmArrays.empty(n)
    s.position[...] = rng.uniform(-1, 2, (n, 3))
    s.velocity[...] = rng.normal(size=(n, 3))
    s.weight[...] = rng.uniform(0, 1, (n, 3))
    s.P[...] = rng.uniform(0, 1e5, n)
    s.cell[...] = np.stack([rng.integers(-1, IM, n), rng.integers(0, JM, n), rng.integers(0, KM, n)], 1)
    s.pid[...] = rng.permutation(n)
    s.status[...] = rng.integers(0, 4, n)
    return s


def _tail(s, t):
    out = SwarmArrays.empty(s.n - t)
    for f in FIELDS:
        getattr(out, f)[...] = getattr(s, f)[t:]
    return out


@pytest.mark.parametrize("form", [FORM_PLAIN_FP64, FORM_FP32])
def test_multi_chunk_transfers(require_gpu, form):
    wl = W.config_sinusoidal(IM=8, JM=8, KM=16, n=10, cfl=1.0, steps=1)
    s = _swarm(N, (8, 8, 16), np.random.default_rng(3))
    s.cell[s.cell[:, 0] < 0] = -1
    with PicContext(0) as ctx:
        ctx.set_form(form)
        ctx.set_grid(wl.coor)
        ctx.set_swarm(s)
        full = ctx.get_swarm()
        ctx.set_swarm(_tail(s, 4_000_000))
        tail = ctx.get_swarm()
    assert full.n == N and tail.n == N - 4_000_000
    for f in FIELDS:
        a, b = getattr(full, f)[4_000_000:], getattr(tail, f)
        assert np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8)), f
    if form == FORM_PLAIN_FP64:
        for f in FIELDS:
            assert np.array_equal(getattr(full, f), getattr(s, f)), f
