"""GPU: fdf_SetSwarm / fdf_GetSwarm move the swarm in chunks of particles on two streams.  A
swarm spanning several chunks round-trips unchanged in the plain form, and in the precision form
every particle converts as it does in a one-chunk transfer of its own tail of the swarm."""
import numpy as np
import pytest

from fdf_gb300 import workloads as W
from fdf_gb300.context import (FORM_FP32, FORM_PLAIN_FP64, TRANSFER_IN_PLACE, TRANSFER_STAGED, PicContext,
                               SwarmArrays)

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


def _pinned(a, offset=0):
    """A page-locked copy of a (torch pinned memory), its data `offset` bytes past a 16-byte boundary."""
    import torch
    t = torch.empty(a.size * a.itemsize + 64, dtype=torch.uint8, pin_memory=True)
    base = t.data_ptr()
    start = (-base) % 16 + offset
    out = t.numpy()[start:start + a.size * a.itemsize].view(a.dtype).reshape(a.shape)
    out[...] = a
    return out, t


def _roundtrip(form, s, pinned, offset=0, launches=None, route=None, routes=None):
    wl = W.config_sinusoidal(IM=8, JM=8, KM=16, n=10, cfl=1.0, steps=1)
    keep = []
    ins = []
    for f in FIELDS:
        a = np.ascontiguousarray(getattr(s, f))
        if pinned:
            a, t = _pinned(a, offset)
            keep.append(t)
        ins.append(a)
    import ctypes
    from fdf_gb300.context import _ptr
    with PicContext(0) as ctx:
        ctx.set_form(form)
        if route is not None:
            ctx.set_transfer_route(route)
        ctx.set_grid(wl.coor)
        l0 = ctx.launches
        ctx._check(ctx.lib.fdf_SetSwarm(ctx.h, s.n, *[_ptr(a) for a in ins]))
        if launches is not None:
            launches.append(ctx.launches - l0)
        outs = []
        for f in FIELDS:
            a = np.zeros_like(np.ascontiguousarray(getattr(s, f)))
            if pinned:
                a, t = _pinned(a, offset)
                keep.append(t)
            outs.append(a)
        got = ctypes.c_int64()
        ctx._check(ctx.lib.fdf_GetSwarm(ctx.h, s.n, ctypes.byref(got), *[_ptr(a) for a in outs]))
        assert got.value == s.n
        if routes is not None:
            routes.append(ctx.transfer_routes())
    return [np.array(a) for a in outs]


@pytest.mark.parametrize("form", [FORM_PLAIN_FP64, FORM_FP32])
def test_page_locked_arrays_in_place(require_gpu, form):
    """With the in-place route, page-locked, 16-byte aligned arrays are read and written in place
    by the layout kernels; the swarm is the staged route's bit for bit (and an unaligned
    page-locked set takes the staged route).  By default (AUTO) the first page-locked transfer of
    each direction times both routes on slices of its particles and finishes with the faster,
    again bit for bit.  4500003 particles: a ragged last tile, and two chunks on the staged
    route."""
    n = 4_500_003
    s = _swarm(n, (8, 8, 16), np.random.default_rng(4))
    s.cell[s.cell[:, 0] < 0] = -1
    counts, routes = [], []
    ref = _roundtrip(form, s, pinned=False, launches=counts, routes=routes)
    direct = _roundtrip(form, s, pinned=True, launches=counts, route=TRANSFER_IN_PLACE)
    skewed = _roundtrip(form, s, pinned=True, offset=8, launches=counts, route=TRANSFER_IN_PLACE)
    default = _roundtrip(form, s, pinned=True, launches=counts, routes=routes)
    staged = _roundtrip(form, s, pinned=True, launches=counts, route=TRANSFER_STAGED)
    # staged: one layout kernel per chunk; in place: one for the swarm; AUTO: a warm-up and a
    # timed slice by each route, then the rest by the faster (one kernel either way)
    assert counts == [2, 1, 2, 5, 2]
    assert routes[0] == (-1, -1)                                  # unpinned: nothing measured
    assert all(r in (TRANSFER_STAGED, TRANSFER_IN_PLACE) for r in routes[1])
    print(f"[transfer] AUTO chose upload {routes[1][0]}, download {routes[1][1]} (0 staged, 1 in place)")
    for f, a, b, c, d, e in zip(FIELDS, ref, direct, skewed, default, staged):
        for x in (b, c, d, e):
            assert np.array_equal(a.view(np.uint8), x.view(np.uint8)), f
