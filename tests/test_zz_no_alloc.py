"""GPU: fdf_SortByCellNoAlloc, the sort by cell for callers that cannot allocate device
memory (their device buffers belong to another allocator, or the call sits where no
allocation may happen), checked against fdf_SortByCell through the C ABI.

Collected last on purpose (file name), so that a stopping-at-first-failure run has
already run every other test.  It passes alone in a fresh process and after the others:
each call clears its shared scratch, so no earlier call's contents leak in.
"""
import ctypes

import numpy as np
import pytest

from fdf_gb300 import _lib

pytestmark = pytest.mark.gpu

MAX_CELLS = 1048576   # FDF_NOALLOC_MAX_CELLS in include/fdf_gb300.h


def _run(fn_name, cells: np.ndarray, ncells: int):
    import torch
    lib = _lib.load()
    dev = torch.device("cuda:0")
    c = torch.from_numpy(cells.astype(np.int32)).to(dev)
    n = len(cells)
    perm = torch.full((max(n, 1),), -1, dtype=torch.int32, device=dev)
    start = torch.full((ncells + 1,), -7, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = getattr(lib, fn_name)(ctypes.c_void_p(c.data_ptr()), n, ncells, ctypes.c_void_p(perm.data_ptr()),
                               ctypes.c_void_p(start.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    torch.cuda.synchronize()
    start_np = start.cpu().numpy().view(np.uint32).astype(np.int64)
    placed = int(start_np[-1]) if rc == 0 else 0
    return rc, perm.cpu().numpy().view(np.uint32)[:placed].astype(np.int64), start_np


def test_no_alloc_sort_matches_allocating_sort_twice(require_gpu):
    rng = np.random.default_rng(11)
    # two calls in a row on different inputs: the second must not see the first's scratch
    cases = [(rng.integers(-2, 300_000 + 2, size=600_000), 300_000),
             (rng.integers(0, MAX_CELLS, size=250_000), MAX_CELLS)]
    for cells, ncells in cases:
        rc_a, perm_a, start_a = _run("fdf_SortByCell", cells, ncells)
        rc_b, perm_b, start_b = _run("fdf_SortByCellNoAlloc", cells, ncells)
        assert rc_a == 0 and rc_b == 0
        assert np.array_equal(start_a, start_b)      # integer outputs: tolerance is exact equality
        assert np.array_equal(perm_a, perm_b)


def test_no_alloc_sort_rejects_too_many_cells(require_gpu):
    cells = np.zeros(10, dtype=np.int64)
    rc, _, _ = _run("fdf_SortByCellNoAlloc", cells, MAX_CELLS + 1)
    assert rc == 63    # FDF_ERR_ARG_OUTOFRANGE, nothing launched
