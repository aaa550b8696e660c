"""GPU: the standalone stable sort by cell (fdf_SortByCell) against numpy's stable argsort."""
import ctypes

import numpy as np
import pytest

from fdf_gb300 import _lib

pytestmark = pytest.mark.gpu


def sort_by_cell_gpu(cells: np.ndarray, ncells: int):
    import torch
    lib = _lib.load()
    dev = torch.device("cuda:0")
    c = torch.from_numpy(cells.astype(np.int32)).to(dev)
    n = len(cells)
    perm = torch.full((max(n, 1),), -1, dtype=torch.int32, device=dev)
    start = torch.zeros(ncells + 1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = lib.fdf_SortByCell(ctypes.c_void_p(c.data_ptr()), n, ncells, ctypes.c_void_p(perm.data_ptr()),
                            ctypes.c_void_p(start.data_ptr()), ctypes.c_void_p(stream.cuda_stream))
    assert rc == 0
    torch.cuda.synchronize()
    start_np = start.cpu().numpy().view(np.uint32).astype(np.int64)
    placed = int(start_np[-1])
    return perm.cpu().numpy().view(np.uint32)[:placed].astype(np.int64), start_np


def reference(cells: np.ndarray, ncells: int):
    valid = np.nonzero((cells >= 0) & (cells < ncells))[0]
    order = valid[np.argsort(cells[valid], kind="stable")]
    counts = np.bincount(cells[valid], minlength=ncells)
    start = np.concatenate([[0], np.cumsum(counts)])
    return order, start


@pytest.mark.parametrize("n,ncells,seed", [(0, 10, 0), (1, 1, 1), (1000, 7, 2), (200_000, 50_000, 3),
                                           (1_000_000, 4_194_304, 4)])
def test_sort_by_cell_matches_stable_argsort(require_gpu, n, ncells, seed):
    rng = np.random.default_rng(seed)
    cells = rng.integers(-3, ncells + 3, size=n)
    perm, start = sort_by_cell_gpu(cells, ncells)
    ref_perm, ref_start = reference(cells, ncells)
    assert np.array_equal(start, ref_start)
    assert np.array_equal(perm, ref_perm)


def test_sort_by_cell_crowded_cells(require_gpu):
    """Long segments (more than 32 slots per cell) take the in-place ordering path."""
    rng = np.random.default_rng(5)
    cells = rng.integers(0, 3, size=5000)
    perm, start = sort_by_cell_gpu(cells, 3)
    ref_perm, ref_start = reference(cells, 3)
    assert np.array_equal(start, ref_start) and np.array_equal(perm, ref_perm)
