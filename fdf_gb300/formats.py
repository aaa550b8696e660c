"""The reference's on-disk formats through the C ABI (host-side; no GPU needed).

``read_grid_file`` / ``write_grid_file``: FDFGRID text grid files (io.c:101-170,
grid.c:356-383).  ``write_petsc_vec`` / ``read_petsc_vec``: PETSc binary Vec files as
VecView writes them on one rank (io.c:653-700), with 64-bit PetscInt headers by default
(the reference's own PETSc build).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib


def _check(code: int, what: str):
    if code != 0:
        raise OSError(f"{what} failed with code {code}")


def read_grid_file(path: str) -> np.ndarray:
    """Node coordinates [KM+1][JM+1][IM+1][3] of the file's first block."""
    lib = _lib.load()
    IM, JM, KM = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    _check(lib.fdf_ReadGridFile(path.encode(), ctypes.byref(IM), ctypes.byref(JM), ctypes.byref(KM), None, 0),
           "fdf_ReadGridFile")
    coor = np.zeros((KM.value + 1, JM.value + 1, IM.value + 1, 3))
    _check(lib.fdf_ReadGridFile(path.encode(), ctypes.byref(IM), ctypes.byref(JM), ctypes.byref(KM),
                                ctypes.c_void_p(coor.ctypes.data), coor.size), "fdf_ReadGridFile")
    return coor


def write_grid_file(path: str, coor: np.ndarray):
    c = np.ascontiguousarray(coor, dtype=np.float64)
    KM, JM, IM = (s - 1 for s in c.shape[:3])
    _check(_lib.load().fdf_WriteGridFile(path.encode(), IM, JM, KM, ctypes.c_void_p(c.ctypes.data)),
           "fdf_WriteGridFile")


def write_petsc_vec(path: str, values: np.ndarray, bs: int = 1, int64_indices: bool = True):
    v = np.ascontiguousarray(values, dtype=np.float64).ravel()
    _check(_lib.load().fdf_WritePetscVec(path.encode(), ctypes.c_void_p(v.ctypes.data), v.size, int(bs),
                                         1 if int64_indices else 0), "fdf_WritePetscVec")


def read_petsc_vec(path: str, int64_indices: bool = True) -> np.ndarray:
    lib = _lib.load()
    n = ctypes.c_int64()
    flag = 1 if int64_indices else 0
    _check(lib.fdf_ReadPetscVec(path.encode(), None, 0, ctypes.byref(n), flag), "fdf_ReadPetscVec")
    out = np.zeros(n.value)
    _check(lib.fdf_ReadPetscVec(path.encode(), ctypes.c_void_p(out.ctypes.data), out.size, ctypes.byref(n), flag),
           "fdf_ReadPetscVec")
    return out
