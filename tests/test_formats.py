"""CPU: the reference's on-disk formats written and read through the C ABI, checked against an
independent numpy restatement of each format.

* PETSc binary Vec (VecView on one rank): big-endian {1211214, N} as PetscInt (8 or 4 bytes),
  then N big-endian doubles; block size > 1 adds "<file>.info" with -vecload_block_size.
* FDFGRID: "FDFGRID", the number of blocks, "IM JM KM" per block, then "x y z" per node,
  i fastest (io.c:101-170, grid.c:356-383).
"""
import os

import numpy as np
import pytest

from fdf_gb300 import formats as F
from fdf_gb300 import workloads as W


def np_write_vec(path, values, int64=True):
    it = ">i8" if int64 else ">i4"
    with open(path, "wb") as f:
        f.write(np.array([1211214, values.size], dtype=it).tobytes())
        f.write(np.asarray(values, dtype=">f8").tobytes())


def np_read_vec(path, int64=True):
    raw = open(path, "rb").read()
    it, ib = (">i8", 8) if int64 else (">i4", 4)
    cls, n = np.frombuffer(raw[:2 * ib], dtype=it)
    assert cls == 1211214
    return np.frombuffer(raw[2 * ib:], dtype=">f8").astype(np.float64), int(n)


@pytest.mark.parametrize("int64", [True, False])
def test_petsc_vec_write_matches_format(tmp_path, int64):
    rng = np.random.default_rng(1)
    v = np.concatenate([rng.standard_normal(3000), [0.0, -0.0, np.inf, -np.inf, 5e-324, 1.7976931348623157e308]])
    v = v[: (len(v) // 3) * 3]
    p = str(tmp_path / "position00005_0.dat")
    F.write_petsc_vec(p, v, bs=3, int64_indices=int64)
    got, n = np_read_vec(p, int64)
    assert n == v.size and np.array_equal(got.view(np.int64), v.view(np.int64))
    assert open(p + ".info").read() == "-vecload_block_size 3\n"
    assert os.path.getsize(p) == (16 if int64 else 8) + 8 * v.size


@pytest.mark.parametrize("int64", [True, False])
def test_petsc_vec_read_of_format(tmp_path, int64):
    v = np.linspace(-3.0, 7.0, 1001) ** 3
    p = str(tmp_path / "P00000_0.dat")
    np_write_vec(p, v, int64)
    got = F.read_petsc_vec(p, int64_indices=int64)
    assert np.array_equal(got.view(np.int64), v.view(np.int64))
    with pytest.raises(OSError):   # the other index width does not see the Vec class id
        F.read_petsc_vec(p, int64_indices=not int64)


def test_petsc_vec_empty_and_scalar_field(tmp_path):
    p = str(tmp_path / "e.dat")
    F.write_petsc_vec(p, np.zeros(0))
    assert F.read_petsc_vec(p).size == 0 and not os.path.exists(p + ".info")


def np_write_grid(path, coor, header=True, nblk=1):
    KM, JM, IM = (s - 1 for s in coor.shape[:3])
    with open(path, "w") as f:
        if header:
            f.write("FDFGRID\n")
        f.write(f"{nblk}\n")
        for b in range(nblk):
            f.write(f"{IM} {JM} {KM}\n")
        for x, y, z in coor.reshape(-1, 3):
            f.write(f"{float(x)!r} {float(y)!r} {float(z)!r}\n")


@pytest.mark.parametrize("header", [True, False])
def test_grid_file_read_of_format(tmp_path, header):
    coor = W.bent_pipe_grid(6, 5, 9)
    p = str(tmp_path / "grid.dat")
    np_write_grid(p, coor, header=header)
    got = F.read_grid_file(p)
    assert got.shape == coor.shape and np.array_equal(got.view(np.int64), coor.view(np.int64))


def test_grid_file_first_block_and_round_trip(tmp_path):
    coor = W.sinusoidal_grid(7, 4, 11)
    p = str(tmp_path / "two.dat")
    np_write_grid(p, coor, nblk=2)          # a second size line; the first block is read
    assert np.array_equal(F.read_grid_file(p), coor)
    q = str(tmp_path / "rt.dat")
    F.write_grid_file(q, coor)
    lines = open(q).read().split("\n")
    assert lines[0] == "FDFGRID" and lines[1] == "1" and lines[2] == "7 4 11"
    parsed = np.array([[float(t) for t in ln.split()] for ln in lines[3:] if ln]).reshape(coor.shape)
    assert np.array_equal(parsed.view(np.int64), coor.view(np.int64))    # 17 digits read back exactly
