"""TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.

ctypes wrapper around oracle/_ref/libpicurv_ref.so: the reference's own particle-path code
(walkingsearch.c, ParticleSwarm.c, interpolation.c, ParticleMotion.c, grid.c, setup.c,
compiled unmodified by oracle/ref_build.py against the one-rank PETSc stand-in in
tests/petsc_stub).  Available only where the reference's sources are present; the tests use it
to pin the CPU restatement (picurv_oracle.c) and to write the golden vectors under
tests/golden/.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import ref_build

_lib = None


def available() -> bool:
    return ref_build.reference_dir() is not None


def lib():
    global _lib
    if _lib is None:
        path = ref_build.build()
        if path is None:
            raise RuntimeError("the reference's sources are not present: oracle/_ref cannot be built")
        L = ctypes.CDLL(path)
        D = ctypes.POINTER(ctypes.c_double)
        I64 = ctypes.POINTER(ctypes.c_int64)
        V = ctypes.c_void_p
        L.ref_last_error.restype = ctypes.c_char_p
        L.ref_ComputeSignedDistanceToPlane.argtypes = [D] * 6 + [ctypes.c_double, D]
        L.ref_GetCellCharacteristicSize.argtypes = [D, D]
        L.ref_CalculateDistancesToCellFaces.argtypes = [D, D, ctypes.c_double, D]
        L.ref_DeterminePointPosition.argtypes = [D, I64]
        L.ref_EvaluateParticlePosition.argtypes = [D, D, ctypes.c_double, D, I64]
        L.ref_UpdateCellIndicesBasedOnDistancesTEST.argtypes = [D, I64]
        L.ref_UpdateParticleWeights.argtypes = [D, D]
        L.ref_sim_create.restype = V
        L.ref_sim_create.argtypes = [ctypes.c_int64] * 3 + [D, D, ctypes.c_double]
        L.ref_sim_bbox.argtypes = [V, D]
        L.ref_sim_set_ucat.argtypes = [V, D]
        L.ref_sim_destroy.argtypes = [V]
        L.ref_sim_destroy.restype = None
        L.ref_locate_point.argtypes = [V, D, I64, I64, D, I64]
        L.ref_swarm_set.argtypes = [V, ctypes.c_int64, D, D, D, D, I64, I64, I64]
        L.ref_swarm_size.argtypes = [V, I64]
        L.ref_swarm_get.argtypes = [V, D, D, D, D, I64, I64, I64]
        L.ref_stage.argtypes = [V, ctypes.c_int, I64]
        L.ref_initial_setup.argtypes = [V]
        L.ref_step.argtypes = [V, I64]
        L.ref_get_scattered.argtypes = [V, D, D]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _i(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


class RefError(RuntimeError):
    def __init__(self, code: int, what: str):
        msg = lib().ref_last_error()
        super().__init__(f"{what}: PETSc error {code} {msg.decode() if msg else ''}")
        self.code = code


def _check(rc: int, what: str):
    if rc:
        err = RefError(rc, what)
        lib().ref_clear_error()
        raise err


# ---- per-cell functions ----
def signed_distance(v1, v2, v3, v4, cc, p, thr):
    a = [np.ascontiguousarray(x, dtype=np.float64) for x in (v1, v2, v3, v4, cc, p)]
    d = np.zeros(1)
    rc = lib().ref_ComputeSignedDistanceToPlane(*[_d(x) for x in a], float(thr), _d(d))
    return rc, float(d[0])


def characteristic_size(verts):
    v = np.ascontiguousarray(verts, dtype=np.float64).reshape(8, 3)
    h = np.zeros(1)
    _check(lib().ref_GetCellCharacteristicSize(_d(v), _d(h)), "GetCellCharacteristicSize")
    return float(h[0])


def distances(verts, p, thr):
    v = np.ascontiguousarray(verts, dtype=np.float64).reshape(8, 3)
    pp = np.ascontiguousarray(p, dtype=np.float64)
    d = np.zeros(6)
    rc = lib().ref_CalculateDistancesToCellFaces(_d(v), _d(pp), float(thr), _d(d))
    return rc, d


def point_position(d):
    dd = np.ascontiguousarray(d, dtype=np.float64).copy()
    r = np.zeros(1, dtype=np.int64)
    _check(lib().ref_DeterminePointPosition(_d(dd), _i(r)), "DeterminePointPosition")
    return int(r[0])


def evaluate_position(verts, p, thr):
    v = np.ascontiguousarray(verts, dtype=np.float64).reshape(8, 3)
    pp = np.ascontiguousarray(p, dtype=np.float64)
    d = np.zeros(6)
    r = np.zeros(1, dtype=np.int64)
    rc = lib().ref_EvaluateParticlePosition(_d(v), _d(pp), float(thr), _d(d), _i(r))
    return rc, d, int(r[0])


def update_indices(d, ijk):
    dd = np.ascontiguousarray(d, dtype=np.float64).copy()
    x = np.ascontiguousarray(ijk, dtype=np.int64).copy()
    _check(lib().ref_UpdateCellIndicesBasedOnDistancesTEST(_d(dd), _i(x)), "UpdateCellIndicesBasedOnDistancesTEST")
    return x


def update_weights(d):
    dd = np.ascontiguousarray(d, dtype=np.float64).copy()
    w = np.zeros(3)
    _check(lib().ref_UpdateParticleWeights(_d(dd), _d(w)), "UpdateParticleWeights")
    return w, dd


@dataclass
class RefSwarm:
    pos: np.ndarray
    vel: np.ndarray
    weight: np.ndarray
    P: np.ndarray
    cell: np.ndarray
    pid: np.ndarray
    status: np.ndarray

    @property
    def n(self) -> int:
        return len(self.pid)

    def sorted_by_pid(self) -> "RefSwarm":
        o = np.argsort(self.pid, kind="stable")
        return RefSwarm(*(getattr(self, f)[o] for f in ("pos", "vel", "weight", "P", "cell", "pid", "status")))


class RefSim:
    """One rank of the reference: grid, node-sized ucat, DMSwarm with its own fields."""

    STAGES = ("reset", "update_positions", "locate", "remove_lost", "remove_out_of_bounds", "interpolate",
              "scatter")

    def __init__(self, coor: np.ndarray, ucat_nodesized: np.ndarray | None = None, dt: float = 0.0):
        self.coor = np.ascontiguousarray(coor, dtype=np.float64)
        KM, JM, IM = (s - 1 for s in self.coor.shape[:3])
        self.dims = (IM, JM, KM)
        self._u = None if ucat_nodesized is None else np.ascontiguousarray(ucat_nodesized, dtype=np.float64)
        h = lib().ref_sim_create(IM, JM, KM, _d(self.coor), _d(self._u) if self._u is not None else None, float(dt))
        if not h:
            raise RefError(-1, "ref_sim_create")
        self.h = ctypes.c_void_p(h)

    def close(self):
        if self.h:
            lib().ref_sim_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def bbox(self) -> np.ndarray:
        b = np.zeros(6)
        lib().ref_sim_bbox(self.h, _d(b))
        return b

    def locate_point(self, p, cell=(-1, -1, -1)):
        pp = np.ascontiguousarray(p, dtype=np.float64)
        ci = np.ascontiguousarray(cell, dtype=np.int64)
        co = np.zeros(3, dtype=np.int64)
        w = np.zeros(3)
        st = np.zeros(1, dtype=np.int64)
        rc = lib().ref_locate_point(self.h, _d(pp), _i(ci), _i(co), _d(w), _i(st))
        return dict(err=rc, cell=co, weights=w, status=int(st[0]))

    def set_swarm(self, pos, vel=None, weight=None, P=None, cell=None, pid=None, status=None):
        n = len(pos)
        a = dict(pos=np.ascontiguousarray(pos, dtype=np.float64).reshape(n, 3),
                 vel=np.zeros((n, 3)) if vel is None else np.ascontiguousarray(vel, dtype=np.float64),
                 weight=np.zeros((n, 3)) if weight is None else np.ascontiguousarray(weight, dtype=np.float64),
                 P=np.full(n, 101325.0) if P is None else np.ascontiguousarray(P, dtype=np.float64),
                 cell=np.full((n, 3), -1, np.int64) if cell is None else np.ascontiguousarray(cell, dtype=np.int64),
                 pid=np.arange(n, dtype=np.int64) if pid is None else np.ascontiguousarray(pid, dtype=np.int64),
                 status=np.full(n, 4, np.int64) if status is None else np.ascontiguousarray(status, dtype=np.int64))
        _check(lib().ref_swarm_set(self.h, n, _d(a["pos"]), _d(a["vel"]), _d(a["weight"]), _d(a["P"]),
                                   _i(a["cell"]), _i(a["pid"]), _i(a["status"])), "ref_swarm_set")

    def swarm(self) -> RefSwarm:
        n = np.zeros(1, dtype=np.int64)
        _check(lib().ref_swarm_size(self.h, _i(n)), "ref_swarm_size")
        m = int(n[0])
        s = RefSwarm(np.zeros((m, 3)), np.zeros((m, 3)), np.zeros((m, 3)), np.zeros(m),
                     np.zeros((m, 3), np.int64), np.zeros(m, np.int64), np.zeros(m, np.int64))
        _check(lib().ref_swarm_get(self.h, _d(s.pos), _d(s.vel), _d(s.weight), _d(s.P), _i(s.cell), _i(s.pid),
                                   _i(s.status)), "ref_swarm_get")
        return s

    def stage(self, name: str) -> int:
        r = np.zeros(1, dtype=np.int64)
        _check(lib().ref_stage(self.h, self.STAGES.index(name), _i(r)), name)
        return int(r[0])

    def initial_setup(self):
        _check(lib().ref_initial_setup(self.h), "initial setup")

    def step(self) -> tuple[int, int]:
        r = np.zeros(2, dtype=np.int64)
        _check(lib().ref_step(self.h, _i(r)), "step")
        return int(r[0]), int(r[1])

    def scattered(self):
        IM, JM, KM = self.dims
        c = np.zeros((KM + 1, JM + 1, IM + 1))
        p = np.zeros((KM + 1, JM + 1, IM + 1))
        _check(lib().ref_get_scattered(self.h, _d(c), _d(p)), "ref_get_scattered")
        return c, p
