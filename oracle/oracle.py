"""TEST INFRASTRUCTURE, NOT PART OF THE PRODUCT.

ctypes wrapper around the CPU restatement of PICurv's particle hot path
(``picurv_oracle.c``).  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` use it, and only as
the checker or the timed CPU baseline -- never as the product path.

The C source restates, function by function, the reference files
``src/walkingsearch.c``, ``src/ParticleSwarm.c``, ``src/ParticleMotion.c`` and
``src/interpolation.c`` (citations in the C source).  The reference itself
cannot be built here (it needs PETSc and MPI), so this restatement is the
oracle; it is pinned by the known-answer tests in ``tests/test_oracle_kats.py``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "picurv_oracle.c")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "libpicurv_oracle.so")

CFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC", "-shared", "-std=c11"]

NEEDS_LOCATION, ACTIVE_AND_LOCATED, MIGRATING_OUT, LOST, UNINITIALIZED = 0, 1, 2, 3, 4
LEFT, RIGHT, BOTTOM, TOP, FRONT, BACK = 0, 1, 2, 3, 4, 5
ERR_USER = 83
ERR_ARG_NULL = 85
ERR_FLOP_COUNT = 90


def build(force: bool = False) -> str:
    """Compile the oracle with gcc (no FMA contraction) into oracle/_build/."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC),
                                             os.path.getmtime(os.path.join(HERE, "picurv_oracle.h")))):
        return LIB
    tmp = LIB + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", *CFLAGS, "-o", tmp, SRC, "-lm"])
    os.replace(tmp, LIB)
    return LIB


class OCmpnts(ctypes.Structure):
    _fields_ = [("x", ctypes.c_double), ("y", ctypes.c_double), ("z", ctypes.c_double)]


class OCell(ctypes.Structure):
    _fields_ = [("vertices", OCmpnts * 8)]


class OGrid(ctypes.Structure):
    _fields_ = [("IM", ctypes.c_int64), ("JM", ctypes.c_int64), ("KM", ctypes.c_int64),
                ("coor", ctypes.POINTER(ctypes.c_double))]


class OSwarm(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64),
                ("pos", ctypes.POINTER(ctypes.c_double)),
                ("vel", ctypes.POINTER(ctypes.c_double)),
                ("weight", ctypes.POINTER(ctypes.c_double)),
                ("P", ctypes.POINTER(ctypes.c_double)),
                ("cell", ctypes.POINTER(ctypes.c_int64)),
                ("pid", ctypes.POINTER(ctypes.c_int64)),
                ("status", ctypes.POINTER(ctypes.c_int64))]


class OStepInfo(ctypes.Structure):
    _fields_ = [("removed_lost", ctypes.c_int64), ("removed_oob", ctypes.c_int64),
                ("evals", ctypes.c_int64), ("n_start", ctypes.c_int64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        L = ctypes.CDLL(path)
        D = ctypes.POINTER(ctypes.c_double)
        I64 = ctypes.POINTER(ctypes.c_int64)
        L.o_GetCellCharacteristicSize.argtypes = [ctypes.POINTER(OCell), D]
        L.o_ComputeSignedDistanceToPlane.argtypes = [OCmpnts] * 6 + [D, ctypes.c_double]
        L.o_CalculateDistancesToCellFaces.argtypes = [OCmpnts, ctypes.POINTER(OCell), D, ctypes.c_double]
        L.o_DeterminePointPosition.argtypes = [D, I64]
        L.o_UpdateCellIndicesBasedOnDistancesTEST.argtypes = [D, I64, I64, I64]
        L.o_UpdateParticleWeights.argtypes = [D, D]
        L.o_EvaluateParticlePosition.argtypes = [ctypes.POINTER(OCell), D, OCmpnts, I64, ctypes.c_double]
        L.o_LocateParticleOrFindMigrationTarget.argtypes = [ctypes.POINTER(OGrid), D, I64, D, I64, I64]
        L.o_LocateAllParticlesInGrid.argtypes = [ctypes.POINTER(OGrid), ctypes.POINTER(OSwarm), ctypes.c_int, I64]
        L.o_UpdateAllParticlePositions.argtypes = [ctypes.POINTER(OSwarm), ctypes.c_double, ctypes.c_int]
        L.o_ResetAllParticleStatuses.argtypes = [ctypes.POINTER(OSwarm)]
        L.o_CheckAndRemoveLostParticles.argtypes = [ctypes.POINTER(OSwarm), I64]
        L.o_CheckAndRemoveOutOfBoundsParticles.argtypes = [ctypes.POINTER(OGrid), ctypes.POINTER(OSwarm), I64]
        L.o_ComputeLocalBoundingBox.argtypes = [ctypes.POINTER(OGrid), D, D]
        L.o_InterpolateFieldFromCenterToCorner_Vector.argtypes = [ctypes.POINTER(OGrid), D, D, ctypes.c_int]
        L.o_TrilinearInterpolation_Vector.argtypes = [ctypes.POINTER(OGrid), D, ctypes.c_int64, ctypes.c_int64,
                                                      ctypes.c_int64, ctypes.c_double, ctypes.c_double,
                                                      ctypes.c_double, D]
        L.o_InterpolateEulerFieldToSwarm.argtypes = [ctypes.POINTER(OGrid), D, ctypes.POINTER(OSwarm), ctypes.c_int]
        L.o_ScatterParticleFieldToEulerField_P.argtypes = [ctypes.POINTER(OGrid), ctypes.POINTER(OSwarm), D, D]
        L.o_DepositParticlesToFaces.argtypes = [ctypes.POINTER(OGrid), ctypes.POINTER(OSwarm), ctypes.c_double,
                                                D, D, D, D, D, D, D, D, D]
        L.o_AdvanceStep.argtypes = [ctypes.POINTER(OGrid), D, D, ctypes.POINTER(OSwarm), ctypes.c_double,
                                    D, D, ctypes.c_int, ctypes.POINTER(OStepInfo)]
        L.o_InitialSetup.argtypes = [ctypes.POINTER(OGrid), D, D, ctypes.POINTER(OSwarm), D, D, ctypes.c_int,
                                     ctypes.POINTER(OStepInfo)]
        L.o_ComputeFaceMetrics.argtypes = [ctypes.POINTER(OGrid), D, D, D]
        L.o_ComputeFaceMetrics.restype = None
        L.o_ComputeCellCenteredJacobianInverse.argtypes = [ctypes.POINTER(OGrid), D]
        L.o_CheckAndFixGridOrientation.argtypes = [ctypes.POINTER(OGrid), D, D, D, D, ctypes.POINTER(ctypes.c_int)]
        L.o_Contra2Cart.argtypes = [ctypes.POINTER(OGrid), D, D, D, D, D]
        _lib = L
    return _lib


def _dp(a):
    if a is None:
        return ctypes.POINTER(ctypes.c_double)()
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


def cmp(v) -> OCmpnts:
    return OCmpnts(float(v[0]), float(v[1]), float(v[2]))


def cell_from_vertices(verts) -> OCell:
    c = OCell()
    for q in range(8):
        c.vertices[q] = cmp(verts[q])
    return c


class Grid:
    """Node coordinates [KM+1][JM+1][IM+1][3] (one-rank DMDA layout)."""

    def __init__(self, coor: np.ndarray):
        assert coor.ndim == 4 and coor.shape[3] == 3
        self.coor = np.ascontiguousarray(coor, dtype=np.float64)
        self.KM, self.JM, self.IM = (s - 1 for s in coor.shape[:3])
        self.c = OGrid(self.IM, self.JM, self.KM, _dp(self.coor))

    @property
    def node_shape(self):
        return (self.KM + 1, self.JM + 1, self.IM + 1)


@dataclass
class Swarm:
    """DMSwarm fields of one rank, AoS like the reference's arrays."""
    pos: np.ndarray
    vel: np.ndarray
    weight: np.ndarray
    P: np.ndarray
    cell: np.ndarray
    pid: np.ndarray
    status: np.ndarray
    n: int = 0

    @classmethod
    def create(cls, pos, pid=None, P=101325.0, cell=None, status=UNINITIALIZED):
        n = len(pos)
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(n, 3).copy()
        return cls(pos=pos,
                   vel=np.zeros((n, 3)),
                   weight=np.zeros((n, 3)),
                   P=np.full(n, P, dtype=np.float64),
                   cell=(np.full((n, 3), -1, dtype=np.int64) if cell is None
                         else np.ascontiguousarray(cell, dtype=np.int64).reshape(n, 3).copy()),
                   pid=(np.arange(n, dtype=np.int64) if pid is None else np.asarray(pid, dtype=np.int64).copy()),
                   status=np.full(n, status, dtype=np.int64),
                   n=n)

    def c(self) -> OSwarm:
        return OSwarm(self.n, _dp(self.pos), _dp(self.vel), _dp(self.weight), _dp(self.P),
                      _ip(self.cell), _ip(self.pid), _ip(self.status))

    def sync(self, cs: OSwarm):
        self.n = int(cs.n)

    def view(self):
        n = self.n
        return dict(pos=self.pos[:n], vel=self.vel[:n], weight=self.weight[:n], P=self.P[:n],
                    cell=self.cell[:n], pid=self.pid[:n], status=self.status[:n])

    def sorted_by_pid(self):
        v = self.view()
        order = np.argsort(v["pid"], kind="stable")
        return {k: a[order] for k, a in v.items()}


def nthreads_default() -> int:
    return os.cpu_count() or 1


def locate_particle(grid: Grid, loc, cell=(-1, -1, -1), weights=(0.0, 0.0, 0.0)):
    L = lib()
    loc = np.asarray(loc, dtype=np.float64).copy()
    cell = np.asarray(cell, dtype=np.int64).copy()
    w = np.asarray(weights, dtype=np.float64).copy()
    st = ctypes.c_int64(0)
    steps = ctypes.c_int64(0)
    err = L.o_LocateParticleOrFindMigrationTarget(ctypes.byref(grid.c), _dp(loc), _ip(cell), _dp(w),
                                                  ctypes.byref(st), ctypes.byref(steps))
    return dict(err=err, cell=cell, weights=w, status=st.value, steps=steps.value)


def locate_all(grid: Grid, s: Swarm, nthreads: int | None = None):
    L = lib()
    cs = s.c()
    ev = ctypes.c_int64(0)
    err = L.o_LocateAllParticlesInGrid(ctypes.byref(grid.c), ctypes.byref(cs), nthreads or nthreads_default(),
                                       ctypes.byref(ev))
    return err, ev.value


def center_to_corner(grid: Grid, ucat_nodesized: np.ndarray, nthreads: int | None = None) -> np.ndarray:
    corner = np.zeros(grid.node_shape + (3,))
    lib().o_InterpolateFieldFromCenterToCorner_Vector(ctypes.byref(grid.c), _dp(np.ascontiguousarray(ucat_nodesized)),
                                                      _dp(corner), nthreads or nthreads_default())
    return corner


def interpolate(grid: Grid, corner: np.ndarray, s: Swarm, nthreads: int | None = None):
    cs = s.c()
    lib().o_InterpolateEulerFieldToSwarm(ctypes.byref(grid.c), _dp(corner), ctypes.byref(cs),
                                         nthreads or nthreads_default())


def scatter_P(grid: Grid, s: Swarm):
    count = np.zeros(grid.node_shape)
    avg = np.zeros(grid.node_shape)
    cs = s.c()
    lib().o_ScatterParticleFieldToEulerField_P(ctypes.byref(grid.c), ctypes.byref(cs), _dp(count), _dp(avg))
    return count, avg


def deposit_faces(grid: Grid, s: Swarm, volume: float = 1.0, momentum: bool = False):
    IM, JM, KM = grid.IM, grid.JM, grid.KM
    fi = np.zeros((KM, JM, IM + 1)); fj = np.zeros((KM, JM + 1, IM)); fk = np.zeros((KM + 1, JM, IM))
    ai = np.zeros_like(fi); aj = np.zeros_like(fj); ak = np.zeros_like(fk)
    mi = mj = mk = None
    if momentum:
        mi = np.zeros(fi.shape + (3,)); mj = np.zeros(fj.shape + (3,)); mk = np.zeros(fk.shape + (3,))
    cs = s.c()
    lib().o_DepositParticlesToFaces(ctypes.byref(grid.c), ctypes.byref(cs), float(volume),
                                    _dp(fi), _dp(fj), _dp(fk), _dp(mi), _dp(mj), _dp(mk),
                                    _dp(ai), _dp(aj), _dp(ak))
    out = dict(fi=fi, fj=fj, fk=fk, abs_i=ai, abs_j=aj, abs_k=ak)
    if momentum:
        out.update(mom_i=mi, mom_j=mj, mom_k=mk)
    return out


def remove_lost(s: Swarm) -> int:
    cs = s.c()
    r = ctypes.c_int64(0)
    lib().o_CheckAndRemoveLostParticles(ctypes.byref(cs), ctypes.byref(r))
    s.sync(cs)
    return r.value


def remove_oob(grid: Grid, s: Swarm) -> int:
    cs = s.c()
    r = ctypes.c_int64(0)
    lib().o_CheckAndRemoveOutOfBoundsParticles(ctypes.byref(grid.c), ctypes.byref(cs), ctypes.byref(r))
    s.sync(cs)
    return r.value


def bounding_box(grid: Grid):
    bmin = np.zeros(3); bmax = np.zeros(3)
    lib().o_ComputeLocalBoundingBox(ctypes.byref(grid.c), _dp(bmin), _dp(bmax))
    return bmin, bmax


class Simulation:
    """The reference's one-rank time loop (simulation.c:202-315) on the oracle."""

    def __init__(self, grid: Grid, ucat_nodesized: np.ndarray, swarm: Swarm, dt: float,
                 nthreads: int | None = None):
        self.grid, self.s, self.dt = grid, swarm, float(dt)
        self.ucat = np.ascontiguousarray(ucat_nodesized, dtype=np.float64)
        self.corner = np.zeros(grid.node_shape + (3,))
        self.count = np.zeros(grid.node_shape)
        self.avg = np.zeros(grid.node_shape)
        self.nthreads = nthreads or nthreads_default()

    def initial_setup(self) -> OStepInfo:
        info = OStepInfo()
        cs = self.s.c()
        err = lib().o_InitialSetup(ctypes.byref(self.grid.c), _dp(self.ucat), _dp(self.corner), ctypes.byref(cs),
                                   _dp(self.count), _dp(self.avg), self.nthreads, ctypes.byref(info))
        self.s.sync(cs)
        if err:
            raise RuntimeError(f"oracle initial setup failed with PETSc error {err}")
        return info

    def step(self, scatter: bool = True) -> OStepInfo:
        info = OStepInfo()
        cs = self.s.c()
        err = lib().o_AdvanceStep(ctypes.byref(self.grid.c), _dp(self.ucat), _dp(self.corner), ctypes.byref(cs),
                                  self.dt, _dp(self.count) if scatter else _dp(None),
                                  _dp(self.avg) if scatter else _dp(None), self.nthreads, ctypes.byref(info))
        self.s.sync(cs)
        if err:
            raise RuntimeError(f"oracle step failed with PETSc error {err}")
        return info


class OracleError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"{what}: PETSc error {code}")
        self.code = code


def grid_metrics(g: Grid):
    """Metric.c:286-460, 491-600 and 195-260 in the reference's order (face metrics, Jacobian
    inverse, orientation check).  Returns (csi, eta, zet, aj, flipped); csi/eta/zet are
    node-sized [KM+1][JM+1][IM+1][3], aj [KM+1][JM+1][IM+1].  Raises OracleError with the
    PETSc code on a near-zero Jacobian (90) or a grid of mixed orientation (83)."""
    L = lib()
    shp = g.node_shape
    csi, eta, zet = (np.zeros(shp + (3,)) for _ in range(3))
    aj = np.zeros(shp)
    L.o_ComputeFaceMetrics(ctypes.byref(g.c), _dp(csi), _dp(eta), _dp(zet))
    rc = L.o_ComputeCellCenteredJacobianInverse(ctypes.byref(g.c), _dp(aj))
    if rc:
        raise OracleError(rc, "ComputeCellCenteredJacobianInverse")
    flipped = ctypes.c_int(0)
    rc = L.o_CheckAndFixGridOrientation(ctypes.byref(g.c), _dp(csi), _dp(eta), _dp(zet), _dp(aj),
                                        ctypes.byref(flipped))
    if rc:
        raise OracleError(rc, "CheckAndFixGridOrientation")
    return csi, eta, zet, aj, bool(flipped.value)


def contra2cart(g: Grid, ucont: np.ndarray, csi, eta, zet, ucat: np.ndarray | None = None) -> np.ndarray:
    """setup.c:1294-1420: node-sized ucat of the interior cells from ucont (node-sized [..][3]);
    entries of `ucat` (zeros when None) outside the interior cells are left as given."""
    L = lib()
    ucont = np.ascontiguousarray(ucont, dtype=np.float64)
    out = np.zeros(g.node_shape + (3,)) if ucat is None else np.array(ucat, dtype=np.float64, copy=True)
    rc = L.o_Contra2Cart(ctypes.byref(g.c), _dp(ucont), _dp(csi), _dp(eta), _dp(zet), _dp(out))
    if rc:
        raise OracleError(rc, "Contra2Cart")
    return out
