"""Host-side mirror of the reference's particle-path interface over the C ABI.

``PicContext`` stands in for PICurv's ``UserCtx`` + DMSwarm on one GPU: it
owns the device-resident grid, velocity field and swarm, and exposes the
reference's operations (``PerformInitialSetup``, ``AdvanceStep`` = one
iteration of ``AdvanceSimulation_TEST``) with the reference's error codes
raised as ``PetscError``.  Arrays cross the boundary in the reference's own
layouts (DMSwarm ``[n][bs]`` fields, DMDA ``[k][j][i]`` arrays).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import FdfStepInfo

ERR_NAMES = {55: "PETSC_ERR_MEM", 56: "PETSC_ERR_SUP", 62: "PETSC_ERR_ARG_WRONG", 63: "PETSC_ERR_ARG_OUTOFRANGE",
             73: "PETSC_ERR_ARG_WRONGSTATE", 76: "PETSC_ERR_LIB", 83: "PETSC_ERR_USER", 85: "PETSC_ERR_ARG_NULL",
             90: "PETSC_ERR_FLOP_COUNT",
             97: "PETSC_ERR_GPU"}
NEEDS_LOCATION, ACTIVE_AND_LOCATED, MIGRATING_OUT, LOST, UNINITIALIZED = 0, 1, 2, 3, 4
FORM_PLAIN_FP64, FORM_FP32, FORM_LEARNED_FP32 = 0, 1, 2
TRANSFER_STAGED, TRANSFER_IN_PLACE, TRANSFER_AUTO = 0, 1, 2
LOCATOR_BF16, LOCATOR_F16 = 0, 1
LOCATOR_NPARAM = 33923


class PetscError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERR_NAMES.get(code, code)} ({code}): {msg}")
        self.code = code


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    return ctypes.c_void_p(a.ctypes.data)


@dataclass
class SwarmArrays:
    """DMSwarm fields in the reference's layout."""
    position: np.ndarray   # [n][3] f64
    velocity: np.ndarray   # [n][3] f64
    weight: np.ndarray     # [n][3] f64
    P: np.ndarray          # [n]    f64
    cell: np.ndarray       # [n][3] i64  DMSwarm_CellID
    pid: np.ndarray        # [n]    i64  DMSwarm_pid
    status: np.ndarray     # [n]    i64  DMSwarm_location_status

    @property
    def n(self) -> int:
        return len(self.pid)

    @classmethod
    def create(cls, position, cell=None, pid=None, P=101325.0, status=UNINITIALIZED) -> "SwarmArrays":
        n = len(position)
        return cls(position=np.ascontiguousarray(position, dtype=np.float64).reshape(n, 3).copy(),
                   velocity=np.zeros((n, 3)), weight=np.zeros((n, 3)), P=np.full(n, P, dtype=np.float64),
                   cell=(np.full((n, 3), -1, dtype=np.int64) if cell is None
                         else np.ascontiguousarray(cell, dtype=np.int64).reshape(n, 3).copy()),
                   pid=(np.arange(n, dtype=np.int64) if pid is None else np.asarray(pid, dtype=np.int64).copy()),
                   status=np.full(n, status, dtype=np.int64))

    @classmethod
    def empty(cls, n: int) -> "SwarmArrays":
        return cls(position=np.zeros((n, 3)), velocity=np.zeros((n, 3)), weight=np.zeros((n, 3)), P=np.zeros(n),
                   cell=np.zeros((n, 3), dtype=np.int64), pid=np.zeros(n, dtype=np.int64),
                   status=np.zeros(n, dtype=np.int64))

    def truncated(self, n: int) -> "SwarmArrays":
        return SwarmArrays(self.position[:n], self.velocity[:n], self.weight[:n], self.P[:n], self.cell[:n],
                           self.pid[:n], self.status[:n])

    def sorted_by_pid(self) -> "SwarmArrays":
        o = np.argsort(self.pid, kind="stable")
        return SwarmArrays(self.position[o], self.velocity[o], self.weight[o], self.P[o], self.cell[o], self.pid[o],
                           self.status[o])


class PicContext:
    """Device-resident grid + swarm on one GPU (the C ABI's FdfContext)."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        rc = self.lib.fdf_ContextCreate(ctypes.byref(h), int(device))
        if rc:
            raise PetscError(rc, "fdf_ContextCreate failed (no usable CUDA device?)")
        self.h = h
        self.dims = None
        self._cap = 0

    # -- lifetime
    def close(self):
        if self.h:
            self.lib.fdf_ContextDestroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc:
            msg = self.lib.fdf_GetLastError(self.h)
            raise PetscError(rc, msg.decode() if msg else "")

    # -- set-up
    def set_grid(self, coor: np.ndarray):
        coor = np.ascontiguousarray(coor, dtype=np.float64)
        KM, JM, IM = (s - 1 for s in coor.shape[:3])
        self._check(self.lib.fdf_SetGrid(self.h, IM, JM, KM, _ptr(coor)))
        self.dims = (IM, JM, KM)

    def set_ucat(self, ucat: np.ndarray):
        ucat = np.ascontiguousarray(ucat, dtype=np.float64)
        IM, JM, KM = self.dims
        if ucat.shape[:3] == (KM + 1, JM + 1, IM + 1):
            node_sized = 1
        elif ucat.shape[:3] == (KM, JM, IM):
            node_sized = 0
        else:
            raise ValueError(f"ucat shape {ucat.shape} matches neither the cell nor the node layout")
        self._check(self.lib.fdf_SetUcat(self.h, _ptr(ucat), node_sized))

    def get_ucat(self, node_sized: bool = True) -> np.ndarray:
        """The context's cell-centred ucat, node-sized [KM+1][JM+1][IM+1][3] (or [KM][JM][IM][3])."""
        IM, JM, KM = self.dims
        shp = (KM + 1, JM + 1, IM + 1, 3) if node_sized else (KM, JM, IM, 3)
        out = np.empty(shp)
        self._check(self.lib.fdf_GetUcat(self.h, _ptr(out), 1 if node_sized else 0))
        return out

    # -- Eulerian input: face velocity -> ucat (Contra2Cart, setup.c:1294-1420)
    def grid_metrics(self):
        """(csi, eta, zet, aj, flipped) of the grid after the orientation check (Metric.c)."""
        IM, JM, KM = self.dims
        shp = (KM + 1, JM + 1, IM + 1)
        csi, eta, zet = (np.empty(shp + (3,)) for _ in range(3))
        aj = np.empty(shp)
        fl = ctypes.c_int(0)
        self._check(self.lib.fdf_GetGridMetrics(self.h, _ptr(csi), _ptr(eta), _ptr(zet), _ptr(aj),
                                                ctypes.byref(fl)))
        return csi, eta, zet, aj, bool(fl.value)

    def set_ucont(self, ucont: np.ndarray):
        """Contravariant face velocity, node-sized [KM+1][JM+1][IM+1][3] (the reference's lUcont)."""
        ucont = np.ascontiguousarray(ucont, dtype=np.float64)
        IM, JM, KM = self.dims
        if ucont.shape != (KM + 1, JM + 1, IM + 1, 3):
            raise ValueError(f"ucont shape {ucont.shape} is not the node-sized [KM+1][JM+1][IM+1][3]")
        self._check(self.lib.fdf_SetUcont(self.h, _ptr(ucont)))

    def contra2cart(self):
        """ucat of the interior cells from the face velocity, on the device (stream-ordered)."""
        self._check(self.lib.fdf_Contra2Cart(self.h))

    def contra2cart_device(self, ucont):
        """Contra2Cart reading a CUDA float64 tensor [KM+1][JM+1][IM+1][3] in place (no copy).
        The tensor's pending writes on PyTorch's current stream are waited for first."""
        import torch
        IM, JM, KM = self.dims
        if not (isinstance(ucont, torch.Tensor) and ucont.is_cuda and ucont.dtype == torch.float64
                and ucont.is_contiguous() and tuple(ucont.shape) == (KM + 1, JM + 1, IM + 1, 3)):
            raise ValueError("ucont must be a contiguous CUDA float64 tensor [KM+1][JM+1][IM+1][3]")
        torch.cuda.current_stream(ucont.device).synchronize()
        self._check(self.lib.fdf_Contra2CartDevice(self.h, ctypes.c_void_p(ucont.data_ptr())))

    def set_transfer_route(self, route: int):
        """TRANSFER_AUTO (the default: per direction, the route measured faster on this machine),
        TRANSFER_STAGED (copy engines through a staging buffer) or TRANSFER_IN_PLACE."""
        self._check(self.lib.fdf_SetTransferRoute(self.h, int(route)))

    def transfer_routes(self) -> tuple[int, int]:
        """(upload, download) routes in use; -1 where AUTO has not measured yet."""
        up, down = ctypes.c_int(), ctypes.c_int()
        self._check(self.lib.fdf_GetTransferRoutes(self.h, ctypes.byref(up), ctypes.byref(down)))
        return up.value, down.value

    def set_form(self, form: int):
        """FORM_PLAIN_FP64 (bit-exact), FORM_FP32 (precision form) or FORM_LEARNED_FP32 (precision
        form with the learned start cell); applies at the next set_swarm / seed_particles."""
        self._check(self.lib.fdf_SetForm(self.h, int(form)))

    def set_dt(self, dt: float):
        self._check(self.lib.fdf_SetTimeStep(self.h, float(dt)))

    def set_volume(self, v: float):
        self._check(self.lib.fdf_SetParticleVolume(self.h, float(v)))

    def reserve(self, cap: int):
        self._check(self.lib.fdf_ReserveParticles(self.h, int(cap)))
        self._cap = max(self._cap, int(cap))

    def set_swarm(self, s: SwarmArrays):
        arrs = [np.ascontiguousarray(a) for a in (s.position, s.velocity, s.weight, s.P, s.cell, s.pid, s.status)]
        assert arrs[0].dtype == np.float64 and arrs[4].dtype == np.int64
        self._check(self.lib.fdf_SetSwarm(self.h, s.n, *[_ptr(a) for a in arrs]))
        self._cap = max(self._cap, s.n)

    def load_workload(self, wl, P: float = 101325.0, form: int | None = None):
        if form is not None:
            self.set_form(form)
        self.set_grid(wl.coor)
        self.set_ucat(wl.ucat)
        self.set_dt(wl.dt)
        self.set_volume(wl.volume)
        if wl.pos is None:
            self.seed_particles(wl.seed_n, wl.meta.get("seed", 0),
                                start_in_generating_cell=not wl.meta.get("corner_start", False), P=P)
        else:
            self.set_swarm(SwarmArrays.create(wl.pos, cell=wl.cell0, P=P))

    def seed_particles(self, n: int, seed: int = 0, start_in_generating_cell: bool = True, pid_base: int = 0,
                       P: float = 101325.0):
        """n particles seeded on the device, bit-identical to workloads.volumetric_particles."""
        self._check(self.lib.fdf_SeedParticles(self.h, int(n), int(seed), 1 if start_in_generating_cell else 0,
                                               int(pid_base), float(P)))
        self._cap = max(self._cap, int(n))

    # -- read back
    def size(self) -> int:
        n = ctypes.c_int64()
        self._check(self.lib.fdf_GetSwarmSize(self.h, ctypes.byref(n)))
        return n.value

    def get_swarm(self) -> SwarmArrays:
        n = self.size()
        out = SwarmArrays.empty(n)
        got = ctypes.c_int64()
        self._check(self.lib.fdf_GetSwarm(self.h, n, ctypes.byref(got), _ptr(out.position), _ptr(out.velocity),
                                          _ptr(out.weight), _ptr(out.P), _ptr(out.cell), _ptr(out.pid),
                                          _ptr(out.status)))
        return out.truncated(got.value)

    def get_scattered(self):
        IM, JM, KM = self.dims
        count = np.zeros((KM + 1, JM + 1, IM + 1))
        avg = np.zeros_like(count)
        self._check(self.lib.fdf_GetScatteredFields(self.h, _ptr(count), _ptr(avg)))
        return count, avg

    def get_corner(self):
        IM, JM, KM = self.dims
        c = np.zeros((KM + 1, JM + 1, IM + 1, 3))
        self._check(self.lib.fdf_GetCornerField(self.h, _ptr(c)))
        return c

    def get_faces(self):
        IM, JM, KM = self.dims
        fi = np.zeros((KM, JM, IM + 1)); fj = np.zeros((KM, JM + 1, IM)); fk = np.zeros((KM + 1, JM, IM))
        self._check(self.lib.fdf_GetFaceDeposits(self.h, _ptr(fi), _ptr(fj), _ptr(fk)))
        return fi, fj, fk

    def write_swarm_field(self, field: str, path: str, int64_indices: bool = True):
        """WriteSwarmField: the field as a PETSc binary Vec file."""
        self._check(self.lib.fdf_WriteSwarmField(self.h, field.encode(), path.encode(), 1 if int64_indices else 0))

    def read_swarm_field(self, field: str, path: str, int64_indices: bool = True):
        """ReadSwarmField: replaces the field from a PETSc binary Vec file of the swarm's length."""
        self._check(self.lib.fdf_ReadSwarmField(self.h, field.encode(), path.encode(), 1 if int64_indices else 0))

    def set_momentum_deposit(self, on: bool = True):
        self._check(self.lib.fdf_SetMomentumDeposit(self.h, 1 if on else 0))

    def get_face_momentum(self):
        IM, JM, KM = self.dims
        mi = np.zeros((KM, JM, IM + 1, 3)); mj = np.zeros((KM, JM + 1, IM, 3)); mk = np.zeros((KM + 1, JM, IM, 3))
        self._check(self.lib.fdf_GetFaceMomentum(self.h, _ptr(mi), _ptr(mj), _ptr(mk)))
        return mi, mj, mk

    # -- the reference's stages one call at a time (ParticleMotion.c, interpolation.c)
    def reset_statuses(self):
        self._check(self.lib.fdf_ResetAllParticleStatuses(self.h))

    def update_positions(self):
        self._check(self.lib.fdf_UpdateAllParticlePositions(self.h))

    def locate(self) -> FdfStepInfo:
        info = FdfStepInfo()
        self._check(self.lib.fdf_LocateAllParticlesInGrid(self.h, ctypes.byref(info)))
        return info

    def remove_lost(self) -> int:
        n = ctypes.c_int64()
        self._check(self.lib.fdf_CheckAndRemoveLostParticles(self.h, ctypes.byref(n)))
        return n.value

    def remove_out_of_bounds(self) -> int:
        n = ctypes.c_int64()
        self._check(self.lib.fdf_CheckAndRemoveOutOfBoundsParticles(self.h, ctypes.byref(n)))
        return n.value

    def interpolate(self):
        self._check(self.lib.fdf_InterpolateAllFieldsToSwarm(self.h))

    def scatter(self):
        self._check(self.lib.fdf_ScatterAllParticleFieldsToEulerFields(self.h))

    def locate_points(self, position: np.ndarray, cell: np.ndarray | None = None):
        """The reference walk for points outside the swarm: (cell [n][3], weight [n][3], status [n])."""
        position = np.ascontiguousarray(position, dtype=np.float64).reshape(-1, 3)
        n = len(position)
        cin = None if cell is None else np.ascontiguousarray(cell, dtype=np.int64).reshape(n, 3)
        cout = np.empty((n, 3), dtype=np.int64)
        w = np.empty((n, 3))
        st = np.empty(n, dtype=np.int64)
        self._check(self.lib.fdf_LocatePoints(self.h, n, _ptr(position), _ptr(cin), _ptr(cout), _ptr(w), _ptr(st)))
        return cout, w, st

    def interpolate_points(self, cell: np.ndarray, weight: np.ndarray) -> np.ndarray:
        """The reference's interpolation for caller-held particles (cells [n][3], weights [n][3]), in order."""
        cell = np.ascontiguousarray(cell, dtype=np.int64).reshape(-1, 3)
        weight = np.ascontiguousarray(weight, dtype=np.float64).reshape(-1, 3)
        vel = np.empty((len(cell), 3))
        self._check(self.lib.fdf_InterpolatePoints(self.h, len(cell), _ptr(cell), _ptr(weight), _ptr(vel)))
        return vel

    # -- k-slab decomposition over several ranks (fdf_gb300/slabs.py)
    def extract_particles(self, k_lo: int, k_hi: int) -> SwarmArrays:
        """The held particles whose cell's k lies outside [k_lo, k_hi) leave the context."""
        n_max = self.size()
        out = SwarmArrays.empty(n_max)
        got = ctypes.c_int64()
        self._check(self.lib.fdf_ExtractParticles(self.h, int(k_lo), int(k_hi), n_max, ctypes.byref(got),
                                                  _ptr(out.position), _ptr(out.velocity), _ptr(out.weight),
                                                  _ptr(out.P), _ptr(out.cell), _ptr(out.pid), _ptr(out.status)))
        return out.truncated(got.value)

    def add_particles(self, s: SwarmArrays):
        """Particles from another rank join the held swarm (their cells, weights, statuses kept)."""
        arrs = [np.ascontiguousarray(a) for a in (s.position, s.velocity, s.weight, s.P, s.cell, s.pid, s.status)]
        self._check(self.lib.fdf_AddParticles(self.h, s.n, *[_ptr(a) for a in arrs]))

    def deposit_k_layer(self, k: int, seed: np.ndarray, seed_momentum: np.ndarray | None = None):
        """The k-faces of layer k summed again from seed[j][i] (the lower cell's part), then the held
        particles of layer k (plain form)."""
        seed = np.ascontiguousarray(seed, dtype=np.float64)
        sm = None if seed_momentum is None else np.ascontiguousarray(seed_momentum, dtype=np.float64)
        self._check(self.lib.fdf_DepositKFaceLayer(self.h, int(k), _ptr(seed), _ptr(sm)))

    # -- the hot path
    def initial_setup(self) -> FdfStepInfo:
        info = FdfStepInfo()
        self._check(self.lib.fdf_PerformInitialSetup(self.h, ctypes.byref(info)))
        return info

    def step(self, info: bool = True) -> FdfStepInfo | None:
        if info:
            inf = FdfStepInfo()
            self._check(self.lib.fdf_AdvanceStep(self.h, ctypes.byref(inf)))
            return inf
        self._check(self.lib.fdf_AdvanceStep(self.h, None))
        return None

    def steps(self, n: int):
        self._check(self.lib.fdf_AdvanceSteps(self.h, int(n)))

    def synchronize(self):
        self._check(self.lib.fdf_Synchronize(self.h))

    @property
    def stream(self) -> int:
        return int(self.lib.fdf_GetStream(self.h) or 0)

    @property
    def launches(self) -> int:
        return int(self.lib.fdf_GetLaunchCount(self.h))

    STAGES = ("center_to_corner", "advect_locate", "sort_by_cell", "wait_corner", "gather_interpolate",
              "deposit", "learned_guess", "guess_walk", "contra2cart")

    def counters(self) -> tuple[int, int, int]:
        """(particle-steps advanced, walk evaluations made, corner nodes computed) since the swarm was set."""
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self._check(self.lib.fdf_GetCounters(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def set_profiling(self, on: bool):
        self._check(self.lib.fdf_SetProfiling(self.h, 1 if on else 0))

    def stage_times(self) -> dict:
        """{stage: (total ms, runs)} since profiling was enabled (CUDA events on the context stream)."""
        ms = np.zeros(len(self.STAGES))
        runs = np.zeros(len(self.STAGES), dtype=np.int64)
        self._check(self.lib.fdf_GetStageTimes(self.h, _ptr(ms), _ptr(runs), len(self.STAGES)))
        return {name: (float(ms[i]), int(runs[i])) for i, name in enumerate(self.STAGES)}

    # -- learned start-cell locator
    def locator_init(self, seed: int = 0):
        self._check(self.lib.fdf_LocatorInit(self.h, int(seed)))

    def locator_train(self, n_samples: int, seed: int = 0, steps: int = 4000, batch: int = 8192,
                      lr: float = 2e-3) -> np.ndarray:
        """Trains the locator on the device; returns the loss of every step."""
        hist = np.zeros(max(int(steps), 1), dtype=np.float32)
        self._check(self.lib.fdf_LocatorTrain(self.h, int(n_samples), int(seed), int(steps), int(batch), float(lr),
                                              _ptr(hist)))
        return hist[:int(steps)]

    def locator_set_params(self, params: np.ndarray):
        p = np.ascontiguousarray(params, dtype=np.float32).ravel()
        self._check(self.lib.fdf_LocatorSetParams(self.h, _ptr(p), p.size))

    def locator_get_params(self) -> np.ndarray:
        p = np.zeros(LOCATOR_NPARAM, dtype=np.float32)
        self._check(self.lib.fdf_LocatorGetParams(self.h, _ptr(p), p.size))
        return p

    def locator_normalization(self) -> tuple[np.ndarray, np.ndarray]:
        c = np.zeros(3, dtype=np.float32)
        h = np.zeros(3, dtype=np.float32)
        self._check(self.lib.fdf_LocatorGetNormalization(self.h, _ptr(c), _ptr(h)))
        return c, h

    def locator_gradients(self, xhat: np.ndarray, target: np.ndarray) -> tuple[np.ndarray, float]:
        x = np.ascontiguousarray(xhat, dtype=np.float32).reshape(-1, 3)
        t = np.ascontiguousarray(target, dtype=np.float32).reshape(-1, 3)
        g = np.zeros(LOCATOR_NPARAM, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        self._check(self.lib.fdf_LocatorGradients(self.h, _ptr(x), _ptr(t), len(x), _ptr(g), _ptr(loss)))
        return g, float(loss[0])

    def locator_predict(self, pos: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
        """(cells [n][3] i64, network outputs [n][3] f32) for host positions [n][3]."""
        p = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        cells = np.zeros((len(p), 3), dtype=np.int64)
        out = np.zeros((len(p), 3), dtype=np.float32)
        self._check(self.lib.fdf_LocatorPredict(self.h, _ptr(p), len(p), _ptr(cells), _ptr(out)))
        return cells, out

    def locator_inference_type(self, kind: int):
        """Inference operands: LOCATOR_BF16 (default) or LOCATOR_F16."""
        self._check(self.lib.fdf_LocatorSetInferenceType(self.h, int(kind)))

    def locator_min_distance(self, cells: float):
        """Particles at least `cells` cells past their previous cell get a network guess."""
        self._check(self.lib.fdf_LocatorSetMinDistance(self.h, float(cells)))

    def locator_stats(self) -> tuple[int, int, int, int]:
        """(particles given a prediction, evaluations of their walks from P1 on the predicted path,
        evaluations of those walks, 0)."""
        a, b, c, d = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self._check(self.lib.fdf_LocatorGetStats(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                                 ctypes.byref(d)))
        return a.value, b.value, c.value, d.value
