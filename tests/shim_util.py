"""Builds and wraps the reference-signature shim (fdf_gb300/shim/picurv_shim.c) for the tests:
the shim, the PETSc stand-in (tests/petsc_stub/minipetsc.c) and the test harness
(tests/shim/shim_harness.c) in one shared library linked against libfdf_gb300.so.
headers="compat" compiles against the stand-ins of the reference's headers
(tests/petsc_stub/picurv); headers="reference" against the reference's own include/ (where
present), which checks that every function the shim defines has the reference's prototype.
Test infrastructure."""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

from fdf_gb300 import build as fdf_build
from oracle import ref_build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SHIM = os.path.join(ROOT, "fdf_gb300", "shim", "picurv_shim.c")
STUB = os.path.join(ROOT, "tests", "petsc_stub")
HARNESS = os.path.join(ROOT, "tests", "shim", "shim_harness.c")
OUT = os.path.join(ROOT, "tests", "_build")
CFLAGS = ["-std=gnu11", "-O2", "-fPIC", "-shared", "-fvisibility=hidden", "-Wall", "-Wextra"]


def header_dir(headers: str) -> str | None:
    if headers == "compat":
        return os.path.join(STUB, "picurv")
    ref = ref_build.reference_dir()
    return os.path.join(ref, "include") if ref else None


def build(headers: str = "compat") -> str:
    inc = header_dir(headers)
    if inc is None:
        raise FileNotFoundError("the reference's headers are not present")
    lib = fdf_build.build()
    os.makedirs(OUT, exist_ok=True)
    out = os.path.join(OUT, f"libshim_{headers}.so")
    srcs = [SHIM, os.path.join(STUB, "minipetsc.c"), HARNESS]
    deps = srcs + [os.path.join(STUB, "minipetsc.h"), lib] + [os.path.join(inc, f) for f in os.listdir(inc)]
    if os.path.exists(out) and all(os.path.getmtime(d) <= os.path.getmtime(out) for d in deps):
        return out
    tmp = out + f".tmp{os.getpid()}"
    cmd = ["gcc", *CFLAGS, "-I", STUB, "-I", inc, "-I", os.path.join(ROOT, "include"), *srcs, "-o", tmp,
           "-L", os.path.dirname(lib), "-lfdf_gb300", f"-Wl,-rpath,{os.path.dirname(lib)}", "-lm"]
    if headers == "reference":
        cmd.insert(len(CFLAGS) + 1, "-Wno-unused-parameter")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"building the shim against {headers} headers failed:\n{r.stderr}")
    os.replace(tmp, out)
    return out


def compile_warnings(headers: str = "compat") -> str:
    """The compiler's diagnostics for the shim alone (-fsyntax-only, -Wall -Wextra)."""
    inc = header_dir(headers)
    cmd = ["gcc", "-std=gnu11", "-fsyntax-only", "-Wall", "-Wextra", "-I", STUB, "-I", inc, "-I",
           os.path.join(ROOT, "include"), SHIM]
    return subprocess.run(cmd, capture_output=True, text=True).stderr


D = ctypes.POINTER(ctypes.c_double)
I64 = ctypes.POINTER(ctypes.c_int64)


def _d(a):
    return a.ctypes.data_as(D)


def _i(a):
    return a.ctypes.data_as(I64)


_libs = {}


def lib(headers: str = "compat"):
    if headers not in _libs:
        L = ctypes.CDLL(build(headers))
        V = ctypes.c_void_p
        L.shim_last_error.restype = ctypes.c_char_p
        L.shim_signed_distance.argtypes = [D] * 6 + [ctypes.c_double, D]
        L.shim_characteristic_size.argtypes = [D, D]
        L.shim_evaluate_position.argtypes = [D, D, ctypes.c_double, D, I64]
        L.shim_point_position.argtypes = [D, I64]
        L.shim_update_indices.argtypes = [D, I64]
        L.shim_update_weights.argtypes = [D, D]
        L.shim_sim_create.restype = V
        L.shim_sim_create.argtypes = [ctypes.c_int64] * 3 + [D, D, ctypes.c_double, ctypes.c_int]
        L.shim_sim_destroy.argtypes = [V]
        L.shim_sim_destroy.restype = None
        L.shim_set_ucat.argtypes = [V, D]
        L.shim_swarm_set.argtypes = [V, ctypes.c_int64, D, D, D, D, I64, I64, I64]
        L.shim_swarm_size.argtypes = [V, I64]
        L.shim_swarm_get.argtypes = [V, D, D, D, D, I64, I64, I64]
        L.shim_stage.argtypes = [V, ctypes.c_int, I64]
        L.shim_locate_point.argtypes = [V, D, I64, D, I64, D, I64]
        L.shim_get_scattered.argtypes = [V, D, D]
        _libs[headers] = L
    return _libs[headers]


class ShimError(RuntimeError):
    def __init__(self, L, code, what):
        msg = L.shim_last_error()
        super().__init__(f"{what}: PETSc error {code} {msg.decode() if msg else ''}")
        self.code = code


class ShimSim:
    """A one-rank PICurv UserCtx driven through the shim's reference-signature functions."""

    STAGES = ("reset", "update_positions", "locate", "remove_lost", "remove_out_of_bounds", "interpolate", "scatter",
              "count")

    def __init__(self, coor, ucat=None, dt=0.0, device=-1, headers="compat"):
        self.L = lib(headers)
        self.coor = np.ascontiguousarray(coor, dtype=np.float64)
        KM, JM, IM = (s - 1 for s in self.coor.shape[:3])
        self.dims = (IM, JM, KM)
        self._u = None if ucat is None else np.ascontiguousarray(ucat, dtype=np.float64)
        h = self.L.shim_sim_create(IM, JM, KM, _d(self.coor), _d(self._u) if self._u is not None else None,
                                   float(dt), int(device))
        if not h:
            raise ShimError(self.L, -1, "shim_sim_create")
        self.h = ctypes.c_void_p(h)

    def close(self):
        if self.h:
            self.L.shim_sim_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc:
            e = ShimError(self.L, rc, what)
            self.L.shim_clear_error()
            raise e

    def set_swarm(self, s):
        a = [np.ascontiguousarray(x) for x in (s.position, s.velocity, s.weight, s.P, s.cell, s.pid, s.status)]
        self._check(self.L.shim_swarm_set(self.h, len(a[5]), _d(a[0]), _d(a[1]), _d(a[2]), _d(a[3]), _i(a[4]),
                                          _i(a[5]), _i(a[6])), "shim_swarm_set")

    def swarm(self):
        n = np.zeros(1, np.int64)
        self._check(self.L.shim_swarm_size(self.h, _i(n)), "size")
        m = int(n[0])
        out = [np.zeros((m, 3)), np.zeros((m, 3)), np.zeros((m, 3)), np.zeros(m), np.zeros((m, 3), np.int64),
               np.zeros(m, np.int64), np.zeros(m, np.int64)]
        self._check(self.L.shim_swarm_get(self.h, _d(out[0]), _d(out[1]), _d(out[2]), _d(out[3]), _i(out[4]),
                                          _i(out[5]), _i(out[6])), "shim_swarm_get")
        return out

    def stage(self, name):
        r = np.zeros(1, np.int64)
        self._check(self.L.shim_stage(self.h, self.STAGES.index(name), _i(r)), name)
        return int(r[0])

    def initial_setup(self):
        for s in ("locate", "interpolate", "scatter"):
            self.stage(s)

    def step(self):
        self.stage("reset")
        self.stage("update_positions")
        self.stage("locate")
        lost = self.stage("remove_lost")
        oob = self.stage("remove_out_of_bounds")
        self.stage("interpolate")
        self.stage("scatter")
        return lost, oob

    def locate_point(self, p, cell, w_in=(0.0, 0.0, 0.0)):
        pp, ci, wi = (np.ascontiguousarray(x, dtype=t) for x, t in ((p, np.float64), (cell, np.int64),
                                                                     (w_in, np.float64)))
        co, w, st = np.zeros(3, np.int64), np.zeros(3), np.zeros(1, np.int64)
        rc = self.L.shim_locate_point(self.h, _d(pp), _i(ci), _d(wi), _i(co), _d(w), _i(st))
        return dict(err=rc, cell=co, weights=w, status=int(st[0]))

    def scattered(self):
        IM, JM, KM = self.dims
        c, p = np.zeros((KM + 1, JM + 1, IM + 1)), np.zeros((KM + 1, JM + 1, IM + 1))
        self._check(self.L.shim_get_scattered(self.h, _d(c), _d(p)), "scattered")
        return c, p
