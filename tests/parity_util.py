"""Shared helpers for the GPU-vs-oracle parity tests (test infrastructure)."""
from __future__ import annotations

import numpy as np

from fdf_gb300.context import SwarmArrays
from oracle import oracle as O


def to_oracle_swarm(s: SwarmArrays) -> O.Swarm:
    n = s.n
    return O.Swarm(pos=s.position.copy(), vel=s.velocity.copy(), weight=s.weight.copy(), P=s.P.copy(),
                   cell=s.cell.copy(), pid=s.pid.copy(), status=s.status.copy(), n=n)


def from_oracle_swarm(o: O.Swarm) -> SwarmArrays:
    v = o.view()
    return SwarmArrays(v["pos"].copy(), v["vel"].copy(), v["weight"].copy(), v["P"].copy(), v["cell"].copy(),
                       v["pid"].copy(), v["status"].copy())


def assert_swarm_bitwise(gpu: SwarmArrays, ref: SwarmArrays, what: str = ""):
    """Same particle set (by PID) with bit-identical fields."""
    a, b = gpu.sorted_by_pid(), ref.sorted_by_pid()
    assert a.n == b.n, f"{what}: particle count {a.n} != {b.n}"
    assert np.array_equal(a.pid, b.pid), f"{what}: PID sets differ"
    for name in ("cell", "status"):
        x, y = getattr(a, name), getattr(b, name)
        bad = np.nonzero((x != y).reshape(len(x), -1).any(axis=1))[0]
        assert len(bad) == 0, f"{what}: {name} differs for {len(bad)} particles, first PID {a.pid[bad[0]]}"
    for name in ("position", "velocity", "weight", "P"):
        x, y = getattr(a, name), getattr(b, name)
        same = (x.view(np.int64) == y.view(np.int64)) | (np.isnan(x) & np.isnan(y))
        bad = np.nonzero(~same.reshape(len(x), -1).all(axis=1))[0]
        assert len(bad) == 0, (f"{what}: {name} not bit-identical for {len(bad)} particles, first PID "
                               f"{a.pid[bad[0]]}: {x[bad[0]]} vs {y[bad[0]]}")


def assert_faces_close(gpu_faces, ref: dict, rel: float = 1e-12, what: str = ""):
    """Face sums within rel * (sum of |contributions|) per face (summation order differs)."""
    for g, key, akey in zip(gpu_faces, ("fi", "fj", "fk"), ("abs_i", "abs_j", "abs_k")):
        r, scale = ref[key], ref[akey]
        err = np.abs(g - r)
        tol = rel * scale + 1e-300
        assert np.all(err <= tol), f"{what}: {key} max err {err.max()} (tol {rel} x |sum|)"


def assert_faces_bitwise(gpu_faces, ref: dict, what: str = ""):
    """Face sums bit-identical: both sides sum in (cell, PID) order from 0.0."""
    for g, key in zip(gpu_faces, ("fi", "fj", "fk")):
        r = ref[key]
        bad = np.nonzero(g.view(np.int64) != r.view(np.int64))
        assert len(bad[0]) == 0, (f"{what}: {key} differs at {len(bad[0])} faces, first {tuple(b[0] for b in bad)}: "
                                  f"{g[tuple(b[0] for b in bad)]} vs {r[tuple(b[0] for b in bad)]}")
