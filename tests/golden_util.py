"""Loader of tests/golden/ref_golden.npz (outputs of the reference's own code, written by
tests/golden/make_ref_golden.py) for the CPU and GPU golden tests (test infrastructure)."""
from __future__ import annotations

import os

import numpy as np

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_golden.npz")
RUNS = ("sinusoidal_cfl1", "bent_pipe_cfl4", "curved_pipe", "uniform_corner_start")
STEPS = 3


def load() -> dict:
    with np.load(PATH) as z:
        return {k: z[k] for k in z.files}


def bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.int64)


def run_inputs(g: dict, name: str):
    p = f"run_{name}/"
    return g[p + "coor"], g[p + "ucat"], float(g[p + "dt"][0]), g[p + "pos0"], g[p + "cell0"], float(g[p + "P0"][0])


def check_state(g: dict, name: str, k: int, pos, vel, weight, P, cell, pid, status, count, avg, what=""):
    """Bit-for-bit comparison of a swarm (any order) and the grid fields with snapshot k."""
    q = f"run_{name}/s{k}/"
    o = np.argsort(pid, kind="stable")
    assert len(pid) == len(g[q + "pid"]), f"{what}: {len(pid)} particles, the reference has {len(g[q + 'pid'])}"
    assert np.array_equal(pid[o], g[q + "pid"]), f"{what}: particle sets differ"
    for f, a in (("cell", cell), ("status", status)):
        bad = np.nonzero(np.asarray(a)[o].reshape(len(o), -1) != g[q + f].reshape(len(o), -1))[0]
        assert len(bad) == 0, f"{what}: {f} differs for {len(bad)} particles, first PID {g[q + 'pid'][bad[0]]}"
    for f, a in (("pos", pos), ("vel", vel), ("weight", weight), ("P", P)):
        bad = np.nonzero((bits(np.asarray(a)[o]) != bits(g[q + f])).reshape(len(o), -1).any(axis=1))[0]
        assert len(bad) == 0, f"{what}: {f} not bit-identical for {len(bad)} particles, first PID {g[q + 'pid'][bad[0]]}"
    assert np.array_equal(bits(count), bits(g[q + "count"])), f"{what}: ParticleCount differs"
    assert np.array_equal(bits(avg), bits(g[q + "avg"])), f"{what}: P average differs"
