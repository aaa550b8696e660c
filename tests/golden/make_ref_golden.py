"""Writes tests/golden/ref_golden.npz: outputs of the reference's own particle-path code
(oracle/_ref/libpicurv_ref.so, the reference's C sources compiled unmodified by
oracle/ref_build.py) on small seeded inputs, for the machines where the reference's sources
are not present (the GPU tests check the CUDA path against these, the CPU tests the oracle).

Contents (every array float64 or int64):
  cells/*      per-cell functions on 300 random hexahedra and points: characteristic size,
               the six signed face distances, DeterminePointPosition, the weights
  walks/*      LocateParticleOrFindMigrationTarget_TEST on a 10x8x24 sinusoidal grid: 600
               points from start cells of every kind -> cell, weights, status
  run_<name>/* whole runs: the grid, node-sized ucat, dt, the initial positions and cells;
               after the initial setup and after each of 3 steps, the swarm sorted by PID
               (positions, velocities, weights, P, cells, statuses), ParticleCount, the P
               average and the removal counts

Run here, where the reference's sources are: python tests/golden/make_ref_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from fdf_gb300 import workloads as W  # noqa: E402
from fdf_gb300.context import SwarmArrays  # noqa: E402
from oracle import ref as R  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_golden.npz")
STEPS = 3

RUNS = {
    "sinusoidal_cfl1": lambda: W.config_sinusoidal(IM=10, JM=8, KM=24, n=600, cfl=1.0, steps=STEPS),
    "bent_pipe_cfl4": lambda: W.config_bent_pipe(8, 6, 20, n=600, cfl=4.0),
    "curved_pipe": lambda: W.config_curved_pipe(8, 8, 24, n=600, cfl=1.0),
    "uniform_corner_start": lambda: W.config1(n=400, IM=5, JM=4, KM=40, steps=STEPS),
}


def cells_section(out: dict):
    rng = np.random.default_rng(2024)
    base = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0], [0, 1, 1], [1, 1, 1], [1, 0, 1], [0, 0, 1]], float)
    n = 300
    verts = base[None] + rng.uniform(-0.3, 0.3, size=(n, 8, 3))
    verts = verts * 10.0 ** rng.uniform(-3, 2, size=(n, 1, 1)) + rng.uniform(-2, 2, size=(n, 1, 3))
    pts = np.empty((n, 3))
    h, d, pos, w = np.zeros(n), np.zeros((n, 6)), np.zeros(n, np.int64), np.zeros((n, 3))
    for q in range(n):
        lo, hi = verts[q].min(0), verts[q].max(0)
        pts[q] = rng.uniform(lo - 0.2 * (hi - lo), hi + 0.2 * (hi - lo))
        if q % 6 == 0:
            pts[q] = verts[q][[0, 3, 2, 1]].mean(0)          # on the k-lower face
        h[q] = R.characteristic_size(verts[q])
        rc, d[q], pos[q] = R.evaluate_position(verts[q], pts[q], 1e-11 * h[q])
        assert rc == 0
        w[q], _ = R.update_weights(d[q])
    out.update({"cells/verts": verts, "cells/points": pts, "cells/h": h, "cells/d": d, "cells/position": pos,
                "cells/weights": w})


def walks_section(out: dict):
    coor = W.sinusoidal_grid(10, 8, 24)
    sim = R.RefSim(coor)
    rng = np.random.default_rng(99)
    n = 600
    pts = rng.uniform(-0.05, 1.05, size=(n, 3))
    pts[:60] = coor.reshape(-1, 3)[rng.integers(0, coor.reshape(-1, 3).shape[0], 60)]
    starts = np.stack([rng.integers(-1, 12, n), rng.integers(-1, 10, n), rng.integers(-1, 26, n)], 1)
    starts[::5] = -1
    cell, wts, st = np.zeros((n, 3), np.int64), np.zeros((n, 3)), np.zeros(n, np.int64)
    for p in range(n):
        r = sim.locate_point(pts[p], starts[p])
        assert r["err"] == 0
        cell[p], wts[p], st[p] = r["cell"], r["weights"], r["status"]
    out.update({"walks/coor": coor, "walks/points": pts, "walks/start": starts, "walks/cell": cell,
                "walks/weights": wts, "walks/status": st})


def run_section(out: dict, name: str, wl):
    s0 = SwarmArrays.create(wl.pos, cell=wl.cell0)
    ucat = wl.ucat_node_sized()
    sim = R.RefSim(wl.coor, ucat, wl.dt)
    sim.set_swarm(s0.position, s0.velocity, s0.weight, s0.P, s0.cell, s0.pid, s0.status)
    p = f"run_{name}/"
    out.update({p + "coor": wl.coor, p + "ucat": ucat, p + "dt": np.array([wl.dt]), p + "pos0": s0.position,
                p + "cell0": s0.cell, p + "P0": np.array([s0.P[0]])})
    removed = []
    for k in range(STEPS + 1):
        if k == 0:
            sim.initial_setup()
        else:
            removed.append(sim.step())
        s = sim.swarm().sorted_by_pid()
        c, a = sim.scattered()
        q = f"{p}s{k}/"
        out.update({q + "pos": s.pos, q + "vel": s.vel, q + "weight": s.weight, q + "P": s.P, q + "cell": s.cell,
                    q + "pid": s.pid, q + "status": s.status, q + "count": c, q + "avg": a})
    out[p + "removed"] = np.array(removed, dtype=np.int64).reshape(-1, 2)


def main():
    if not R.available():
        raise SystemExit("the reference's sources are not present: nothing to generate")
    out: dict = {}
    cells_section(out)
    walks_section(out)
    for name, make in RUNS.items():
        run_section(out, name, make())
    np.savez_compressed(OUT, **out)
    print(f"wrote {OUT}: {os.path.getsize(OUT) / 1e6:.2f} MB, {len(out)} arrays")


if __name__ == "__main__":
    main()
