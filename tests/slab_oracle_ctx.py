"""A rank's context for the k-slab driver's CPU tests: PicContext's stage methods over the CPU
oracle (test infrastructure).  The seeded k-face layer sum restates fdf_DepositKFaceLayer: the
seed, then the held particles of the layer's cells in (cell, PID) order adding (1 - a) V/3 (and
its products with the velocity)."""
from __future__ import annotations

import numpy as np

from fdf_gb300.context import SwarmArrays
from oracle import oracle as O


class OracleRankCtx:
    def __init__(self, wl, momentum: bool = False):
        self.g = O.Grid(wl.coor)
        self.ucat = wl.ucat_node_sized()
        self.dt, self.volume, self.momentum = wl.dt, wl.volume, momentum
        self.dims = wl.dims
        self.s = O.Swarm.create(np.zeros((0, 3)))
        self.faces = None

    def reserve(self, cap):
        pass

    def set_swarm(self, a: SwarmArrays):
        self.s = O.Swarm(pos=a.position.copy(), vel=a.velocity.copy(), weight=a.weight.copy(), P=a.P.copy(),
                         cell=a.cell.copy(), pid=a.pid.copy(), status=a.status.copy(), n=a.n)

    def size(self):
        return self.s.n

    def get_swarm(self) -> SwarmArrays:
        v = self.s.view()
        return SwarmArrays(*(v[k].copy() for k in ("pos", "vel", "weight", "P", "cell", "pid", "status")))

    def add_particles(self, a: SwarmArrays):
        self.set_swarm(SwarmArrays(*(np.concatenate([getattr(self.get_swarm(), f), getattr(a, f)])
                                     for f in ("position", "velocity", "weight", "P", "cell", "pid", "status"))))

    def extract_particles(self, k_lo, k_hi) -> SwarmArrays:
        s = self.get_swarm()
        has = np.all(s.cell >= 0, axis=1)
        out = has & ((s.cell[:, 2] < k_lo) | (s.cell[:, 2] >= k_hi))
        keep = ~out
        self.set_swarm(SwarmArrays(*(getattr(s, f)[keep] for f in ("position", "velocity", "weight", "P", "cell",
                                                                     "pid", "status"))))
        return SwarmArrays(*(getattr(s, f)[out] for f in ("position", "velocity", "weight", "P", "cell", "pid",
                                                          "status")))

    def reset_statuses(self):
        st = self.s.status[:self.s.n]
        st[st == O.ACTIVE_AND_LOCATED] = O.NEEDS_LOCATION

    def update_positions(self):
        import ctypes
        cs = self.s.c()
        O.lib().o_UpdateAllParticlePositions(ctypes.byref(cs), self.dt, 1)

    def locate(self):
        err, _ = O.locate_all(self.g, self.s, 1)
        assert err == 0

    def remove_lost(self):
        return O.remove_lost(self.s)

    def remove_out_of_bounds(self):
        return O.remove_oob(self.g, self.s)

    def interpolate(self):
        O.interpolate(self.g, O.center_to_corner(self.g, self.ucat, 1), self.s, 1)

    def scatter(self):
        self.count, self.avg = O.scatter_P(self.g, self.s)
        self.faces = O.deposit_faces(self.g, self.s, volume=self.volume, momentum=self.momentum)

    def get_scattered(self):
        return self.count, self.avg

    def get_faces(self):
        return self.faces["fi"], self.faces["fj"], self.faces["fk"]

    def get_face_momentum(self):
        return self.faces["mom_i"], self.faces["mom_j"], self.faces["mom_k"]

    def deposit_k_layer(self, k, seed, seed_momentum=None):
        IM, JM, KM = self.dims
        third = self.volume / 3.0
        fk = self.faces["fk"]
        fk[k] = seed
        mk = self.faces.get("mom_k")
        if mk is not None:
            mk[k] = 0.0 if seed_momentum is None else seed_momentum
        if k >= KM:
            return
        s = self.get_swarm()
        sel = np.all(s.cell >= 0, axis=1) & (s.cell[:, 2] == k)
        lin = s.cell[sel, 1] * IM + s.cell[sel, 0]
        order = np.lexsort((s.pid[sel], lin))
        a3, u, cells = s.weight[sel, 2][order], s.velocity[sel][order], s.cell[sel][order]
        for q in range(len(order)):
            i, j = int(cells[q, 0]), int(cells[q, 1])
            x = (1.0 - a3[q]) * third
            fk[k, j, i] = fk[k, j, i] + x
            if mk is not None:
                for c in range(3):
                    mk[k, j, i, c] = mk[k, j, i, c] + x * u[q, c]
