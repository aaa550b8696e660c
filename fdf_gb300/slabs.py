"""The particle path over several GPUs, one process per GPU, by k-slabs of cells.

The reference spreads a swarm over MPI ranks by subdomain and moves particles with
DMSwarmMigrate inside LocateAllParticlesInGrid_TEST's walk-and-handoff passes
(ParticleMotion.c:1931-2135).  Here every rank holds the whole grid (plane tables, ucat) and the
particles whose cell lies in its k-slab [k0, k1) of cells, and each step runs:

    reset, advect, walk (over the whole grid), remove LOST, remove out of bounds  -- every rank
    migration: the particles whose new cell lies in another slab move to that slab's rank
    interpolate, scatter, face deposit                                             -- every rank
    the k-faces between two slabs: the upper rank sums them again starting from the lower rank's
    partial sums (fdf_DepositKFaceLayer)

After the migration every cell's particles are on one rank, so ParticleCount, the P average and
every i-, j- and interior k-face are that rank's sums; a k-face on a slab boundary is the lower
cell's particles summed by the rank below, continued with the upper cell's by the rank above, in
the one-rank order.  The ranks' results together are therefore the one-rank results bit for bit
(plain FP64 form), and the removal counts add up to the one-rank counts.

The exchanges are host-side (the particles that cross a slab boundary in a step, and one layer of
k-faces per boundary), over a torch.distributed process group for CPU tensors (gloo).  `ctx` is a
PicContext (or any object with its stage methods), one per rank.
"""
from __future__ import annotations

import numpy as np

from .context import SwarmArrays

FIELDS = ("position", "velocity", "weight", "P", "cell", "pid", "status")
_WIDTH = {"position": 3, "velocity": 3, "weight": 3, "P": 1, "cell": 3, "pid": 1, "status": 1}   # 8-B values


class SlabDecomposition:
    """k-slabs of cells: rank r owns cells with k in [bounds[r], bounds[r+1])."""

    def __init__(self, KM: int, nranks: int):
        if nranks < 1 or nranks > KM:
            raise ValueError("need 1 <= ranks <= KM")
        self.KM, self.nranks = int(KM), int(nranks)
        self.bounds = [(r * self.KM) // self.nranks for r in range(self.nranks + 1)]

    def slab(self, rank: int) -> tuple[int, int]:
        return self.bounds[rank], self.bounds[rank + 1]

    def owner(self, k: np.ndarray) -> np.ndarray:
        return np.searchsorted(self.bounds, np.asarray(k), side="right") - 1


def _pack(s: SwarmArrays) -> np.ndarray:
    """Particles as rows of 15 8-byte values (DMSwarm fields in order)."""
    if s.n == 0:
        return np.zeros((0, 15), np.int64)
    cols = [np.ascontiguousarray(getattr(s, f)).reshape(s.n, _WIDTH[f]).view(np.int64) for f in FIELDS]
    return np.concatenate(cols, axis=1)


def _unpack(rows: np.ndarray) -> SwarmArrays:
    n = len(rows)
    out, c = [], 0
    for f in FIELDS:
        w = _WIDTH[f]
        a = np.ascontiguousarray(rows[:, c:c + w])
        a = a.view(np.float64) if f in ("position", "velocity", "weight", "P") else a
        out.append(a.reshape(n, 3) if w == 3 else a.reshape(n))
        c += w
    return SwarmArrays(*out)


class SlabRun:
    """One rank's part of a k-slab decomposition (see the module docstring)."""

    def __init__(self, ctx, dist, group=None, momentum: bool = False):
        self.ctx, self.dist, self.group = ctx, dist, group
        self.rank = dist.get_rank(group) if dist is not None else 0
        self.size = dist.get_world_size(group) if dist is not None else 1
        IM, JM, KM = ctx.dims
        self.dims = (IM, JM, KM)
        self.dec = SlabDecomposition(KM, self.size)
        self.k0, self.k1 = self.dec.slab(self.rank)
        self.momentum = momentum
        self.migrated = 0   # particles this rank has sent to other ranks

    # -- the initial distribution
    def set_swarm(self, s: SwarmArrays, capacity: int | None = None):
        """Every rank passes the whole initial swarm; each keeps the particles of its slab (those
        without a cell start on rank 0, which walks them from the corner cell as the reference
        does).  capacity: particles a rank may hold (default: all of them)."""
        k = s.cell[:, 2]
        has = np.all(s.cell >= 0, axis=1)
        own = np.where(has, self.dec.owner(np.where(has, k, 0)) == self.rank, self.rank == 0)
        mine = SwarmArrays(*(getattr(s, f)[own] for f in FIELDS))
        self.ctx.reserve(int(capacity or s.n))
        self.ctx.set_swarm(mine)

    # -- collectives over the host group
    def _alltoallv(self, rows_per_rank: list[np.ndarray]) -> np.ndarray:
        import torch
        sizes = torch.tensor([len(r) for r in rows_per_rank], dtype=torch.int64)
        table = [torch.zeros(self.size, dtype=torch.int64) for _ in range(self.size)]
        self.dist.all_gather(table, sizes, group=self.group)
        recv_counts = [int(table[src][self.rank]) for src in range(self.size)]
        send = torch.from_numpy(np.ascontiguousarray(np.concatenate(rows_per_rank).view(np.uint8).ravel()))
        recv = torch.empty(sum(recv_counts) * 120, dtype=torch.uint8)
        self.dist.all_to_all_single(recv, send, [c * 120 for c in recv_counts],
                                    [len(r) * 120 for r in rows_per_rank], group=self.group)
        return recv.numpy().view(np.int64).reshape(-1, 15)

    def _sum(self, values: list[int]) -> list[int]:
        if self.dist is None:
            return values
        import torch
        t = torch.tensor(values, dtype=torch.int64)
        self.dist.all_reduce(t, group=self.group)
        return [int(x) for x in t]

    # -- the steps
    def _migrate(self):
        """The particles whose cell left this rank's slab go to the slab's rank."""
        if self.size == 1:
            return
        out = self.ctx.extract_particles(self.k0, self.k1)
        self.migrated += out.n
        dest = self.dec.owner(out.cell[:, 2]) if out.n else np.zeros(0, np.int64)
        rows = _pack(out)
        arrived = self._alltoallv([rows[dest == r] for r in range(self.size)])
        if len(arrived):
            self.ctx.add_particles(_unpack(arrived))

    def _join_boundary_faces(self):
        """The k-faces on the slab boundary below this rank: the lower rank's partial sums, then
        this rank's particles (plain form)."""
        if self.size == 1:
            return
        import torch
        reqs = []
        if self.rank + 1 < self.size:
            fk = self.ctx.get_faces()[2][self.k1]
            parts = [torch.from_numpy(np.ascontiguousarray(fk))]
            if self.momentum:
                parts.append(torch.from_numpy(np.ascontiguousarray(self.ctx.get_face_momentum()[2][self.k1])))
            reqs = [self.dist.isend(p, self.rank + 1, group=self.group) for p in parts]
        if self.rank > 0:
            IM, JM, _ = self.dims
            seed = torch.empty((JM, IM), dtype=torch.float64)
            self.dist.recv(seed, self.rank - 1, group=self.group)
            seed_m = None
            if self.momentum:
                seed_m = torch.empty((JM, IM, 3), dtype=torch.float64)
                self.dist.recv(seed_m, self.rank - 1, group=self.group)
            self.ctx.deposit_k_layer(self.k0, seed.numpy(), None if seed_m is None else seed_m.numpy())
        for r in reqs:
            r.wait()

    def initial_setup(self):
        """PerformInitialSetup_TEST's path: locate (LOST particles kept), migrate, interpolate, scatter."""
        self.ctx.locate()
        self._migrate()
        self.ctx.interpolate()
        self.ctx.scatter()
        self._join_boundary_faces()

    def step(self) -> tuple[int, int]:
        """One step of AdvanceSimulation_TEST's loop; returns the removal counts of all ranks."""
        c = self.ctx
        c.reset_statuses()
        c.update_positions()
        c.locate()
        lost = c.remove_lost()
        oob = c.remove_out_of_bounds()
        self._migrate()
        c.interpolate()
        c.scatter()
        self._join_boundary_faces()
        lost, oob = self._sum([lost, oob])
        return lost, oob

    # -- output
    def owned_fields(self) -> dict:
        """This rank's layers of the grid outputs: cells k0..k1-1 (node layers of ParticleCount and P,
        i-, j- and lower k-faces), plus the top k-face layer on the last rank."""
        k0, k1 = self.k0, self.k1
        top = k1 + 1 if self.rank == self.size - 1 else k1
        count, avg = self.ctx.get_scattered()
        fi, fj, fk = self.ctx.get_faces()
        out = {"count": count[k0:k1], "avg": avg[k0:k1], "fi": fi[k0:k1], "fj": fj[k0:k1], "fk": fk[k0:top]}
        if self.momentum:
            mi, mj, mk = self.ctx.get_face_momentum()
            out.update(mi=mi[k0:k1], mj=mj[k0:k1], mk=mk[k0:top])
        return out

    def gather(self, root: int = 0):
        """The whole swarm and the whole grid outputs on `root` (output steps); None elsewhere."""
        mine = {"swarm": _pack(self.ctx.get_swarm()), **self.owned_fields()}
        parts = [None] * self.size if self.rank == root else None
        if self.dist is None:
            parts = [mine]
        else:
            self.dist.gather_object(mine, parts, dst=root, group=self.group)
        if self.rank != root:
            return None
        IM, JM, KM = self.dims
        res = {"swarm": _unpack(np.concatenate([p["swarm"] for p in parts]))}
        for key in ("count", "avg"):
            full = np.zeros((KM + 1, JM + 1, IM + 1))
            full[:KM] = np.concatenate([p[key] for p in parts])
            res[key] = full
        for key in ("fi", "fj", "fk") + (("mi", "mj", "mk") if self.momentum else ()):
            res[key] = np.concatenate([p[key] for p in parts])
        return res
