"""Synthetic workloads for the particle hot path (host-side, FP64, seeded).

The reference publishes no dataset for this path; every grid, velocity field
and particle set here is generated from a formula and a counter-based
splitmix64 stream, so the same call gives the same bits on any machine.

Families
--------
``uniform``    Cartesian box [0,1]^3, nodes ``i/IM`` (grid.c:265-283,386-396 with L=1).
``sinusoidal`` curvilinear box: x = xi + A sin(2 pi eta) sin(2 pi zeta), cyclic in (y, z).
``bent_pipe``  O-type disk cross-section swept along a 90 degree bend.
``curved_pipe`` O-type disk cross-section swept along a planar curve.

Velocity fields are evaluated at the cell centroid (mean of the 8 nodes).
Particles are placed like the reference's volumetric initialisation
(ParticleSwarm.c:229-312): a random cell, random logical coordinates in [0,1)
clamped to 1-1e-7, mapped by the trilinear blend of Metric.c:48-62.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

TWO_PI = 2.0 * np.pi
_GOLDEN = np.uint64(0x9E3779B97F4A7C15)


def _mix64(z: np.ndarray) -> np.ndarray:
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def uniform01(seed: int, stream: int, n: int, start: int = 0) -> np.ndarray:
    """n doubles in [0,1) from the splitmix64 sequence (seed, stream), element start.."""
    with np.errstate(over="ignore"):
        base = _mix64(np.uint64(seed) * np.uint64(0xD1B54A32D192ED03) + np.uint64(stream) * np.uint64(0xA24BAED4963EE407)
                      + np.uint64(0x632BE59BD9B4E019))
        idx = np.arange(start, start + n, dtype=np.uint64)
        z = _mix64(base + (idx + np.uint64(1)) * _GOLDEN)
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


# ----------------------------------------------------------------------------- grids

def uniform_grid(IM: int, JM: int, KM: int) -> np.ndarray:
    xi = np.arange(IM + 1, dtype=np.float64) / IM
    eta = np.arange(JM + 1, dtype=np.float64) / JM
    zeta = np.arange(KM + 1, dtype=np.float64) / KM
    Z, Y, X = np.meshgrid(zeta, eta, xi, indexing="ij")
    return np.ascontiguousarray(np.stack([X, Y, Z], axis=-1))


def sinusoidal_grid(IM: int, JM: int, KM: int, amp: float = 0.04) -> np.ndarray:
    xi = np.arange(IM + 1, dtype=np.float64) / IM
    eta = np.arange(JM + 1, dtype=np.float64) / JM
    zeta = np.arange(KM + 1, dtype=np.float64) / KM
    Z, Y, X = np.meshgrid(zeta, eta, xi, indexing="ij")
    sx, sy, sz = np.sin(TWO_PI * X), np.sin(TWO_PI * Y), np.sin(TWO_PI * Z)
    x = X + amp * sy * sz
    y = Y + amp * sz * sx
    z = Z + amp * sx * sy
    return np.ascontiguousarray(np.stack([x, y, z], axis=-1))


def _square_to_disk(a: np.ndarray, b: np.ndarray):
    """Elliptical square->disk map of [-1,1]^2 (smooth inside, corners on the circle)."""
    return a * np.sqrt(1.0 - 0.5 * b * b), b * np.sqrt(1.0 - 0.5 * a * a)


def bent_pipe_grid(IM: int, JM: int, KM: int, radius: float = 0.5, bend_radius: float = 3.0,
                   angle: float = 0.5 * np.pi) -> np.ndarray:
    """O-type disk (i, j) swept over theta in [0, angle] (k) about the z axis.

    The cross-section point (u, v) sits at distance bend_radius + u from the bend
    axis and height v; the sweep runs counter-clockwise so (i, j, k) is right-handed.
    """
    a = np.linspace(-1.0, 1.0, IM + 1)
    b = np.linspace(-1.0, 1.0, JM + 1)
    th = np.linspace(0.0, angle, KM + 1)
    B, A = np.meshgrid(b, a, indexing="ij")            # [JM+1][IM+1]
    u, v = _square_to_disk(A, B)
    u, v = radius * u, radius * v
    r = bend_radius + u                                 # [JM+1][IM+1]
    cos_t, sin_t = np.cos(th), np.sin(th)               # [KM+1]
    x = r[None] * cos_t[:, None, None]
    y = r[None] * sin_t[:, None, None]
    z = np.broadcast_to(v[None], x.shape)
    # (i: radial-ish u, j: height v, k: +theta) -- u x v = +z_local; check handedness below
    g = np.stack([x, y, z], axis=-1)
    return np.ascontiguousarray(_make_right_handed(g))


def curved_pipe_grid(IM: int, JM: int, KM: int, radius: float = 0.5, length: float = 8.0,
                     wiggle: float = 1.0) -> np.ndarray:
    """O-type disk swept along the planar curve c(s) = (wiggle*sin(pi s / L), 0, s), s in [0, L]."""
    a = np.linspace(-1.0, 1.0, IM + 1)
    b = np.linspace(-1.0, 1.0, JM + 1)
    s = np.linspace(0.0, length, KM + 1)
    B, A = np.meshgrid(b, a, indexing="ij")
    u, v = _square_to_disk(A, B)
    u, v = radius * u, radius * v
    cx = wiggle * np.sin(np.pi * s / length)
    dcx = wiggle * (np.pi / length) * np.cos(np.pi * s / length)
    tn = np.sqrt(1.0 + dcx * dcx)
    # unit tangent (dcx, 0, 1)/tn ; in-plane normal (1, 0, -dcx)/tn ; binormal (0, 1, 0)
    nx, nz = 1.0 / tn, -dcx / tn
    x = cx[:, None, None] + u[None] * nx[:, None, None]
    y = np.broadcast_to(v[None], x.shape)
    z = s[:, None, None] + u[None] * nz[:, None, None]
    g = np.stack([x, y, np.broadcast_to(z, x.shape)], axis=-1)
    return np.ascontiguousarray(_make_right_handed(g))


def _make_right_handed(g: np.ndarray) -> np.ndarray:
    """Flip the i direction if (e_i x e_j) . e_k < 0 at the first cell."""
    e_i = g[0, 0, 1] - g[0, 0, 0]
    e_j = g[0, 1, 0] - g[0, 0, 0]
    e_k = g[1, 0, 0] - g[0, 0, 0]
    if np.dot(np.cross(e_i, e_j), e_k) < 0:
        g = g[:, :, ::-1, :]
    return g


def uniform_flow_fluxes(u, csi: np.ndarray, eta: np.ndarray, zet: np.ndarray) -> np.ndarray:
    """Contravariant face velocity (the reference's ucont layout, node-sized [..][3]) of the
    constant velocity u through the face metric vectors: (csi . u, eta . u, zet . u)."""
    u = np.asarray(u, dtype=np.float64)
    out = np.empty(csi.shape)
    out[..., 0] = csi[..., 0] * u[0] + csi[..., 1] * u[1] + csi[..., 2] * u[2]
    out[..., 1] = eta[..., 0] * u[0] + eta[..., 1] * u[1] + eta[..., 2] * u[2]
    out[..., 2] = zet[..., 0] * u[0] + zet[..., 1] * u[1] + zet[..., 2] * u[2]
    return out


def cell_centroids(coor: np.ndarray) -> np.ndarray:
    c = (coor[:-1, :-1, :-1] + coor[:-1, :-1, 1:] + coor[:-1, 1:, :-1] + coor[:-1, 1:, 1:]
         + coor[1:, :-1, :-1] + coor[1:, :-1, 1:] + coor[1:, 1:, :-1] + coor[1:, 1:, 1:])
    return c / 8.0


def min_edge_length(coor: np.ndarray) -> float:
    ei = np.linalg.norm(np.diff(coor, axis=2), axis=-1).min()
    ej = np.linalg.norm(np.diff(coor, axis=1), axis=-1).min()
    ek = np.linalg.norm(np.diff(coor, axis=0), axis=-1).min()
    return float(min(ei, ej, ek))


def node_sized(ucat_cells: np.ndarray) -> np.ndarray:
    """Cell array [KM][JM][IM][3] -> the reference's node-sized DMDA layout."""
    KM, JM, IM, _ = ucat_cells.shape
    out = np.zeros((KM + 1, JM + 1, IM + 1, 3))
    out[:KM, :JM, :IM] = ucat_cells
    return out


# ----------------------------------------------------------------------------- fields

def field_config1(cent: np.ndarray) -> np.ndarray:
    x, y, z = cent[..., 0], cent[..., 1], cent[..., 2]
    return np.stack([0.1 * np.sin(TWO_PI * y), 0.1 * np.sin(TWO_PI * z), 1.0 + 0.1 * np.sin(TWO_PI * x)], axis=-1)


def field_taylor_green(cent: np.ndarray, U0: float = 1.0, w: float = 1.0) -> np.ndarray:
    x, y = cent[..., 0], cent[..., 1]
    u = U0 * np.sin(TWO_PI * x) * np.cos(TWO_PI * y)
    v = -U0 * np.cos(TWO_PI * x) * np.sin(TWO_PI * y)
    return np.stack([u, v, np.full_like(u, w)], axis=-1)


def field_pipe(coor: np.ndarray, cent: np.ndarray, U: float = 1.0, radius: float = 0.5,
               secondary: float = 0.2) -> np.ndarray:
    """Poiseuille profile 2U(1 - r^2/R^2) along the local k direction plus a
    Taylor-Green-like secondary swirl of amplitude `secondary` in the cross-section."""
    KM, JM, IM = cent.shape[:3]
    # local frame from the grid: axis = centreline tangent, r from the section centre
    ctr = 0.5 * (coor[:, JM // 2, IM // 2] + coor[:, (JM + 1) // 2, (IM + 1) // 2])   # node ring centre [KM+1][3]
    ctr_c = 0.5 * (ctr[:-1] + ctr[1:])
    tang = ctr[1:] - ctr[:-1]
    tang /= np.linalg.norm(tang, axis=-1, keepdims=True)
    rel = cent - ctr_c[:, None, None, :]
    rel_ax = np.sum(rel * tang[:, None, None, :], axis=-1, keepdims=True)
    rvec = rel - rel_ax * tang[:, None, None, :]
    r2 = np.sum(rvec * rvec, axis=-1)
    ax = 2.0 * U * np.clip(1.0 - r2 / (radius * radius), 0.0, None)
    # secondary: rotate rvec by 90 degrees about the tangent, modulated by the radius
    swirl = np.cross(tang[:, None, None, :], rvec)
    sec = secondary * U * np.sin(np.pi * np.sqrt(r2) / radius)[..., None] * swirl / radius
    return ax[..., None] * tang[:, None, None, :] + sec


# ----------------------------------------------------------------------------- particles

def trilinear_blend(coor: np.ndarray, ci, cj, ck, xi, eta, zta) -> np.ndarray:
    """MetricLogicalToPhysical (Metric.c:48-80): bit-ordered vertices, same operation order."""
    x = np.zeros(len(ci)); y = np.zeros(len(ci)); z = np.zeros(len(ci))
    for c in range(8):
        ii = ci + (1 if c & 1 else 0)
        jj = cj + (1 if c & 2 else 0)
        kk = ck + (1 if c & 4 else 0)
        N = ((xi if c & 1 else 1.0 - xi) * (eta if c & 2 else 1.0 - eta)) * (zta if c & 4 else 1.0 - zta)
        V = coor[kk, jj, ii]
        x = x + N * V[:, 0]
        y = y + N * V[:, 1]
        z = z + N * V[:, 2]
    return np.stack([x, y, z], axis=-1)


def volumetric_particles(coor: np.ndarray, n: int, seed: int = 0):
    """Random cell + random logical coordinates (ParticleSwarm.c:229-312).

    Returns (positions [n][3], generating cell [n][3])."""
    KM, JM, IM = (s - 1 for s in coor.shape[:3])
    ri, rj, rk = uniform01(seed, 0, n), uniform01(seed, 1, n), uniform01(seed, 2, n)
    ci = np.clip((ri * IM).astype(np.int64), 0, IM - 1)
    cj = np.clip((rj * JM).astype(np.int64), 0, JM - 1)
    ck = np.clip((rk * KM).astype(np.int64), 0, KM - 1)
    lim = 1.0 - 1.0e-7
    xi = np.maximum(np.minimum(uniform01(seed, 3, n), lim), 0.0)
    eta = np.maximum(np.minimum(uniform01(seed, 4, n), lim), 0.0)
    zta = np.maximum(np.minimum(uniform01(seed, 5, n), lim), 0.0)
    pos = trilinear_blend(coor, ci, cj, ck, xi, eta, zta)
    return pos, np.stack([ci, cj, ck], axis=-1)


def box_particles(n: int, seed: int = 0) -> np.ndarray:
    return np.stack([uniform01(seed, 0, n), uniform01(seed, 1, n), uniform01(seed, 2, n)], axis=-1)


# ----------------------------------------------------------------------------- configs

@dataclass
class Workload:
    name: str
    coor: np.ndarray            # [KM+1][JM+1][IM+1][3]
    ucat: np.ndarray            # [KM][JM][IM][3] cell-centred
    pos: np.ndarray | None      # [n][3]; None: seeded on the device (seed_n particles, meta seed)
    cell0: np.ndarray | None    # [n][3] initial DMSwarm_CellID (-1 = walk from the corner)
    dt: float
    steps: int
    volume: float = 1.0
    meta: dict = field(default_factory=dict)
    seed_n: int = 0

    @property
    def dims(self):
        KM, JM, IM = (s - 1 for s in self.coor.shape[:3])
        return IM, JM, KM

    @property
    def n(self):
        return len(self.pos) if self.pos is not None else self.seed_n

    def sample(self, m: int):
        """The first m particles (an i.i.d. sample) as host arrays: (pos, cell0, pid)."""
        if self.pos is not None:
            return self.pos[:m], self.cell0[:m], np.arange(min(m, self.n))
        pos, cell = volumetric_particles(self.coor, min(m, self.seed_n), self.meta.get("seed", 0))
        return pos, cell, np.arange(len(pos))

    def ucat_node_sized(self) -> np.ndarray:
        return node_sized(self.ucat)


def config1(n: int = 10_000, IM: int = 20, JM: int = 20, KM: int = 280, steps: int = 10, seed: int = 0) -> Workload:
    """Uniform [0,1]^3 box; ucat = (0,0,1) + 0.1 (sin 2pi y, sin 2pi z, sin 2pi x); dt = 0.1 dz;
    particles uniform in the box, located from the corner cell as the reference does."""
    coor = uniform_grid(IM, JM, KM)
    ucat = field_config1(cell_centroids(coor))
    pos = box_particles(n, seed)
    return Workload("uniform_%dx%dx%d_n%d" % (IM, JM, KM, n), coor, ucat, pos,
                    np.full((n, 3), -1, dtype=np.int64), dt=0.1 / KM, steps=steps,
                    meta=dict(family="uniform", cfl=None, seed=seed, corner_start=True), seed_n=n)


def _particles(coor, n, seed, materialize):
    if not materialize:
        return None, None
    return volumetric_particles(coor, n, seed)


def config_sinusoidal(IM: int = 64, JM: int = 64, KM: int = 1024, n: int = 1_000_000, cfl: float = 0.5,
                      steps: int = 50, seed: int = 0, corner_start: bool = False, materialize: bool = True) -> Workload:
    """Curvilinear box (amplitude 0.04) with a Taylor-Green vortex plus w = 1; particles
    uniform in (xi, eta, zeta); dt = cfl * min edge / max |ucat|."""
    coor = sinusoidal_grid(IM, JM, KM)
    ucat = field_taylor_green(cell_centroids(coor))
    pos, cell = _particles(coor, n, seed, materialize)
    umax = float(np.sqrt((ucat ** 2).sum(-1)).max())
    dt = cfl * min_edge_length(coor) / umax
    if corner_start and cell is not None:
        cell = np.full((n, 3), -1, dtype=np.int64)
    return Workload("sinusoidal_%dx%dx%d_n%d_cfl%g" % (IM, JM, KM, n, cfl), coor, ucat, pos, cell, dt=dt,
                    steps=steps, meta=dict(family="sinusoidal", cfl=cfl, seed=seed, corner_start=corner_start),
                    seed_n=n)


def config_bent_pipe(IM: int = 96, JM: int = 96, KM: int = 1536, n: int = 64_000_000, cfl: float = 4.0,
                     steps: int = 50, seed: int = 0, materialize: bool = True) -> Workload:
    """90-degree bend (pipe radius 0.5, bend radius 3), O-type 96x96 section, Poiseuille
    axial flow 2U(1 - r^2/R^2) along the bend; dt = cfl * min edge / max |ucat|."""
    coor = bent_pipe_grid(IM, JM, KM)
    cent = cell_centroids(coor)
    ucat = field_pipe(coor, cent, secondary=0.0)
    pos, cell = _particles(coor, n, seed, materialize)
    umax = float(np.sqrt((ucat ** 2).sum(-1)).max())
    dt = cfl * min_edge_length(coor) / umax
    return Workload("bent_pipe_%dx%dx%d_n%d_cfl%g" % (IM, JM, KM, n, cfl), coor, ucat, pos, cell, dt=dt,
                    steps=steps, meta=dict(family="bent_pipe", cfl=cfl, seed=seed), seed_n=n)


def config_curved_pipe(IM: int = 128, JM: int = 128, KM: int = 2048, n: int = 128_000_000, cfl: float = 1.0,
                       steps: int = 200, seed: int = 0, materialize: bool = True) -> Workload:
    """Curved pipe (radius 0.5) along a planar curve, Poiseuille axial flow plus a
    Taylor-Green-like secondary swirl of amplitude 0.2; dt = cfl * min edge / max |ucat|."""
    coor = curved_pipe_grid(IM, JM, KM)
    cent = cell_centroids(coor)
    ucat = field_pipe(coor, cent, secondary=0.2)
    pos, cell = _particles(coor, n, seed, materialize)
    umax = float(np.sqrt((ucat ** 2).sum(-1)).max())
    dt = cfl * min_edge_length(coor) / umax
    return Workload("curved_pipe_%dx%dx%d_n%d_cfl%g" % (IM, JM, KM, n, cfl), coor, ucat, pos, cell, dt=dt,
                    steps=steps, meta=dict(family="curved_pipe", cfl=cfl, seed=seed), seed_n=n)
