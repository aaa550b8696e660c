"""TEST INFRASTRUCTURE: a second, independent restatement of the reference walk
in plain Python (IEEE doubles, no FMA), for small cases only.

It is written from the reference source (src/walkingsearch.c:25-59, 102-227,
271-389, 407-462, 521-549, 882-959, 1094-1242; src/ParticleSwarm.c:1010-1047)
separately from oracle/picurv_oracle.c; agreement of the two restatements bit for
bit is one of the pins on the oracle.
"""
from __future__ import annotations

import math

LEFT, RIGHT, BOTTOM, TOP, FRONT, BACK = range(6)
EDGES = [(0, 1), (1, 2), (2, 3), (3, 0), (4, 5), (5, 6), (6, 7), (7, 4), (0, 7), (1, 6), (2, 5), (3, 4)]
VOFF = [(0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0), (0, 1, 1), (1, 1, 1), (1, 0, 1), (0, 0, 1)]
FACES = [(BACK, (0, 3, 2, 1)), (FRONT, (4, 7, 6, 5)), (BOTTOM, (0, 1, 6, 7)), (TOP, (3, 4, 5, 2)),
         (LEFT, (0, 7, 4, 3)), (RIGHT, (1, 2, 5, 6))]


class Degenerate(Exception):
    pass


def cell_vertices(coor, i, j, k):
    return [tuple(float(c) for c in coor[k + dk][j + dj][i + di]) for (di, dj, dk) in VOFF]


def cell_size(v):
    tot = 0.0
    for a, b in EDGES:
        dx = v[b][0] - v[a][0]; dy = v[b][1] - v[a][1]; dz = v[b][2] - v[a][2]
        tot += math.sqrt(dx * dx + dy * dy + dz * dz)
    return tot / 12.0


def signed_distance(v1, v2, v3, v4, cc, p, thr):
    e1 = (v2[0] - v1[0], v2[1] - v1[1], v2[2] - v1[2])
    e2 = (v4[0] - v1[0], v4[1] - v1[1], v4[2] - v1[2])
    nx = e1[1] * e2[2] - e1[2] * e2[1]
    ny = e1[2] * e2[0] - e1[0] * e2[2]
    nz = e1[0] * e2[1] - e1[1] * e2[0]
    mag = math.sqrt(nx * nx + ny * ny + nz * nz)
    if mag < 1.0e-12:
        raise Degenerate()
    fc = tuple(0.25 * (v1[c] + v2[c] + v3[c] + v4[c]) for c in range(3))
    t = (cc[0] - fc[0], cc[1] - fc[1], cc[2] - fc[2])
    dot = nx * t[0] + ny * t[1] + nz * t[2]
    if dot > 1.0e-9:
        nx, ny, nz = -nx, -ny, -nz
    nx /= mag; ny /= mag; nz /= mag
    d = (fc[0] - p[0]) * nx + (fc[1] - p[1]) * ny + (fc[2] - p[2]) * nz
    if abs(d) < thr:
        d = 0.0
    return d


def distances(p, v, thr):
    cc = [0.0, 0.0, 0.0]
    for q in range(8):
        for c in range(3):
            cc[c] += v[q][c]
    cc = [c / 8.0 for c in cc]
    d = [0.0] * 6
    for f, (a, b, c, e) in FACES:
        d[f] = signed_distance(v[a], v[b], v[c], v[e], cc, p, thr)
    return d


def position(d):
    inside = all(not (x < 0.0) for x in d)
    zeros = sum(1 for x in d if x == 0.0)
    if inside:
        return 0
    if zeros:
        return min(zeros, 3)
    return -1


def weights(d):
    d = [1e-14 if x <= 1e-14 else x for x in d]
    return (d[LEFT] / (d[LEFT] + d[RIGHT]), d[BOTTOM] / (d[BOTTOM] + d[TOP]), d[BACK] / (d[FRONT] + d[BACK]))


def locate(coor, p, cell=(-1, -1, -1)):
    """Returns (cell, weights or None, status, steps); status 1 = located, 3 = LOST."""
    KM, JM, IM = len(coor) - 1, len(coor[0]) - 1, len(coor[0][0]) - 1
    i, j, k = cell
    if not (0 <= i < IM and 0 <= j < JM and 0 <= k < KM):
        i, j, k = 0, 0, 0
    steps = 0
    while steps < 1000:
        steps += 1
        if not (0 <= i < IM and 0 <= j < JM and 0 <= k < KM):
            return (-1, -1, -1), None, 3, steps
        v = cell_vertices(coor, i, j, k)
        d = distances(p, v, 1e-11 * cell_size(v))
        if position(d) >= 0:
            return (i, j, k), weights(d), 1, steps
        if d[FRONT] < 0.0:
            k += 1
        elif d[BACK] < 0.0:
            k -= 1
        if d[LEFT] < 0.0:
            i -= 1
        elif d[RIGHT] < 0.0:
            i += 1
        if d[BOTTOM] < 0.0:
            j -= 1
        elif d[TOP] < 0.0:
            j += 1
    return (-1, -1, -1), None, 3, steps
