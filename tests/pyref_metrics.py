"""TEST INFRASTRUCTURE: an independent numpy restatement of the grid metrics and of
Contra2Cart, written from the reference source separately from oracle/picurv_oracle.c:

    src/Metric.c:286-460    ComputeFaceMetrics (Csi, Eta, Zet + boundary extrapolation)
    src/Metric.c:491-600    ComputeCellCenteredJacobianInverse (Aj + extrapolation)
    src/Metric.c:195-260    CheckAndFixGridOrientation
    src/setup.c:1294-1420   Contra2Cart

numpy evaluates every elementwise expression with IEEE double operations in the written
order and never fuses a*b+c, so agreement bit for bit with the C restatement pins both.
Arrays are node-sized, indexed [k][j][i].
"""
from __future__ import annotations

import numpy as np


class MetricError(Exception):
    def __init__(self, code: int):
        super().__init__(f"PETSc error {code}")
        self.code = code


def _P(coor, di, dj, dk):
    """coor[k+dk][j+dj][i+di] over the interior block k, j, i >= 1 (dk, dj, di in {0, -1})."""
    K, J, I = coor.shape[:3]
    return coor[1 + dk:K + dk, 1 + dj:J + dj, 1 + di:I + di]


def face_metrics(coor):
    K, J, I = coor.shape[:3]
    csi = np.zeros_like(coor)
    eta = np.zeros_like(coor)
    zet = np.zeros_like(coor)
    # Csi on k >= 1, j >= 1, every i
    a, b = coor[1:, 1:], coor[:-1, 1:]          # (k, j), (k-1, j)
    c, d = coor[1:, :-1], coor[:-1, :-1]        # (k, j-1), (k-1, j-1)
    de = 0.5 * (a + b - c - d)
    dz = 0.5 * (c + a - d - b)
    csi[1:, 1:, :, 0] = de[..., 1] * dz[..., 2] - de[..., 2] * dz[..., 1]
    csi[1:, 1:, :, 1] = de[..., 2] * dz[..., 0] - de[..., 0] * dz[..., 2]
    csi[1:, 1:, :, 2] = de[..., 0] * dz[..., 1] - de[..., 1] * dz[..., 0]
    # Eta on k >= 1, i >= 1, every j
    a, b = coor[1:, :, 1:], coor[:-1, :, 1:]    # (k, i), (k-1, i)
    c, d = coor[1:, :, :-1], coor[:-1, :, :-1]  # (k, i-1), (k-1, i-1)
    dx = 0.5 * (a + b - c - d)
    dz = 0.5 * (a + c - b - d)
    eta[1:, :, 1:, 0] = dz[..., 1] * dx[..., 2] - dz[..., 2] * dx[..., 1]
    eta[1:, :, 1:, 1] = dz[..., 2] * dx[..., 0] - dz[..., 0] * dx[..., 2]
    eta[1:, :, 1:, 2] = dz[..., 0] * dx[..., 1] - dz[..., 1] * dx[..., 0]
    # Zet on j >= 1, i >= 1, every k
    a, b = coor[:, 1:, 1:], coor[:, :-1, 1:]    # (j, i), (j-1, i)
    c, d = coor[:, 1:, :-1], coor[:, :-1, :-1]  # (j, i-1), (j-1, i-1)
    dx = 0.5 * (a + b - c - d)
    de = 0.5 * (a + c - b - d)
    zet[:, 1:, 1:, 0] = dx[..., 1] * de[..., 2] - dx[..., 2] * de[..., 1]
    zet[:, 1:, 1:, 1] = dx[..., 2] * de[..., 0] - dx[..., 0] * de[..., 2]
    zet[:, 1:, 1:, 2] = dx[..., 0] * de[..., 1] - dx[..., 1] * de[..., 0]
    # extrapolation: i faces (Eta, Zet), then j (Csi, Zet), then k (Csi, Eta)
    for arr in (eta, zet):
        arr[:, :, 0] = arr[:, :, 1]
        arr[:, :, I - 1] = arr[:, :, I - 2]
    for arr in (csi, zet):
        arr[:, 0] = arr[:, 1]
        arr[:, J - 1] = arr[:, J - 2]
    for arr in (csi, eta):
        arr[0] = arr[1]
        arr[K - 1] = arr[K - 2]
    return csi, eta, zet


def jacobian_inverse(coor):
    K, J, I = coor.shape[:3]
    p = {(di, dj, dk): _P(coor, di, dj, dk) for di in (0, -1) for dj in (0, -1) for dk in (0, -1)}
    dxi = 0.25 * ((p[0, 0, 0] + p[0, -1, 0] + p[0, 0, -1] + p[0, -1, -1]) -
                  (p[-1, 0, 0] + p[-1, -1, 0] + p[-1, 0, -1] + p[-1, -1, -1]))
    deta = 0.25 * ((p[0, 0, 0] + p[-1, 0, 0] + p[0, 0, -1] + p[-1, 0, -1]) -
                   (p[0, -1, 0] + p[-1, -1, 0] + p[0, -1, -1] + p[-1, -1, -1]))
    dzeta = 0.25 * ((p[0, 0, 0] + p[0, -1, 0] + p[-1, 0, 0] + p[-1, -1, 0]) -
                    (p[0, 0, -1] + p[0, -1, -1] + p[-1, 0, -1] + p[-1, -1, -1]))
    x, y, z = (lambda v: v[..., 0]), (lambda v: v[..., 1]), (lambda v: v[..., 2])
    jac = (x(dxi) * (y(deta) * z(dzeta) - z(deta) * y(dzeta))
           - y(dxi) * (x(deta) * z(dzeta) - z(deta) * x(dzeta))
           + z(dxi) * (x(deta) * y(dzeta) - y(deta) * x(dzeta)))
    if np.any(np.abs(jac) < 1.0e-12):
        raise MetricError(90)
    aj = np.zeros(coor.shape[:3])
    aj[1:, 1:, 1:] = 1.0 / jac
    aj[:, :, 0] = aj[:, :, 1]
    aj[:, :, I - 1] = aj[:, :, I - 2]
    aj[:, 0] = aj[:, 1]
    aj[:, J - 1] = aj[:, J - 2]
    aj[0] = aj[1]
    aj[K - 1] = aj[K - 2]
    return aj


def metrics(coor):
    """(csi, eta, zet, aj, flipped) after the orientation check."""
    csi, eta, zet = face_metrics(coor)
    aj = jacobian_inverse(coor)
    lo, hi = aj.min(), aj.max()
    if lo < 0.0 and hi > 0.0:
        raise MetricError(83)
    if hi < 0.0:
        return -csi, -eta, -zet, -aj, True
    return csi, eta, zet, aj, False


def contra2cart(ucont, csi, eta, zet, ucat):
    """Interior cells 1..IM-1 x 1..JM-1 x 1..KM-1 of a copy of ucat (node-sized)."""
    out = np.array(ucat, dtype=np.float64, copy=True)
    K, J, I = ucont.shape[:3]   # KM+1, JM+1, IM+1
    s = (slice(1, K - 1), slice(1, J - 1), slice(1, I - 1))
    si = (slice(1, K - 1), slice(1, J - 1), slice(0, I - 2))
    sj = (slice(1, K - 1), slice(0, J - 2), slice(1, I - 1))
    sk = (slice(0, K - 2), slice(1, J - 1), slice(1, I - 1))
    m = [[0.5 * (csi[si + (c,)] + csi[s + (c,)]) for c in range(3)],
         [0.5 * (eta[sj + (c,)] + eta[s + (c,)]) for c in range(3)],
         [0.5 * (zet[sk + (c,)] + zet[s + (c,)]) for c in range(3)]]
    q0 = 0.5 * (ucont[si + (0,)] + ucont[s + (0,)])
    q1 = 0.5 * (ucont[sj + (1,)] + ucont[s + (1,)])
    q2 = 0.5 * (ucont[sk + (2,)] + ucont[s + (2,)])
    det = (m[0][0] * (m[1][1] * m[2][2] - m[1][2] * m[2][1])
           - m[0][1] * (m[1][0] * m[2][2] - m[1][2] * m[2][0])
           + m[0][2] * (m[1][0] * m[2][1] - m[1][1] * m[2][0]))
    if np.any(np.abs(det) < 1.0e-18):
        raise MetricError(90)
    det_inv = 1.0 / det
    det0 = (q0 * (m[1][1] * m[2][2] - m[1][2] * m[2][1])
            - q1 * (m[0][1] * m[2][2] - m[0][2] * m[2][1])
            + q2 * (m[0][1] * m[1][2] - m[0][2] * m[1][1]))
    det1 = (-q0 * (m[1][0] * m[2][2] - m[1][2] * m[2][0])
            + q1 * (m[0][0] * m[2][2] - m[0][2] * m[2][0])
            - q2 * (m[0][0] * m[1][2] - m[0][2] * m[1][0]))
    det2 = (q0 * (m[1][0] * m[2][1] - m[1][1] * m[2][0])
            - q1 * (m[0][0] * m[2][1] - m[0][1] * m[2][0])
            + q2 * (m[0][0] * m[1][1] - m[0][1] * m[1][0]))
    out[s + (0,)] = det0 * det_inv
    out[s + (1,)] = det1 * det_inv
    out[s + (2,)] = det2 * det_inv
    return out


def ucont_of_uniform_flow(u, csi, eta, zet):
    """Face fluxes of the constant velocity u through the metric vectors: (csi.u, eta.u, zet.u)."""
    u = np.asarray(u, dtype=np.float64)
    out = np.empty(csi.shape)
    out[..., 0] = csi[..., 0] * u[0] + csi[..., 1] * u[1] + csi[..., 2] * u[2]
    out[..., 1] = eta[..., 0] * u[0] + eta[..., 1] * u[1] + eta[..., 2] * u[2]
    out[..., 2] = zet[..., 0] * u[0] + zet[..., 1] * u[1] + zet[..., 2] * u[2]
    return out
