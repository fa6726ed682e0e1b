"""Literal dense restatement of the reference's element matrices (numpy).

TEST INFRASTRUCTURE ONLY.  Follows the reference's code structure as written:
dense strain-displacement matrices, B^T C B products at each integration point,
dense 6x6 / 12x12 / 24x24 rotation matrices and T^T K T.  It uses numpy's
LU-based inverse/determinant and the axis-angle (acos / cos / sin) form of the
alignment rotation, so it shares no evaluation order with fem_oracle.c; the
tests use it to check the oracle's restructured formulas at 1e-12.
"""
from __future__ import annotations

import math

import numpy as np

F32_PI = float(np.float32(math.pi))


def _cwt(v, abs_tol):  # math_functions.rs:3-12
    return 0.0 if abs(v) < abs_tol else v


def align_rotation(a, b, abs_tol):
    """rotation taking a onto b, axis-angle form (extended_matrix, not vendored)."""
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    na, nb = np.linalg.norm(a), np.linalg.norm(b)
    axis = np.cross(a, b)
    if not np.any(axis):
        if np.dot(a, b) > 0:
            return np.eye(3)
        ez, ex = np.array([0.0, 0.0, 1.0]), np.array([1.0, 0.0, 0.0])
        n = np.cross(a / na, ez)
        if not np.any(n):
            n = np.cross(a / na, ex)
        n = n / np.linalg.norm(n)
        R = 2.0 * np.outer(n, n) - np.eye(3)
        return np.vectorize(lambda v: _cwt(v, abs_tol))(R)
    cosang = min(1.0, max(-1.0, float(np.dot(a, b) / (na * nb))))
    ang = math.acos(cosang)
    n = axis / np.linalg.norm(axis)
    c, s, t = math.cos(ang), math.sin(ang), 1.0 - math.cos(ang)
    x, y, z = n
    R = np.array([[t * x * x + c, t * x * y - z * s, t * x * z + y * s],
                  [t * x * y + z * s, t * y * y + c, t * y * z - x * s],
                  [t * x * z - y * s, t * y * z + x * s, t * z * z + c]])
    return np.vectorize(lambda v: _cwt(v, abs_tol))(R)


def _blockdiag(R, n):
    T = np.zeros((3 * n, 3 * n))
    for k in range(n):
        T[3 * k:3 * k + 3, 3 * k:3 * k + 3] = R
    return T


# --------------------------------------------------------------------------
# truss (structs/truss.rs)
# --------------------------------------------------------------------------

def truss_global_matrix(x1, x2, E, A, A2=None, rel_tol=1e-12, abs_tol=1e-12):
    d = np.asarray(x2, float) - np.asarray(x1, float)
    L = float(np.linalg.norm(d))
    R = align_rotation(d, [L, 0.0, 0.0], abs_tol)
    T = np.zeros((6, 6))
    T[0:3, 0:3] = R
    T[3:6, 3:6] = R
    r, alpha = 0.0, 2.0
    jac = L / 2.0
    B = np.array([[-0.5, 0, 0, 0.5, 0, 0]]) / jac
    area = A if A2 is None else (A2 - A) / 2.0 * r + A - (A2 - A) / 2.0 * -1.0
    k = B.T @ B * (area * E * jac * alpha)
    return T.T @ k @ T


# --------------------------------------------------------------------------
# beam (structs/beam.rs)
# --------------------------------------------------------------------------

def beam_principal(i11, i22, i12, rel_tol):
    if i11 != i22:
        angle = math.atan(2 * i12 / (i22 - i11)) / 2
    else:
        if i22 < i11:
            i11m, i22m = i11, (abs(i22) - abs(i22) * rel_tol) * i22 / abs(i22)
        else:
            i11m, i22m = (abs(i11) - abs(i11) * rel_tol) * i11 / abs(i11), i22
        angle = math.atan(2 * i12 / (i22m - i11m)) / 2
    f = lambda a: (i11 * math.cos(a) ** 2 + i22 * math.sin(a) ** 2 - i12 * math.sin(2 * a),
                   i11 * math.sin(a) ** 2 + i22 * math.cos(a) ** 2 + i12 * math.sin(2 * a))
    p1, p2 = f(angle)
    i = 1
    while p1 < p2 and i <= 8:
        angle = (math.atan(2 * i12 / (i22 - i11)) + F32_PI * i) / 2
        p1, p2 = f(angle)
        i += 1
    return p1, p2, angle


def beam_rotation(x1, x2, i11, i22, i12, axis, rel_tol=1e-12, abs_tol=1e-12):
    p1, p2, angle = beam_principal(i11, i22, i12, rel_tol)
    d = np.asarray(x2, float) - np.asarray(x1, float)
    L = float(np.linalg.norm(d))
    Ri = align_rotation(d, [L, 0, 0], abs_tol)
    ax = np.asarray(axis, float)
    proj = ax - np.dot(ax, d) / np.dot(d, d) * d
    tp = Ri @ proj
    cosang = min(1.0, max(-1.0, tp[2] / np.linalg.norm(tp)))
    total = angle + math.acos(cosang)
    cx, cy, cz = (_cwt(v / L, abs_tol) for v in d)
    cxz = _cwt(math.sqrt(cx * cx + cz * cz), abs_tol)
    c, s = _cwt(math.cos(total), abs_tol), _cwt(math.sin(total), abs_tol)
    if cxz != 0:
        R = np.array([[cx, cy, cz],
                      [(-cx * cy * c - cz * s) / cxz, cxz * c, (-cy * cz * c + cx * s) / cxz],
                      [(cx * cy * s - cz * c) / cxz, -cxz * s, (cy * cz * s + cx * c) / cxz]])
    else:
        R = np.array([[0, cy, 0], [-cy * c, 0, s], [cy * s, 0, c]])
    return R, p1, p2


def beam_global_matrix(x1, x2, E, nu, A, i11, i22, i12, it, k_s, axis, rel_tol=1e-12, abs_tol=1e-12):
    R, i11p, i22p = beam_rotation(x1, x2, i11, i22, i12, axis, rel_tol, abs_tol)
    d = np.asarray(x2, float) - np.asarray(x1, float)
    L = float(np.linalg.norm(d))
    r, alpha = 0.0, 2.0
    jac = L / 2
    inv = 1 / jac
    dh1, dh2, h1, h2 = -0.5, 0.5, 0.5 * (1 - r), 0.5 * (1 + r)

    def row(entries):
        v = np.zeros((1, 12))
        for idx, val in entries:
            v[0, idx] = val
        return v

    Bu = row([(0, dh1 * inv), (6, dh2 * inv)])
    Bv = row([(1, dh1 * inv), (7, dh2 * inv)]) - row([(5, h1), (11, h2)])
    Bw = row([(2, dh1 * inv), (8, dh2 * inv)]) - row([(4, h1), (10, h2)])
    Btu = row([(3, dh1 * inv), (9, dh2 * inv)])
    Btv = row([(4, dh1 * inv), (10, dh2 * inv)])
    Btw = row([(5, dh1 * inv), (11, dh2 * inv)])
    G = E / (2 * (1 + nu))
    k = (Bu.T @ Bu * (A * E * jac * alpha) + Bv.T @ Bv * (G * A * k_s * jac * alpha)
         + Bw.T @ Bw * (G * A * k_s * jac * alpha) + Btu.T @ Btu * (G * it * jac * alpha)
         + Btv.T @ Btv * (E * i22p * jac * alpha) + Btw.T @ Btw * (E * i11p * jac * alpha))
    T = _blockdiag(R, 4)
    return T.T @ k @ T


# --------------------------------------------------------------------------
# plate (structs/plate.rs, quadrilateral_4n_element_functions.rs)
# --------------------------------------------------------------------------

def plate_rotation(x2, x3, x4, abs_tol=1e-12):
    e34 = np.asarray(x4, float) - np.asarray(x3, float)
    e32 = np.asarray(x2, float) - np.asarray(x3, float)
    n = np.cross(e34, e32)
    return align_rotation(n, [0.0, 0.0, float(np.linalg.norm(n))], abs_tol)


def plate_global_matrix(x1, x2, x3, x4, E, nu, t, k_s, rel_tol=1e-12, abs_tol=1e-12):
    X = [np.asarray(v, float) for v in (x1, x2, x3, x4)]
    R = plate_rotation(X[1], X[2], X[3], abs_tol)
    loc = {i: R @ (X[i] - X[2]) for i in (0, 1, 3)}
    xs = [loc[0][0], loc[1][0], 0.0, loc[3][0]]
    ys = [loc[0][1], loc[1][1], 0.0, loc[3][1]]
    g = math.sqrt(float(np.float32(1.0) / np.float32(3.0)))
    ips = [(g, g), (-g, g), (-g, -g), (g, -g)]
    K = np.zeros((24, 24))
    Cm = E * t / (1 - nu ** 2) * np.array([[1, nu, 0], [nu, 1, 0], [0, 0, (1 - nu) / 2]])
    Cb = E * t ** 3 / (12 * (1 - nu ** 2)) * np.array([[1, nu, 0], [nu, 1, 0], [0, 0, (1 - nu) / 2]])
    x1l, x2l, x3l, x4l = xs
    y1l, y2l, y3l, y4l = ys
    a_x, b_x, c_x = x1l - x2l - x3l + x4l, x1l - x2l + x3l - x4l, x1l + x2l - x3l - x4l
    a_y, b_y, c_y = y1l - y2l - y3l + y4l, y1l - y2l + y3l - y4l, y1l + y2l - y3l - y4l
    for r, s in ips:
        dhr = 0.25 * np.array([1 + s, -(1 + s), -(1 - s), 1 - s])
        dhs = 0.25 * np.array([1 + r, 1 - r, -(1 - r), -(1 + r)])
        J = np.array([[dhr @ xs, dhr @ ys], [dhs @ xs, dhs @ ys]])
        det = np.linalg.det(J)
        dxy = np.linalg.inv(J) @ np.vstack([dhr, dhs])
        Bm = np.zeros((3, 24))
        Bb = np.zeros((3, 24))
        for i in range(4):
            Bm[0, 6 * i] = dxy[0, i]
            Bm[1, 6 * i + 1] = dxy[1, i]
            Bm[2, 6 * i] = dxy[1, i]
            Bm[2, 6 * i + 1] = dxy[0, i]
            Bb[0, 6 * i + 4] = -dxy[0, i]
            Bb[1, 6 * i + 3] = dxy[1, i]
            Bb[2, 6 * i + 3] = dxy[0, i]
            Bb[2, 6 * i + 4] = -dxy[1, i]
        mr = math.sqrt((c_x + r * b_x) ** 2 + (c_y + r * b_y) ** 2) / (8 * det)
        ms = math.sqrt((a_x + s * b_x) ** 2 + (a_y + s * b_y) ** 2) / (8 * det)
        Bs = np.zeros((2, 24))
        # gamma_rz row (plate.rs:452-480)
        Bs[0, 2], Bs[0, 3], Bs[0, 4] = (1 + s) / 2 * mr, -(1 + s) * (y1l - y2l) / 4 * mr, (1 + s) * (x1l - x2l) / 4 * mr
        Bs[0, 8], Bs[0, 9], Bs[0, 10] = -(1 + s) / 2 * mr, -(1 + s) * (y1l - y2l) / 4 * mr, (1 + s) * (x1l - x2l) / 4 * mr
        Bs[0, 14], Bs[0, 15], Bs[0, 16] = -(1 - s) / 2 * mr, -(1 - s) * (y4l - y3l) / 4 * mr, (1 - s) * (x4l - x3l) / 4 * mr
        Bs[0, 20], Bs[0, 21], Bs[0, 22] = (1 - s) / 2 * mr, -(1 - s) * (y4l - y3l) / 4 * mr, (1 - s) * (x4l - x3l) / 4 * mr
        # gamma_sz row (plate.rs:481-508)
        Bs[1, 2], Bs[1, 3], Bs[1, 4] = (1 + r) / 2 * ms, -(1 + r) * (y1l - y4l) / 4 * ms, (1 + r) * (x1l - x4l) / 4 * ms
        Bs[1, 8], Bs[1, 9], Bs[1, 10] = (1 - r) / 2 * ms, -(1 - r) * (y2l - y3l) / 4 * ms, (1 - r) * (x2l - x3l) / 4 * ms
        Bs[1, 14], Bs[1, 15], Bs[1, 16] = -(1 - r) / 2 * ms, -(1 - r) * (y2l - y3l) / 4 * ms, (1 - r) * (x2l - x3l) / 4 * ms
        Bs[1, 20], Bs[1, 21], Bs[1, 22] = -(1 + r) / 2 * ms, -(1 + r) * (y1l - y4l) / 4 * ms, (1 + r) * (x1l - x4l) / 4 * ms
        Cs = np.eye(2) * (E * t * k_s / (2 * (1 + nu)))
        K += Bm.T @ Cm @ Bm * det + Bb.T @ Cb @ Bb * det + Bs.T @ Cs @ Bs * det
    for i in range(4):
        K[6 * i + 5, 6 * i + 5] += 1.0  # KROT6
    T = _blockdiag(R, 8)
    return T.T @ K @ T
