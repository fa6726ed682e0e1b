"""Literal dense restatement of the reference's element matrices.

TEST INFRASTRUCTURE ONLY.  Follows the reference's code structure as written:
dense strain-displacement matrices, B^T C B products at each integration point,
dense 6x6 / 12x12 / 24x24 rotation matrices and T^T K T (structs/truss.rs,
structs/beam.rs, structs/plate.rs, bar_2n_element_functions.rs,
quadrilateral_4n_element_functions.rs).  It uses the closed-form 2x2
inverse/determinant and the axis-angle (acos / cos / sin) form of the alignment
rotation, so it shares no evaluation order with fem_oracle.c; the tests use it
to check the oracle's restructured formulas at 1e-12.

The arithmetic runs on a backend: plain floats (default), or mpmath at a
chosen precision (`Backend.mp(dps)`), which tests/golden/make_golden.py uses to
write high-precision golden element matrices.
"""
from __future__ import annotations

import math

import numpy as np

F32_PI = float(np.float32(math.pi))
G_F32 = float(np.float32(1.0) / np.float32(3.0))  # 1f32 / 3f32 widened (plate.rs:1066-1091)


class Backend:
    def __init__(self, num, sqrt, acos, cos, sin, atan):
        self.num, self.sqrt, self.acos, self.cos, self.sin, self.atan = num, sqrt, acos, cos, sin, atan

    @staticmethod
    def floats():
        return Backend(float, math.sqrt, math.acos, math.cos, math.sin, math.atan)

    @staticmethod
    def mp(dps=50):
        import mpmath

        mpmath.mp.dps = dps
        return Backend(mpmath.mpf, mpmath.sqrt, mpmath.acos, mpmath.cos, mpmath.sin, mpmath.atan)

    def vec(self, v):
        return np.array([self.num(float(x)) if isinstance(x, (float, int, np.floating, np.integer)) else x
                         for x in v], dtype=object)

    def zeros(self, n, m):
        z = np.empty((n, m), dtype=object)
        z[...] = self.num(0)
        return z

    def eye(self, n):
        z = self.zeros(n, n)
        for i in range(n):
            z[i, i] = self.num(1)
        return z

    def norm(self, v):
        return self.sqrt(sum(x * x for x in v))


FLOAT = Backend.floats()


def _cwt(v, abs_tol):  # math_functions.rs:3-12
    return 0 * v if abs(v) < abs_tol else v


def _cross(a, b):
    return np.array([a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]], dtype=object)


def _dot(a, b):
    return sum(x * y for x, y in zip(a, b))


def _out(M, bk):
    return np.array(M, dtype=float) if bk is FLOAT else M


def align_rotation(a, b, abs_tol, bk=FLOAT):
    """rotation taking a onto b, axis-angle form (extended_matrix's rotation_matrix_to_align_with_vector,
    not vendored; called at structs/truss.rs:80, beam.rs:179, quadrilateral_4n_element_functions.rs:158)."""
    a, b = bk.vec(a), bk.vec(b)
    na, nb = bk.norm(a), bk.norm(b)
    axis = _cross(a, b)
    if all(x == 0 for x in axis):
        if _dot(a, b) > 0:
            return bk.eye(3)
        ez, ex = bk.vec([0.0, 0.0, 1.0]), bk.vec([1.0, 0.0, 0.0])
        n = _cross(a / na, ez)
        if all(x == 0 for x in n):
            n = _cross(a / na, ex)
        n = n / bk.norm(n)
        R = 2 * np.outer(n, n) - bk.eye(3)
        return np.vectorize(lambda v: _cwt(v, abs_tol), otypes=[object])(R)
    cosang = _dot(a, b) / (na * nb)
    cosang = min(bk.num(1), max(bk.num(-1), cosang))
    ang = bk.acos(cosang)
    n = axis / bk.norm(axis)
    c, s = bk.cos(ang), bk.sin(ang)
    t = 1 - c
    x, y, z = n
    R = np.array([[t * x * x + c, t * x * y - z * s, t * x * z + y * s],
                  [t * x * y + z * s, t * y * y + c, t * y * z - x * s],
                  [t * x * z - y * s, t * y * z + x * s, t * z * z + c]], dtype=object)
    return np.vectorize(lambda v: _cwt(v, abs_tol), otypes=[object])(R)


def _blockdiag(R, n, bk):
    T = bk.zeros(3 * n, 3 * n)
    for k in range(n):
        T[3 * k:3 * k + 3, 3 * k:3 * k + 3] = R
    return T


# --------------------------------------------------------------------------
# truss (structs/truss.rs)
# --------------------------------------------------------------------------

def truss_global_matrix(x1, x2, E, A, A2=None, rel_tol=1e-12, abs_tol=1e-12, bk=FLOAT):
    x1, x2 = bk.vec(x1), bk.vec(x2)
    d = x2 - x1
    L = bk.norm(d)
    R = align_rotation(d, [L, 0, 0], abs_tol, bk)
    T = _blockdiag(R, 2, bk)
    r, alpha = bk.num(0), bk.num(2)
    jac = L / 2
    B = bk.vec([-0.5, 0, 0, 0.5, 0, 0]).reshape(1, 6) / jac  # truss.rs:95-118
    E, A = bk.num(E), bk.num(A)
    area = A if A2 is None else (bk.num(A2) - A) / 2 * r + A - (bk.num(A2) - A) / 2 * -1  # truss.rs:120-130
    k = B.T.dot(B) * (area * E * jac * alpha)  # truss.rs:132-189
    return _out(T.T.dot(k).dot(T), bk)


# --------------------------------------------------------------------------
# beam (structs/beam.rs)
# --------------------------------------------------------------------------

def beam_principal(i11, i22, i12, rel_tol, bk=FLOAT):
    """find_principal_moments_of_inertia, beam.rs:119-160"""
    i11, i22, i12 = bk.num(i11), bk.num(i22), bk.num(i12)
    if i11 != i22:
        angle = bk.atan(2 * i12 / (i22 - i11)) / 2
    else:
        if i22 < i11:
            i11m, i22m = i11, (abs(i22) - abs(i22) * rel_tol) * i22 / abs(i22)
        else:
            i11m, i22m = (abs(i11) - abs(i11) * rel_tol) * i11 / abs(i11), i22
        angle = bk.atan(2 * i12 / (i22m - i11m)) / 2
    f = lambda a: (i11 * bk.cos(a) ** 2 + i22 * bk.sin(a) ** 2 - i12 * bk.sin(2 * a),
                   i11 * bk.sin(a) ** 2 + i22 * bk.cos(a) ** 2 + i12 * bk.sin(2 * a))
    p1, p2 = f(angle)
    i = 1
    while p1 < p2 and i <= 8:
        angle = (bk.atan(2 * i12 / (i22 - i11)) + bk.num(F32_PI) * i) / 2
        p1, p2 = f(angle)
        i += 1
    return p1, p2, angle


def beam_rotation(x1, x2, i11, i22, i12, axis, rel_tol=1e-12, abs_tol=1e-12, bk=FLOAT):
    """find_rotation_matrix_elements, beam.rs:162-258"""
    p1, p2, angle = beam_principal(i11, i22, i12, rel_tol, bk)
    x1, x2 = bk.vec(x1), bk.vec(x2)
    d = x2 - x1
    L = bk.norm(d)
    Ri = align_rotation(d, [L, 0, 0], abs_tol, bk)
    ax = bk.vec(axis)
    proj = ax - _dot(ax, d) / _dot(d, d) * d
    tp = Ri.dot(proj)
    cosang = min(bk.num(1), max(bk.num(-1), tp[2] / bk.norm(tp)))
    total = angle + bk.acos(cosang)
    cx, cy, cz = (_cwt(v / L, abs_tol) for v in d)
    cxz = _cwt(bk.sqrt(cx * cx + cz * cz), abs_tol)
    c, s = _cwt(bk.cos(total), abs_tol), _cwt(bk.sin(total), abs_tol)
    if cxz != 0:
        R = np.array([[cx, cy, cz],
                      [(-cx * cy * c - cz * s) / cxz, cxz * c, (-cy * cz * c + cx * s) / cxz],
                      [(cx * cy * s - cz * c) / cxz, -cxz * s, (cy * cz * s + cx * c) / cxz]], dtype=object)
    else:
        z = bk.num(0)
        R = np.array([[z, cy, z], [-cy * c, z, s], [cy * s, z, c]], dtype=object)
    return R, p1, p2


def beam_global_matrix(x1, x2, E, nu, A, i11, i22, i12, it, k_s, axis, rel_tol=1e-12, abs_tol=1e-12, bk=FLOAT):
    R, i11p, i22p = beam_rotation(x1, x2, i11, i22, i12, axis, rel_tol, abs_tol, bk)
    d = bk.vec(x2) - bk.vec(x1)
    L = bk.norm(d)
    r, alpha = bk.num(0), bk.num(2)
    jac = L / 2
    inv = 1 / jac
    dh1, dh2, h1, h2 = bk.num(-0.5), bk.num(0.5), (1 - r) / 2, (1 + r) / 2

    def row(entries):
        v = bk.zeros(1, 12)
        for idx, val in entries:
            v[0, idx] = val
        return v

    # beam.rs:260-493
    Bu = row([(0, dh1 * inv), (6, dh2 * inv)])
    Bv = row([(1, dh1 * inv), (7, dh2 * inv)]) - row([(5, h1), (11, h2)])
    Bw = row([(2, dh1 * inv), (8, dh2 * inv)]) - row([(4, h1), (10, h2)])
    Btu = row([(3, dh1 * inv), (9, dh2 * inv)])
    Btv = row([(4, dh1 * inv), (10, dh2 * inv)])
    Btw = row([(5, dh1 * inv), (11, dh2 * inv)])
    E, nu, A, it, k_s = (bk.num(v) for v in (E, nu, A, it, k_s))
    G = E / (2 * (1 + nu))  # beam.rs:519
    k = (Bu.T.dot(Bu) * (A * E * jac * alpha) + Bv.T.dot(Bv) * (G * A * k_s * jac * alpha)
         + Bw.T.dot(Bw) * (G * A * k_s * jac * alpha) + Btu.T.dot(Btu) * (G * it * jac * alpha)
         + Btv.T.dot(Btv) * (E * i22p * jac * alpha) + Btw.T.dot(Btw) * (E * i11p * jac * alpha))
    T = _blockdiag(R, 4, bk)
    return _out(T.T.dot(k).dot(T), bk)


# --------------------------------------------------------------------------
# plate (structs/plate.rs, quadrilateral_4n_element_functions.rs)
# --------------------------------------------------------------------------

def plate_rotation(x2, x3, x4, abs_tol=1e-12, bk=FLOAT):
    """find_rotation_matrix_elements_of_quadrilateral, quad.rs:131-171"""
    e34 = bk.vec(x4) - bk.vec(x3)
    e32 = bk.vec(x2) - bk.vec(x3)
    n = _cross(e34, e32)
    return align_rotation(n, [0, 0, bk.norm(n)], abs_tol, bk)


def plate_global_matrix(x1, x2, x3, x4, E, nu, t, k_s, rel_tol=1e-12, abs_tol=1e-12, bk=FLOAT):
    X = [bk.vec(v) for v in (x1, x2, x3, x4)]
    R = plate_rotation(X[1], X[2], X[3], abs_tol, bk)
    loc = {i: R.dot(X[i] - X[2]) for i in (0, 1, 3)}  # quad.rs:340-378
    z = bk.num(0)
    xs = [loc[0][0], loc[1][0], z, loc[3][0]]
    ys = [loc[0][1], loc[1][1], z, loc[3][1]]
    g = bk.sqrt(bk.num(G_F32))
    ips = [(g, g), (-g, g), (-g, -g), (g, -g)]  # plate.rs:1066-1091
    E, nu, t, k_s = (bk.num(v) for v in (E, nu, t, k_s))
    K = bk.zeros(24, 24)
    cmat = np.array([[1, nu, 0], [nu, 1, 0], [0, 0, (1 - nu) / 2]], dtype=object)
    Cm = E * t / (1 - nu ** 2) * cmat  # plate.rs:532-548
    Cb = E * t ** 3 / (12 * (1 - nu ** 2)) * cmat  # plate.rs:580-597
    x1l, x2l, x3l, x4l = xs
    y1l, y2l, y3l, y4l = ys
    a_x, b_x, c_x = x1l - x2l - x3l + x4l, x1l - x2l + x3l - x4l, x1l + x2l - x3l - x4l  # plate.rs:424-429
    a_y, b_y, c_y = y1l - y2l - y3l + y4l, y1l - y2l + y3l - y4l, y1l + y2l - y3l - y4l
    q = bk.num(0.25)
    for r, s in ips:
        dhr = [q * (1 + s), -q * (1 + s), -q * (1 - s), q * (1 - s)]  # quad.rs:505-583
        dhs = [q * (1 + r), q * (1 - r), -q * (1 - r), -q * (1 + r)]
        J = [[_dot(dhr, xs), _dot(dhr, ys)], [_dot(dhs, xs), _dot(dhs, ys)]]  # quad.rs:380-446
        det = J[0][0] * J[1][1] - J[0][1] * J[1][0]
        Ji = [[J[1][1] / det, -J[0][1] / det], [-J[1][0] / det, J[0][0] / det]]
        dxy = [[Ji[a][0] * dhr[i] + Ji[a][1] * dhs[i] for i in range(4)] for a in range(2)]  # quad.rs:613-653
        Bm = bk.zeros(3, 24)  # plate.rs:160-274
        Bb = bk.zeros(3, 24)  # plate.rs:276-390
        for i in range(4):
            Bm[0, 6 * i] = dxy[0][i]
            Bm[1, 6 * i + 1] = dxy[1][i]
            Bm[2, 6 * i] = dxy[1][i]
            Bm[2, 6 * i + 1] = dxy[0][i]
            Bb[0, 6 * i + 4] = -dxy[0][i]
            Bb[1, 6 * i + 3] = dxy[1][i]
            Bb[2, 6 * i + 3] = dxy[0][i]
            Bb[2, 6 * i + 4] = -dxy[1][i]
        mr = bk.sqrt((c_x + r * b_x) ** 2 + (c_y + r * b_y) ** 2) / (8 * det)  # plate.rs:443-447
        ms = bk.sqrt((a_x + s * b_x) ** 2 + (a_y + s * b_y) ** 2) / (8 * det)
        Bs = bk.zeros(2, 24)
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
        Cs = bk.eye(2) * (E * t * k_s / (2 * (1 + nu)))  # plate.rs:629-636
        K = K + Bm.T.dot(Cm).dot(Bm) * det + Bb.T.dot(Cb).dot(Bb) * det + Bs.T.dot(Cs).dot(Bs) * det
    for i in range(4):
        K[6 * i + 5, 6 * i + 5] = K[6 * i + 5, 6 * i + 5] + 1  # KROT6 (plate.rs:25, :716-721)
    T = _blockdiag(R, 8, bk)
    return _out(T.T.dot(K).dot(T), bk)


# --------------------------------------------------------------------------
# element results (methods_for_element_analysis.rs:27-58)
#
# Each function returns (values, scale): the results as the reference writes
# them (dense B matrices summed over the integration / corner points, times
# the rotated displacements, times C) and the same expression with every
# factor replaced by its absolute value -- the magnitude a rounding error is
# measured against.
# --------------------------------------------------------------------------

def _both(M, bk):
    return M, np.array([abs(v) for v in np.asarray(M, dtype=object).ravel()], dtype=object).reshape(np.shape(M))


def truss_results(x1, x2, E, A, A2, u6, rel_tol=1e-12, abs_tol=1e-12, bk=FLOAT):
    """truss.rs:281-333"""
    x1, x2 = bk.vec(x1), bk.vec(x2)
    d = x2 - x1
    L = bk.norm(d)
    R = align_rotation(d, [L, 0, 0], abs_tol, bk)
    T, Ta = _both(_blockdiag(R, 2, bk), bk)
    u, ua = _both(bk.vec(u6), bk)
    r = bk.num(0)
    B, Ba = _both(bk.vec([-0.5, 0, 0, 0.5, 0, 0]) * (1 / (L / 2)), bk)  # truss.rs:95-118
    E, A = bk.num(E), bk.num(A)
    area = bk.num(0) + (A if A2 is None else (bk.num(A2) - A) / 2 * r + A - (bk.num(A2) - A) / 2 * -1)
    f = E * area / 1
    return [B.dot(T.dot(u)) * f], [Ba.dot(Ta.dot(ua)) * abs(f)]


def beam_results(x1, x2, E, nu, A, i11, i22, i12, it, k_s, axis, u12, rel_tol=1e-12, abs_tol=1e-12, bk=FLOAT):
    """beam.rs:803-993"""
    R, i11p, i22p = beam_rotation(x1, x2, i11, i22, i12, axis, rel_tol, abs_tol, bk)
    d = bk.vec(x2) - bk.vec(x1)
    L = bk.norm(d)
    r = bk.num(0)
    inv = 1 / (L / 2)
    dh1, dh2, h1, h2 = bk.num(-0.5), bk.num(0.5), (1 - r) / 2, (1 + r) / 2

    def row(entries):
        v = bk.zeros(1, 12)
        for idx, val in entries:
            v[0, idx] = val
        return v[0]

    T, Ta = _both(_blockdiag(R, 4, bk), bk)
    u, ua = _both(bk.vec(u12), bk)
    ul, ula = T.dot(u), Ta.dot(ua)
    E, nu, A, it, k_s = (bk.num(v) for v in (E, nu, A, it, k_s))
    G = E / (2 * (1 + nu))
    rows = [  # beam.rs:260-493
        (row([(0, dh1 * inv), (6, dh2 * inv)]), E * A / 1),
        (row([(1, dh1 * inv), (7, dh2 * inv)]) - row([(5, h1), (11, h2)]), G * A * k_s / 1),
        (row([(2, dh1 * inv), (8, dh2 * inv)]) - row([(4, h1), (10, h2)]), G * A * k_s / 1),
        (row([(3, dh1 * inv), (9, dh2 * inv)]), G * it / 1),
        (row([(4, dh1 * inv), (10, dh2 * inv)]), E * i22p / 1),
        (row([(5, dh1 * inv), (11, dh2 * inv)]), E * i11p / 1),
    ]
    v = [B.dot(ul) * c for B, c in rows]
    s = [np.array([abs(x) for x in B], dtype=object).dot(ula) * abs(c) for B, c in rows]
    fr, fs, ft, mr, ms, mt = v
    sr, ss, st, smr, sms, smt = s
    vals = [fr, fs, ft, mr, ms + L * ft / 2, ms, ms - L * ft / 2, mt + L * fs / 2, mt, mt - L * fs / 2]
    scale = [sr, ss, st, smr, sms + L * st / 2, sms, sms + L * st / 2, smt + L * ss / 2, smt, smt + L * ss / 2]
    return vals, scale


def plate_results(x1, x2, x3, x4, E, nu, t, k_s, u24, rel_tol=1e-12, abs_tol=1e-12, bk=FLOAT):
    """plate.rs:1196-1409: B matrices (plate.rs:160-511) summed over the corner points"""
    X = [bk.vec(v) for v in (x1, x2, x3, x4)]
    R = plate_rotation(X[1], X[2], X[3], abs_tol, bk)
    loc = {i: R.dot(X[i] - X[2]) for i in (0, 1, 3)}
    z = bk.num(0)
    xs = [loc[0][0], loc[1][0], z, loc[3][0]]
    ys = [loc[0][1], loc[1][1], z, loc[3][1]]
    x1l, x2l, x3l, x4l = xs
    y1l, y2l, y3l, y4l = ys
    a_x, b_x, c_x = x1l - x2l - x3l + x4l, x1l - x2l + x3l - x4l, x1l + x2l - x3l - x4l
    a_y, b_y, c_y = y1l - y2l - y3l + y4l, y1l - y2l + y3l - y4l, y1l + y2l - y3l - y4l
    q = bk.num(0.25)
    Bm, Bb, Bs = bk.zeros(3, 24), bk.zeros(3, 24), bk.zeros(2, 24)
    one = bk.num(1)
    for r, s in [(one, one), (-one, one), (-one, -one), (one, -one)]:  # plate.rs:1248-1253
        dhr = [q * (1 + s), -q * (1 + s), -q * (1 - s), q * (1 - s)]
        dhs = [q * (1 + r), q * (1 - r), -q * (1 - r), -q * (1 + r)]
        J = [[_dot(dhr, xs), _dot(dhr, ys)], [_dot(dhs, xs), _dot(dhs, ys)]]
        det = J[0][0] * J[1][1] - J[0][1] * J[1][0]
        Ji = [[J[1][1] / det, -J[0][1] / det], [-J[1][0] / det, J[0][0] / det]]
        dxy = [[Ji[a][0] * dhr[i] + Ji[a][1] * dhs[i] for i in range(4)] for a in range(2)]
        for i in range(4):
            Bm[0, 6 * i] += dxy[0][i]
            Bm[1, 6 * i + 1] += dxy[1][i]
            Bm[2, 6 * i] += dxy[1][i]
            Bm[2, 6 * i + 1] += dxy[0][i]
            Bb[0, 6 * i + 4] += -dxy[0][i]
            Bb[1, 6 * i + 3] += dxy[1][i]
            Bb[2, 6 * i + 3] += dxy[0][i]
            Bb[2, 6 * i + 4] += -dxy[1][i]
        mr = bk.sqrt((c_x + r * b_x) ** 2 + (c_y + r * b_y) ** 2) / (8 * det)
        ms = bk.sqrt((a_x + s * b_x) ** 2 + (a_y + s * b_y) ** 2) / (8 * det)
        for (c, w, sg, ex, ey) in ((0, 1 + s, 1, x1l - x2l, y1l - y2l), (1, 1 + s, -1, x1l - x2l, y1l - y2l),
                                   (2, 1 - s, -1, x4l - x3l, y4l - y3l), (3, 1 - s, 1, x4l - x3l, y4l - y3l)):
            Bs[0, 6 * c + 2] += sg * w / 2 * mr
            Bs[0, 6 * c + 3] += -w * ey / 4 * mr
            Bs[0, 6 * c + 4] += w * ex / 4 * mr
        for (c, w, sg, ex, ey) in ((0, 1 + r, 1, x1l - x4l, y1l - y4l), (1, 1 - r, 1, x2l - x3l, y2l - y3l),
                                   (2, 1 - r, -1, x2l - x3l, y2l - y3l), (3, 1 + r, -1, x1l - x4l, y1l - y4l)):
            Bs[1, 6 * c + 2] += sg * w / 2 * ms
            Bs[1, 6 * c + 3] += -w * ey / 4 * ms
            Bs[1, 6 * c + 4] += w * ex / 4 * ms
    T, Ta = _both(_blockdiag(R, 8, bk), bk)
    u, ua = _both(bk.vec(u24), bk)
    ul, ula = T.dot(u), Ta.dot(ua)
    E, nu, t, k_s = (bk.num(v) for v in (E, nu, t, k_s))
    cmat = np.array([[1, nu, 0], [nu, 1, 0], [0, 0, (1 - nu) / 2]], dtype=object)
    Cm = cmat * (E / (1 - nu ** 2))
    Cb = cmat * (E * t / (2 * (1 - nu ** 2)))
    Cs = bk.eye(2) * (E / (2 * (1 + nu)))
    fm = Cm.dot(Bm.dot(ul)) * (t / 4)
    fb = Cb.dot(Bb.dot(ul)) * (t ** 2 / 24)
    fs = Cs.dot(Bs.dot(ul)) * (t * k_s / 4)
    ab = lambda M: np.array([abs(x) for x in np.asarray(M, dtype=object).ravel()], dtype=object).reshape(np.shape(M))
    sm = ab(Cm).dot(ab(Bm).dot(ula)) * (t / 4)
    sb = ab(Cb).dot(ab(Bb).dot(ula)) * (t ** 2 / 24)
    ss = ab(Cs).dot(ab(Bs).dot(ula)) * abs(t * k_s / 4)
    vals = [fm[0], fm[1], fm[2], fb[1], fb[0], fb[2], fs[0], fs[1]]
    scale = [sm[0], sm[1], sm[2], sb[1], sb[0], sb[2], ss[0], ss[1]]
    return vals, scale
