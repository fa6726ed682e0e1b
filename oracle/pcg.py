"""CPU restatement of the reference's sparse solution path.

TEST INFRASTRUCTURE ONLY: imported by tests/ and by bench.py's CPU legs,
never by the product package.

find_b_sparse and find_r_r_sparse follow src/fem/methods_for_global_analysis.rs:27-48
and :100-133 loop by loop; build_block_starts follows :140-159.  The conjugate
gradient itself is in the unvendored iterative_solvers_smpl 0.1.5, so `pcg` is the
textbook preconditioned recurrence from x = 0 with the stopping rule
||r||_2 <= max(rel_tol ||b||_2, abs_tol) after every iteration -- the rule the GPU
path states -- with the diagonal (Jacobi) or the node blocks (block Jacobi) of A.
"""
from __future__ import annotations

import numpy as np
import scipy.sparse as sp


def find_b_sparse(r_a, k_ab, u_b):
    """b = r_a - K_ab u_b, one subtraction per triplet (k_ab: (rows, cols, values))"""
    b = np.array(r_a, dtype=np.float64)
    for i, j, a in zip(*k_ab):
        b[i] = b[i] - a * u_b[j]
    return b


def find_r_r_sparse(k_ba, u_a, k_bb, u_b, r_b):
    n_bb = len(r_b)
    y_ba = np.zeros(n_bb)
    for i, j, a in zip(*k_ba):
        y_ba[i] = y_ba[i] + a * u_a[j]
    y_bb = np.zeros(n_bb)
    for i, j, a in zip(*k_bb):
        y_bb[i] = y_bb[i] + a * u_b[j]
    return (y_ba + y_bb) - np.asarray(r_b)


def build_block_starts(k_aa_indexes):
    starts = []
    cur = None
    for i, g in enumerate(k_aa_indexes):
        if g // 6 != cur:
            starts.append(i)
            cur = g // 6
    return starts


def pcg(k_aa, b, rel_tol, abs_tol, max_iter, block_starts=None):
    """(x, iterations, converged) for K_aa x = b; k_aa: (rows, cols, values), n = len(b)"""
    n = len(b)
    A = sp.csr_matrix((k_aa[2], (k_aa[0], k_aa[1])), shape=(n, n))
    if block_starts is None:
        block_starts = list(range(n))
    bounds = list(block_starts) + [n]
    inv = [np.linalg.inv(A[s:e, s:e].toarray()) for s, e in zip(bounds[:-1], bounds[1:])]

    def precond(r):
        return np.concatenate([m @ r[s:e] for m, s, e in zip(inv, bounds[:-1], bounds[1:])]) if n else r

    x = np.zeros(n)
    r = np.array(b, dtype=np.float64)
    tol = max(rel_tol * np.sqrt(r @ r), abs_tol)
    if not np.sqrt(r @ r) > tol:
        return x, 0, True
    z = precond(r)
    p = z.copy()
    rz = r @ z
    for it in range(1, max_iter + 1):
        q = A @ p
        alpha = rz / (p @ q)
        x += alpha * p
        r -= alpha * q
        if not np.sqrt(r @ r) > tol:
            return x, it, True
        z = precond(r)
        rz_new = r @ z
        p = z + (rz_new / rz) * p
        rz = rz_new
    return x, max_iter, False
