"""CPU restatement of the reference's sparse stiffness separation.

TEST INFRASTRUCTURE ONLY: imported by tests/ and by bench.py's CPU legs,
never by the product package.

`separate_sparse` follows separate_stiffness_matrix_sparse_iterative
(src/fem/methods_for_separate_stiffness_matrix.rs:217-320) line by line, on
the stored entries of the global stiffness given as CSR (the keys of the
reference's SquareMatrix, zero-valued kept keys included).
"""
from __future__ import annotations

import numpy as np

from .fem_oracle import OracleError

DOF_PARAMETERS = ("X", "Y", "Z", "ThX", "ThY", "ThZ")  # methods_for_bc_data_handle.rs:7-14
ERR_DISPLACEMENT, ERR_NO_RESTRAINTS, ERR_EMPTY_KAA = 22, 23, 24
BLOCKS = ("k_aa", "k_ab", "k_ba", "k_bb")


def separate_sparse(row_ptr, col_idx, values, imposed, index_node_numbers):
    """Returns (k_aa_indexes, k_bb_indexes, {block: (rows, cols, values)}), each block's triplets sorted by
    (row, column); raises OracleError with the reference's messages."""
    row_ptr = np.asarray(row_ptr, np.int64)
    col_idx = np.asarray(col_idx, np.int64)
    values = np.asarray(values, np.float64)
    imposed = np.asarray(imposed).astype(bool)
    n = len(row_ptr) - 1  # get_indexes(): every DOF of nodes_number nodes
    rows = np.repeat(np.arange(n), np.diff(row_ptr))
    # :221-226 the diagonal, 0 where K has no (i, i) entry
    diag = np.zeros(n)
    on_diag = rows == col_idx
    diag[rows[on_diag]] = values[on_diag]
    # :231-253 DOFs in ascending order: zero diagonal -> error if imposed, else excluded; then b or a
    zero = diag == 0.0
    bad = np.flatnonzero(zero & imposed)
    if bad.size:
        idx = int(bad[0])
        node = idx // 6
        number = int(index_node_numbers[node]) if node < len(index_node_numbers) else 0
        raise OracleError(ERR_DISPLACEMENT, f"There are no stiffness to withstand displacement "
                                            f"{DOF_PARAMETERS[idx % 6]} applied to node {number}!")
    bb = np.flatnonzero(~zero & imposed)
    aa = np.flatnonzero(~zero & ~imposed)
    if bb.size == 0:  # :255-257
        raise OracleError(ERR_NO_RESTRAINTS, "No restraints")
    # :262-270 local positions
    aa_pos = np.full(n, -1, np.int64)
    bb_pos = np.full(n, -1, np.int64)
    aa_pos[aa] = np.arange(aa.size)
    bb_pos[bb] = np.arange(bb.size)
    # :277-303 every non-zero stored entry with both DOFs kept, into one of the four blocks
    nz = values != 0.0
    i_aa, j_aa, i_bb, j_bb = aa_pos[rows], aa_pos[col_idx], bb_pos[rows], bb_pos[col_idx]
    sel = {
        "k_aa": nz & (i_aa >= 0) & (j_aa >= 0),
        "k_ab": nz & (i_aa >= 0) & (j_bb >= 0),
        "k_ba": nz & (i_bb >= 0) & (j_aa >= 0),
        "k_bb": nz & (i_bb >= 0) & (j_bb >= 0),
    }
    loc = {"k_aa": (i_aa, j_aa), "k_ab": (i_aa, j_bb), "k_ba": (i_bb, j_aa), "k_bb": (i_bb, j_bb)}
    blocks = {}
    for name in BLOCKS:
        m = sel[name]
        r, c = loc[name]
        blocks[name] = (r[m], c[m], values[m])  # CSR order: sorted by (row, column)
    if blocks["k_aa"][0].size == 0:  # :305-309
        raise OracleError(ERR_EMPTY_KAA, "Sparse separation: K_aa is empty (structure has no free stiffness?)")
    return aa, bb, blocks
