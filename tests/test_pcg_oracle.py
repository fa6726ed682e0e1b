"""The CPU restatement of the solution path against the reference's integration tests
(src/tests/fem/test_fem.rs:83-225): a truss with node 1 fixed in X and 100 at node 2 gives
u_2x = 0.0015 (0.0014999999 in f32) after one iteration and the reaction -100 at node 1."""
import numpy as np
import pytest

from oracle import fem_oracle as fo
from oracle.pcg import build_block_starts, find_b_sparse, find_r_r_sparse, pcg
from oracle.separate import separate_sparse


@pytest.mark.parametrize("block", [False, True])
def test_reference_truss_solution(block):
    m = fo.OracleFEM(1e-4, 1e-12, 2)
    m.add_node(1, 0.0, 0.0, 0.0)
    m.add_node(2, 30.0, 0.0, 0.0)
    m.add_truss(1, 1, 2, 1e6, 2.0)
    imposed = np.zeros(12, np.uint8)
    imposed[0] = 1
    f = np.zeros(12)
    f[6] = 100.0
    aa, bb, blocks = separate_sparse(*m.csr(), imposed, m.index_node_numbers())
    r_a, u_b = f[aa], np.zeros(len(bb))
    b = find_b_sparse(r_a, blocks["k_ab"], u_b)
    x, it, ok = pcg(blocks["k_aa"], b, 1e-4, 1e-12, 1000, build_block_starts(aa) if block else None)
    assert ok and it == 1
    assert x[0] == pytest.approx(0.0015, rel=1e-12)  # 0.0014999999 in the reference's f32 arithmetic
    r_r = find_r_r_sparse(blocks["k_ba"], x, blocks["k_bb"], u_b, f[bb])
    assert r_r[0] == pytest.approx(-100.0, rel=1e-12)


def test_block_starts():
    assert build_block_starts([0, 1, 2, 6, 8, 13]) == [0, 3, 5]
