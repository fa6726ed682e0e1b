"""The CPU restatement of the sparse separation against the reference's own test case
(src/tests/fem/test_fem.rs:66-81 and the PCG tests at :83-225, whose single free DOF has
K_aa = 100 / 0.0015 = 66666.67) and its error paths."""
import numpy as np
import pytest

from oracle import fem_oracle as fo
from oracle.separate import separate_sparse


def truss_model():
    m = fo.OracleFEM(1e-4, 1e-12, 2)
    m.add_node(1, 0.0, 0.0, 0.0)
    m.add_node(2, 30.0, 0.0, 0.0)
    m.add_truss(1, 1, 2, 1e6, 2.0)
    return m


def test_reference_truss_case():
    m = truss_model()
    rp, ci, va = m.csr()
    imposed = np.zeros(12, np.uint8)
    imposed[0] = 1  # add_displacement(1, X, 0.0)
    aa, bb, blocks = separate_sparse(rp, ci, va, imposed, m.index_node_numbers())
    assert aa.tolist() == [6] and bb.tolist() == [0]
    k = 1e6 * 2.0 / 30.0
    for name, sign in (("k_aa", 1), ("k_ab", -1), ("k_ba", -1), ("k_bb", 1)):
        r, c, v = blocks[name]
        assert r.tolist() == [0] and c.tolist() == [0]
        assert v[0] == pytest.approx(sign * k, rel=1e-15)
    # the reference's PCG result for the free DOF: u = f / K_aa with f = 100
    assert 100.0 / blocks["k_aa"][2][0] == pytest.approx(0.0015, rel=1e-12)


def test_displacement_on_a_dof_without_stiffness():
    m = truss_model()
    rp, ci, va = m.csr()
    imposed = np.zeros(12, np.uint8)
    imposed[[0, 3]] = 1  # node 1: X and ThX (a truss has no rotational stiffness)
    with pytest.raises(fo.OracleError, match=r"^There are no stiffness to withstand displacement ThX applied to "
                                             r"node 1!$"):
        separate_sparse(rp, ci, va, imposed, m.index_node_numbers())


def test_no_restraints():
    m = truss_model()
    rp, ci, va = m.csr()
    with pytest.raises(fo.OracleError, match="^No restraints$"):
        separate_sparse(rp, ci, va, np.zeros(12, np.uint8), m.index_node_numbers())


def test_empty_kaa():
    m = truss_model()
    rp, ci, va = m.csr()
    imposed = np.zeros(12, np.uint8)
    imposed[[0, 6]] = 1  # both translational DOFs with stiffness restrained
    with pytest.raises(fo.OracleError, match=r"K_aa is empty"):
        separate_sparse(rp, ci, va, imposed, m.index_node_numbers())
