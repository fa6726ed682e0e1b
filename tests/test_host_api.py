"""CPU checks of the host mirror's FEM::reset (fem.rs:155-169): no device work happens before the first
add, so the handle swap, the new sizes and the kept node limit are checked here without a GPU."""
import numpy as np

from finite_element_method_gb300 import FEM


def test_reset_sizes_vectors_and_keeps_tolerances_and_limit():
    g = FEM(1e-9, 1e-11, 5)
    h0 = g.handle.value
    g.reset(8)
    assert g.handle.value and g.handle.value != h0
    assert (g.rel_tol, g.abs_tol, g.nodes_number) == (1e-9, 1e-11, 8)
    assert g._node_limit == 5
    assert g.node_count() == 0 and g.element_counts() == (0, 0, 0)
    assert np.array_equal(g.displacements_vector(), np.zeros(48))
    g.reset(2)
    assert g.nodes_number == 2 and g._node_limit == 5
    assert g.displacements_vector().shape == (12,)
    g.close()
    assert g.handle is None
