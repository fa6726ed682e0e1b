"""Bulk add_* calls large enough for the threaded registry checks (>= 32768 items): the first
failure, its message and the state after it match the oracle's sequential calls, for every kind of
duplicate the reference rejects; after the failure the rest of the model is added and the CSR
compared bit for bit."""
import numpy as np
import pytest

from finite_element_method_gb300 import FEM, FEMError, meshes
from oracle import fem_oracle as fo

pytestmark = pytest.mark.gpu

N = 201  # 201 x 201 = 40,401 nodes, 40,000 plates, 80,400 grid bars


def grid():
    ii, jj = np.meshgrid(np.arange(N), np.arange(N), indexing="xy")
    xyz = np.stack([ii.ravel() * 0.5, jj.ravel() * 0.5, np.zeros(N * N)], -1)
    numbers = np.arange(1, N * N + 1, dtype=np.uint32)
    node = lambda i, j: 1 + i + N * j
    j, i = np.meshgrid(np.arange(N - 1), np.arange(N - 1), indexing="ij")
    quads = np.stack([node(i + 1, j + 1), node(i, j + 1), node(i, j), node(i + 1, j)], -1).reshape(-1, 4)
    bars = np.concatenate([np.stack([node(i, j), node(i + 1, j)], -1).reshape(-1, 2),
                           np.stack([node(i, j), node(i, j + 1)], -1).reshape(-1, 2)])
    return numbers, xyz, quads.astype(np.uint32), bars.astype(np.uint32)


def both(n_nodes):
    return FEM(1e-12, 1e-12, n_nodes), fo.OracleFEM(1e-12, 1e-12, n_nodes)


def expect_same_failure(call_g, call_o):
    with pytest.raises(FEMError) as eg:
        call_g()
    with pytest.raises(fo.OracleError) as eo:
        call_o()
    assert str(eg.value) == str(eo.value)
    return str(eg.value)


@pytest.mark.parametrize("case", ["number", "coords", "number_before_coords", "limit", "nan"])
def test_bulk_nodes(case):
    numbers, xyz, quads, _ = grid()
    numbers, xyz = numbers.copy(), xyz.copy()
    n_nodes = len(numbers)
    if case == "number":
        numbers[30000] = numbers[123]
    elif case == "coords":
        xyz[30000] = xyz[456]
        numbers[35000] = numbers[7]
    elif case == "number_before_coords":
        numbers[30000] = numbers[5]
        xyz[30000] = xyz[9]
    elif case == "limit":
        n_nodes = 33333
    else:  # two NaN coordinates never collide; a duplicate after them still fails
        xyz[31000] = np.nan
        xyz[31001] = np.nan
        xyz[36000] = xyz[31002]
    g, o = both(n_nodes)
    msg = expect_same_failure(lambda: g.add_nodes(numbers, xyz), lambda: o.add_nodes(numbers, xyz))
    assert g.node_count() == len(o.index_node_numbers())
    np.testing.assert_array_equal(g.index_node_numbers(), o.index_node_numbers())
    assert msg


def test_bulk_nodes_then_continue_and_assemble():
    numbers, xyz, quads, _ = grid()
    bad = numbers.copy()
    bad[25000] = bad[10]
    g, o = both(len(numbers))
    expect_same_failure(lambda: g.add_nodes(bad, xyz), lambda: o.add_nodes(bad, xyz))
    k = g.node_count()
    assert k == 25000
    g.add_nodes(numbers[k:], xyz[k:])
    o.add_nodes(numbers[k:], xyz[k:])
    E, nu, t, ks = 70e9, 0.3, 0.02, 5 / 6
    g.add_plates(np.arange(1, len(quads) + 1), quads, E, nu, t, ks)
    o.add_plates(np.arange(1, len(quads) + 1), quads, E, nu, t, ks)
    g.assemble()
    for a, b in zip(g.stiffness_csr(), o.csr()):
        np.testing.assert_array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("kind", ["truss", "beam"])
@pytest.mark.parametrize("case", ["number", "pair", "reversed_pair", "missing_node", "order",
                                  "young_before_number", "number_before_young", "young_after_missing_node"])
def test_bulk_two_node_elements(kind, case):
    """Bulk calls stop where the sequential calls would (the validation runs on the GPU while the host
    checks the numbers, over the items before the first missing node)."""
    numbers, xyz, _, bars = grid()
    bars = bars.copy()
    m = len(bars)
    enums = np.arange(1, m + 1, dtype=np.uint32)
    young = np.full(m, 200e9 if kind == "truss" else 210e9)
    if case == "young_before_number":
        young[40000] = 0.0
        enums[45000] = enums[3]
    elif case == "number_before_young":
        enums[40000] = enums[3]
        young[45000] = -1.0
    elif case == "young_after_missing_node":
        bars[40000, 1] = 10 ** 7
        young[45000] = 0.0
    elif case == "number":
        enums[40000] = enums[3]
    elif case == "pair":
        bars[40000] = bars[77]
    elif case == "reversed_pair":
        bars[40000] = bars[77][::-1]
    elif case == "missing_node":
        bars[40000, 1] = 10 ** 7
    else:  # a pair duplicate before a number duplicate
        bars[50000] = bars[1]
        enums[60000] = enums[2]
    g, o = both(len(numbers))
    g.add_nodes(numbers, xyz)
    o.add_nodes(numbers, xyz)
    if kind == "truss":
        add_g = lambda: g.add_trusses(enums, bars, young, 3e-4)
        add_o = lambda: o.add_trusses(enums, bars, young, 3e-4)
    else:
        args = (0.3, 1e-2, 3e-5, 8e-5, 0.0, 2e-5, 5 / 6, [0.0, 0.0, 1.0])
        add_g = lambda: g.add_beams(enums, bars, young, *args)
        add_o = lambda: o.add_beams(enums, bars, young, *args)
    expect_same_failure(add_g, add_o)
    counts = g.element_counts()
    assert counts[0 if kind == "truss" else 1] == (50000 if case == "order" else 40000)
    g.assemble()
    for a, b in zip(g.stiffness_csr(), o.csr()):
        np.testing.assert_array_equal(a.view(np.uint8), b.view(np.uint8))


@pytest.mark.parametrize("case", ["number", "same_nodes", "missing_node", "repeated_node_numbers",
                                  "young_before_number", "number_before_young", "line_before_number",
                                  "young_before_missing_node", "young_after_missing_node"])
def test_bulk_plates(case):
    """Bulk calls stop where the sequential calls would: the validation of a bulk call runs on the GPU while
    the host checks the numbers, over the items before the first missing node, and the first failure in
    item order wins (a number or node-set failure before an invalid plate, and the reverse)."""
    numbers, xyz, quads, _ = grid()
    quads = quads.copy()
    m = len(quads)
    pnums = np.arange(1, m + 1, dtype=np.uint32)
    young = np.full(m, 70e9)
    if case == "number":
        pnums[35000] = pnums[100]
    elif case == "same_nodes":
        quads[35000] = quads[100][[2, 3, 0, 1]]
    elif case == "missing_node":
        quads[35000, 2] = 10 ** 7
    elif case == "repeated_node_numbers":  # a plate whose node list repeats a number: the sequential path decides
        quads[20000] = [quads[5][0], quads[5][1], quads[5][1], quads[5][2]]
    elif case == "young_before_number":
        young[20000] = 0.0
        pnums[35000] = pnums[100]
    elif case == "number_before_young":
        pnums[20000] = pnums[100]
        young[35000] = -1.0
    elif case == "line_before_number":  # the third node moved onto the line of the first two (an inner plate)
        a, b = int(quads[20050, 0]), int(quads[20050, 1])
        quads[20050, 2] = b + (b - a)
        pnums[35000] = pnums[100]
    elif case == "young_before_missing_node":
        young[20000] = 0.0
        quads[35000, 2] = 10 ** 7
    else:  # young_after_missing_node
        quads[30000, 2] = 10 ** 7
        young[35000] = 0.0
    g, o = both(len(numbers))
    g.add_nodes(numbers, xyz)
    o.add_nodes(numbers, xyz)
    nu, t, ks = 0.3, 0.02, 5 / 6
    expect_same_failure(lambda: g.add_plates(pnums, quads, young, nu, t, ks),
                        lambda: o.add_plates(pnums, quads, young, nu, t, ks))
    g.assemble()
    for a, b in zip(g.stiffness_csr(), o.csr()):
        np.testing.assert_array_equal(a.view(np.uint8), b.view(np.uint8))


# -- the registries of bulk calls are checked on the GPU and built on the host only when a later call needs
#    them: every mix of bulk and single calls must still see every earlier node and plate

def two_layers():
    """the grid twice, the second layer at z = 1 (node numbers continue), each with its quads"""
    numbers, xyz, quads, _ = grid()
    n = len(numbers)
    xyz2 = xyz.copy()
    xyz2[:, 2] = 1.0
    return numbers, xyz, quads, numbers + n, xyz2, quads + n


def test_bulk_then_single_and_second_bulk_nodes():
    n1, x1, _, n2, x2, _ = two_layers()
    g, o = both(len(n1) + len(n2) + 50000)
    for m in (g, o):
        m.add_nodes(n1, x1)
    # a single node at the coordinates of a bulk-added node, then a fresh one
    expect_same_failure(lambda: g.add_node(10 ** 6, *x1[1234]), lambda: o.add_node(10 ** 6, *x1[1234]))
    for m in (g, o):
        m.add_node(10 ** 6, 1e3, 1e3, 0.0)
    # a second bulk call whose item 30000 repeats the coordinates of a first-call node
    bad = x2.copy()
    bad[30000] = x1[77]
    expect_same_failure(lambda: g.add_nodes(n2, bad), lambda: o.add_nodes(n2, bad))
    np.testing.assert_array_equal(g.index_node_numbers(), o.index_node_numbers())
    assert g.node_count() == len(n1) + 1 + 30000
    # and a duplicate of the single node inside a bulk call
    more_n = np.arange(2 * 10 ** 6, 2 * 10 ** 6 + 40000, dtype=np.uint32)
    more_x = np.stack([np.arange(40000) * 0.25 + 5e3, np.zeros(40000), np.zeros(40000)], -1)
    more_x[35000] = [1e3, 1e3, -0.0]  # -0.0 == 0.0
    expect_same_failure(lambda: g.add_nodes(more_n, more_x), lambda: o.add_nodes(more_n, more_x))
    np.testing.assert_array_equal(g.index_node_numbers(), o.index_node_numbers())


def test_bulk_then_single_and_second_bulk_plates():
    n1, x1, q1, n2, x2, q2 = two_layers()
    m = len(q1)
    E, nu, t, ks = 70e9, 0.3, 0.02, 5 / 6
    g, o = both(len(n1) + len(n2))
    for x in (g, o):
        x.add_nodes(n1, x1)
        x.add_nodes(n2, x2)
        x.add_plates(np.arange(1, m + 1), q1, E, nu, t, ks)
    # a single plate on the node set of a bulk-added plate (other order)
    q = q1[321][[1, 2, 3, 0]]
    expect_same_failure(lambda: g.add_plate(10 ** 6, *q, E, nu, t, ks), lambda: o.add_plate(10 ** 6, *q, E, nu, t, ks))
    # a second bulk call whose item 17000 repeats a first-call plate's node set
    bad = q2.copy()
    bad[17000] = q1[4321][[3, 2, 1, 0]]
    expect_same_failure(lambda: g.add_plates(np.arange(m + 1, 2 * m + 1), bad, E, nu, t, ks),
                        lambda: o.add_plates(np.arange(m + 1, 2 * m + 1), bad, E, nu, t, ks))
    assert g.element_counts()[2] == m + 17000
    # the single path sees the second bulk call's plates too
    q = q2[5][[2, 3, 0, 1]]
    expect_same_failure(lambda: g.add_plate(10 ** 6 + 1, *q, E, nu, t, ks),
                        lambda: o.add_plate(10 ** 6 + 1, *q, E, nu, t, ks))
    g.assemble()
    for a, b in zip(g.stiffness_csr(), o.csr()):
        np.testing.assert_array_equal(a.view(np.uint8), b.view(np.uint8))


def test_moved_nodes_are_checked_at_their_new_coordinates():
    numbers, xyz, _, _ = grid()
    g = FEM(1e-12, 1e-12, len(numbers) + 2)
    g.add_nodes(numbers, xyz)
    moved = xyz.copy()
    moved[500] = [7e3, 7e3, 7e3]
    g.set_node_coordinates(moved)
    g.add_node(10 ** 6, *xyz[500])  # the old place is free now
    with pytest.raises(FEMError, match="already exists"):
        g.add_node(10 ** 6 + 1, 7e3, 7e3, 7e3)


@pytest.mark.parametrize("kind", ["truss", "beam"])
def test_bulk_then_single_and_second_bulk_two_node_elements(kind):
    numbers, xyz, _, bars = grid()
    m = len(bars)
    half = m // 2  # 40,200 per call: both calls take the bulk path
    enums = np.arange(1, m + 1, dtype=np.uint32)
    g, o = both(len(numbers))
    for x in (g, o):
        x.add_nodes(numbers, xyz)
    if kind == "truss":
        add = lambda x, nums, prs: x.add_trusses(nums, prs, 200e9, 3e-4)
        one = lambda x, num, u, v: x.add_truss(num, u, v, 200e9, 3e-4)
    else:
        args = (210e9, 0.3, 1e-2, 3e-5, 8e-5, 0.0, 2e-5, 5 / 6, [0.0, 0.0, 1.0])
        add = lambda x, nums, prs: x.add_beams(nums, prs, *args)
        one = lambda x, num, u, v: x.add_beam(num, u, v, *args)
    for x in (g, o):
        add(x, enums[:half], bars[:half])
    # a single element on a bulk-added pair (reversed), then a second bulk call repeating a first-call pair
    u, v = bars[999]
    expect_same_failure(lambda: one(g, 10 ** 6, v, u), lambda: one(o, 10 ** 6, v, u))
    rest = bars[half:].copy()
    rest[33000] = bars[5][::-1]
    expect_same_failure(lambda: add(g, enums[half:], rest), lambda: add(o, enums[half:], rest))
    assert g.element_counts()[0 if kind == "truss" else 1] == half + 33000
    u, v = rest[7]
    expect_same_failure(lambda: one(g, 10 ** 6 + 1, u, v), lambda: one(o, 10 ** 6 + 1, u, v))
    g.assemble()
    for a, b in zip(g.stiffness_csr(), o.csr()):
        np.testing.assert_array_equal(a.view(np.uint8), b.view(np.uint8))
