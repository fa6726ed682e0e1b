"""The batch built from host arrays (fem_gpu_batch_create_from_arrays) against
one plain call sequence per structure (FEM + add_nodes + add_* + assemble):
every structure's CSR (row_ptr, col_idx and the values' bits) must be the one
its plain assembly gives, and a structure whose calls would fail must make the
batch fail with that call's code and message."""
import numpy as np
import pytest

from finite_element_method_gb300 import FEM, FEMError, meshes
from finite_element_method_gb300.fem import Batch
from oracle.fem_oracle import OracleFEM

pytestmark = pytest.mark.gpu

TOL = (meshes.REL_TOL, meshes.ABS_TOL)


def plain_csr(m):
    g = FEM(*TOL, m.nodes_number)
    meshes.load(g, m)
    g.assemble()
    out = g.stiffness_csr()
    g.close()
    return out


def assert_same_csr(a, b):
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    np.testing.assert_array_equal(np.asarray(a[2]).view(np.uint64), np.asarray(b[2]).view(np.uint64))


def test_batch_from_meshes_matches_plain_calls():
    structures = meshes.batch_structures(11, lo=150, hi=4000, seed=18)
    kinds = {m.name.split("_")[0] for m in structures}
    assert kinds == {"truss", "beam", "plate"}
    b = Batch.from_meshes(structures, *TOL)
    assert len(b) == len(structures)
    refs = [plain_csr(m) for m in structures]
    for i, r in enumerate(refs):
        assert_same_csr(b.csr(i), r)
    # further numeric passes, default and autotuned configuration
    b.assemble()
    table = b.autotune(reps=2)
    assert table["best_ms"] > 0
    b.assemble()
    for i, r in enumerate(refs):
        assert_same_csr(b.csr(i), r)
    # two against the oracle
    for i in (0, len(structures) - 1):
        o = OracleFEM(*TOL, structures[i].nodes_number)
        meshes.load(o, structures[i])
        assert_same_csr(b.csr(i), o.csr())
    b.close()


def test_batch_mixed_kinds_and_spare_node_slots():
    """structures holding trusses, beams and plates together, with room for more nodes than they add
    (empty rows, as FEM::create(nodes_number) gives them)"""
    ms = [meshes.adjoint_model(frame=(3, 3, 2), slab=(20, 20), seed=s) for s in (3, 4)]
    lat = meshes.truss_lattice(4, seed=9)
    lat.trusses["area_2"] = np.where(np.arange(len(lat.trusses["numbers"])) % 2 == 0, np.nan,
                                     lat.trusses["area"] * 0.7)
    structures = [ms[0], lat, ms[1]]
    room = [m.nodes_number + extra for m, extra in zip(structures, (5, 0, 17))]
    b = Batch.from_meshes(structures, *TOL, nodes_number=room)
    for i, m in enumerate(structures):
        g = FEM(*TOL, room[i])
        meshes.load(g, m)
        g.assemble()
        assert_same_csr(b.csr(i), g.stiffness_csr())
        g.close()
    b.close()


def _plain_error(m, nodes_number=None):
    g = FEM(*TOL, m.nodes_number if nodes_number is None else nodes_number)
    try:
        meshes.load(g, m)
    except FEMError as e:
        return e.code, str(e)
    finally:
        g.close()
    return None


@pytest.mark.parametrize("fault", ["node_number", "coordinates", "element_number", "missing_node", "node_pair",
                                   "plate_set", "thickness", "not_convex", "too_many_nodes"])
def test_batch_reports_first_failing_structure(fault):
    structures = meshes.batch_structures(6, lo=100, hi=600, seed=23, kinds=("beam", "plate"))
    plates = [i for i, m in enumerate(structures) if m.plates is not None]
    beams = [i for i, m in enumerate(structures) if m.beams is not None]
    assert plates and beams
    room = None
    if fault in ("node_number", "coordinates", "missing_node", "too_many_nodes"):
        s = 2
    elif fault == "node_pair" or fault == "element_number":
        s = beams[-1]
    else:
        s = plates[-1]
    m = structures[s]
    if fault == "node_number":
        m.node_numbers = m.node_numbers.copy()
        m.node_numbers[7] = m.node_numbers[3]
    elif fault == "coordinates":
        m.xyz = m.xyz.copy()
        m.xyz[9] = m.xyz[4]
    elif fault == "element_number":
        m.beams["numbers"] = m.beams["numbers"].copy()
        m.beams["numbers"][5] = m.beams["numbers"][1]
    elif fault == "missing_node":
        d = m.plates if m.plates is not None else m.beams
        d["nodes"] = d["nodes"].copy()
        d["nodes"][2, 1] = 10 ** 7
    elif fault == "node_pair":
        m.beams["nodes"] = m.beams["nodes"].copy()
        m.beams["nodes"][6] = m.beams["nodes"][2][::-1]
    elif fault == "plate_set":
        m.plates["nodes"] = m.plates["nodes"].copy()
        m.plates["nodes"][4] = np.roll(m.plates["nodes"][1], 1)
    elif fault == "thickness":
        m.plates["thickness"] = m.plates["thickness"].copy()
        m.plates["thickness"][3] = -0.01
    elif fault == "not_convex":
        m.xyz = m.xyz.copy()
        q = m.plates["nodes"][5] - 1
        m.xyz[q[0], :2] = 0.5 * (m.xyz[q[1], :2] + m.xyz[q[3], :2]) + 0.3 * (m.xyz[q[2], :2] - m.xyz[q[0], :2])
    elif fault == "too_many_nodes":
        room = [x.nodes_number for x in structures]
        room[s] -= 1
    want = _plain_error(m, None if room is None else room[s])
    assert want is not None, "the planted fault must make the plain calls fail"
    with pytest.raises(FEMError) as ei:
        Batch.from_meshes(structures, *TOL, nodes_number=room)
    assert ei.value.code == want[0]
    assert str(ei.value) == f"structure {s}: {want[1]}"


@pytest.mark.slow
def test_batch_full_config_matches_plain_calls():
    """512 structures (config 4: log-uniform 1e3..2e5 elements, seeded kind mix): every structure bit for bit
    against its own plain call sequence, two of them against the oracle."""
    structures = meshes.batch_structures()
    b = Batch.from_meshes(structures, *TOL)
    assert len(b) == 512
    for i, m in enumerate(structures):
        assert_same_csr(b.csr(i), plain_csr(m))
    small = sorted(range(512), key=lambda i: structures[i].n_elements)[:2]
    for i in small:
        o = OracleFEM(*TOL, structures[i].nodes_number)
        meshes.load(o, structures[i])
        assert_same_csr(b.csr(i), o.csr())
    b.close()
