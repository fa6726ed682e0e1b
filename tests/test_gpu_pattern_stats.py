"""Pattern sizes (fem_gpu_get_pattern_stats) against counts made from the mesh's
connectivity: node-pair blocks, element pair contributions, packed scratch entries
and block-sum slots.  On a flat plate mesh every block is packed (13 entries off the
diagonal, 14 on it), so the scratch holds 134 entries a plate; the 14th word that
pads each 13-entry contribution is not counted."""
import numpy as np
import pytest

from finite_element_method_gb300 import FEM, meshes

pytestmark = pytest.mark.gpu

PAIRS4 = [(0, 0), (0, 1), (0, 2), (0, 3), (1, 1), (1, 2), (1, 3), (2, 2), (2, 3), (3, 3)]


def expected_stats(nodes):
    """(blocks, contributions, packed entries, sum slots) of a flat plate mesh from its connectivity
    (nodes: (n_plates, 4) node indexes)."""
    keys = []
    for i, j in PAIRS4:
        a, b = nodes[:, i], nodes[:, j]
        keys.append(np.minimum(a, b).astype(np.int64) << 32 | np.maximum(a, b).astype(np.int64))
    keys = np.concatenate(keys)
    uniq, count = np.unique(keys, return_counts=True)
    diag = (uniq >> 32) == (uniq & 0xFFFFFFFF)
    size = np.where(diag, 14, 13)
    contributions = len(keys)
    entries = int((size * count).sum())
    sum_slots = int(size[count >= 2].sum())
    return len(uniq), contributions, entries, sum_slots


@pytest.mark.parametrize("nx,ny", [(6, 5), (40, 31)])
def test_plate_pattern_stats_match_connectivity(nx, ny):
    mesh = meshes.plate_mesh(nx, ny, size=2.0)
    g = FEM(meshes.REL_TOL, meshes.ABS_TOL, mesh.nodes_number)
    meshes.load(g, mesh)
    g.assemble()
    got = g.pattern_stats()
    nodes = mesh.plates["nodes"].astype(np.int64) - 1  # node numbers are 1-based indexes here
    want = expected_stats(nodes)
    g.close()
    assert got == want
    assert got[2] == 134 * len(nodes)
