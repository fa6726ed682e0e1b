"""CPU restatement of the reference's equivalent nodal loads (beam.rs:775-797, plate.rs:1145-1185)
against closed forms: q L / 2 per beam node; for a parallelogram plate the four shares are equal and
sum to q times its area (the Jacobian is constant); for a general quad they sum to q times its area."""
import numpy as np
import pytest

from oracle import fem_oracle as fo
from oracle.loads import forces_vector


def test_beam_line_load():
    f = fo.beam_line_load([0.0, 0.0, 0.0], [3.0, 4.0, 0.0], 10.0)
    assert f.tolist() == [25.0, 25.0]


def test_plate_surface_load_parallelogram_and_tilt():
    rng = np.random.default_rng(0)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    quad = np.array([[3.0, 2.0, 0.0], [1.0, 2.0, 0.0], [0.0, 0.0, 0.0], [2.0, 0.0, 0.0]])  # area 4
    for rot in (np.eye(3), q):
        f = fo.plate_surface_load(*(quad @ rot.T), 5.0)
        np.testing.assert_allclose(f, [5.0, 5.0, 5.0, 5.0], rtol=1e-14)


def test_plate_surface_load_general_quad_total():
    quad = np.array([[1.2, 0.9, 0.0], [-0.8, 1.1, 0.0], [-1.0, -1.0, 0.0], [0.9, -1.2, 0.0]])
    x, y = quad[:, 0], quad[:, 1]
    area = 0.5 * abs(np.dot(x, np.roll(y, -1)) - np.dot(y, np.roll(x, -1)))
    f = fo.plate_surface_load(*quad, 3.0)
    assert f.sum() == pytest.approx(3.0 * area, rel=1e-13)


def test_forces_in_call_order():
    xyz = np.array([[0.0, 0.0, 0.0], [2.0, 0.0, 0.0], [2.0, 2.0, 0.0], [0.0, 2.0, 0.0]])
    loads = [("node", 1, 2, -7.0), ("line", 0, 2, 4.0), ("surface", 0, 2, 1.0), ("node", 1, 2, 0.5)]
    f = forces_vector(4, xyz, loads, beam_nodes=[(0, 1)], plate_nodes=[(2, 3, 0, 1)])
    # node 1, Z: -7 + (4 * 2 / 2) + (1 * 4 / 4) + 0.5
    assert f[6 * 1 + 2] == ((-7.0 + 4.0) + 1.0) + 0.5
    assert f[2] == 4.0 + 1.0 and f.sum() == -7.0 + 8.0 + 4.0 + 0.5
