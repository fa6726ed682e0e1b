"""Batch.structures -- the host arrays of many meshes laid out one after another for
fem_gpu_batch_create_from_arrays (fem_gpu_structures_t) -- checked on the CPU: per-structure offsets,
node and element arrays concatenated in mesh order, the NaN fill of absent second truss areas, kinds a
batch leaves NULL, and the forms of nodes_number.  No device work: the layout is host-side only."""
import numpy as np
import pytest

from finite_element_method_gb300 import Batch, meshes


def _read(p, n, dtype):
    return np.array([p[i] for i in range(n)], dtype=dtype)


def _meshes():
    lat = meshes.truss_lattice(4, seed=9)
    lat.trusses["area_2"] = np.where(np.arange(len(lat.trusses["numbers"])) % 2 == 0, np.nan,
                                     lat.trusses["area"] * 0.7)
    return [meshes.adjoint_model(frame=(3, 3, 2), slab=(20, 20), seed=3), lat, meshes.plate_mesh(5, 4, size=2.0),
            meshes.truss_lattice(3, seed=2)]


def test_offsets_and_arrays_in_mesh_order():
    ms = _meshes()
    st, _keep = Batch.structures(ms)
    S = len(ms)
    assert st.n_structures == S
    nn = [m.nodes_number for m in ms]
    np.testing.assert_array_equal(_read(st.nodes_number, S, np.uint32), nn)
    node_off = _read(st.node_off, S + 1, np.int64)
    np.testing.assert_array_equal(node_off, np.concatenate([[0], np.cumsum(nn)]))
    N = int(node_off[-1])
    np.testing.assert_array_equal(_read(st.node_numbers, N, np.uint32),
                                  np.concatenate([m.node_numbers for m in ms]))
    np.testing.assert_array_equal(_read(st.xyz, 3 * N, np.float64),
                                  np.concatenate([np.asarray(m.xyz).reshape(-1) for m in ms]))
    for kind, prefix, width in (("trusses", "truss", 2), ("beams", "beam", 2), ("plates", "plate", 4)):
        counts = [0 if getattr(m, kind) is None else len(getattr(m, kind)["numbers"]) for m in ms]
        off = _read(getattr(st, prefix + "_off"), S + 1, np.int64)
        np.testing.assert_array_equal(off, np.concatenate([[0], np.cumsum(counts)]), err_msg=kind)
        E = int(off[-1])
        parts = [getattr(m, kind) for m in ms if getattr(m, kind) is not None]
        np.testing.assert_array_equal(_read(getattr(st, prefix + "_numbers"), E, np.uint32),
                                      np.concatenate([d["numbers"] for d in parts]), err_msg=kind)
        np.testing.assert_array_equal(_read(getattr(st, prefix + "_nodes"), width * E, np.uint32),
                                      np.concatenate([np.asarray(d["nodes"]).reshape(-1) for d in parts]),
                                      err_msg=kind)
        np.testing.assert_array_equal(_read(getattr(st, prefix + "_young"), E, np.float64),
                                      np.concatenate([np.broadcast_to(d["young"], (len(d["numbers"]),))
                                                      for d in parts]), err_msg=kind)


def test_absent_second_areas_are_nan():
    ms = _meshes()
    st, _keep = Batch.structures(ms)
    E = int(_read(st.truss_off, len(ms) + 1, np.int64)[-1])
    a2 = _read(st.truss_area2, E, np.float64)
    want = np.concatenate([np.full(len(m.trusses["numbers"]), np.nan) if m.trusses.get("area_2") is None
                           else m.trusses["area_2"] for m in ms if m.trusses is not None])
    np.testing.assert_array_equal(a2, want)  # NaN where NaN (assert_array_equal treats NaN as equal)
    assert np.isnan(a2).any() and not np.isnan(a2).all()


def test_kinds_absent_from_every_mesh_stay_null():
    st, _keep = Batch.structures([meshes.plate_mesh(4, 3, size=1.0), meshes.plate_mesh(3, 3, size=1.0, seed=5)])
    assert not st.truss_off and not st.truss_numbers and not st.beam_off and not st.beam_local_axis
    assert st.plate_off and st.plate_nodes


def test_nodes_number_per_mesh_or_one_for_all():
    ms = _meshes()
    S = len(ms)
    room = [m.nodes_number + k for k, m in enumerate(ms)]
    st, _keep = Batch.structures(ms, room)
    np.testing.assert_array_equal(_read(st.nodes_number, S, np.uint32), room)
    big = max(m.nodes_number for m in ms) + 3
    st, _keep = Batch.structures(ms, big)
    np.testing.assert_array_equal(_read(st.nodes_number, S, np.uint32), [big] * S)
    with pytest.raises(ValueError, match="one per mesh"):
        Batch.structures(ms, room[:-1])


def test_kinds_must_come_trusses_beams_plates():
    m = meshes.adjoint_model(frame=(3, 3, 2), slab=(20, 20), seed=3)
    m.order = ("plates", "beams", "trusses")
    with pytest.raises(ValueError, match="trusses, then beams, then plates"):
        Batch.structures([m])
