"""CPU restatement of the reference's load application.

TEST INFRASTRUCTURE ONLY: imported by tests/ and by bench.py's CPU legs,
never by the product package.

add_concentrated_load, add_uniformly_distributed_line_load and
add_uniformly_distributed_surface_load (src/fem/methods_for_bc_data_handle.rs:20-175)
add their nodal contributions to the forces vector in call order, one `+=`
each (node 1 first); the element parts are the C oracle's orc_beam_line_load
and orc_plate_surface_load.
"""
from __future__ import annotations

import numpy as np

from . import fem_oracle as fo


def forces_vector(nodes_number, xyz, loads, beam_nodes=None, plate_nodes=None, rel_tol=1e-12, abs_tol=1e-12):
    """loads: call-ordered list of (kind, index, dof, value); kind 'node' (index = node index), 'line' (index =
    beam index into beam_nodes, pairs of node indices) or 'surface' (plate index into plate_nodes)."""
    f = [0.0] * (6 * nodes_number)
    for kind, i, dof, value in loads:
        if kind == "node":
            f[6 * i + dof] = f[6 * i + dof] + float(value)
            continue
        if kind == "line":
            n = beam_nodes[i]
            c = fo.beam_line_load(xyz[n[0]], xyz[n[1]], float(value))
        else:
            n = plate_nodes[i]
            c = fo.plate_surface_load(*[xyz[k] for k in n], float(value), rel_tol, abs_tol)
        for k, node in enumerate(n):
            f[6 * int(node) + dof] = f[6 * int(node) + dof] + float(c[k])
    return np.array(f)
