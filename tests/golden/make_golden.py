"""Writes tests/golden/element_matrices.json: element matrices of the reference
formulas (oracle/literal.py, a literal dense restatement of structs/truss.rs,
structs/beam.rs and structs/plate.rs) evaluated in 50-digit mpmath arithmetic.

The reference crate cannot be compiled in this environment (no Rust toolchain,
unvendored `extended_matrix`), so these high-precision evaluations of its
formulas pin the FP64 oracle's restructured evaluation order.  Run:
    python tests/golden/make_golden.py
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import literal  # noqa: E402

BK = literal.Backend.mp(50)


def mstr(M):
    return [str(v) if v != 0 else "0" for v in np.asarray(M, dtype=object).ravel()]


def main():
    cases = []
    # trusses
    for name, a in [
        ("truss_reference_test", dict(x1=[0.0, 0.0, 0.0], x2=[30.0, 0.0, 0.0], young=1e6, area=2.0)),
        ("truss_skew", dict(x1=[0.1, -0.3, 0.7], x2=[1.3, 0.4, -0.2], young=200e9, area=3.2e-4)),
        ("truss_tapered", dict(x1=[0.0, 0.0, 0.0], x2=[0.0, 2.5, 1.0], young=200e9, area=3e-4, area_2=1e-4)),
        ("truss_antiparallel", dict(x1=[2.0, 0.0, 0.0], x2=[-1.0, 0.0, 0.0], young=200e9, area=2e-4)),
    ]:
        M = literal.truss_global_matrix(a["x1"], a["x2"], a["young"], a["area"], a.get("area_2"), bk=BK)
        cases.append(dict(name=name, kind="truss", args=a, shape=[6, 6], matrix=mstr(M), axis_aligned="skew" not in name
                          and "tapered" not in name))
    # beams
    base = dict(young=210e9, poisson=0.3, area=1.2e-2, i11=8e-5, i22=3e-5, i12=0.0, it=2e-5, shear_factor=5 / 6)
    for name, geo in [
        ("beam_x_axis", dict(x1=[0.0, 0.0, 0.0], x2=[3.0, 0.0, 0.0], axis=[0.0, 0.0, 1.0])),
        ("beam_skew", dict(x1=[0.2, 0.1, -0.4], x2=[2.9, 1.7, 0.8], axis=[0.0, 0.0, 1.0])),
        ("beam_vertical_z", dict(x1=[0.0, 0.0, 0.0], x2=[0.05, -0.08, 3.0], axis=[1.0, 0.0, 0.0])),
        ("beam_vertical_y", dict(x1=[1.0, 0.0, 0.0], x2=[1.0, 2.0, 0.0], axis=[1.0, 0.0, 1.0])),
        ("beam_i12", dict(x1=[0.0, 0.0, 0.0], x2=[2.0, 1.0, 0.5], axis=[0.0, 1.0, 0.0], i12=1e-5)),
        ("beam_equal_i", dict(x1=[0.0, 0.0, 0.0], x2=[2.0, 0.0, 1.0], axis=[0.0, 0.0, 1.0], i11=5e-5, i22=5e-5)),
    ]:
        a = dict(base)
        a.update(geo)
        M = literal.beam_global_matrix(a["x1"], a["x2"], a["young"], a["poisson"], a["area"], a["i11"], a["i22"],
                                       a["i12"], a["it"], a["shear_factor"], a["axis"], bk=BK)
        cases.append(dict(name=name, kind="beam", args=a, shape=[12, 12], matrix=mstr(M),
                          axis_aligned=name == "beam_x_axis"))
    # plates
    pbase = dict(young=70e9, poisson=0.3, thickness=0.02, shear_factor=5 / 6)
    for name, geo in [
        ("plate_unit_square", dict(x1=[1.0, 1.0, 0.0], x2=[0.0, 1.0, 0.0], x3=[0.0, 0.0, 0.0], x4=[1.0, 0.0, 0.0])),
        ("plate_distorted_flat", dict(x1=[0.12, 0.09, 0.0], x2=[-0.02, 0.11, 0.0], x3=[0.01, -0.015, 0.0],
                                      x4=[0.105, 0.003, 0.0])),
        ("plate_rectangle_xz", dict(x1=[2.0, 0.0, 1.0], x2=[0.0, 0.0, 1.0], x3=[0.0, 0.0, 0.0], x4=[2.0, 0.0, 0.0])),
        ("plate_tilted", dict(x1=[1.1, 0.9, 0.3], x2=[-0.8, 1.2, 0.5], x3=[-1.0, -1.0, -0.2],
                              x4=[0.9, -1.1, -0.4])),
    ]:
        a = dict(pbase)
        a.update(geo)
        if name == "plate_tilted":  # make node 1 lie exactly on the plane of nodes 2, 3, 4 in double arithmetic
            p2, p3, p4 = (np.array(a[k]) for k in ("x2", "x3", "x4"))
            a["x1"] = list(map(float, p2 + p4 - p3))
        M = literal.plate_global_matrix(a["x1"], a["x2"], a["x3"], a["x4"], a["young"], a["poisson"], a["thickness"],
                                        a["shear_factor"], bk=BK)
        cases.append(dict(name=name, kind="plate", args=a, shape=[24, 24], matrix=mstr(M),
                          axis_aligned=name in ("plate_unit_square", "plate_distorted_flat")))
    out = dict(generator="tests/golden/make_golden.py", precision_digits=50, cases=cases)
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "element_matrices.json"), "w") as f:
        json.dump(out, f, indent=0)


if __name__ == "__main__":
    main()
