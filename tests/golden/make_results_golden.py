"""Writes tests/golden/element_results.json: element results of the reference
formulas (oracle/literal.py: dense strain-displacement matrices summed over the
integration / corner points as structs/truss.rs:281-333, structs/beam.rs:803-993
and structs/plate.rs:1196-1409 write them) evaluated in 50-digit mpmath
arithmetic, for seeded displacement vectors, together with the magnitude scale
of each value (the same expression over absolute values).

The reference crate cannot be compiled in this environment (no Rust toolchain,
unvendored `extended_matrix`), so these high-precision evaluations of its
formulas pin the FP64 oracle's restated evaluation order.  Run:
    python tests/golden/make_results_golden.py
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import literal  # noqa: E402

BK = literal.Backend.mp(50)


def strs(v):
    return [str(x) if x != 0 else "0" for x in v]


def main():
    rng = np.random.default_rng(20261204)
    cases = []

    def disp(n, kind):
        if kind == "random":
            return [float(x) for x in rng.standard_normal(n) * 1e-3]
        return None

    # trusses: geometry, properties, displacement vectors (3 per node)
    for name, a in [
        ("truss_reference_test", dict(x1=[0.0, 0.0, 0.0], x2=[30.0, 0.0, 0.0], young=1e6, area=2.0)),
        ("truss_skew", dict(x1=[0.1, -0.3, 0.7], x2=[1.3, 0.4, -0.2], young=200e9, area=3.2e-4)),
        ("truss_tapered", dict(x1=[0.0, 0.0, 0.0], x2=[0.0, 2.5, 1.0], young=200e9, area=3e-4, area_2=1e-4)),
        ("truss_antiparallel", dict(x1=[2.0, 0.0, 0.0], x2=[-1.0, 0.0, 0.0], young=200e9, area=2e-4)),
    ]:
        us = [[0.0, 0.0, 0.0, 0.0015, 0.0, 0.0]] if name == "truss_reference_test" else []
        us += [disp(6, "random") for _ in range(2)]
        for k, u in enumerate(us):
            v, s = literal.truss_results(a["x1"], a["x2"], a["young"], a["area"], a.get("area_2"), u, bk=BK)
            cases.append(dict(name=f"{name}_{k}", kind="truss", args=a, u=u, values=strs(v), scale=strs(s)))
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
        for k in range(2):
            u = disp(12, "random")
            v, s = literal.beam_results(a["x1"], a["x2"], a["young"], a["poisson"], a["area"], a["i11"], a["i22"],
                                        a["i12"], a["it"], a["shear_factor"], a["axis"], u, bk=BK)
            cases.append(dict(name=f"{name}_{k}", kind="beam", args=a, u=u, values=strs(v), scale=strs(s)))
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
        if name == "plate_tilted":  # node 1 exactly on the plane of nodes 2, 3, 4 in double arithmetic
            p2, p3, p4 = (np.array(a[k]) for k in ("x2", "x3", "x4"))
            a["x1"] = list(map(float, p2 + p4 - p3))
        for k in range(2):
            u = disp(24, "random")
            v, s = literal.plate_results(a["x1"], a["x2"], a["x3"], a["x4"], a["young"], a["poisson"],
                                         a["thickness"], a["shear_factor"], u, bk=BK)
            cases.append(dict(name=f"{name}_{k}", kind="plate", args=a, u=u, values=strs(v), scale=strs(s)))
    out = dict(generator="tests/golden/make_results_golden.py", precision_digits=50, cases=cases)
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "element_results.json"), "w") as f:
        json.dump(out, f, indent=0)


if __name__ == "__main__":
    main()
