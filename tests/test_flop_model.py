"""The bench's algorithmic FP64 work per plate (bench.PLATE_FLOPS, the roofline's numerator) against an
operation count of the device arithmetic itself: tests/flops/count_element_ops.cpp compiles
element_math.cuh on the host with a counting number type (adds, multiplications, divisions and square
roots one flop, a fused multiply-add two) and runs the plate's rotation and local coordinates, its
element core and its ten node-pair blocks, for a plate in a global plane (R = I) and one off the planes;
the beam's blocks (bench.BEAM_FLOPS) for the four section cases: I12 != 0 or I12 = 0, each with
I11 >= I22 or I11 < I22; and the truss block of an oblique bar (bench.WORK["truss"])."""
import os
import re
import shutil
import subprocess
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)


def counts(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "count_element_ops")
    subprocess.run([cxx, "-std=c++17", "-O1", "-o", exe, os.path.join(HERE, "flops", "count_element_ops.cpp")],
                   check=True, capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    res, case = {}, None
    for line in out.splitlines():
        m = re.match(r"(\w+) (identity|ok)=(\d)", line)
        if m:
            case = m.group(1)
            res[case] = {m.group(2): m.group(3) == "1"}
            continue
        m = re.match(r"\s+(\w+) add=(\d+) mul=(\d+) fma=(\d+) div=(\d+) sqrt=(\d+) flops=(\d+)", line)
        if m:
            res[case][m.group(1)] = dict(zip(("add", "mul", "fma", "div", "sqrt", "flops"), map(int, m.groups()[1:])))
            continue
        m = re.match(r"\s+total=(\d+)", line)
        if m:
            res[case]["total"] = int(m.group(1))
    return res


def test_plate_flop_model_matches_the_device_arithmetic(tmp_path):
    import bench

    c = counts(tmp_path)
    assert c["flat"]["identity"] and not c["tilted"]["identity"]
    assert c["flat"]["total"] == bench.PLATE_FLOPS["flat"] == 932
    assert c["tilted"]["total"] == bench.PLATE_FLOPS["tilted"] == 2480
    # the element core is the same on both paths; only the rotation and the blocks differ
    assert c["flat"]["core"] == c["tilted"]["core"]
    assert c["flat"]["core"]["flops"] == 583


def test_beam_flop_model_matches_the_device_arithmetic(tmp_path):
    import bench

    c = counts(tmp_path)
    for case in ("general", "general_turn", "aligned", "aligned_turn"):
        assert c["beam_" + case]["ok"]
        assert c["beam_" + case]["blocks"]["flops"] == bench.BEAM_FLOPS[case], case
    assert bench.WORK["beam"]["elem_flops"] == bench.BEAM_FLOPS["general"]


def test_truss_flop_model_matches_the_device_arithmetic(tmp_path):
    import bench

    c = counts(tmp_path)
    assert all(c["truss_" + k]["ok"] for k in ("general", "general_area2", "along_x"))
    assert c["truss_general"]["blocks"]["flops"] == bench.WORK["truss"]["elem_flops"] == 92
    # a second area adds its mean (one subtraction, one product, one addition); a bar along x has R = I
    assert c["truss_general_area2"]["blocks"]["flops"] == 95
    assert c["truss_along_x"]["blocks"]["flops"] == 69
