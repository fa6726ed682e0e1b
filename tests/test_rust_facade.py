"""CPU checks of the Rust facade under rust/ (no Rust toolchain in this image,
so the crate is checked as source): its raw `extern "C"` block is exactly what
rust/gen_ffi.py derives from include/fem_gpu.h, it binds every entry point, and
the `FEM` wrapper keeps the reference's method names and parameter lists."""
import os
import re
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RUST = os.path.join(ROOT, "rust")
sys.path.insert(0, RUST)

import gen_ffi  # noqa: E402


def _read(*p):
    with open(os.path.join(RUST, *p)) as f:
        return f.read()


def test_ffi_is_generated_from_header():
    assert _read("src", "ffi.rs") == gen_ffi.render(), "rust/src/ffi.rs is stale: run python rust/gen_ffi.py"


def test_ffi_binds_every_entry_point_with_its_arity():
    ffi = _read("src", "ffi.rs")
    decl = {m.group(1): m.group(2) for m in re.finditer(r"pub fn (fem_gpu_\w+)\((.*?)\) ->", ffi)}
    protos = {name: params for _, name, params in gen_ffi.prototypes()}
    assert set(decl) == set(protos)
    for name, params in protos.items():
        n_rust = 0 if not decl[name].strip() else decl[name].count(":")
        assert n_rust == len(params), name


def test_facade_calls_only_declared_entry_points():
    lib = _read("src", "lib.rs")
    used = set(re.findall(r"ffi::(fem_gpu_\w+)", lib))
    protos = {name for _, name, _ in gen_ffi.prototypes()}
    assert used and used <= protos, used - protos


# parameter lists of the reference's FEM methods (after &self / &mut self)
REFERENCE_METHODS = {
    # src/fem/fem.rs:34
    "create": ["rel_tol", "abs_tol", "nodes_number"],
    # src/fem/methods_for_node_data_handle.rs:66
    "add_node": ["number", "x", "y", "z"],
    # src/fem/methods_for_truss_data_handle.rs:49-57
    "add_truss": ["number", "node_1_number", "node_2_number", "young_modulus", "area", "optional_area_2"],
    # src/fem/methods_for_beam_data_handle.rs:49-63
    "add_beam": ["number", "node_1_number", "node_2_number", "young_modulus", "poisson_ratio", "area", "i11", "i22",
                 "i12", "it", "shear_factor", "local_axis_1_direction"],
    # src/fem/methods_for_plate_data_handle.rs:62-73
    "add_plate": ["number", "node_1_number", "node_2_number", "node_3_number", "node_4_number", "young_modulus",
                  "poisson_ratio", "thickness", "shear_factor"],
    # src/fem/fem.rs:171-202
    "get_truss_rotation_matrix_elements": ["number"],
    "get_beam_rotation_matrix_elements": ["number"],
    "get_plate_rotation_matrix_elements": ["number"],
}


def test_facade_keeps_reference_signatures():
    lib = _read("src", "lib.rs")
    for name, params in REFERENCE_METHODS.items():
        m = re.search(r"pub fn " + name + r"\s*\((.*?)\)\s*->\s*([^{]+)\{", lib, flags=re.S)
        assert m, name
        args = [a.strip() for a in m.group(1).split(",") if a.strip()]
        args = [a for a in args if not a.startswith("&")]
        assert [a.split(":")[0].strip() for a in args] == params, name
        ret = m.group(2).strip()
        if name == "create":
            assert ret == "Self"
        elif name.startswith("get_"):
            assert ret == "Result<[f64; 9], String>", name
        else:
            assert ret == "Result<(), String>", name


def test_crate_links_the_library():
    cargo = _read("Cargo.toml")
    assert 'links = "fem_gpu"' in cargo and 'build = "build.rs"' in cargo
    build = _read("build.rs")
    assert "rustc-link-lib=dylib=fem_gpu" in build
