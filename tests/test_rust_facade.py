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
    # src/fem/fem.rs:154
    "reset": ["nodes_number"],
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
    # src/fem/methods_for_bc_data_handle.rs:34-39, 58-63, 103-108, 176-181
    "add_concentrated_load": ["node_number", "dof_parameter", "value"],
    "add_uniformly_distributed_line_load": ["beam_element_number", "dof_parameter", "value"],
    "add_uniformly_distributed_surface_load": ["plate_element_number", "dof_parameter", "value"],
    "add_displacement": ["node_number", "dof_parameter", "value"],
    # src/fem/methods_for_separate_stiffness_matrix.rs:217-219, 322, 333
    "separate_stiffness_matrix_sparse_iterative": [],
    "compose_r_a_vector": ["k_aa_indexes"],
    "compose_u_b_vector": ["k_bb_indexes"],
    # src/fem/methods_for_global_analysis.rs:189-195, 235-241, 306-311, 335-341, 361
    "find_ua_vector_iterative_pcg_jacobi_sparse": ["separated_stiffness_matrix_sparse", "r_a_vector", "u_b_vector",
                                                   "max_iter"],
    "find_ua_vector_iterative_pcg_block_jacobi_sparse": ["separated_stiffness_matrix_sparse", "r_a_vector",
                                                         "u_b_vector", "max_iter"],
    "find_r_r_vector_sparse": ["sep", "u_a_vector", "u_b_vector"],
    "compose_global_analysis_result": ["k_aa_indexes", "k_bb_indexes", "u_a_vector", "r_r_vector"],
    "extract_global_analysis_result": [],
    # src/fem/methods_for_element_analysis.rs:27-29
    "extract_elements_analysis_result": [],
}

# return types other than Result<(), String> (the crate's Vector<V> is a Vec<f64> here)
REFERENCE_RETURNS = {
    "create": "Self",
    "reset": None,
    "get_truss_rotation_matrix_elements": "Result<[f64; 9], String>",
    "get_beam_rotation_matrix_elements": "Result<[f64; 9], String>",
    "get_plate_rotation_matrix_elements": "Result<[f64; 9], String>",
    "separate_stiffness_matrix_sparse_iterative": "Result<SeparatedStiffnessMatrixSparse, String>",
    "compose_r_a_vector": "Result<Vec<f64>, String>",
    "compose_u_b_vector": "Result<Vec<f64>, String>",
    "find_ua_vector_iterative_pcg_jacobi_sparse": "Result<(Vec<f64>, usize), String>",
    "find_ua_vector_iterative_pcg_block_jacobi_sparse": "Result<(Vec<f64>, usize), String>",
    "find_r_r_vector_sparse": "Result<Vec<f64>, String>",
    "extract_global_analysis_result": "Result<Vec<(u32, DOFParameter, f64, f64)>, String>",
    "extract_elements_analysis_result": "Result<Vec<(u32, Vec<(ElementForceComponent, f64)>)>, String>",
}


def test_facade_keeps_reference_signatures():
    lib = _read("src", "lib.rs")
    for name, params in REFERENCE_METHODS.items():
        m = re.search(r"pub fn " + name + r"\s*\((.*?)\)\s*(?:->\s*([^{]+))?\{", lib, flags=re.S)
        assert m, name
        args = [a.strip() for a in m.group(1).split(",") if a.strip()]
        args = [a for a in args if not a.startswith("&")]
        assert [a.split(":")[0].strip() for a in args] == params, name
        ret = " ".join(m.group(2).split()) if m.group(2) else None
        assert ret == REFERENCE_RETURNS.get(name, "Result<(), String>"), name


def test_facade_keeps_reference_enums():
    """DOFParameter and ElementForceComponent with the crate's variants (DOFParameter in DOF order)"""
    lib = _read("src", "lib.rs")
    for enum, variants in (("DOFParameter", ["X = 0", "Y = 1", "Z = 2", "ThX = 3", "ThY = 4", "ThZ = 5"]),
                           ("ElementForceComponent", ["ForceR", "ForceS", "ForceT", "MembraneForceR",
                                                      "MembraneForceS", "MembraneForceRS", "ShearForceRT",
                                                      "ShearForceST", "MomentR", "MomentS", "MomentT",
                                                      "BendingMomentR", "BendingMomentS", "BendingMomentRS"])):
        m = re.search(r"pub enum " + enum + r"\s*\{(.*?)\}", lib, flags=re.S)
        assert m, enum
        assert [v.strip() for v in m.group(1).split(",") if v.strip()] == variants, enum


def test_crate_links_the_library():
    cargo = _read("Cargo.toml")
    assert 'links = "fem_gpu"' in cargo and 'build = "build.rs"' in cargo
    build = _read("build.rs")
    assert "rustc-link-lib=dylib=fem_gpu" in build


def test_integration_tests_call_only_facade_methods():
    """rust/tests/*.rs (the crate's own integration tests through the facade) call methods that lib.rs
    defines, with the reference's enums"""
    lib = _read("src", "lib.rs")
    defined = set(re.findall(r"pub fn (\w+)", lib))
    tests_dir = os.path.join(RUST, "tests")
    files = sorted(f for f in os.listdir(tests_dir) if f.endswith(".rs"))
    assert files
    for f in files:
        src = _read("tests", f)
        called = set(re.findall(r"\b(?:model|sep|rec|batch)\.(\w+)\(", src)) | \
            set(re.findall(r"\b(?:FEM|Batch|Structures)::(\w+)\(", src))
        assert called and called <= defined, (f, called - defined)
        for enum in set(re.findall(r"\b(DOFParameter|ElementForceComponent)::(\w+)", src)):
            assert re.search(r"pub enum " + enum[0] + r"\s*\{[^}]*\b" + enum[1] + r"\b", lib) or \
                enum[1] in defined, enum


def test_integration_notes_declare_entry_points_as_the_header():
    """the Rust declarations shown in INTEGRATION.md (the binding a maintainer would add to the reference
    crate) name real entry points with the header's parameter and return types, in order"""
    def decls(text):
        out = {}
        for m in re.finditer(r"fn (fem_gpu_\w+)\((.*?)\)\s*->\s*([^;]+);", text, flags=re.S):
            types = [p.split(":", 1)[1].strip() for p in m.group(2).split(",") if p.strip()]
            out[m.group(1)] = (types, " ".join(m.group(3).split()))
        return out

    with open(os.path.join(ROOT, "INTEGRATION.md")) as f:
        shown = decls(f.read())
    ffi = decls(_read("src", "ffi.rs"))
    assert len(shown) >= 20
    for name, sig in shown.items():
        assert name in ffi, name
        assert sig == ffi[name], (name, sig, ffi[name])


def test_structures_builder_fills_every_field():
    """Structures::layout sets every field of the generated fem_gpu_structures_t, in its order"""
    ffi = _read("src", "ffi.rs")
    fields = re.findall(r"pub (\w+): ", re.search(r"pub struct FemGpuStructures \{(.*?)\}", ffi, re.S).group(1))
    lib = _read("src", "lib.rs")
    init = re.search(r"^\s*ffi::FemGpuStructures \{\n(.*?)\n\s*\}", lib, re.S | re.M).group(1)
    assert re.findall(r"^\s*(\w+):", init, re.M) == fields
