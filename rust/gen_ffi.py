"""Writes rust/src/ffi.rs: the `extern "C"` declarations of every entry point in
include/fem_gpu.h, with each C parameter type mapped to its Rust FFI type.

Run `python rust/gen_ffi.py` after changing the header; tests/test_rust_facade.py
checks that the committed ffi.rs is what this script produces."""
from __future__ import annotations

import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
HEADER = os.path.join(os.path.dirname(HERE), "include", "fem_gpu.h")
OUT = os.path.join(HERE, "src", "ffi.rs")

TYPES = {
    "double": "f64",
    "float*": "*mut f32",
    "int": "c_int",
    "int*": "*mut c_int",
    "size_t": "usize",
    "size_t*": "*mut usize",
    "const size_t*": "*const usize",
    "uint32_t": "u32",
    "uint32_t*": "*mut u32",
    "const uint32_t*": "*const u32",
    "int32_t*": "*mut i32",
    "const int32_t*": "*const i32",
    "const int32_t**": "*mut *const i32",
    "int64_t": "i64",
    "int64_t*": "*mut i64",
    "const int64_t**": "*mut *const i64",
    "uint8_t*": "*mut u8",
    "const uint8_t*": "*const u8",
    "double*": "*mut f64",
    "const double*": "*const f64",
    "const double**": "*mut *const f64",
    "char*": "*mut c_char",
    "const char*": "*const c_char",
    "void*": "*mut c_void",
    "void**": "*mut *mut c_void",
    "fem_gpu_t*": "*mut FemGpu",
    "const fem_gpu_t*": "*const FemGpu",
    "fem_gpu_t**": "*mut *mut FemGpu",
    "fem_gpu_t* const*": "*const *mut FemGpu",
    "fem_gpu_batch_t*": "*mut FemGpuBatch",
    "const fem_gpu_batch_t*": "*const FemGpuBatch",
    "fem_gpu_batch_t**": "*mut *mut FemGpuBatch",
    "const fem_gpu_structures_t*": "*const FemGpuStructures",
}
RETURNS = {"int": "c_int", "const char*": "*const c_char"}
KEYWORDS = {"type", "ref", "move", "fn", "in", "match", "loop", "use", "mod", "box"}


def prototypes(path: str = HEADER):
    """[(return C type, name, [(C type, parameter name)])] in header order."""
    src = re.sub(r"/\*.*?\*/", "", open(path).read(), flags=re.S)
    out = []
    for ret, name, args in re.findall(r"(int|const char\s*\*)\s*(fem_gpu_\w+)\s*\(([^;]*?)\)\s*;", src, flags=re.S):
        params = []
        for a in args.split(","):
            a = " ".join(a.split())
            if not a or a == "void":
                continue
            m = re.match(r"(.*?)\s*(\w+)$", a)
            params.append((m.group(1).strip().replace(" *", "*"), m.group(2)))
        out.append((" ".join(ret.replace("*", " *").split()).replace(" *", "*"), name, params))
    return out


def structs(path: str = HEADER):
    """[(C typedef name, [(C type, field name)])] of the header's plain-data structs."""
    src = re.sub(r"/\*.*?\*/", "", open(path).read(), flags=re.S)
    out = []
    for body, name in re.findall(r"typedef struct \w+ \{(.*?)\}\s*(\w+)\s*;", src, flags=re.S):
        fields = []
        for decl in body.split(";"):
            decl = " ".join(decl.split())
            if not decl:
                continue
            m = re.match(r"(.*?)\s*(\w+)$", decl)
            fields.append((m.group(1).strip().replace(" *", "*"), m.group(2)))
        out.append((name, fields))
    return out


RUST_STRUCT = {"fem_gpu_structures_t": "FemGpuStructures"}


def render(path: str = HEADER) -> str:
    lines = [
        "// ffi.rs -- raw declarations of the C ABI in include/fem_gpu.h (libfem_gpu.so).",
        "// Generated by rust/gen_ffi.py from the header; do not edit by hand.",
        "#![allow(non_camel_case_types, dead_code)]",
        "",
        "use std::os::raw::{c_char, c_int, c_void};",
        "",
        "/// The library's model handle (`fem_gpu_t`): opaque, owned through `FEM`.",
        "#[repr(C)]",
        "pub struct FemGpu {",
        "    _opaque: [u8; 0],",
        "}",
        "",
        "/// A batch of structures (`fem_gpu_batch_t`): opaque.",
        "#[repr(C)]",
        "pub struct FemGpuBatch {",
        "    _opaque: [u8; 0],",
        "}",
        "",
    ]
    for cname, fields in structs(path):
        lines.append(f"/// `{cname}`: plain data, laid out as the C struct.")
        lines.append("#[repr(C)]")
        lines.append(f"pub struct {RUST_STRUCT[cname]} {{")
        for ctype, fname in fields:
            if ctype not in TYPES:
                raise KeyError(f"{cname}.{fname}: no Rust type for C type {ctype!r}")
            lines.append(f"    pub {fname}: {TYPES[ctype]},")
        lines.append("}")
        lines.append("")
    lines += [
        'unsafe extern "C" {',
    ]
    for ret, name, params in prototypes(path):
        ps = []
        for ctype, pname in params:
            if ctype not in TYPES:
                raise KeyError(f"{name}: no Rust type for C type {ctype!r}")
            if pname in KEYWORDS:
                pname += "_"
            ps.append(f"{pname}: {TYPES[ctype]}")
        lines.append(f"    pub fn {name}({', '.join(ps)}) -> {RETURNS[ret]};")
    lines.append("}")
    lines.append("")
    return "\n".join(lines)


if __name__ == "__main__":
    with open(OUT, "w") as f:
        f.write(render())
    print(OUT)
