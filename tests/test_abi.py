"""CPU checks of the C ABI: the library builds for sm_103a, loads, and exports
every entry point include/*.h declares (no compute calls: no GPU here)."""
import ctypes
import glob
import os
import re

from finite_element_method_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(fem_gpu_\w+)\s*\(", src))
    return names


def test_library_exports_every_declared_symbol():
    lib = _lib.load()
    names = declared_symbols()
    assert len(names) >= 27
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    """every declared entry point has a ctypes signature (and no stale ones remain)."""
    assert set(_lib.SIGNATURES) == declared_symbols()



def test_no_gpu_call_surface_without_device():
    """creating a handle allocates nothing on the device and succeeds without a GPU."""
    lib = _lib.load()
    h = ctypes.c_void_p()
    assert lib.fem_gpu_create(1e-12, 1e-12, 4, ctypes.byref(h)) == 0
    assert lib.fem_gpu_destroy(h) == 0


def test_library_exports_nothing_undeclared():
    """the reverse direction: every fem_gpu_* symbol the library exports is declared in include/*.h"""
    import shutil
    import subprocess

    import pytest

    nm = shutil.which("nm")
    if nm is None:
        pytest.skip("nm not available")
    from finite_element_method_gb300 import build

    _lib.load()
    out = subprocess.run([nm, "-D", "--defined-only", build.LIB_PATH], capture_output=True, text=True,
                         check=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.split() and line.split()[-1].startswith("fem_gpu_")}
    assert exported == declared_symbols()


def test_structures_layout_matches_header():
    """the ctypes mirror of fem_gpu_structures_t lists the header's fields in the header's order"""
    import sys

    sys.path.insert(0, os.path.join(ROOT, "rust"))
    import gen_ffi

    (name, fields), = [s for s in gen_ffi.structs() if s[0] == "fem_gpu_structures_t"]
    assert [f for _, f in fields] == [f for f, _ in _lib.Structures._fields_]
    sizes = {"size_t": ctypes.sizeof(ctypes.c_size_t)}
    assert ctypes.sizeof(_lib.Structures) == sum(sizes.get(t, ctypes.sizeof(ctypes.c_void_p)) for t, _ in fields)


def test_python_binding_types_match_header():
    """every ctypes signature has the header's argument and return types: scalars exactly (a size_t bound
    as a 32-bit int would truncate), pointers as c_void_p or a pointer to the header's element type"""
    import sys
    from ctypes import (POINTER, c_char_p, c_double, c_float, c_int, c_int32, c_int64, c_size_t, c_uint8, c_uint32,
                        c_void_p)

    sys.path.insert(0, os.path.join(ROOT, "rust"))
    import gen_ffi

    scalar = {"double": c_double, "uint32_t": c_uint32, "size_t": c_size_t, "int": c_int, "int64_t": c_int64}
    elem = {"double": c_double, "float": c_float, "int64_t": c_int64, "int32_t": c_int32, "uint32_t": c_uint32,
            "uint8_t": c_uint8, "size_t": c_size_t, "int": c_int}

    def matches(decl, ct):
        t = decl.replace("const", "").replace(" ", "")
        base = t.rstrip("*")
        stars = len(t) - len(base)
        if stars == 0:
            return ct is scalar[base]
        if base == "char" and stars == 1:
            return ct is c_char_p
        if ct is c_void_p:
            return True
        if stars == 1:
            return base in elem and ct is POINTER(elem[base])
        return stars == 2 and ct is POINTER(c_void_p)

    protos = gen_ffi.prototypes()
    assert len(protos) == len(_lib.SIGNATURES)
    for ret, name, params in protos:
        res, args = _lib.SIGNATURES[name]
        assert matches(ret, res), (name, ret, res)
        assert len(args) == len(params), name
        for (decl, pname), ct in zip(params, args):
            assert matches(decl, ct), (name, pname, decl, ct)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    """without the CUDA library there is no fallback: loading it raises"""
    import pytest

    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib._build, "LIB_PATH", str(tmp_path / "libfem_gpu.so"))
    with pytest.raises(RuntimeError, match="CUDA assembly library not found"):
        _lib.load(build_if_missing=False)


def test_product_never_imports_the_oracle():
    """the package's Python modules import nothing from oracle/ (the oracle is the checker, never the path),
    and its CUDA/C++ sources include nothing from there"""
    import ast

    pkg = os.path.join(ROOT, "finite_element_method_gb300")
    for path in glob.glob(os.path.join(pkg, "**", "*.py"), recursive=True):
        tree = ast.parse(open(path).read(), path)
        for node in ast.walk(tree):
            if isinstance(node, ast.Import):
                names = [a.name for a in node.names]
            elif isinstance(node, ast.ImportFrom):
                names = [node.module or ""]
            else:
                continue
            assert not any(n == "oracle" or n.startswith("oracle.") for n in names), (path, names)
    for path in glob.glob(os.path.join(pkg, "csrc", "*")):
        assert "oracle" not in "".join(re.findall(r'#include\s*[<"][^>"]*[>"]', open(path).read())), path
