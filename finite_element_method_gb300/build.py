"""In-tree build of the CUDA assembly library (libfem_gpu.so) for sm_103a.

The library is plain C ABI (include/fem_gpu.h) compiled with nvcc; nothing
here depends on PyTorch.  `--fmad=false` is part of the arithmetic contract:
the kernels contain explicit fma() calls only, so every product and sum is
rounded exactly where the source says.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB_DIR = os.path.join(HERE, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libfem_gpu.so")
# the same library with the device-side index checks of the assembly path (-DFEM_GPU_DEBUG)
DEBUG_LIB_PATH = os.path.join(LIB_DIR, "libfem_gpu_debug.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "--fmad=false", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "-diag-suppress", "550"]

SOURCES = ["fem_gpu.cu", "fem_noalloc.cu"]  # the .cuh parts (batch, adjoint, loads, separation, solve, results) are included by fem_gpu.cu


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA assembly library cannot be built")


def _sources():
    return [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]


def _stale(path: str) -> bool:
    if not os.path.exists(path):
        return True
    t = os.path.getmtime(path)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return any(os.path.getmtime(d) > t for d in deps)


VARIANTS = {LIB_PATH: ("obj", []), DEBUG_LIB_PATH: ("obj_debug", ["-DFEM_GPU_DEBUG"])}


def _extra_flags():
    """tuning flags from the environment (for instance FEM_GPU_NVCC_EXTRA="-DFEM_PLATE_MAXNREG=168
    -DFEM_PLATE_BLOCK=128"); rebuild with force=True after changing them"""
    return os.environ.get("FEM_GPU_NVCC_EXTRA", "").split()


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile every translation unit of both libraries (release and index-checked) in parallel and link
    libfem_gpu.so and libfem_gpu_debug.so; returns the release library's path."""
    todo = [path for path in VARIANTS if force or _stale(path)]
    if not todo:
        return LIB_PATH
    nvcc = _nvcc()
    procs, objs = [], {}
    for path in todo:
        sub, extra = VARIANTS[path]
        obj_dir = os.path.join(LIB_DIR, sub)
        os.makedirs(obj_dir, exist_ok=True)
        objs[path] = []
        for src in _sources():
            obj = os.path.join(obj_dir, os.path.splitext(src)[0] + ".o")
            objs[path].append(obj)
            cmd = [nvcc, *ARCH, *NVCC_FLAGS, *extra, *_extra_flags(), "-I", INCLUDE, "-c", os.path.join(CSRC, src),
                   "-o", obj]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
            procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append(f"{src}:\n{out.decode(errors='replace')}")
        elif verbose:
            print(out.decode(errors="replace"))
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(failed))
    for path in todo:
        tmp = path + ".tmp"
        subprocess.run([nvcc, *ARCH, "-shared", "-o", tmp, *objs[path]], check=True, capture_output=True)
        os.replace(tmp, path)
    return LIB_PATH


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
