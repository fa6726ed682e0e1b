// Links the CUDA assembly library built by finite_element_method_gb300/build.py
// (libfem_gpu.so, CUDA runtime linked in statically).  FEM_GPU_LIB_DIR
// overrides where it is looked for; by default the in-tree build directory.
use std::env;
use std::path::PathBuf;

fn main() {
    let dir = match env::var("FEM_GPU_LIB_DIR") {
        Ok(d) => PathBuf::from(d),
        Err(_) => {
            let manifest = PathBuf::from(env::var("CARGO_MANIFEST_DIR").expect("cargo sets CARGO_MANIFEST_DIR"));
            manifest.join("..").join("finite_element_method_gb300").join("lib")
        }
    };
    println!("cargo:rustc-link-search=native={}", dir.display());
    println!("cargo:rustc-link-lib=dylib=fem_gpu");
    // the shared library is found next to the binary at run time through this rpath
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", dir.display());
    println!("cargo:rerun-if-env-changed=FEM_GPU_LIB_DIR");
    println!("cargo:rerun-if-changed=../include/fem_gpu.h");
}
