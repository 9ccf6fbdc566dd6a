// Links libmczi_gpu.so.  The library is built by `python -m mczi_gb300.build`
// into mczi_gb300/lib/; MCZI_GPU_LIB_DIR overrides the search directory.
use std::env;
use std::path::PathBuf;

fn main() {
    let dir = env::var("MCZI_GPU_LIB_DIR").map(PathBuf::from).unwrap_or_else(|_| {
        PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap()).join("../../mczi_gb300/lib")
    });
    println!("cargo:rerun-if-env-changed=MCZI_GPU_LIB_DIR");
    println!("cargo:rustc-link-search=native={}", dir.display());
    println!("cargo:rustc-link-lib=dylib=mczi_gpu");
    // the CUDA runtime the library was linked against
    if let Ok(cuda) = env::var("CUDA_HOME") {
        println!("cargo:rustc-link-search=native={}/lib64", cuda);
    }
}
