// Links libsoftrender_gb300.so, built in place by
// `python rust-softrender_gb300/build.py` (nvcc, sm_103a).  SOFTRENDER_GB300_LIB
// overrides the directory that holds it.
use std::env;
use std::path::PathBuf;

fn main() {
    let dir = env::var("SOFTRENDER_GB300_LIB").map(PathBuf::from).unwrap_or_else(|_| {
        PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap())
            .join("../../rust-softrender_gb300/lib")
    });
    println!("cargo:rustc-link-search=native={}", dir.display());
    println!("cargo:rustc-link-lib=dylib=softrender_gb300");
    println!("cargo:rerun-if-env-changed=SOFTRENDER_GB300_LIB");
}
