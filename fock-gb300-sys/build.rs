//! Links libfock_gb300.so, built by `python fock-rs_gb300/build.py`.
//! FOCK_GB300_LIB_DIR names the directory that holds it (default: the
//! in-tree build output next to this crate); the CUDA runtime libraries it
//! depends on are found through its own run path.
use std::env;
use std::path::PathBuf;

fn main() {
    let dir = env::var("FOCK_GB300_LIB_DIR").map(PathBuf::from).unwrap_or_else(|_| {
        PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap())
            .join("..")
            .join("fock-rs_gb300")
            .join("lib")
    });
    println!("cargo:rustc-link-search=native={}", dir.display());
    println!("cargo:rustc-link-lib=dylib=fock_gb300");
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", dir.display());
    println!("cargo:rerun-if-env-changed=FOCK_GB300_LIB_DIR");
}
