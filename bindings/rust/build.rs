//! Links the crate against libbendy2d_gb300.so, the shared library that
//! `python -c "import __graft_entry__ as g; g.build()"` produces in
//! `bendy2d_gb300/_build/`.  `BENDY2D_GB300_LIB_DIR` overrides the directory.
use std::env;
use std::path::PathBuf;

fn main() {
    let dir = match env::var("BENDY2D_GB300_LIB_DIR") {
        Ok(d) => PathBuf::from(d),
        Err(_) => {
            let manifest = PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap());
            manifest.join("../../bendy2d_gb300/_build")
        }
    };
    println!("cargo:rerun-if-env-changed=BENDY2D_GB300_LIB_DIR");
    println!("cargo:rustc-link-search=native={}", dir.display());
    println!("cargo:rustc-link-lib=dylib=bendy2d_gb300");
    // find the library at run time without LD_LIBRARY_PATH
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", dir.display());
}
