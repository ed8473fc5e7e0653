// Links libsigops.so.  SIGOPS_LIB_DIR names the directory that holds it
// (python wgpu-sigops_gb300/build_ext.py writes it into wgpu-sigops_gb300/);
// without it the crate's own parent directory is searched.
fn main() {
    let dir = std::env::var("SIGOPS_LIB_DIR").unwrap_or_else(|_| {
        let here = std::env::var("CARGO_MANIFEST_DIR").expect("cargo sets CARGO_MANIFEST_DIR");
        format!("{here}/..")
    });
    println!("cargo:rerun-if-env-changed=SIGOPS_LIB_DIR");
    println!("cargo:rustc-link-search=native={dir}");
    println!("cargo:rustc-link-lib=dylib=sigops");
    // the library's directory on the run-time search path of tests and binaries
    println!("cargo:rustc-link-arg=-Wl,-rpath,{dir}");
}
