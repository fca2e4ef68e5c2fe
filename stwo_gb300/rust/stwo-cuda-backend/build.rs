// Links libstwo_gb300.so (built in-tree by `python -c "import __graft_entry__ as g; g.build()"`).
fn main() {
    let dir = std::env::var("STWO_GB300_LIB_DIR")
        .expect("set STWO_GB300_LIB_DIR to the directory of libstwo_gb300.so");
    println!("cargo:rustc-link-search=native={dir}");
    println!("cargo:rustc-link-lib=dylib=stwo_gb300");
    println!("cargo:rerun-if-env-changed=STWO_GB300_LIB_DIR");
}
