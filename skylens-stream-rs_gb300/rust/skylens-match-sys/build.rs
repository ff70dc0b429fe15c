// Links libslm.so. SLM_LIB_DIR points at the directory holding it
// (skylens-stream-rs_gb300/build after `python -c "import __graft_entry__ as g; g.build()"`).
fn main() {
    let dir = std::env::var("SLM_LIB_DIR").unwrap_or_else(|_| "../../build".to_string());
    println!("cargo:rustc-link-search=native={dir}");
    println!("cargo:rustc-link-lib=dylib=slm");
    println!("cargo:rerun-if-env-changed=SLM_LIB_DIR");
}
