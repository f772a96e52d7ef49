// Links libbacon_gb300.so.  BACON_GB300_LIB_DIR names the folder that holds
// it (bacon_gb300/_lib after `python -m bacon_gb300.build_ext`).
fn main() {
    println!("cargo:rerun-if-env-changed=BACON_GB300_LIB_DIR");
    if let Ok(dir) = std::env::var("BACON_GB300_LIB_DIR") {
        println!("cargo:rustc-link-search=native={dir}");
    }
    println!("cargo:rustc-link-lib=dylib=bacon_gb300");
}
