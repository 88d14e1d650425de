// build.rs for the reference crate's `gpu` feature (see src/gpu.rs): links
// libsdegpu.so, found in SDEGPU_LIB_DIR (the directory that
// `python -c "import __graft_entry__ as g; g.build()"` leaves it in,
// sde-sim-rs_gb300/sde_sim_rs/).  Not compiled in this repository (no cargo).
fn main() {
    if std::env::var_os("CARGO_FEATURE_GPU").is_none() {
        return;
    }
    println!("cargo:rerun-if-env-changed=SDEGPU_LIB_DIR");
    if let Some(dir) = std::env::var_os("SDEGPU_LIB_DIR") {
        let dir = dir.to_string_lossy().into_owned();
        println!("cargo:rustc-link-search=native={dir}");
        println!("cargo:rustc-link-arg=-Wl,-rpath,{dir}");
    }
    println!("cargo:rustc-link-lib=dylib=sdegpu");
}
