//! Builds libcoupe_gpu.so with nvcc (coupe_gb300/build.py, sm_103a) and links it.
use std::path::PathBuf;
use std::process::Command;

fn main() {
    let root = PathBuf::from(env!("CARGO_MANIFEST_DIR")).join("..").join("..");
    let status = Command::new("python3")
        .arg(root.join("coupe_gb300").join("build.py"))
        .status()
        .expect("python3 is needed to drive nvcc");
    assert!(status.success(), "building libcoupe_gpu.so failed");
    println!("cargo:rustc-link-search=native={}", root.join("coupe_gb300").display());
    println!("cargo:rustc-link-lib=dylib=coupe_gpu");
    println!("cargo:rerun-if-changed={}", root.join("coupe_gb300").join("csrc").display());
}
