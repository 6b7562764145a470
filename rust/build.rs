// Builds libribo_world.so with nvcc (sm_103a) through the library's own
// build script and links it.  RIBO_GB300_DIR names the checkout (default:
// the parent of this crate).
use std::env;
use std::path::PathBuf;
use std::process::Command;

fn main() {
    let root = env::var("RIBO_GB300_DIR")
        .map(PathBuf::from)
        .unwrap_or_else(|_| PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap()).join(".."));
    let script = root.join("ribossome-v2_gb300").join("build.py");
    let status = Command::new("python3").arg(&script).status().expect("running build.py (nvcc)");
    assert!(status.success(), "build.py failed");
    let lib_dir = root.join("ribossome-v2_gb300").join("_build");
    println!("cargo:rustc-link-search=native={}", lib_dir.display());
    println!("cargo:rustc-link-lib=dylib=ribo_world");
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", lib_dir.display());
    println!("cargo:rerun-if-changed={}", root.join("ribossome-v2_gb300").join("csrc").display());
    println!("cargo:rerun-if-changed={}", root.join("include").join("ribo_world.h").display());
}
