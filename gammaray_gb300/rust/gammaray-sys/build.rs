// Links libgammaray_gpu.so.  GAMMARAY_GPU_DIR names the directory that holds it (the
// in-tree build writes gammaray_gb300/libgammaray_gpu.so); by default the directory two
// levels above this crate, which is gammaray_gb300/ in this repository.
use std::env;
use std::path::PathBuf;

fn main() {
    let dir = match env::var("GAMMARAY_GPU_DIR") {
        Ok(d) => PathBuf::from(d),
        Err(_) => {
            let manifest = PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap());
            manifest.join("..").join("..")
        }
    };
    println!("cargo:rustc-link-search=native={}", dir.display());
    println!("cargo:rustc-link-lib=dylib=gammaray_gpu");
    println!("cargo:rerun-if-env-changed=GAMMARAY_GPU_DIR");
}
