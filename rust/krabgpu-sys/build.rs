// Links the prebuilt libkrabgpu.so (sm_103a kernels + C ABI host runtime).
// KRABGPU_DIR names the folder that holds it (`make -C krabmaga_gb300` builds
// it in place); without it the library is looked for beside this crate.
use std::env;
use std::path::PathBuf;

fn main() {
    let dir = match env::var("KRABGPU_DIR") {
        Ok(d) => PathBuf::from(d),
        Err(_) => PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap())
            .join("..")
            .join("..")
            .join("krabmaga_gb300"),
    };
    if !dir.join("libkrabgpu.so").exists() {
        panic!("libkrabgpu.so not found in {}: build it (make -C krabmaga_gb300) or set KRABGPU_DIR",
               dir.display());
    }
    println!("cargo:rustc-link-search=native={}", dir.display());
    println!("cargo:rustc-link-lib=dylib=krabgpu");
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", dir.display());
    println!("cargo:rerun-if-env-changed=KRABGPU_DIR");
    println!("cargo:rerun-if-changed=../../include/krabgpu.h");
}
