//! Links libquantr_gpu.so. With QUANTR_GPU_LIB_DIR set, the library found there is used;
//! otherwise it is compiled in-tree by the repository's build script (nvcc for sm_103a, the same
//! translation units `python -m quantr_gb300.build` compiles) and linked from quantr_gb300/lib.
use std::env;
use std::path::PathBuf;
use std::process::Command;

fn main() {
    let manifest = PathBuf::from(env::var("CARGO_MANIFEST_DIR").expect("CARGO_MANIFEST_DIR"));
    let repo = manifest.join("..").join("..");
    let lib_dir = match env::var("QUANTR_GPU_LIB_DIR") {
        Ok(dir) => PathBuf::from(dir),
        Err(_) => {
            let python = env::var("PYTHON").unwrap_or_else(|_| String::from("python3"));
            let status = Command::new(python)
                .args(["-m", "quantr_gb300.build"])
                .current_dir(&repo)
                .status()
                .expect("could not run `python -m quantr_gb300.build` (nvcc is required)");
            assert!(status.success(), "building libquantr_gpu.so failed");
            repo.join("quantr_gb300").join("lib")
        }
    };
    println!("cargo:rustc-link-search=native={}", lib_dir.display());
    println!("cargo:rustc-link-lib=dylib=quantr_gpu");
    println!("cargo:rustc-link-arg=-Wl,-rpath,{}", lib_dir.display());
    println!("cargo:rerun-if-env-changed=QUANTR_GPU_LIB_DIR");
    println!("cargo:rerun-if-changed={}", repo.join("include").join("qgpu.h").display());
    println!("cargo:rerun-if-changed={}", repo.join("quantr_gb300").join("csrc").display());
}
