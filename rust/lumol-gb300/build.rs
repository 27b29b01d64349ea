//! Builds the engine's CUDA sources for sm_103a with nvcc and links the
//! resulting shared library, as `lumol_gb300/build.py` does for the Python
//! package: every translation unit of `lumol_gb300/csrc` compiled with
//! `-gencode arch=compute_103a,code=sm_103a`, linked with cudart.
use std::env;
use std::path::PathBuf;
use std::process::Command;

const SOURCES: &[&str] = &[
    "nlist.cu", "forces.cu", "mixed.cu", "persist.cu", "md.cu", "diag.cu", "mc.cu", "noalloc.cu", "lower.cu",
    "runtime.cu", "capi.cu", "capi_mc.cu",
];

fn main() {
    let manifest = PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap());
    let csrc = manifest.join("../../lumol_gb300/csrc");
    let out = PathBuf::from(env::var("OUT_DIR").unwrap());
    let nvcc = env::var("NVCC").unwrap_or_else(|_| "nvcc".into());
    let mut objects = Vec::new();
    for src in SOURCES {
        let path = csrc.join(src);
        println!("cargo:rerun-if-changed={}", path.display());
        let obj = out.join(src.replace(".cu", ".o"));
        let status = Command::new(&nvcc)
            .args(["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17"])
            .args(["-Xcompiler", "-fPIC,-ffp-contract=off", "-c"])
            .arg(&path)
            .arg("-o")
            .arg(&obj)
            .status()
            .expect("nvcc must be on PATH (or NVCC set) to build the engine");
        assert!(status.success(), "nvcc failed on {}", src);
        objects.push(obj);
    }
    let lib = out.join("liblumol_gb300.so");
    let status = Command::new(&nvcc)
        .arg("-shared")
        .arg("-o")
        .arg(&lib)
        .args(&objects)
        .arg("-lcudart")
        .status()
        .expect("nvcc link");
    assert!(status.success(), "linking liblumol_gb300.so failed");
    println!("cargo:rerun-if-changed={}", manifest.join("../../include/lumol_gb300.h").display());
    println!("cargo:rustc-link-search=native={}", out.display());
    println!("cargo:rustc-link-lib=dylib=lumol_gb300");
}
