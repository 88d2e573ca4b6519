//! Builds libnalgebra_cuda.so from the CUDA sources beside this crate
//! (../nalgebra_gb300/csrc, nvcc for sm_103a, the CUDA runtime linked
//! statically) into OUT_DIR and links it, unless NALGEBRA_CUDA_LIB_DIR names a
//! directory that already holds the library (the one `python -m
//! nalgebra_gb300.build` writes, for instance).
use std::env;
use std::path::PathBuf;
use std::process::Command;

fn main() {
    println!("cargo:rerun-if-env-changed=NALGEBRA_CUDA_LIB_DIR");
    if let Ok(dir) = env::var("NALGEBRA_CUDA_LIB_DIR") {
        println!("cargo:rustc-link-search=native={dir}");
        println!("cargo:rustc-link-lib=dylib=nalgebra_cuda");
        return;
    }
    let manifest = PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap());
    let root = manifest.parent().unwrap().to_path_buf();
    let csrc = root.join("nalgebra_gb300").join("csrc");
    let include = root.join("include");
    let out = PathBuf::from(env::var("OUT_DIR").unwrap());
    let nvcc = env::var("NVCC").unwrap_or_else(|_| "nvcc".to_string());
    let mut objs = Vec::new();
    let mut sources: Vec<PathBuf> = std::fs::read_dir(&csrc)
        .expect("CUDA sources")
        .filter_map(|e| e.ok().map(|e| e.path()))
        .filter(|p| p.extension().map_or(false, |x| x == "cu"))
        .collect();
    sources.sort();
    for src in &sources {
        println!("cargo:rerun-if-changed={}", src.display());
        let obj = out.join(src.file_stem().unwrap()).with_extension("o");
        let status = Command::new(&nvcc)
            .args(["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-DNACU_ARCH=103"])
            .arg(format!("-I{}", include.display()))
            .arg("-c").arg(src).arg("-o").arg(&obj)
            .status()
            .expect("nvcc (the CUDA toolkit) is required to build nalgebra-cuda");
        assert!(status.success(), "nvcc failed for {}", src.display());
        objs.push(obj);
    }
    let lib = out.join("libnalgebra_cuda.so");
    let status = Command::new(&nvcc)
        .args(["-gencode", "arch=compute_103a,code=sm_103a", "-shared", "-cudart", "static", "-o"])
        .arg(&lib)
        .args(&objs)
        .status()
        .expect("nvcc link");
    assert!(status.success(), "nvcc link failed");
    println!("cargo:rustc-link-search=native={}", out.display());
    println!("cargo:rustc-link-lib=dylib=nalgebra_cuda");
}
