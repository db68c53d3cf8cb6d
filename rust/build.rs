//! Compiles the CUDA pipeline (../rusterizer_gb300/csrc) for sm_103a with nvcc into a static
//! library and links it with the static CUDA runtime. The flags match rusterizer_gb300/build.py:
//! bit-exact parity with the reference needs --fmad=false, IEEE division and square root, and
//! -ffp-contract=off for host code.
use std::env;
use std::path::PathBuf;
use std::process::Command;

const SOURCES: &[&str] = &[
    "rast_kernels.cu",
    "rast_api.cu",
    "rast_noalloc.cu",
    "rast_batch.cu",
    "rast_server.cu",
];

fn main() {
    let root = PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap()).join("..");
    let csrc = root.join("rusterizer_gb300").join("csrc");
    let include = root.join("include");
    let out = PathBuf::from(env::var("OUT_DIR").unwrap());
    let cuda = env::var("CUDA_HOME").unwrap_or_else(|_| "/usr/local/cuda".to_string());
    let nvcc = PathBuf::from(&cuda).join("bin").join("nvcc");

    let mut objs = Vec::new();
    for src in SOURCES {
        let obj = out.join(src.replace(".cu", ".o"));
        let status = Command::new(&nvcc)
            .args(["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-std=c++17"])
            .args(["--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"])
            .args(["-Xcompiler", "-fPIC,-ffp-contract=off"])
            .arg(format!("-I{}", include.display()))
            .arg("-c")
            .arg(csrc.join(src))
            .arg("-o")
            .arg(&obj)
            .status()
            .expect("failed to run nvcc");
        assert!(status.success(), "nvcc failed on {src}");
        objs.push(obj);
        println!("cargo:rerun-if-changed={}", csrc.join(src).display());
    }
    for h in ["rast_device.cuh", "rast_types.h", "rast_kernels.h", "rast_internal.h"] {
        println!("cargo:rerun-if-changed={}", csrc.join(h).display());
    }
    println!("cargo:rerun-if-changed={}", include.join("rast.h").display());

    // device code is relocatable-free (whole-program per file), so `nvcc -lib` is enough
    let lib = out.join("librast_gb300.a");
    let status = Command::new(&nvcc)
        .args(["-gencode", "arch=compute_103a,code=sm_103a", "-lib", "-o"])
        .arg(&lib)
        .args(&objs)
        .status()
        .expect("failed to run nvcc -lib");
    assert!(status.success(), "nvcc -lib failed");

    println!("cargo:rustc-link-search=native={}", out.display());
    println!("cargo:rustc-link-lib=static=rast_gb300");
    println!("cargo:rustc-link-search=native={}/lib64", cuda);
    println!("cargo:rustc-link-search=native={}/targets/sbsa-linux/lib", cuda);
    println!("cargo:rustc-link-search=native={}/targets/x86_64-linux/lib", cuda);
    println!("cargo:rustc-link-lib=static=cudart_static");
    for l in ["stdc++", "dl", "rt", "pthread"] {
        println!("cargo:rustc-link-lib=dylib={l}");
    }
}
