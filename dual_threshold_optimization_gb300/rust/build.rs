//! Compiles libdto (the CUDA kernels and the C ABI of include/dto.h) for
//! sm_103a with nvcc into a static archive and links it with the CUDA
//! runtime.  The sources are the package's csrc/ directory next to this
//! crate; NVCC (or CUDA_HOME/bin/nvcc, else /usr/local/cuda/bin/nvcc) is the
//! compiler.
use std::env;
use std::fs;
use std::path::{Path, PathBuf};
use std::process::Command;

fn nvcc() -> PathBuf {
    if let Ok(p) = env::var("NVCC") {
        return PathBuf::from(p);
    }
    if let Ok(h) = env::var("CUDA_HOME") {
        return Path::new(&h).join("bin").join("nvcc");
    }
    PathBuf::from("/usr/local/cuda/bin/nvcc")
}

fn main() {
    let crate_dir = PathBuf::from(env::var("CARGO_MANIFEST_DIR").unwrap());
    let pkg = crate_dir.parent().expect("crate inside the package").to_path_buf();
    let csrc = pkg.join("csrc");
    let include = pkg.parent().expect("package inside the repository").join("include");
    let out = PathBuf::from(env::var("OUT_DIR").unwrap());
    let nvcc = nvcc();
    println!("cargo:rerun-if-changed={}", csrc.display());
    println!("cargo:rerun-if-changed={}", include.join("dto.h").display());
    println!("cargo:rerun-if-env-changed=NVCC");
    println!("cargo:rerun-if-env-changed=CUDA_HOME");

    let mut sources: Vec<PathBuf> = fs::read_dir(&csrc)
        .expect("csrc directory")
        .filter_map(|e| e.ok().map(|e| e.path()))
        .filter(|p| matches!(p.extension().and_then(|e| e.to_str()), Some("cu") | Some("cpp")))
        .collect();
    sources.sort();
    let mut objects = Vec::new();
    for src in &sources {
        let obj = out.join(format!("{}.o", src.file_name().unwrap().to_string_lossy()));
        let status = Command::new(&nvcc)
            .args(["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "-std=c++17"])
            .args(["-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"])
            .arg("-I")
            .arg(&include)
            .arg("-I")
            .arg(&csrc)
            .arg("-c")
            .arg(src)
            .arg("-o")
            .arg(&obj)
            .status()
            .expect("running nvcc");
        assert!(status.success(), "nvcc failed on {}", src.display());
        objects.push(obj);
    }
    // device code is whole-program per translation unit (no -rdc), so a
    // plain archive of the objects links like any host library
    let lib = out.join("libdto.a");
    let status = Command::new(&nvcc)
        .args(["-gencode", "arch=compute_103a,code=sm_103a", "-lib", "-o"])
        .arg(&lib)
        .args(&objects)
        .status()
        .expect("running nvcc -lib");
    assert!(status.success(), "nvcc -lib failed");

    let cuda_lib = nvcc
        .parent()
        .and_then(|b| b.parent())
        .map(|h| h.join("lib64"))
        .unwrap_or_else(|| PathBuf::from("/usr/local/cuda/lib64"));
    println!("cargo:rustc-link-search=native={}", out.display());
    println!("cargo:rustc-link-search=native={}", cuda_lib.display());
    println!("cargo:rustc-link-lib=static=dto");
    println!("cargo:rustc-link-lib=dylib=cudart");
    println!("cargo:rustc-link-lib=dylib=stdc++");
    println!("cargo:rustc-link-lib=dylib=pthread");
}
