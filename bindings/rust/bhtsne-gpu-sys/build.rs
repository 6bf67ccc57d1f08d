// Links libbhtsne_gpu.so. BHTSNE_GPU_LIB_DIR names the directory that holds it
// (the package directory bhtsne_gb300/ after `python bhtsne_gb300/build.py`);
// the CUDA runtime comes from CUDA_HOME (default /usr/local/cuda).
use std::env;

fn main() {
    println!("cargo:rerun-if-env-changed=BHTSNE_GPU_LIB_DIR");
    println!("cargo:rerun-if-env-changed=CUDA_HOME");
    if let Ok(dir) = env::var("BHTSNE_GPU_LIB_DIR") {
        println!("cargo:rustc-link-search=native={dir}");
        println!("cargo:rustc-link-arg=-Wl,-rpath,{dir}");
    }
    let cuda = env::var("CUDA_HOME").unwrap_or_else(|_| "/usr/local/cuda".to_string());
    for sub in ["lib64", "lib", "targets/sbsa-linux/lib", "targets/x86_64-linux/lib"] {
        println!("cargo:rustc-link-search=native={cuda}/{sub}");
    }
    println!("cargo:rustc-link-lib=dylib=bhtsne_gpu");
    println!("cargo:rustc-link-lib=dylib=cudart");
}
