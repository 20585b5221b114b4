fn main() {
    if let Ok(dir) = std::env::var("FUZZYBLUE_CUDA_LIB_DIR") {
        println!("cargo:rustc-link-search=native={}", dir);
    }
    println!("cargo:rustc-link-lib=dylib=fuzzyblue_cuda");
    println!("cargo:rerun-if-env-changed=FUZZYBLUE_CUDA_LIB_DIR");
}
