// Link libraydar_cuda.so.  RAYDAR_CUDA_LIB_DIR names the directory that holds
// it (the raydar_gb300/ folder of this repository after its build step).
fn main() {
    println!("cargo:rerun-if-env-changed=RAYDAR_CUDA_LIB_DIR");
    if let Ok(dir) = std::env::var("RAYDAR_CUDA_LIB_DIR") {
        println!("cargo:rustc-link-search=native={dir}");
        println!("cargo:rustc-link-arg=-Wl,-rpath,{dir}");
    }
    println!("cargo:rustc-link-lib=dylib=raydar_cuda");
}
