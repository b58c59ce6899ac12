// Links libchfft_gb300.so (built by `python -m chfft_gb300._build` into
// chfft_gb300/_lib/). CHFFT_GB300_LIB_DIR names that directory.
fn main() {
    let dir = std::env::var("CHFFT_GB300_LIB_DIR")
        .unwrap_or_else(|_| concat!(env!("CARGO_MANIFEST_DIR"), "/../../chfft_gb300/_lib").to_string());
    println!("cargo:rustc-link-search=native={}", dir);
    println!("cargo:rustc-link-lib=dylib=chfft_gb300");
    println!("cargo:rerun-if-env-changed=CHFFT_GB300_LIB_DIR");
}
