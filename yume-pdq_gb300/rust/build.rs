//! Links libyumepdq_gb300.so, built by `python -c "import __graft_entry__ as g; g.build()"`
//! into yume-pdq_gb300/_build/. YPDQ_GB300_LIB_DIR overrides the search directory.
fn main() {
    let dir = std::env::var("YPDQ_GB300_LIB_DIR").unwrap_or_else(|_| {
        let here = std::path::PathBuf::from(std::env::var("CARGO_MANIFEST_DIR").unwrap());
        here.join("../_build").to_string_lossy().into_owned()
    });
    println!("cargo:rerun-if-env-changed=YPDQ_GB300_LIB_DIR");
    println!("cargo:rustc-link-search=native={dir}");
    println!("cargo:rustc-link-lib=dylib=yumepdq_gb300");
}
