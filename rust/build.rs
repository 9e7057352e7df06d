// Build script of qvnt's `gb300` feature: links the GB300 engine (libqvnt_gb300.so, the C ABI of
// include/qvnt_gb300.h).  Two ways:
//   QVNT_GB300_LIB_DIR=<dir holding libqvnt_gb300.so>   link the library built by the engine's own
//                                                         build (python -m qvnt_gb300.build);
//   QVNT_GB300_SRC=<checkout of the engine>             compile qvnt_gb300/csrc with the `cc` crate
//                                                         (nvcc for the .cu units, sm_103a).
// Without the feature nothing is linked and the crate builds as before.
fn main() {
    if std::env::var_os("CARGO_FEATURE_GB300").is_none() {
        return;
    }
    println!("cargo:rerun-if-env-changed=QVNT_GB300_LIB_DIR");
    println!("cargo:rerun-if-env-changed=QVNT_GB300_SRC");
    if let Ok(dir) = std::env::var("QVNT_GB300_LIB_DIR") {
        println!("cargo:rustc-link-search=native={dir}");
        println!("cargo:rustc-link-lib=dylib=qvnt_gb300");
        println!("cargo:rustc-link-arg=-Wl,-rpath,{dir}");
        return;
    }
    let root = std::path::PathBuf::from(
        std::env::var("QVNT_GB300_SRC").expect("set QVNT_GB300_LIB_DIR or QVNT_GB300_SRC for the gb300 feature"),
    );
    let csrc = root.join("qvnt_gb300").join("csrc");
    let include = root.join("include");
    // Units as the engine's own build compiles them; the plain engine and the register-wide passes
    // are built without FMA contraction (they round like qvnt's arithmetic).
    let cuda_units: [(&str, bool); 7] = [
        ("abi.cu", true),
        ("fused.cu", true),
        ("gates_plain.cu", false),
        ("measure.cu", false),
        ("serve.cu", true),
        ("precision.cu", true),
        ("tensor64.cu", true),
    ];
    for (unit, fmad) in cuda_units.iter() {
        let mut b = cc::Build::new();
        b.cuda(true)
            .cudart("static")
            .flag("-gencode=arch=compute_103a,code=sm_103a")
            .flag("-std=c++17")
            .flag("--expt-relaxed-constexpr")
            .flag("-O3")
            .include(&include)
            .file(csrc.join(unit));
        if !fmad {
            b.flag("--fmad=false");
        }
        b.compile(&format!("qvnt_gb300_{}", unit.trim_end_matches(".cu")));
        println!("cargo:rerun-if-changed={}", csrc.join(unit).display());
    }
    cc::Build::new()
        .cpp(true)
        .std("c++17")
        .flag("-ffp-contract=off")
        .include(&include)
        .files(["builders.cpp", "wire.cpp", "program.cpp", "qasm.cpp"].iter().map(|f| csrc.join(f)))
        .compile("qvnt_gb300_host");
    println!("cargo:rustc-link-lib=dylib=stdc++");
}
