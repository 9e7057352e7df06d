"""Builds the engine's shared library, libqvnt_gb300.so, for sm_103a (GB300).

Each translation unit is compiled by its own nvcc/g++ process, in parallel; the library links the
CUDA runtime statically.  Outputs go to qvnt_gb300/_build/ (git-ignored).

    python -m qvnt_gb300.build            # or: python qvnt_gb300/build.py
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libqvnt_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2", "--expt-relaxed-constexpr",
                      "-I" + os.path.join(HERE, "..", "include")]

# (source, extra flags).  The plain engine and the register-wide passes round every product and
# sum separately, as qvnt's own arithmetic does, so they are built without FMA contraction.
UNITS = [
    ("abi.cu", []),
    ("fused.cu", []),
    ("gates_plain.cu", ["--fmad=false"]),
    ("measure.cu", ["--fmad=false"]),
    ("serve.cu", []),
    ("precision.cu", []),
    ("tensor64.cu", []),
    ("builders.cpp", None),
    ("wire.cpp", None),
    ("program.cpp", None),
    ("qasm.cpp", None),
]


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _compile(unit, extra, verbose):
    src = os.path.join(CSRC, unit)
    obj = os.path.join(OUT, "obj", unit + ".o")
    if extra is None:
        cmd = ["g++", "-O2", "-fPIC", "-std=c++17", "-Wall", "-ffp-contract=off", "-c", src, "-o", obj]
    else:
        cmd = [_nvcc()] + NVCC_COMMON + extra + ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    if verbose and (r.stderr.strip() or r.stdout.strip()):
        print(r.stdout + r.stderr, flush=True)
    return obj


def build(verbose=False, extra_units=()):
    os.makedirs(os.path.join(OUT, "obj"), exist_ok=True)
    units = list(UNITS) + list(extra_units)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(lambda u: _compile(u[0], u[1], verbose), units))
    cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
