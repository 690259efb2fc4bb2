"""Builds libeuc_gb300.so (the C ABI + sm_103a kernels) in-tree.

    python -m euc_gb300.build

Flags that matter for parity with euc's CPU arithmetic:
  -fmad=false      no multiply-add contraction (Rust never contracts)
  -prec-div=true   IEEE round-to-nearest division and reciprocal
  -prec-sqrt=true  IEEE round-to-nearest sqrt
  -ftz=false       keep denormals
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libeuc_gb300.so")
SOURCES = [os.path.join(HERE, "csrc", f) for f in ("euc_capi.cu", "euc_server.cu")]
HEADERS = [os.path.join(HERE, "csrc", f) for f in ("euc_device.cuh", "euc_kernels.cuh")] + [
    os.path.join(ROOT, "include", "euc_gb300.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-strict-aliasing", "-shared", "--expt-relaxed-constexpr"]


def nvcc():
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def build(force=False, verbose=False, extra=()):
    os.makedirs(OUT_DIR, exist_ok=True)
    deps = SOURCES + HEADERS
    if not force and os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(d) for d in deps):
        return LIB
    tmp = LIB + ".tmp%d" % os.getpid()
    compile_flags = [f for f in NVCC_FLAGS if f != "-shared"]
    objs, procs = [], []
    for src in SOURCES:  # translation units compile in parallel
        obj = os.path.join(OUT_DIR, os.path.basename(src) + ".%d.o" % os.getpid())
        cmd = [nvcc()] + ARCH + compile_flags + list(extra) + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        procs.append(subprocess.Popen(cmd))
        objs.append(obj)
    failed = [p.args for p in procs if p.wait() != 0]
    try:
        if failed:
            raise subprocess.CalledProcessError(1, failed[0])
        cmd = [nvcc()] + ARCH + ["-shared", "-Xcompiler", "-fPIC"] + objs + ["-o", tmp]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    finally:
        for o in objs:
            if os.path.exists(o):
                os.remove(o)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    extra = [a for a in sys.argv[1:] if a.startswith("-X") or a.startswith("--resource")]
    print(build(force="--force" in sys.argv, verbose=True, extra=extra))
