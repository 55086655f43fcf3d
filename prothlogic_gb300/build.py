"""Build libprothgpu.so (the engine) for sm_103a with nvcc, in-tree.

The library is the product: CUDA kernels + host engine + C ABI.  It is
written to prothlogic_gb300/_build/libprothgpu.so (git-ignored).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libprothgpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["pg_engine.cu", "pg_prefilter.cu", "pg_bigint.cpp"]
DEPS = SOURCES + ["pg_kernels.cuh", "pg_resident.cuh", "pg_internal.h", "pg_bigint.h", "pg_engine_more.inc", "pg_tune.inc",
                  os.path.join("..", "..", "include", "prothgpu.h")]


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


COMPAT_LIB = os.path.join(OUT_DIR, "libprothgpu_compat.a")
COMPAT_DRIVER = os.path.join(OUT_DIR, "compat_driver")


def build_compat():
    """The reference-API shim (fft_init / fft_square_karatsuba / fft_destroy) and its test driver."""
    comp = os.path.join(HERE, "compat")
    obj = os.path.join(OUT_DIR, "fft_engine_gpu.o")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-fPIC", "-c", os.path.join(comp, "fft_engine_gpu.cpp"),
                           "-o", obj])
    subprocess.check_call(["ar", "rcs", COMPAT_LIB, obj])
    subprocess.check_call(["g++", "-std=c++17", "-O2", os.path.join(comp, "compat_driver.cpp"), COMPAT_LIB,
                           "-L" + OUT_DIR, "-lprothgpu", "-Wl,-rpath," + OUT_DIR, "-o", COMPAT_DRIVER])
    return COMPAT_DRIVER


def needs_build():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    if not os.path.exists(COMPAT_DRIVER):
        return True
    return any(os.path.getmtime(os.path.join(CSRC, d)) > t for d in DEPS)


def build(force=False, verbose=False):
    if not force and not needs_build():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    objs = []
    procs = []
    for src in SOURCES:
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        cmd = [nvcc(), "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-c",
               os.path.join(CSRC, src), "-o", obj] + ARCH
        if src.endswith(".cu") and verbose:
            cmd += ["-Xptxas", "-v"]
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            sys.stderr.write(out.decode(errors="replace"))
            raise RuntimeError("nvcc failed: " + " ".join(cmd))
        if verbose:
            sys.stderr.write(out.decode(errors="replace"))
    tmp = LIB + ".tmp"
    link = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-lcudart"]
    subprocess.check_call(link)
    os.replace(tmp, LIB)
    build_compat()
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print(LIB)
