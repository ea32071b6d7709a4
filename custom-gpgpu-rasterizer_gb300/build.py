"""Build recipe for libgbr.so (the C ABI in include/gbr.h) for sm_103a.

The translation units compile in parallel with nvcc; the library lands in
custom-gpgpu-rasterizer_gb300/_build/ (git-ignored) and is rebuilt when a
source is newer.  Device code uses -fmad=false: every fused multiply-add in
the kernels is explicit, which keeps culling, bin rectangles and texel
addresses bit-identical to the roundings they are specified by.
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgbr.so")
SOURCES = ["gbr_kernels.cu", "gbr_scan.cu", "gbr_api.cu", "gbr_batch.cu", "gbr_noalloc.cu", "gbr_predict.cu", "gbr_draw.cu", "gbr_obj.cpp"]
HEADERS = ["gbr_device.cuh", "gbr_shade.cuh", "gbr_kernels.h", "gbr_predict.h", "gbr_internal.h"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else (shutil.which("nvcc") or "nvcc")


def _inputs():
    files = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    files.append(os.path.join(ROOT, "include", "gbr.h"))
    files.append(os.path.join(ROOT, "include", "gbr_cudarenderer.hpp"))
    files.append(os.path.join(ROOT, "tests", "cpp", "facade_render.cpp"))
    files.append(os.path.abspath(__file__))
    return files


def up_to_date() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(FACADE_BIN):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _inputs())


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    common = [nvcc(), "-O3", "-std=c++17", *ARCH, "-lineinfo", "-fmad=false",
              "-Xcompiler", "-fPIC,-ffp-contract=off,-Wall", "-I", os.path.join(ROOT, "include")]
    if verbose:
        common += ["-Xptxas", "-v"]
    procs, objs = [], []
    for src in SOURCES:
        obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        objs.append(obj)
        procs.append((src, subprocess.Popen(common + ["-c", os.path.join(CSRC, src), "-o", obj],
                                            stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)))
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode != 0:
            sys.stderr.write(out)
        if p.returncode != 0:
            failed.append(src)
    if failed:
        raise RuntimeError(f"nvcc failed for {failed}")
    tmp = LIB + ".tmp"
    subprocess.run([nvcc(), "-shared", *ARCH, *objs, "-o", tmp, "-lcudart"], check=True)
    os.replace(tmp, LIB)
    build_facade_demo()
    return LIB


FACADE_SRC = os.path.join(ROOT, "tests", "cpp", "facade_render.cpp")
FACADE_BIN = os.path.join(OUT_DIR, "facade_render")


def build_facade_demo() -> str:
    """Compiles the C++ host-API driver (tests/cpp/facade_render.cpp) with the
    host compiler against include/gbr_cudarenderer.hpp and libgbr.so."""
    if not os.path.exists(FACADE_SRC):
        return ""
    cxx = os.environ.get("CXX", "g++")
    subprocess.run([cxx, "-O2", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "include"), FACADE_SRC,
                    "-L", OUT_DIR, "-lgbr", "-Wl,-rpath," + OUT_DIR, "-o", FACADE_BIN], check=True)
    return FACADE_BIN


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
