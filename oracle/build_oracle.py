"""Build recipe for the CPU oracle (test infrastructure).

Compiles oracle/gbr_oracle.c into oracle/_build/libgbr_oracle.so with the
host C compiler.  -ffp-contract=off keeps the host compiler from fusing
multiply-adds on its own (GCC fuses by default on aarch64); the fusions the
reference's GPU build performs are written out as fmaf() in the source.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgbr_oracle.so")
SRC = os.path.join(HERE, "gbr_oracle.c")


def build(force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    hdr = os.path.join(HERE, "gbr_oracle.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(hdr))):
        return LIB
    cc = os.environ.get("CC", "gcc")
    cmd = [cc, "-O2", "-std=c11", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-pthread", "-Wall", "-Wno-unused-function", SRC, "-o", LIB + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
