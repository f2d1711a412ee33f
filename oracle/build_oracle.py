"""Compile oracle/tm_oracle.c into oracle/_build/libtm_oracle.so (gcc, OpenMP).

Portable flags only (the library must build the same way on x86_64 and
aarch64).  Test infrastructure.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "tm_oracle.c")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libtm_oracle.so")


def build() -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O3", "-std=c99", "-fPIC", "-shared", "-fopenmp", SRC, "-o", LIB, "-lm"]
    subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build())
    sys.exit(0)
