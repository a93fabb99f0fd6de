"""Builds the CPU test oracle (oracle/cs_oracle.c) into oracle/_build/liboracle_cs.so.

Plain C, compiled without floating-point contraction so that it rounds like
the reference's x86 build on any host (gcc on aarch64 would otherwise fuse
multiply-adds)."""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cs_oracle.c")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "liboracle_cs.so")
HDR = os.path.join(HERE, "..", "crystalscatter_gb300", "csrc", "cs_prepared.h")


def build(force=False):
    os.makedirs(OUT, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(HDR)):
        return LIB
    cmd = ["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-fPIC", "-shared", "-ffp-contract=off", "-Wall", SRC, "-o",
           LIB, "-lpthread", "-lm"]
    subprocess.run(cmd, check=True)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
