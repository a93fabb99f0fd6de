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
PROBE = os.path.join(OUT, "liboracle_cs_probe.so")
COUNT = os.path.join(OUT, "liboracle_cs_count.so")
COUNT_SRC = os.path.join(HERE, "count_ops.cpp")
QUAD = os.path.join(OUT, "liboracle_cs_quad.so")
QUAD_SRC = os.path.join(HERE, "quad_oracle.cpp")
HDR = os.path.join(HERE, "..", "crystalscatter_gb300", "csrc", "cs_prepared.h")


def _compile(out, extra):
    cmd = ["gcc", "-O2", "-std=c11", "-D_GNU_SOURCE", "-fPIC", "-shared", "-ffp-contract=off", "-Wall"] + extra + [
        SRC, "-o", out, "-lpthread", "-lm"]
    subprocess.run(cmd, check=True)


def build(force=False):
    """liboracle_cs.so (the oracle) and liboracle_cs_probe.so (the same code
    with the one-ulp conditioning probe compiled in)."""
    os.makedirs(OUT, exist_ok=True)
    newest = max(os.path.getmtime(SRC), os.path.getmtime(HDR))
    for out, extra in ((LIB, []), (PROBE, ["-DCS_ORACLE_PROBE"])):
        if force or not os.path.exists(out) or os.path.getmtime(out) < newest:
            _compile(out, extra)
    # operation-counting build (count_ops.cpp includes cs_oracle.c unchanged)
    if force or not os.path.exists(COUNT) or os.path.getmtime(COUNT) < max(newest, os.path.getmtime(COUNT_SRC)):
        subprocess.run(["g++", "-O1", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-w", COUNT_SRC, "-o",
                        COUNT, "-lpthread"], check=True)
    # quadruple-precision build (quad_oracle.cpp includes cs_oracle.c unchanged)
    if force or not os.path.exists(QUAD) or os.path.getmtime(QUAD) < max(newest, os.path.getmtime(QUAD_SRC)):
        import platform
        libs = [] if platform.machine() in ("aarch64", "arm64") else ["-lquadmath"]
        # optional: only the golden-fixture generator needs it; a host whose
        # compiler lacks binary128 support goes on without it
        r = subprocess.run(["g++", "-O2", "-std=gnu++17", "-fPIC", "-shared", "-ffp-contract=off", "-w", QUAD_SRC,
                            "-o", QUAD, "-lpthread"] + libs, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            print("quadruple-precision oracle not built on this host:\n" + r.stdout[-2000:], file=sys.stderr)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
