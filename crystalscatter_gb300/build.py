"""Build of the native library libcrystalscatter.so (sm_103a) in-tree.

Host C++ (preparation, parameters, C ABI) is compiled by g++ without
floating-point contraction, so that the preparation rounds like the
reference's x86 build; the CUDA translation unit is compiled by nvcc for
sm_103a only. Translation units compile in parallel; the result lands in
crystalscatter_gb300/_lib/.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libcrystalscatter.so")

HOST_SOURCES = ["cs_prep.cpp", "cs_params.cpp", "cs_capi.cpp", "cs_batch.cpp", "cs_simplex.cpp"]
CUDA_SOURCES = ["cs_kernels.cu", "cs_mixed.cu", "cs_noalloc.cu", "cs_mlp.cu", "cs_peaks.cu", "cs_postproc.cu"]
# cs_fp64_unit.cu is compiled once per dispatch key (the FP64 drop-in kernels
# of that key), so that the keys' kernels compile in parallel
FP64_UNIT = "cs_fp64_unit.cu"
UNIT_KEYS = ["CS_KEY_SPHERE_NONE_ISO", "CS_KEY_SPHERE_GAUSS_FCC_GAUSS", "CS_KEY_CYL_NONE_GAUSS",
             "CS_KEY_CYL_NONE_ZDIR", "CS_KEY_CYL_GAUSS_BCT_ZDIR", "CS_KEY_CUBE_NONE_ISO", "CS_KEY_GENERIC"]
# No automatic multiply-add contraction in either unit: the FP64 drop-in keeps
# the reference's separate multiply and add roundings, and the mixed kernels
# share its FP64 functions (pixel geometry, power series, math library calls),
# which must round identically there; FP32 code asks for fmaf where it wants one
FMAD = {"cs_kernels.cu": "false", "cs_mixed.cu": "false", "cs_noalloc.cu": "false", "cs_mlp.cu": "true",
        "cs_peaks.cu": "true", "cs_postproc.cu": "false", FP64_UNIT: "false"}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _cuda_home():
    nv = _nvcc()
    return os.path.dirname(os.path.dirname(os.path.realpath(nv)))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    cuda_inc = os.path.join(_cuda_home(), "include")
    headers = [os.path.join(SRC, f) for f in os.listdir(SRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "crystalscatter.h"))
    jobs = []
    objs = []
    for f in HOST_SOURCES:
        src = os.path.join(SRC, f)
        obj = os.path.join(OUT, f + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append(["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-I" + cuda_inc,
                         "-c", src, "-o", obj])
    units = [(f, f + ".o", []) for f in CUDA_SOURCES]
    units += [(FP64_UNIT, "cs_fp64_unit_" + k[len("CS_KEY_"):].lower() + ".o", ["-DCS_UNIT_KEY=" + k])
              for k in UNIT_KEYS]
    for f, oname, defs in units:
        src = os.path.join(SRC, f)
        obj = os.path.join(OUT, oname)
        objs.append(obj)
        if force or _stale(obj, [src] + headers):
            jobs.append([_nvcc()] + ARCH + ["-O3", "-lineinfo", "-std=c++17", "--fmad=" + FMAD[f]] + defs +
                        ["-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills", "-c", src, "-o", obj])
    # longest units first (the generic pixel function's kernels)
    jobs.sort(key=lambda j: 0 if any("GENERIC" in a for a in j) else 1)
    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            if o.strip():
                print(o)
    if force or _stale(LIB, objs):
        _run([_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    return LIB


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
