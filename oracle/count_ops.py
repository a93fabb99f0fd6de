"""Algorithmic operations per pixel of the benchmark workloads, counted on
the oracle (MEASUREMENT INFRASTRUCTURE).

The counting build of the oracle (count_ops.cpp: cs_oracle.c compiled
unchanged with a tallying double type) runs sampled pixels of each workload
and reports how many FP64 adds/subtracts, multiplies, divides and math-library
calls the reference's per-pixel algorithm performs. A fixed cost table turns
the tallies into FP64-equivalent flops (an FMA counts as its multiply and its
add, 2 flops; a library call counts as the flops of a typical FP64
implementation of it). The result is frozen in
crystalscatter_gb300/config_ops.json, which bench.py reads for the compute
roofline: achieved flop/s = pixels/s x flops/pixel.

    python oracle/count_ops.py            # all workloads, ~1-2 minutes
"""
import ctypes
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

from oracle import build_oracle, cpu_oracle  # noqa: E402
from crystalscatter_gb300 import configs as C  # noqa: E402

FIELDS = ["add", "mul", "div", "sqrt", "exp", "log", "sin", "cos", "tan", "atan", "atan2", "pow", "acos"]
# FP64-equivalent flops per operation. add/sub and mul: 1 each (an FMA is 2).
# Library calls and divide/sqrt: the flop count of a typical FP64 GPU
# implementation (range reduction + polynomial / Newton steps, ~2 flops per
# DFMA-pipe instruction).
COST = {"add": 1, "mul": 1, "div": 16, "sqrt": 16, "exp": 32, "log": 32, "sin": 40, "cos": 40, "tan": 48,
        "atan": 48, "atan2": 56, "pow": 80, "acos": 48}
OUT = os.path.join(ROOT, "crystalscatter_gb300", "config_ops.json")


def load():
    build_oracle.build()
    lib = ctypes.CDLL(build_oracle.COUNT)
    lib.ops_pixel.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_ulonglong)]
    lib.ops_pixel.restype = ctypes.c_double
    return lib


def sample_pixels(P, n_target):
    xs = np.arange(P.zzmin, P.zzmax)
    ys = np.arange(P.iimin, P.iimax)
    total = len(xs) * len(ys)
    step = max(1, int(np.sqrt(total / max(n_target, 1))))
    # odd offsets so the sample does not sit on the axes only
    return [(int(x), int(y)) for y in ys[step // 2::step] for x in xs[step // 3::step]], total


def count(lib, params, ign_cbs, n_target, check_oracle=True):
    P = cpu_oracle.prepare(params, ign_cbs)
    pix, total = sample_pixels(P, n_target)
    t = (ctypes.c_ulonglong * 13)()
    vals = []
    for (x, y) in pix:
        vals.append(lib.ops_pixel(ctypes.byref(P), x, y, t))
    if check_oracle:
        ol = cpu_oracle.load()
        ref = [ol.oracle_pixel(ctypes.byref(P), x, y) for (x, y) in pix]
        a, b = np.array(vals), np.array(ref)
        same = (a == b) | (np.isnan(a) & np.isnan(b))
        assert same.all(), "counting build disagrees with the oracle"
    n = len(pix)
    per = {f: t[k] / n for k, f in enumerate(FIELDS)}
    flops = sum(per[f] * COST[f] for f in FIELDS)
    return {"pixels_sampled": n, "pixels_image": total, "per_pixel": per, "flops_per_pixel": flops}


def main():
    lib = load()
    res = {}
    t0 = time.time()
    for name, n in (("sphere", 4096), ("cyl_gauss", 4096), ("cyl_gauss_x", 1024), ("sphere_fcc", 4096)):
        res[name] = count(lib, C.WORKLOADS[name], 0, n)
        print(name, round(res[name]["flops_per_pixel"], 1), f"{time.time() - t0:.1f}s", flush=True)
    # sweep: pixel-weighted mean over a sample of its parameter sets
    sets, tot_pix, tot_flops = [], 0, 0.0
    for k in range(16):
        r = count(lib, C.bct_set(k), 1, 256)
        sets.append({"set": k, "pixels_image": r["pixels_image"], "flops_per_pixel": r["flops_per_pixel"]})
        tot_pix += r["pixels_image"]
        tot_flops += r["pixels_image"] * r["flops_per_pixel"]
    res["bct_sweep"] = {"sets_sampled": 16, "per_set": sets, "flops_per_pixel": tot_flops / tot_pix}
    print("bct_sweep", round(res["bct_sweep"]["flops_per_pixel"], 1), f"{time.time() - t0:.1f}s", flush=True)
    out = {"unit": "FP64-equivalent flops per pixel (algorithmic, counted on the oracle)", "cost_table": COST,
           "note": "add/sub and mul 1 flop each (FMA = 2); div/sqrt/library calls at the flops of a typical FP64 "
                   "implementation", "workloads": res}
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
