"""Console entry: compute one image on the GPU.

    python -m crystalscatter_gb300.cli --workload cyl_gauss_x --grid 64 --repeat 3
    python -m crystalscatter_gb300.cli --mcpval "cbparticle=sphere;radius=10;gridpoints=128" --out img.dat
    python -m crystalscatter_gb300.cli --sweep 16 --mode mixed --repeat 2

The parameter set is a named workload (crystalscatter_gb300.configs), optionally
rescaled to another grid with the same q-range, then modified by a console
``--mcpval`` key/value string (the rules of the console front end,
Source/sc_mainCons.cpp:858-900). ``--out`` writes the raw image format of the
reference (Source/widimage.cpp:1480-1500): a 19-byte text header
"minX maxX minY maxY" (each %4d) followed by the doubles row by row.
"""
import argparse
import json
import sys
import time

import numpy as np

from . import CS_MODE_FP64, CS_MODE_MIXED, SasCalc_GENERIC_calculation, SasCalcBatch
from . import configs as C


def write_dat(path, img, x0, x1, y0, y1):
    header = f"{x0:4d} {x1:4d} {y0:4d} {y1:4d}".encode()
    with open(path, "wb") as f:
        f.write(header)
        f.write(np.ascontiguousarray(img, dtype="<f8").tobytes())


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", default="sphere", choices=sorted(C.WORKLOADS) + ["bct0"])
    ap.add_argument("--grid", type=int, default=0, help="GridPoints (half the image edge); 0 = workload size")
    ap.add_argument("--mcpval", default="", help="console key/value string applied after the workload")
    ap.add_argument("--mode", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--repeat", type=int, default=1)
    ap.add_argument("--ign-cbs", action="store_true")
    ap.add_argument("--out", default="")
    ap.add_argument("--sweep", type=int, default=0,
                    help="instead of one image: the first N parameter sets of the cylinder/BCT sweep as one batch")
    ap.add_argument("--schedule", default="",
                    help="sweep: CHUNK,BLOCKS_PER_SM of the mixed persistent kernel (0,0 = block tiles at full "
                         "occupancy) instead of the autotuner's choice")
    a = ap.parse_args(argv)
    if a.sweep:
        return sweep(a)
    params = C.bct_set(0) if a.workload == "bct0" else C.WORKLOADS[a.workload]
    if a.grid:
        params = C.scaled(params, a.grid)
    ign = a.ign_cbs or (params.get("ComboBoxParticle") == 1 and params.get("LType") == 8)
    calc = SasCalc_GENERIC_calculation()
    calc.setParams(params)
    if a.mcpval:
        calc.setKeyValues(a.mcpval)
    mode = CS_MODE_MIXED if a.mode == "mixed" else CS_MODE_FP64
    times = []
    for _ in range(max(1, a.repeat)):
        t0 = time.perf_counter()
        calc.doCalculation(0, False, ign, mode=mode)
        times.append(time.perf_counter() - t0)
    img = calc.data()
    x0, x1, y0, y1 = calc.minX(), calc.maxX(), calc.minY(), calc.maxY()
    if a.out:
        write_dat(a.out, img, x0, x1, y0, y1)
    fin = np.isfinite(img)
    print(json.dumps({"workload": a.workload, "dims": [x0, x1, y0, y1], "mode": a.mode,
                      "min": float(img[fin].min()) if fin.any() else None,
                      "max": float(img[fin].max()) if fin.any() else None,
                      "nonfinite": int((~fin).sum()), "seconds": times,
                      "prep_ms": calc.higResTimerElapsedPrep, "calc_ms": calc.higResTimerElapsedCalc}))
    calc.cleanup()
    return 0


def sweep(a):
    """the first a.sweep sets of the cylinder/BCT sweep in one batch
    (persistent launch per dispatch key), a.repeat times"""
    mode = CS_MODE_MIXED if a.mode == "mixed" else CS_MODE_FP64
    b = SasCalcBatch()
    t0 = time.perf_counter()
    b.prepare(C.bct_sweep(a.sweep), bIgnoreCbs=True)
    t_prep = time.perf_counter() - t0
    if a.schedule:
        chunk, bps = (int(v) for v in a.schedule.split(","))
        b.set_schedule(chunk, bps)
    times = []
    for _ in range(max(1, a.repeat)):
        t0 = time.perf_counter()
        flat = b.run_host(mode)
        times.append(time.perf_counter() - t0)
    total, pixels, groups = b.info()
    redo = b.redo_pixels()[0] if mode == CS_MODE_MIXED else 0
    nonfinite = sum(int((~np.isfinite(img)).sum()) for img in b.split(flat))
    print(json.dumps({"sweep_sets": a.sweep, "pixels": pixels, "key_groups": groups, "mode": a.mode,
                      "prep_seconds": t_prep, "seconds": times, "redo_pixels": redo, "nonfinite": nonfinite}))
    b.cleanup()
    return 0


if __name__ == "__main__":
    sys.exit(main())
