"""Executed work per pixel of a kernel, from an ncu capture (measurement
support for the compute roofline that bench.py reports).

Reads the raw page of an ncu report exported as CSV
(``ncu -i X.ncu-rep --page raw --csv``), takes the kernel's thread-level
FP32 and FP64 instruction counts and its special-function (XU) pipe
instructions, divides by the pixels the captured launch computed, and stores
the per-pixel figures in crystalscatter_gb300/kernel_work.json under the
dispatch key:

* fp32_flops_per_pixel  2 FFMA + FADD + FMUL (+ 4 FFMA2 + 2 FADD2 + 2 FMUL2)
* fp64_flops_per_pixel  2 DFMA + DADD + DMUL
* mufu_ops_per_pixel    XU warp instructions x active threads per instruction
* dram_bytes_per_pixel  DRAM read + write bytes

    python -m crystalscatter_gb300.kernel_work RAW.csv --key 0x01020806 --pixels N --source "..."
"""
import argparse
import csv
import json
import os

HERE = os.path.dirname(os.path.abspath(__file__))
PATH = os.path.join(HERE, "kernel_work.json")

M = "sm__sass_thread_inst_executed_op_{}_pred_on.sum"


def per_pixel(raw_csv, pixels, kernel_regex=None):
    import re
    rows = list(csv.reader(open(raw_csv)))
    hdr, units, data = rows[0], rows[1], rows[2:]
    for row in data:
        d = dict(zip(hdr, row))
        if kernel_regex and not re.search(kernel_regex, d.get("Kernel Name", "")):
            continue

        def v(name):
            x = d.get(name, "0").replace(",", "")
            u = units[hdr.index(name)] if name in hdr else ""
            f = float(x) if x not in ("", "n/a") else 0.0
            scale = {"Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "byte": 1.0}.get(u, 1.0)
            return f * scale

        fp32 = (2 * v(M.format("ffma")) + v(M.format("fadd")) + v(M.format("fmul")) + 4 * v(M.format("ffma2")) +
                2 * v(M.format("fadd2")) + 2 * v(M.format("fmul2")))
        fp64 = 2 * v(M.format("dfma")) + v(M.format("dadd")) + v(M.format("dmul"))
        xu = v("sm__inst_executed_pipe_xu.sum") * v("smsp__thread_inst_executed_per_inst_executed.ratio")
        dram = v("dram__bytes_read.sum") + v("dram__bytes_write.sum")
        return {"kernel": d.get("Kernel Name", "")[:80], "fp32_flops_per_pixel": fp32 / pixels,
                "fp64_flops_per_pixel": fp64 / pixels, "mufu_ops_per_pixel": xu / pixels,
                "dram_bytes_per_pixel": dram / pixels,
                "fp64_pipe_pct": v("sm__pipe_fp64_cycles_active.avg.pct_of_peak_sustained_active"),
                "fma_pipe_pct": v("sm__pipe_fma_cycles_active.avg.pct_of_peak_sustained_active"),
                "xu_pipe_pct": v("sm__inst_executed_pipe_xu.avg.pct_of_peak_sustained_active"),
                "registers": v("launch__registers_per_thread"),
                "warps_active_pct": v("sm__warps_active.avg.pct_of_peak_sustained_active")}
    raise ValueError("no matching kernel in " + raw_csv)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("raw_csv")
    ap.add_argument("--key", required=True)
    ap.add_argument("--pixels", type=int, required=True)
    ap.add_argument("--kernel", default=None)
    ap.add_argument("--source", default="")
    a = ap.parse_args()
    w = per_pixel(a.raw_csv, a.pixels, a.kernel)
    w["source"] = a.source
    data = json.load(open(PATH)) if os.path.exists(PATH) else {}
    data[a.key] = w
    with open(PATH, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    print(json.dumps(w, indent=1))


if __name__ == "__main__":
    main()
