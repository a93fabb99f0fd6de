#!/usr/bin/env python3
"""Benchmark: detector pixels per second of the 2D scattering-pattern
calculation on one GB300 (or N replicas on N GPUs).

Workload (one step = one full image): cylinders, no lattice, Gaussian
orientation (pCyl_lNon_oGau), 512x512 detector, pixel 0.5 mm, 4 m, 0.6 nm,
radius 5 nm / length 60 nm (Schulz sigma 0.10), axis in the detector plane at
azimuth 30 deg, orientation width 15 deg (crystalscatter_gb300.configs
"cyl_gauss"). Reported:

* value   pixels/s with the prepared parameter set resident in device memory
          (kernel launches only), summed over all ranks
* e2e     pixels/s through the drop-in call with host buffers: host
          preparation, upload of the prepared block, kernel, image download
* roofline / cpu_baseline / clocks as the benchmark contract asks
* extra   per-workload kernel rates for the other workloads (sphere, the
          x-axis cylinder that runs the full orientation integral, FCC)

``--impl reference`` times the reference's algorithm on the host cores: the
CPU port of the reference in oracle/ (the reference's own sources cannot be
built on the GPU host), with all host threads, on the same workload.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "pixels/s at <=1e-5 rel err vs FP64"
UNIT = "pixels/s"
WORKLOAD = "cyl_gauss"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--no-extra", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--sweep-sets", type=int, default=4096, help="parameter sets of the batched sweep (0 = skip)")
    ap.add_argument("--sweep-steps", type=int, default=2)
    ap.add_argument("--surrogate", default="", help="surrogate-seeded fits of this family ('2', '2x'); off by default")
    ap.add_argument("--surrogate-train", type=int, default=32768)
    ap.add_argument("--surrogate-epochs", type=int, default=200)
    ap.add_argument("--surrogate-targets", type=int, default=8)
    return ap.parse_args()


def max_over_ranks(values, world, device):
    """Per-rank timings reduced to their maximum over the ranks (the job's
    time: every rank waits for the slowest); the values themselves on one
    rank."""
    if world <= 1:
        return list(values)
    import torch
    import torch.distributed as dist
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def replica_rate(units_per_rank, world, seconds):
    """Whole-job rate of `world` independent replicas that each process
    units_per_rank units, over the slowest replica's time."""
    return units_per_rank * world / seconds


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        sm.sort()
        med = sm[len(sm) // 2] if sm else None
        return {"sm_mhz": med, "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def time_kernel(calc, torch, d_out, n, steps, warmup, flush, mode=0):
    """Device-resident launches of the prepared calculation on a dedicated
    stream: per step an L2 flush outside the timed events, then one launch
    between two events recorded on that same stream. Returns (total seconds
    over steps, per-step list)."""
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    assert sp != 0, "run on a created stream: handle 0 would select the library's own stream"
    for _ in range(warmup):
        calc.launch_prepared(d_out.data_ptr(), n, sp, mode=mode)
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        flush.fill_(1.0)  # 256 MB write: evicts the 129 MB L2 between steps
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        calc.launch_prepared(d_out.data_ptr(), n, sp, mode=mode)
        b.record(stream)
        b.synchronize()
        times.append(a.elapsed_time(b) / 1e3)
    return sum(times), times


def fp_peaks():
    """Nominal arithmetic peaks of the GPU from its SM count and clock: FP64
    (2 DFMA per SM per clock, FMA = 2 flops) and FP32 (128 lanes per SM)."""
    import torch
    props = torch.cuda.get_device_properties(torch.cuda.current_device())
    sms = props.multi_processor_count
    mhz = 2070.0
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            mhz = float(json.load(f).get("sm_max_mhz", mhz))
    return {"fp64_tflops": sms * 2 * 2 * mhz * 1e6 / 1e12, "fp32_tflops": sms * 128 * 2 * mhz * 1e6 / 1e12,
            "sms": sms, "sm_mhz": mhz, "kind": "nominal (SMs x lanes x max clock)"}


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# the headline kernel, k_image_mixed on the 512x512 cylinder, from an ncu
# capture of three launches on a GB300 (the median; the image stays in L2
# during the launch and reaches DRAM after it)
TRAFFIC_BYTES_PER_LAUNCH = 95232


def load_ops():
    p = os.path.join(ROOT, "crystalscatter_gb300", "config_ops.json")
    with open(p) as f:
        return json.load(f)["workloads"]


def rel_stats(img, ref):
    import numpy as np
    with np.errstate(invalid="ignore", divide="ignore"):
        rel = np.abs(img - ref) / np.maximum(np.abs(ref), 1e-300)
    fin = np.isfinite(ref) & np.isfinite(img)
    mism = int(((~np.isfinite(ref)) != (~np.isfinite(img))).sum())
    r = rel[fin]
    return {"max": float(r.max()) if r.size else 0.0, "median": float(np.median(r)) if r.size else 0.0,
            "p99_99": float(np.quantile(r, 0.9999)) if r.size else 0.0, "nonfinite_mismatch": mism}


def config_row(cs, torch, name, params, flush, ops, peaks, steps):
    """Mixed and FP64 kernel rates of one workload, accuracy of mixed vs FP64
    over the full image, and the compute roofline fractions."""
    c = cs.SasCalc_GENERIC_calculation()
    c.setParams(params)
    c.doCalculation(0, False, False, mode=cs.CS_MODE_FP64)
    ref = c.data()
    c.doCalculation(0, False, False, mode=cs.CS_MODE_MIXED)
    img = c.data()
    redo = c.mixed_redo_pixels()
    n = img.size
    npix = c.prepared_pixels()
    d = torch.empty(n, dtype=torch.float64, device="cuda")
    row = {"pixels": npix, "accuracy_mixed_vs_fp64": rel_stats(img, ref), "fp64_redo_pixels": redo}
    for mname, mode, k in (("mixed", cs.CS_MODE_MIXED, steps), ("fp64", cs.CS_MODE_FP64, max(2, steps // 4))):
        tk, _ = time_kernel(c, torch, d, n, k, 2, flush, mode=mode)
        row[mname + "_pixels_per_s"] = npix * k / tk
        row[mname + "_ms_per_image"] = 1e3 * tk / k
    row["speedup_mixed_over_fp64"] = row["mixed_pixels_per_s"] / row["fp64_pixels_per_s"]
    fl = ops[name]["flops_per_pixel"]
    row["compute"] = {"flops_per_pixel": fl,
                      "fp64_dropin_tflops": row["fp64_pixels_per_s"] * fl / 1e12,
                      "fp64_dropin_frac_of_fp64_peak": row["fp64_pixels_per_s"] * fl / 1e12 / peaks["fp64_tflops"],
                      "mixed_tflops": row["mixed_pixels_per_s"] * fl / 1e12,
                      "mixed_frac_of_fp32_peak": row["mixed_pixels_per_s"] * fl / 1e12 / peaks["fp32_tflops"]}
    c.cleanup()
    return row


def sweep(cs, torch, C, nsets, ops, peaks, steps):
    """Config 4: nsets seeded cylinder/BCT parameter sets of detector size
    128..1024 in one batch; one persistent launch per step (captured as a CUDA
    graph) against one plain launch per set, in both precision modes."""
    import numpy as np
    sets = C.bct_sweep(nsets)
    b = cs.SasCalcBatch()
    t0 = time.perf_counter()
    b.prepare(sets, bIgnoreCbs=True)
    t_prep = time.perf_counter() - t0
    total, npix, groups = b.info()
    out = torch.empty(total, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream()
    sp = s.cuda_stream

    def timed(fn, k):
        fn()
        s.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        a.record(s)
        for _ in range(k):
            fn()
        e.record(s)
        e.synchronize()
        return a.elapsed_time(e) / 1e3 / k

    row = {"sets": nsets, "pixels": npix, "key_groups": groups, "host_prep_s": t_prep,
           "image_buffer_gb": total * 8 / 1e9}
    b.capture(out.data_ptr(), total, mode=cs.CS_MODE_MIXED, schedule=cs.CS_SCHED_PERSISTENT)
    row["graph_nodes_persistent"] = b.graph_nodes()
    t_graph = timed(lambda: b.replay(sp), steps)
    redo, cap = b.redo_pixels(sp)
    mixed = out.cpu().numpy()
    t_mp = timed(lambda: b.launch(out.data_ptr(), total, sp, cs.CS_MODE_MIXED, cs.CS_SCHED_PLAIN), 1)
    t_fp = timed(lambda: b.launch(out.data_ptr(), total, sp, cs.CS_MODE_FP64, cs.CS_SCHED_PERSISTENT), 1)
    fp64 = out.cpu().numpy()
    t_fplain = timed(lambda: b.launch(out.data_ptr(), total, sp, cs.CS_MODE_FP64, cs.CS_SCHED_PLAIN), 1)
    fl = ops["bct_sweep"]["flops_per_pixel"]
    row.update({
        "mixed_persistent_graph_s": t_graph, "mixed_persistent_graph_pixels_per_s": npix / t_graph,
        "mixed_plain_launches_s": t_mp, "fp64_persistent_s": t_fp, "fp64_plain_launches_s": t_fplain,
        "fp64_plain_launches_pixels_per_s": npix / t_fplain,
        "speedup_graph_mixed_over_plain_fp64": t_fplain / t_graph,
        "speedup_persistent_over_plain_fp64": t_fplain / t_fp,
        "fp64_redo_pixels": redo, "accuracy_mixed_vs_fp64": rel_stats(mixed, fp64),
        "compute": {"flops_per_pixel_sampled": fl,
                    "mixed_frac_of_fp32_peak": npix / t_graph * fl / 1e12 / peaks["fp32_tflops"],
                    "fp64_plain_frac_of_fp64_peak": npix / t_fplain * fl / 1e12 / peaks["fp64_tflops"]},
        "launches": {"persistent_graph": 2 * groups, "plain": nsets},
    })
    b.cleanup()
    del out
    return row, redo


def surrogate_fits(args):
    """Config 5: the surrogate trained on simulator patterns, then plain fits
    (FP64, one vertex at a time, random start) against surrogate-seeded fits
    (batched, mixed precision) run until they reach the plain fit's chi^2."""
    from crystalscatter_gb300 import surrogate as S
    fam = S.Family(args.surrogate)
    t0 = time.perf_counter()
    U, Y = S.training_set(fam, args.surrogate_train, seed=11)
    t_data = time.perf_counter() - t0
    sur = S.Surrogate(fam, seed=11)
    info = sur.train(U, Y, epochs=args.surrogate_epochs)
    res = S.compare_fits(fam, sur, n_targets=args.surrogate_targets, seed=101)
    res.update({"train_patterns": args.surrogate_train, "pattern_seconds": t_data, "training": info})
    return res


def native(args):
    import numpy as np
    import torch
    import crystalscatter_gb300 as cs
    from crystalscatter_gb300 import configs as C

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    work_stream = torch.cuda.Stream()
    torch.cuda.set_stream(work_stream)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    params = C.WORKLOADS[WORKLOAD]
    ops = load_ops()
    peaks = fp_peaks()

    calc = cs.SasCalc_GENERIC_calculation()
    calc.setParams(params)
    # one drop-in call to prepare (and validate) the parameter set
    calc.doCalculation(0, False, False)
    ref_img = calc.data()
    n = ref_img.size
    npix = calc.prepared_pixels()
    d_out = torch.empty(n, dtype=torch.float64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    # correctness of the device-resident launches against the drop-in image
    calc.launch_prepared(d_out.data_ptr(), n, stream.cuda_stream)
    torch.cuda.synchronize()
    assert np.array_equal(d_out.cpu().numpy().reshape(ref_img.shape), ref_img, equal_nan=True)

    # mixed path (FP32 bulk, FP64 guards): the metric's <= 1e-5 bar, checked here
    calc.doCalculation(0, False, False, mode=cs.CS_MODE_MIXED)
    mixed_img = calc.data()
    redo = calc.mixed_redo_pixels()
    acc = rel_stats(mixed_img, ref_img)
    assert acc["max"] <= 1e-5 and acc["nonfinite_mismatch"] == 0, f"mixed path exceeds 1e-5 vs FP64: {acc}"

    clocks = ClockSampler(local)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    t_kernel, per_step = time_kernel(calc, torch, d_out, n, args.steps, args.warmup, flush, mode=cs.CS_MODE_MIXED)
    t_fp64, _ = time_kernel(calc, torch, d_out, n, args.steps, args.warmup, flush, mode=cs.CS_MODE_FP64)
    # end-to-end: the drop-in call with host buffers (prep + upload + kernel + download)
    for _ in range(args.warmup):
        calc.doCalculation(0, False, False, mode=cs.CS_MODE_MIXED)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        calc.doCalculation(0, False, False, mode=cs.CS_MODE_MIXED)
        _ = calc.data()
    t_e2e = time.perf_counter() - t0
    prep_ms = calc.higResTimerElapsedPrep
    clk = clocks.stop()
    t_kernel, t_e2e, t_fp64 = max_over_ranks([t_kernel, t_e2e, t_fp64], world, "cuda")

    value = replica_rate(npix * args.steps, world, t_kernel)
    e2e = replica_rate(npix * args.steps, world, t_e2e)
    ms_per_step = 1e3 * t_kernel / args.steps

    # roofline: algorithmic HBM bytes per launch = the image (8 B per pixel)
    peak, peak_kind = load_peaks()
    launch_s = t_kernel / args.steps
    bytes_per_launch = 8.0 * npix
    achieved = bytes_per_launch / launch_s / 1e9
    fl = ops[WORKLOAD]["flops_per_pixel"]
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded parameter sets, no dataset)",
        "config": {"workload": "pCyl_lNon_oGau 512x512 (cylinder r=5 L=60, Gaussian 15 deg, phi=30)",
                   "pixels_per_step": npix, "mode": "mixed FP32/FP64, <=1e-5 vs FP64",
                   "l2": "256 MB write between timed steps (flush)", "parallelism": f"replicas x{world}"},
        "accuracy": {"mixed_vs_fp64": acc, "fp64_redo_pixels": redo},
        "fp64_dropin": {"value": npix * args.steps * world / t_fp64, "unit": UNIT,
                        "ms_per_step": 1e3 * t_fp64 / args.steps},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(calc._lib.cs_prepared_size()),
                "d2h_bytes_per_step": int(8 * n), "host_prep_ms": prep_ms},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": TRAFFIC_BYTES_PER_LAUNCH,
                     "note": f"peak {peak_kind}; 8 B written per pixel: the kernels are bound by arithmetic, "
                             f"see compute_roofline and profiles/"},
        "compute_roofline": {"flops_per_pixel": fl, "achieved_tflops": value * fl / 1e12,
                             "fp32_peak_tflops": peaks["fp32_tflops"],
                             "frac_of_fp32_peak": value * fl / 1e12 / peaks["fp32_tflops"],
                             "fp64_peak_tflops": peaks["fp64_tflops"], "peaks": peaks["kind"],
                             "flops_source": "crystalscatter_gb300/config_ops.json (counted on the oracle)"},
        "gpu_launches": 2 * args.steps,
        "clocks": clk,
    }
    if not args.no_extra and rank == 0:
        rows = {}
        for name in ("sphere", "cyl_gauss", "cyl_gauss_x", "sphere_fcc"):
            rows[name] = config_row(cs, torch, name, C.WORKLOADS[name], flush, ops, peaks, max(3, args.steps // 2))
        result["configs"] = rows
        if args.sweep_sets > 0:
            result["sweep"], _ = sweep(cs, torch, C, args.sweep_sets, ops, peaks, max(1, args.sweep_steps))
    if args.surrogate and rank == 0:
        result["surrogate"] = surrogate_fits(args)
    if rank == 0:
        result["cpu_baseline"] = cpu_baseline(params, args.cpu_seconds)
        print(json.dumps(result))
    calc.cleanup()
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


def cpu_baseline(params, seconds):
    """The oracle port of the reference on all host cores, on a bounded sample
    of the same workload: whole calculations (host preparation, as the
    reference's doCalculation runs it, then the image) repeated until
    `seconds` elapse."""
    from oracle import cpu_oracle
    nthreads = os.cpu_count() or 1
    t0 = time.perf_counter()
    pix = 0
    reps = 0
    while True:
        P = cpu_oracle.prepare(params)
        _, n = cpu_oracle.image_prepared(P, nthreads)
        pix += n
        reps += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": pix / dt, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"{reps} full 512x512 calculations (preparation + image) of the same workload, {dt:.1f} s"}


def reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return
    from crystalscatter_gb300 import configs as C
    from oracle import cpu_oracle
    params = C.WORKLOADS[WORKLOAD]
    nthreads = os.cpu_count() or 1
    for _ in range(args.warmup):
        cpu_oracle.image_prepared(cpu_oracle.prepare(params), nthreads)
    t0 = time.perf_counter()
    pix = 0
    for _ in range(args.steps):
        P = cpu_oracle.prepare(params)  # doCalculation prepares on every call
        _, n = cpu_oracle.image_prepared(P, nthreads)
        pix += n
    dt = time.perf_counter() - t0
    value = pix / dt
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded parameter sets, no dataset)",
        "config": {"workload": "pCyl_lNon_oGau 512x512 (cylinder r=5 L=60, Gaussian 15 deg, phi=30)",
                   "pixels_per_step": pix // args.steps, "parallelism": f"{nthreads} host threads"},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": f"{args.steps} full calculations (host preparation + image), the reference's "
                                   f"algorithm restated in C (oracle/cs_oracle.c), row-parallel over host threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def main():
    args = parse()
    if args.impl == "reference":
        reference(args)
    else:
        native(args)


if __name__ == "__main__":
    main()
