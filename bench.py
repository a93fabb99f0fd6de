#!/usr/bin/env python3
"""Benchmark: detector pixels per second of the 2D scattering-pattern
calculation on one GB300 (or N replicas on N GPUs).

Headline workload (one step = one pass over the whole batch): the batched
sweep of cylinders on a BCT lattice with z-direction orientation
(pCyl_pGau_lBCT_oZDi), 4096 seeded parameter sets of detector size
128^2..1024^2 (crystalscatter_gb300.configs.bct_sweep: radius, length, lattice
constants, Schulz widths and orientation width drawn per set), wavelength
0.154 nm, 3 m, pixel 0.172 mm, HKLmax 3 -- 1.41e9 pixels per step. The
mixed-precision kernels run all sets in one persistent launch per step,
replayed as a CUDA graph. Reported:

* value        pixels/s of the graph replays with the prepared batch resident
               in device memory, summed over all ranks
* e2e          the same through the C-ABI host-buffer batch call: host
               parameters in, host preparation, upload, kernels, download of
               all images into pinned host memory, per step
* roofline     the dominant kernel (k_batch_mixed of the sweep's key) against
               the measured issue rate of the pipe that bounds it
               (cs_measure_pipe_peaks), from its executed instructions per
               pixel (ncu, crystalscatter_gb300/kernel_work.json) and its
               CUDA-event duration measured here
* accuracy     mixed vs the FP64 GPU drop-in over every pixel of the sweep,
               and vs the CPU oracle (the reference's algorithm in C, on the
               reference's own prepared constants) on 64 sample sets
* configs      per configuration (sphere 256^2, cylinder 512^2 at phi = 30 and
               phi = 0, FCC spheres 1024^2): mixed and FP64 kernel rates,
               accuracy vs FP64 and vs the CPU oracle, a CPU baseline
* cpu_baseline the CPU oracle on all host cores on a bounded sample of the
               sweep (64 reference-prepared sample sets)

``--impl reference`` times the reference's algorithm on the host cores: the
CPU oracle (oracle/cs_oracle.c, the reference's per-pixel code restated in C;
the reference's own sources cannot travel to the GPU host) on the
reference-prepared sample sets of the same sweep, all host threads, one
sample set per step. It loads no part of this library.
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
SINGLE = ("sphere", "cyl_gauss", "cyl_gauss_x", "sphere_fcc")
WORKLOAD_TEXT = {
    "sphere": "pSph_lNon_oIso 256x256 (sphere r=10, sigma 0.10)",
    "cyl_gauss": "pCyl_lNon_oGau 512x512 (cylinder r=5 L=60, Gaussian 15 deg, phi=30)",
    "cyl_gauss_x": "pCyl_lNon_oGau 512x512 (the same at phi=0: full orientation integral)",
    "sphere_fcc": "pSph_pGau_lFCC_oGau 1024x1024 (sphere r=8 on FCC a=40, HKLmax 5)",
}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--sweep-sets", type=int, default=4096, help="parameter sets of the headline sweep")
    ap.add_argument("--e2e-steps", type=int, default=2, help="steps of the host-buffer (e2e) timing")
    ap.add_argument("--no-extra", action="store_true", help="skip the per-config table")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison legs of the sweep")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--surrogate", default="2,2x",
                    help="config 5: surrogate-seeded fits of these families ('2' as specified, '2x' its phi = 0 "
                         "variant), comma-separated; '' skips them")
    ap.add_argument("--surrogate-train", default="30000,8192",
                    help="training patterns per family (the specification's 200000 for family 2 take ~5 minutes of "
                         "host preparation on a 16-core host: pass them explicitly)")
    ap.add_argument("--surrogate-grid", default="256,64",
                    help="GridPoints of the training patterns per family (256: the 512x512 detector)")
    ap.add_argument("--surrogate-epochs", default="60,150", help="training epochs per family")
    ap.add_argument("--surrogate-targets", default="16,4", help="fit targets per family (of the 1000 specified)")
    return ap.parse_args()


# ------------------------------------------------------------------ helpers

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


def sweep_pixels(nsets):
    """Calculated pixels of the first nsets sweep sets (N^2 each), from the
    seeded parameter draws alone."""
    from crystalscatter_gb300 import configs as C
    return sum(C.bct_set(k)["EditPixelNoX"] ** 2 for k in range(nsets))


def headline_config(nsets, world):
    """The workload description both arms print (identical by construction)."""
    return {"workload": f"pCyl_pGau_lBCT_oZDi batched sweep: {nsets} seeded parameter sets (configs.bct_set), "
                        f"detector 128^2..1024^2, 0.154 nm, 3 m, HKLmax 3",
            "sets_per_step": nsets, "pixels_per_step": sweep_pixels(nsets),
            "mode": "mixed FP32/FP64, <=1e-5 vs FP64",
            "l2": "no flush: each step writes the whole image buffer (11.3 GB for 4096 sets, > 129 MB L2)",
            "parallelism": f"replicas x{world}"}


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


def rel_stats(img, ref, cond=None):
    """max / median / p99.99 of |img - ref| / max(|ref|, tau), tau = 1e-30
    max|ref|, over pixels finite in both; non-finite class mismatches counted.
    With a conditioning map: the count of ill-conditioned pixels (the
    reference's own value moves by more than 1e-12 / 1e-6 under one-ulp
    changes of the math library) and the maximum over the others."""
    import numpy as np
    fin_r = np.isfinite(ref)
    tau = 1e-30 * (np.max(np.abs(ref[fin_r])) if fin_r.any() else 1.0)
    with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
        rel = np.abs(img - ref) / np.maximum(np.abs(ref), tau)
    fin = fin_r & np.isfinite(img)
    mism = int((np.isnan(ref) != np.isnan(img)).sum() + ((np.isinf(ref) | np.isinf(img)) & (ref != img)).sum())
    r = rel[fin]
    out = {"pixels": int(ref.size), "max": float(r.max()) if r.size else 0.0,
           "median": float(np.median(r)) if r.size else 0.0,
           "p99_99": float(np.quantile(r, 0.9999)) if r.size else 0.0, "nonfinite_mismatch": mism}
    if cond is not None:
        good = fin & (cond <= 1e-6)
        out["ill_conditioned_1e-12"] = int((cond > 1e-12).sum())
        out["ill_conditioned_1e-6"] = int((cond > 1e-6).sum())
        out["max_where_cond_le_1e-6"] = float(rel[good].max()) if good.any() else 0.0
    return out


def rel_stats_device(img, ref):
    """rel_stats (without conditioning) of two device tensors, chunked."""
    import torch
    fin_r = torch.isfinite(ref)
    amax = torch.where(fin_r, ref.abs(), torch.zeros_like(ref)).max().item()
    tau = 1e-30 * (amax if amax > 0 else 1.0)
    mx, mism, n = 0.0, 0, 0
    sample = []
    step = 1 << 27
    for a in range(0, ref.numel(), step):
        r = ref[a:a + step]
        g = img[a:a + step]
        fin = torch.isfinite(r) & torch.isfinite(g)
        rel = ((g - r).abs() / torch.clamp(r.abs(), min=tau))[fin]
        if rel.numel():
            mx = max(mx, rel.max().item())
            sample.append(rel[:: max(1, rel.numel() // 200000)].cpu())
        mism += int((torch.isnan(r) != torch.isnan(g)).sum().item())
        mism += int(((torch.isinf(r) | torch.isinf(g)) & (r != g)).sum().item())
        n += r.numel()
    s = torch.cat(sample) if sample else torch.zeros(1, dtype=torch.float64)
    return {"pixels": n, "max": mx, "median": float(s.median().item()),
            "p99_99": float(torch.quantile(s.float(), 0.9999).item()), "nonfinite_mismatch": mism,
            "note": "median and p99.99 from an even subsample of ~200k pixels per 128M"}


def cpu_threads():
    return os.cpu_count() or 1


def load_kernel_work():
    p = os.path.join(ROOT, "crystalscatter_gb300", "kernel_work.json")
    if not os.path.exists(p):
        return {}
    with open(p) as f:
        return json.load(f)


def roofline(work, key, pixels, seconds, peaks, traffic_per_pixel=None):
    """Compute roofline of one kernel launch: executed FP32 / FP64 flops and
    special-function ops per pixel (ncu counts, kernel_work.json) times the
    pixels of the launch over its CUDA-event duration, against the measured
    pipe peaks; the bound is the pipe with the largest fraction."""
    w = work.get(key)
    if not w:
        return None
    fp32_peak = max(peaks["fp32_tflops"], peaks["fp32x2_tflops"])
    rates = {
        "fp32": (w["fp32_flops_per_pixel"] * pixels / seconds / 1e12, fp32_peak, "TFLOP/s"),
        "fp64": (w["fp64_flops_per_pixel"] * pixels / seconds / 1e12, peaks["fp64_tflops"], "TFLOP/s"),
        "sfu": (w["mufu_ops_per_pixel"] * pixels / seconds / 1e12, peaks["mufu_tops"], "Tops/s"),
    }
    bound = max(rates, key=lambda k: rates[k][0] / rates[k][1])
    a, p, u = rates[bound]
    t = w.get("dram_bytes_per_pixel")
    return {"bound": bound, "achieved": a, "peak": p, "unit": u, "frac": a / p,
            "traffic": (t * pixels) if t is not None else None,
            "algorithmic_bytes": 8.0 * pixels,
            "pipes": {k: {"achieved": v[0], "peak": v[1], "unit": v[2], "frac": v[0] / v[1]} for k, v in rates.items()},
            # issue-slot view of the same kernel (ncu, the capture that gave
            # the counts): a DADD or DMUL fills an FP64 issue slot but counts
            # one flop, so the flop fraction reads below the pipe's busy share
            "pipe_active_pct_ncu": {"fp64": w.get("fp64_pipe_pct"), "fma": w.get("fma_pipe_pct"),
                                    "xu": w.get("xu_pipe_pct")},
            "kernel": w.get("kernel"), "kernel_ms": seconds * 1e3, "pixels": pixels,
            "peaks": "measured here (cs_measure_pipe_peaks: FFMA, FFMA2, DFMA, MUFU.EX2 chains)",
            "work_source": w.get("source")}


# ------------------------------------------------------------ CPU baseline

def cpu_baseline_blocks(names, seconds, whole=True):
    """The CPU oracle on all host cores over reference-prepared blocks, whole
    images, cycling through `names` until `seconds` elapse."""
    from oracle import ref_prepared as R
    blocks = [R.load(n) for n in names]
    nt = cpu_threads()
    t0 = time.perf_counter()
    pix, reps, i = 0, 0, 0
    while True:
        _, n = blocks[i % len(blocks)].image(nt)
        pix += n
        reps += 1
        i += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    return {"value": pix / dt, "unit": UNIT, "cores": nt, "kind": "port",
            "sample": f"{reps} whole images ({pix} pixels) of {len(blocks)} reference-prepared parameter set(s), "
                      f"{dt:.1f} s, the reference's per-pixel algorithm restated in C (oracle/cs_oracle.c), "
                      f"rows over {nt} host threads"}


def sweep_sample_names(nsets=None):
    """the reference-prepared sample sets of the sweep (k = 0, 64, ..., 4032),
    those below nsets when given"""
    from oracle import ref_prepared as R
    return [f"bct_set{k:04d}" for k in R.sweep_sample() if nsets is None or k < nsets]


# --------------------------------------------------------------- native arm

def time_kernel(calc, torch, d_out, n, steps, warmup, flush, mode=0):
    """Device-resident launches of the prepared calculation: per step an L2
    flush outside the timed events, then one launch between two events on the
    launching stream. Returns (total seconds over steps, per-step list)."""
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


def config_row(cs, torch, name, flush, steps, cpu_seconds):
    """Mixed and FP64 kernel rates of one workload; accuracy of mixed vs FP64
    (GPU) and of both vs the CPU oracle on the reference-prepared block (whole
    image, or a row sample for the orientation-averaged cylinder); a CPU
    baseline on that block."""
    import numpy as np
    from crystalscatter_gb300 import configs as C
    from oracle import ref_prepared as R
    c = cs.SasCalc_GENERIC_calculation()
    c.setParams(C.WORKLOADS[name])
    c.doCalculation(0, False, False, mode=cs.CS_MODE_FP64)
    ref = c.data()
    c.doCalculation(0, False, False, mode=cs.CS_MODE_MIXED)
    img = c.data()
    redo = c.mixed_redo_pixels()
    n = img.size
    npix = c.prepared_pixels()
    d = torch.empty(n, dtype=torch.float64, device="cuda")
    row = {"workload": WORKLOAD_TEXT[name], "pixels": npix, "accuracy_mixed_vs_fp64": rel_stats(img, ref),
           "fp64_redo_pixels": redo}
    for mname, mode, k in (("mixed", cs.CS_MODE_MIXED, steps), ("fp64", cs.CS_MODE_FP64, max(2, steps // 4))):
        tk, _ = time_kernel(c, torch, d, n, k, 2, flush, mode=mode)
        row[mname + "_pixels_per_s"] = npix * k / tk
        row[mname + "_ms_per_image"] = 1e3 * tk / k
    row["speedup_mixed_over_fp64"] = row["mixed_pixels_per_s"] / row["fp64_pixels_per_s"]
    c.cleanup()
    # main kernel vs FP64 redo: the same set as a one-set batch (persistent
    # kernels), CUDA events around each (cs_batch_profile)
    b = cs.SasCalcBatch()
    b.prepare([C.WORKLOADS[name]])
    total = b.info()[0]
    db = torch.empty(total, dtype=torch.float64, device="cuda")
    prof = [b.profile(db.data_ptr(), total) for _ in range(3)]
    m_ms, r_ms = min(p[0] for p in prof), min(p[1] for p in prof)
    row["split_one_set_batch_ms"] = {"main": m_ms, "redo": r_ms, "redo_share": r_ms / (m_ms + r_ms),
                                     "redo_pixels": b.redo_pixels()[0], "schedule": b.schedule(0)}
    b.cleanup()
    # the CPU oracle on the reference's own prepared constants
    blk = R.load(name)
    nt = cpu_threads()
    if name == "cyl_gauss_x":
        rows = R.sample_rows(blk, 48)
        o, _ = blk.image_rows(rows, nt)
        cond = blk.condition(rows, nt, base=o)
        sel = np.zeros(blk.shape, dtype=bool)
        sel[:, np.asarray(rows) - blk.xmin] = True
        sample = f"{len(rows)} evenly spaced ihex rows ({int(sel.sum())} pixels)"
    else:
        o, _ = blk.image(nt)
        rows = list(range(blk.zzmin, blk.zzmax))
        cond = blk.condition(rows, nt, base=o)
        sel = np.ones(blk.shape, dtype=bool)
        sample = "whole image"
    row["accuracy_vs_cpu"] = {"sample": sample,
                              "mixed": rel_stats(img[sel], o[sel], cond[sel]),
                              "fp64": rel_stats(ref[sel], o[sel], cond[sel])}
    row["cpu_baseline"] = cpu_baseline_blocks([name], cpu_seconds)
    return row


def sweep_accuracy_vs_cpu(b, out_host_view, names, rows_per_set=8):
    """Mixed sweep images vs the CPU oracle on the reference-prepared sample
    sets (row samples), with the oracle's conditioning probe."""
    import numpy as np
    from oracle import ref_prepared as R
    nt = cpu_threads()
    gi, ri, ci = [], [], []
    worst = None  # largest error where the reference is stable to 1e-6: (err, set, ihex, i, got, ref, cond)
    for name in names:
        k = int(name[len("bct_set"):])
        blk = R.load(name)
        rows = R.sample_rows(blk, rows_per_set)
        o, _ = blk.image_rows(rows, nt)
        cond = blk.condition(rows, nt, base=o)
        off, x0, x1, y0, y1 = b.layout(k)
        g = out_host_view(off, (x1 - x0) * (y1 - y0)).reshape(y1 - y0, x1 - x0)
        cols = np.asarray(rows) - blk.xmin
        gs, rs, cs_ = g[:, cols], o[:, cols], cond[:, cols]
        with np.errstate(invalid="ignore", divide="ignore", over="ignore"):
            e = np.abs(gs - rs) / np.maximum(np.abs(rs), 1e-300)
        e = np.where((cs_ <= 1e-6) & np.isfinite(e), e, 0.0)
        j = np.unravel_index(np.argmax(e), e.shape)
        if worst is None or e[j] > worst[0]:
            worst = (float(e[j]), k, int(rows[j[1]]), int(j[0] + blk.ymin), float(gs[j]), float(rs[j]), float(cs_[j]))
        gi.append(gs.ravel())
        ri.append(rs.ravel())
        ci.append(cs_.ravel())
    st = rel_stats(np.concatenate(gi), np.concatenate(ri), np.concatenate(ci))
    if worst is not None:
        st["worst_where_cond_le_1e-6"] = dict(zip(("rel", "set", "ihex", "i", "gpu", "cpu", "cond"), worst))
    st["sample"] = f"{len(names)} reference-prepared sets (k = 0, 64, ...), {rows_per_set} ihex rows each"
    return st


def sweep(cs, torch, C, args, world, peaks, work, clocks_start):
    """The headline: the batched BCT sweep. Returns (result dict, timings)."""
    nsets = args.sweep_sets
    sets = C.bct_sweep(nsets)
    params = [cs.params_from_mapping(s) for s in sets]
    b = cs.SasCalcBatch()
    t0 = time.perf_counter()
    b.prepare(params, bIgnoreCbs=True)
    t_prep = time.perf_counter() - t0
    total, npix, groups = b.info()
    out = torch.empty(total, dtype=torch.float64, device="cuda")
    s = torch.cuda.current_stream()
    sp = s.cuda_stream
    row = {"sets": nsets, "pixels": npix, "key_groups": groups, "host_prep_s": t_prep,
           "image_buffer_gb": total * 8 / 1e9}
    b.capture(out.data_ptr(), total, mode=cs.CS_MODE_MIXED, schedule=cs.CS_SCHED_PERSISTENT)
    row["graph_nodes_persistent"] = b.graph_nodes()

    # timed region: graph replays (persistent mixed kernels + FP64 redo)
    clocks = clocks_start()
    for _ in range(args.warmup):
        b.replay(sp)
    s.synchronize()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    times = []
    for _ in range(args.steps):
        a = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        a.record(s)
        b.replay(sp)
        e.record(s)
        e.synchronize()
        times.append(a.elapsed_time(e) / 1e3)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    t_kernel = sum(times)
    redo, cap = b.redo_pixels(sp)

    def timed(fn):
        fn()
        s.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        e = torch.cuda.Event(enable_timing=True)
        a.record(s)
        fn()
        e.record(s)
        e.synchronize()
        return a.elapsed_time(e) / 1e3

    # the autotuned schedule against the fixed one (block tiles of 256 pixels
    # at the occupancy limit), one persistent launch each
    row["schedule"] = b.schedule(0)
    t_tuned = timed(lambda: b.launch(out.data_ptr(), total, sp, cs.CS_MODE_MIXED, cs.CS_SCHED_PERSISTENT))
    b.set_schedule(0, 0)
    t_fixed = timed(lambda: b.launch(out.data_ptr(), total, sp, cs.CS_MODE_MIXED, cs.CS_SCHED_PERSISTENT))
    b.set_schedule(-1, 0)
    row["schedule_comparison"] = {"tuned_s": t_tuned, "fixed_block_tile_256_s": t_fixed,
                                  "speedup_tuned_over_fixed": t_fixed / t_tuned}
    # the dominant kernel alone: CUDA events around it on its stream
    prof = [b.profile(out.data_ptr(), total, sp, cs.CS_MODE_MIXED) for _ in range(2)]
    main_ms = min(p[0] for p in prof)
    redo_ms = min(p[1] for p in prof)
    row.update({"mixed_persistent_graph_s": t_kernel / args.steps, "step_seconds": times,
                "mixed_kernel_ms": main_ms, "redo_kernel_ms": redo_ms, "fp64_redo_pixels": redo,
                "launches_per_step": {"persistent_graph": 2 * groups}})
    # FP64 drop-in: one plain launch per set (the drop-in's own call pattern)
    if not args.no_fp64:
        ref = torch.empty_like(out)
        t_fplain = timed(lambda: b.launch(ref.data_ptr(), total, sp, cs.CS_MODE_FP64, cs.CS_SCHED_PLAIN))
        t_mplain = timed(lambda: b.launch(out.data_ptr(), total, sp, cs.CS_MODE_MIXED, cs.CS_SCHED_PLAIN))
        b.launch(out.data_ptr(), total, sp, cs.CS_MODE_MIXED, cs.CS_SCHED_PERSISTENT)
        s.synchronize()
        row.update({"fp64_plain_launches_s": t_fplain, "fp64_plain_launches_pixels_per_s": npix / t_fplain,
                    "mixed_plain_launches_s": t_mplain,
                    "speedup_mixed_graph_over_fp64_plain": t_fplain / (t_kernel / args.steps),
                    "speedup_persistent_graph_over_plain_mixed": t_mplain / (t_kernel / args.steps),
                    "accuracy_mixed_vs_fp64": rel_stats_device(out, ref)})
        row["launches_per_step"]["plain"] = nsets
        del ref
    # accuracy vs the CPU oracle on the reference-prepared sample sets
    host = out.cpu()
    hv = host.numpy()
    row["accuracy_vs_cpu"] = sweep_accuracy_vs_cpu(b, lambda o, n: hv[o:o + n], sweep_sample_names(args.sweep_sets))
    del host, hv
    # e2e: the C-ABI host-buffer call, host parameters in, images out
    pinned = torch.empty(total, dtype=torch.float64, pin_memory=True)
    pv = pinned.numpy()
    b2 = cs.SasCalcBatch()
    b2.prepare(params, bIgnoreCbs=True)
    b2.run_host(cs.CS_MODE_MIXED, out=pv)  # warm-up (allocations)
    t0 = time.perf_counter()
    for _ in range(args.e2e_steps):
        b2.prepare(params, bIgnoreCbs=True)
        b2.run_host(cs.CS_MODE_MIXED, out=pv)
    t_e2e = time.perf_counter() - t0
    up = b2.upload_bytes()
    b2.cleanup()
    del pinned, pv
    b.cleanup()
    del out
    return row, {"t_kernel": t_kernel, "t_e2e": t_e2e, "npix": npix, "clocks": clk, "main_ms": main_ms,
                 "upload_bytes": up, "total_doubles": total}


def surrogate_fits(args):
    """Config 5, per family: the surrogate (8 -> 512 -> 512 -> 512 -> 64x64)
    trained on simulator patterns generated on the GPU and averaged to 64 x 64
    there; then per target (Poisson noise, 1e4 counts at the peak, 256 x 256)
    the plain fit (FP64, one vertex at a time, random start), the
    surrogate-seeded fit (batched, mixed precision, until it reaches the plain
    fit's chi^2) and the same batched mixed fit from the random start."""
    from crystalscatter_gb300 import surrogate as S
    fams = [f for f in args.surrogate.split(",") if f]
    def per(v, i, conv):
        parts = str(v).split(",")
        return conv(parts[min(i, len(parts) - 1)])
    out = {}
    for i, name in enumerate(fams):
        n_train = per(args.surrogate_train, i, int)
        grid = per(args.surrogate_grid, i, int)
        epochs = per(args.surrogate_epochs, i, int)
        n_targets = per(args.surrogate_targets, i, int)
        fam = S.Family(name, train_grid=grid)
        t0 = time.perf_counter()
        U, Y, t_prep = S.training_set_device(fam, n_train, seed=11)
        t_data = time.perf_counter() - t0
        sur = S.Surrogate(fam, seed=11)
        info = sur.train(U, Y, epochs=epochs)
        del U, Y
        res = S.compare_fits(fam, sur, n_targets=n_targets, seed=101)
        res.update({"train_patterns": n_train, "pattern_detector": f"{2 * grid}x{2 * grid}",
                    "pattern_seconds": t_data, "pattern_host_prep_seconds": t_prep,
                    "training": {k: v for k, v in info.items() if k != "loss_per_epoch"},
                    "final_loss": info["loss_per_epoch"][-1] if info["loss_per_epoch"] else None,
                    "targets_note": f"{n_targets} of the 1000 specified targets (seeded), the rest not run",
                    "patterns_note": f"{n_train} training patterns (specified: 200000 of family 2)"})
        out[name] = res
    return out


def native(args):
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
    peaks = cs.measure_pipe_peaks()
    work = load_kernel_work()

    def clocks_start():
        c = ClockSampler(local)
        c.start()
        time.sleep(0.3)
        return c

    row, T = sweep(cs, torch, C, args, world, peaks, work, clocks_start)
    t_kernel, t_e2e = max_over_ranks([T["t_kernel"], T["t_e2e"]], world, "cuda")
    npix = T["npix"]
    value = replica_rate(npix * args.steps, world, t_kernel)
    e2e = replica_rate(npix * args.e2e_steps, world, t_e2e)
    key = "0x01020806"
    rl = roofline(work, key, npix, T["main_ms"] / 1e3, peaks)
    result = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_kernel / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64",
        "data": "synthetic (seeded parameter sets, no dataset)",
        "config": headline_config(args.sweep_sets, world),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(T["upload_bytes"]),
                "d2h_bytes_per_step": int(8 * T["total_doubles"]), "steps": args.e2e_steps,
                "path": "SasCalcBatch.prepare(host parameters) + run_host(CS_MODE_MIXED, pinned host buffer): "
                        "cs_batch_prepare (host preparation on all host threads, upload) + cs_batch_run_host "
                        "(persistent kernels, FP64 redo, image download)"},
        "roofline": rl,
        "pipe_peaks": peaks,
        "sweep": row,
        # per replay: the persistent mixed kernel and its FP64 redo kernel per key group
        "gpu_launches": 2 * row["key_groups"] * args.steps,
        "clocks": T["clocks"],
    }
    if rank == 0 and not args.no_extra:
        flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
        result["configs"] = {name: config_row(cs, torch, name, flush, max(3, args.steps // 2),
                                              min(5.0, args.cpu_seconds)) for name in SINGLE}
        del flush
    if args.surrogate and rank == 0:
        result["surrogate"] = surrogate_fits(args)
    if rank == 0:
        result["cpu_baseline"] = cpu_baseline_blocks(sweep_sample_names(), args.cpu_seconds)
        print(json.dumps(result))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# ------------------------------------------------------------ reference arm

def reference(args):
    """The reference's algorithm on the host cores: the CPU oracle on the
    reference-prepared sample sets of the sweep, one whole image per step,
    cycling through the sample (k = 0, 64, ..., 4032)."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    from oracle import ref_prepared as R
    names = sweep_sample_names()
    blocks = [R.load(n) for n in names]
    nt = cpu_threads()
    for i in range(args.warmup):
        blocks[i % len(blocks)].image(nt)
    t0 = time.perf_counter()
    pix = 0
    for i in range(args.steps):
        _, n = blocks[(args.warmup + i) % len(blocks)].image(nt)
        pix += n
    dt = time.perf_counter() - t0
    value = pix / dt
    sample = (f"{args.steps} whole images ({pix} pixels) of the reference-prepared sweep sample sets, one per step, "
              f"the reference's per-pixel algorithm restated in C (oracle/cs_oracle.c), rows over {nt} host threads")
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded parameter sets, no dataset)",
        "config": headline_config(args.sweep_sets, world),
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nt, "kind": "port", "sample": sample},
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
