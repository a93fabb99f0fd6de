"""Prepared blocks made by the reference's own host preparation.

TEST INFRASTRUCTURE: the benchmark's reference arm and CPU baseline and the
full-size accuracy checks evaluate the CPU oracle (oracle/cs_oracle.c) on these
blocks, so they depend on neither this library's preparation nor its shared
library. The blocks are fixtures (tests/golden/ref_prepared/*.npz) written by
tests/golden/make_ref_prepared.py from the reference's prepareCalculation
(Source/sc_calc_generic_cpu.cpp:319-988) through oracle/ref_driver.cpp's
ref_export_prepared; loading them needs only numpy and the oracle library.
"""
import ctypes
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DIR = os.path.join(os.path.dirname(HERE), "tests", "golden", "ref_prepared")


def index():
    with open(os.path.join(DIR, "index.json")) as f:
        return json.load(f)


def sweep_sample():
    """Set numbers k of the cylinder/BCT sweep that have a reference block."""
    return list(index()["sweep_sample"])


class Block:
    """One prepared parameter set: the raw block (a ctypes buffer the oracle
    reads), its parameters, extents and calculated region."""

    def __init__(self, name):
        d = np.load(os.path.join(DIR, name + ".npz"))
        raw = d["block"].tobytes()
        self.name = name
        self.buf = ctypes.create_string_buffer(raw, len(raw))
        self.params = json.loads(str(d["params"]))
        self.ign_cbs = int(d["ign_cbs"])
        from oracle import cpu_oracle
        lib = cpu_oracle.load()
        e = (ctypes.c_int * 9)()
        lib.oracle_extents(self.buf, e)
        self.xmin, self.xmax, self.ymin, self.ymax, self.zzmin, self.zzmax, self.iimin, self.iimax, self.key = list(e)

    @property
    def shape(self):
        return (self.ymax - self.ymin, self.xmax - self.xmin)

    @property
    def pixels(self):
        """calculated pixels"""
        return (self.zzmax - self.zzmin) * (self.iimax - self.iimin)

    def image(self, nthreads=None, rows=None):
        """The oracle's image (all ihex rows, or rows [r0, r1)); returns
        (image, pixels computed)."""
        from oracle import cpu_oracle
        lib = cpu_oracle.load()
        out = np.zeros(self.shape, dtype=np.float64)
        r0, r1 = rows if rows else (0, 0)
        n = lib.oracle_image_rows(self.buf, out.ctypes.data, int(r0), int(r1), int(nthreads or os.cpu_count() or 1))
        return out, n


    def image_rows(self, rows, nthreads=None, probe_mode=None):
        """The oracle's values on the listed ihex rows (a sample of the image;
        other pixels stay 0); probe_mode: evaluate with the one-ulp math
        library probe (oracle/cs_oracle.c) in that mode. Returns (image, pixels
        computed)."""
        from oracle import cpu_oracle
        rl = np.ascontiguousarray(rows, dtype=np.int32)
        out = np.zeros(self.shape, dtype=np.float64)
        nt = int(nthreads or os.cpu_count() or 1)
        if probe_mode is None:
            lib = cpu_oracle.load()
        else:
            lib = cpu_oracle.load_probe()
            lib.oracle_set_probe(int(probe_mode))
        n = lib.oracle_image_rowlist(self.buf, out.ctypes.data, rl.ctypes.data, len(rl), nt)
        if probe_mode is not None:
            lib.oracle_set_probe(0)
        return out, n

    def condition(self, rows, nthreads=None, base=None):
        """Per-pixel sensitivity of the reference computation on the listed
        rows to one-ulp changes of the math library: the largest
        |I_mode - I| / max(|I|, tau) over the probe modes (tau = 1e-30 max|I|);
        a non-finite disagreement counts as inf. Pixels off the rows are 0."""
        from oracle import cpu_oracle
        if base is None:
            base, _ = self.image_rows(rows, nthreads)
        cond = np.zeros(base.shape)
        fin = np.isfinite(base)
        tau = 1e-30 * (np.max(np.abs(base[fin])) if fin.any() else 1.0)
        for m in cpu_oracle.PROBE_MODES:
            out, _ = self.image_rows(rows, nthreads, probe_mode=m)
            with np.errstate(invalid="ignore", over="ignore"):
                d = np.abs(out - base) / np.maximum(np.abs(base), tau)
            same_nf = (~np.isfinite(base)) & ((np.isnan(base) & np.isnan(out)) | (base == out))
            d[same_nf] = 0.0
            d[~np.isfinite(d)] = np.inf
            cond = np.maximum(cond, d)
        return cond


def sample_rows(block, count):
    """`count` ihex rows spread evenly over the block's calculated region
    (all rows when it has fewer)."""
    n = block.zzmax - block.zzmin
    if count >= n:
        return list(range(block.zzmin, block.zzmax))
    return sorted(set(block.zzmin + (np.arange(count) * n) // count))


def load(name):
    return Block(name)
