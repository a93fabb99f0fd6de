"""Generates the prepared blocks of the benchmark workloads from the
reference's own host preparation (tests/golden/ref_prepared/*.npz).

The reference's CPU path (oracle/_ref/libscref.so, built from the reference
sources by oracle/build_ref.sh) prepares each parameter set
(checkAllParameters + prepareCalculation); oracle/ref_driver.cpp's
ref_export_prepared writes its constants into the prepared-block layout that
the CPU oracle evaluates. The benchmark's reference arm and CPU baseline, and
the full-size accuracy checks, run the oracle on these blocks, so neither
depends on this library's own preparation. Each file holds the block as raw
bytes, the image extents and the parameter dictionary.

Workloads: the four single-image workloads of crystalscatter_gb300.configs
(sphere 256^2, cylinder 512^2 at phi = 30 and phi = 0, FCC spheres 1024^2) and
a fixed sample of the cylinder/BCT sweep: sets k = 0, 64, ..., 4032 of
configs.bct_set (64 sets, every detector size). Usage (needs the reference
sources and the built oracle/_ref):

    python tests/golden/make_ref_prepared.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from crystalscatter_gb300 import configs as C  # noqa: E402
from oracle import refbind  # noqa: E402

OUT = os.path.join(HERE, "ref_prepared")
SWEEP_SAMPLE = list(range(0, 4096, 64))


def workloads():
    w = {name: (p, 0) for name, p in C.WORKLOADS.items()}
    for k in SWEEP_SAMPLE:
        w[f"bct_set{k:04d}"] = (C.bct_set(k), 1)  # cylinder on BCT needs bIgnoreCbs
    return w


def main():
    if not refbind.available():
        sys.exit("oracle/_ref/libscref.so not built (oracle/build_ref.sh)")
    os.makedirs(OUT, exist_ok=True)
    index = {}
    for name, (p, ign_cbs) in workloads().items():
        blob, err = refbind.prepared_block(p, 0, ign_cbs)
        assert blob is not None, (name, err)
        r = refbind.RefCalc(p)
        r.close()
        np.savez_compressed(os.path.join(OUT, name + ".npz"), block=np.frombuffer(blob, dtype=np.uint8),
                            params=json.dumps(p, sort_keys=True), ign_cbs=ign_cbs)
        index[name] = {"ign_cbs": ign_cbs, "bytes": len(blob)}
        print(name, len(blob))
    with open(os.path.join(OUT, "index.json"), "w") as f:
        json.dump({"sweep_sample": SWEEP_SAMPLE, "blocks": index}, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
