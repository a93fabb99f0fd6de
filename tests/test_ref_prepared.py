"""The reference-prepared blocks (tests/golden/ref_prepared, written by
tests/golden/make_ref_prepared.py from the reference's own
prepareCalculation) that the benchmark's reference arm, its CPU baselines and
the full-size accuracy checks evaluate with the CPU oracle:

* they load, and the oracle evaluates them, in a process that never maps this
  library (the reference arm must not depend on it);
* on every benchmark workload and a spread of sweep sets, the oracle's values
  from the reference's block equal, bit for bit, its values from this
  library's own preparation of the same parameters (which pins the export as
  well as the library's preparation);
* the benchmark's two arms describe the same workload."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from oracle import cpu_oracle, ref_prepared as R  # noqa: E402


def test_index_covers_the_sweep_sample_and_workloads():
    idx = R.index()
    assert idx["sweep_sample"] == list(range(0, 4096, 64))
    for name in ["sphere", "cyl_gauss", "cyl_gauss_x", "sphere_fcc"] + [f"bct_set{k:04d}" for k in idx["sweep_sample"]]:
        assert name in idx["blocks"], name


def test_blocks_evaluate_without_the_library():
    code = (
        "import sys; sys.path.insert(0, %r)\n"
        "from oracle import ref_prepared as R\n"
        "b = R.load('bct_set0064'); img, n = b.image_rows(R.sample_rows(b, 4), 2)\n"
        "assert n == 4 * (b.iimax - b.iimin) and (img != 0).any()\n"
        "maps = open('/proc/self/maps').read()\n"
        "assert 'libcrystalscatter' not in maps, 'library mapped'\n"
        "print('ok')\n" % ROOT)
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stderr


@pytest.mark.parametrize("name", ["sphere", "cyl_gauss", "cyl_gauss_x", "sphere_fcc", "bct_set0000", "bct_set0448",
                                  "bct_set1984", "bct_set4032"])
def test_reference_block_equals_library_preparation(name):
    blk = R.load(name)
    P = cpu_oracle.prepare(blk.params, blk.ign_cbs)
    rows = R.sample_rows(blk, 3)
    a, _ = blk.image_rows(rows, 4)
    lib = cpu_oracle.load()
    b = np.zeros_like(a)
    rl = np.asarray(rows, dtype=np.int32)
    import ctypes
    lib.oracle_image_rowlist(ctypes.byref(P), b.ctypes.data, rl.ctypes.data, len(rl), 4)
    assert np.array_equal(a, b, equal_nan=True), name


def test_bench_arms_share_the_workload_description():
    import bench
    c = bench.headline_config(4096, 1)
    assert c == bench.headline_config(4096, 1)
    assert c["pixels_per_step"] == 1408368640
