"""Batches of parameter sets (cs_batch_*): one persistent launch per dispatch
key over a device tile queue, the per-set plain schedule, and CUDA-graph
capture/replay.

Every batch image must equal, bit for bit, the image the single-set call
computes for the same parameter set in the same precision mode (the pixel
arithmetic is the same code; only the scheduling differs), and the golden
cases must meet the same bars as the single-set tests (1e-10 FP64, 1e-5
mixed; where the reference is ill-conditioned, against the quadruple-precision
value of its algorithm, helpers.compare_with_exact)."""
import numpy as np
import pytest

import crystalscatter_gb300 as cs
from crystalscatter_gb300 import configs as C
from helpers import compare_with_exact, golden, golden_cases, written_mask

pytestmark = pytest.mark.gpu

CASES = golden_cases()["images"]
NAMES = sorted(CASES)


def single(params, ign_cbs, mode):
    c = cs.SasCalc_GENERIC_calculation()
    c.setParams(params)
    c.doCalculation(0, False, bool(ign_cbs), mode=mode)
    img = c.data()
    c.cleanup()
    return img


def same_bits(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def golden_batch():
    # every golden case in one batch: several dispatch keys (several persistent
    # launches), mirrored quadrants, beam offsets, midpoint geometry
    sets = [CASES[n]["params"] for n in NAMES]
    b = cs.SasCalcBatch()
    b.prepare(sets, bIgnoreCbs=True)
    return b


@pytest.fixture(scope="module")
def gbatch():
    b = golden_batch()
    yield b
    b.cleanup()


def test_layout(gbatch):
    total, pixels, groups = gbatch.info()
    assert groups >= 4
    end = 0
    for k, n in enumerate(NAMES):
        o, x0, x1, y0, y1 = gbatch.layout(k)
        assert o % 32 == 0 and o >= end
        end = o + (x1 - x0) * (y1 - y0)
        assert [x0, x1, y0, y1] == [int(v) for v in golden(n)["dims"]]
    assert end <= total


@pytest.mark.parametrize("mode", [cs.CS_MODE_FP64, cs.CS_MODE_MIXED])
def test_batch_equals_single_calls_and_reference(gbatch, mode):
    imgs = gbatch.split(gbatch.run_host(mode))
    tol = 1e-10 if mode == cs.CS_MODE_FP64 else 1e-5
    for n, img in zip(NAMES, imgs):
        case = CASES[n]
        ref = single(case["params"], case["ign_cbs"], mode)
        assert same_bits(img, ref), n
        g = golden(n)
        r = compare_with_exact(img, g, mask=written_mask(case["params"], img.shape), tol=tol)
        assert r["n_bad"] == 0, (n, r)
        assert r["max_rel_well"] <= tol, (n, r)


@pytest.mark.parametrize("mode", [cs.CS_MODE_FP64, cs.CS_MODE_MIXED])
def test_plain_schedule_graph_and_persistent_agree(gbatch, mode):
    import torch
    total = gbatch.info()[0]
    s = torch.cuda.Stream()
    outs = []
    for sched in (cs.CS_SCHED_PLAIN, cs.CS_SCHED_PERSISTENT):
        d = torch.full((total,), -1.0, dtype=torch.float64, device="cuda")
        gbatch.launch(d.data_ptr(), total, s.cuda_stream, mode=mode, schedule=sched)
        s.synchronize()
        outs.append(d.cpu().numpy())
    ref = gbatch.run_host(mode)
    imgs = [gbatch.split(o) for o in outs] + [gbatch.split(ref)]
    for k in range(len(NAMES)):
        assert same_bits(imgs[0][k], imgs[2][k]), NAMES[k]
        assert same_bits(imgs[1][k], imgs[2][k]), NAMES[k]
    # captured once, replayed twice into a buffer that is poisoned in between
    for sched in (cs.CS_SCHED_PLAIN, cs.CS_SCHED_PERSISTENT):
        d = torch.full((total,), -1.0, dtype=torch.float64, device="cuda")
        gbatch.capture(d.data_ptr(), total, mode=mode, schedule=sched)
        nodes = gbatch.graph_nodes()
        assert nodes >= (len(NAMES) if sched == cs.CS_SCHED_PLAIN else 2)
        for _ in range(2):
            d.fill_(-1.0)
            torch.cuda.synchronize()
            gbatch.replay(s.cuda_stream)
            s.synchronize()
            got = gbatch.split(d.cpu().numpy())
            for k in range(len(NAMES)):
                assert same_bits(got[k], imgs[2][k]), (sched, NAMES[k])


def test_sweep_sets_of_uneven_size():
    # parameter sets of the cylinder/BCT sweep at four detector sizes in one
    # persistent launch; each image equals its single-set call
    sets = [C.scaled(C.bct_set(k), g) for k, g in zip(range(8), (8, 16, 24, 32, 8, 16, 24, 32))]
    b = cs.SasCalcBatch()
    for mode in (cs.CS_MODE_FP64, cs.CS_MODE_MIXED):
        imgs = b.calc(sets, bIgnoreCbs=True, mode=mode)
        for p, img in zip(sets, imgs):
            assert same_bits(img, single(p, 1, mode))
    b.cleanup()


def test_rejected_set_fails_batch_with_index():
    bad = dict(C.scaled(C.bct_set(1), 8))  # cylinder on BCT without bIgnoreCbs
    sets = [C.scaled(C.SPHERE, 8), bad]
    b = cs.SasCalcBatch()
    with pytest.raises(cs.CrystalScatterError) as e:
        b.prepare(sets, bIgnoreCbs=False)
    assert e.value.code == cs.CS_ERR_PARAM
    assert str(e.value).find("set 1:") >= 0
    b.cleanup()


def test_redo_overflow_is_reported_and_recovered():
    import torch
    sets = [C.scaled(C.CYL_GAUSS_X, 16), C.scaled(C.CYL_GAUSS_X, 24)]
    b = cs.SasCalcBatch()
    b.prepare(sets)
    ref = b.run_host(cs.CS_MODE_MIXED)
    n, cap = b.redo_pixels()
    b.set_redo_capacity(1)
    total = b.info()[0]
    d = torch.zeros(total, dtype=torch.float64, device="cuda")
    b.launch(d.data_ptr(), total, 0, mode=cs.CS_MODE_MIXED)
    if n > 1:
        with pytest.raises(cs.CrystalScatterError) as e:
            b.redo_pixels()
        assert e.value.code == cs.CS_ERR_SIZE
    # the host form grows the list and runs again
    got = b.run_host(cs.CS_MODE_MIXED)
    assert same_bits(got, ref)
    b.cleanup()
