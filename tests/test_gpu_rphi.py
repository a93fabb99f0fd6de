"""The GPU r-phi transform (cs_rphi_device) against the reference's own
generateRphi outputs (tests/golden/rphi.npz) and against the numpy
restatement postproc.rphi on larger images."""
import os
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import crystalscatter_gb300 as cs  # noqa: E402
from crystalscatter_gb300 import postproc  # noqa: E402

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from make_rphi_golden import CASES, image  # noqa: E402

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "rphi.npz")


def _flags(f):
    return dict(scale=bool(f & 1), clip=bool(f & 2), clip40=bool(f & 4))


@pytest.mark.parametrize("k", range(len(CASES)))
def test_rphi_device_matches_reference_golden(k):
    z = np.load(GOLDEN)
    ref = z[f"ref{k}"]
    x0, x1, y0, y1, xc, yc, s, f = (int(v) for v in z[f"args{k}"])
    d = image(x1 - x0, y1 - y0, 100 + k)
    got = cs.rphi_device(torch.from_numpy(d).cuda(), x0, x1, y0, y1, xc, yc, s, **_flags(f)).cpu().numpy()
    written = ~np.isnan(ref)
    assert written.sum() > 0.8 * s * s
    # entries the reference leaves unwritten are 0 here (after clip: 0 maps to 0)
    assert np.all(got[~written] == 0.0)
    # FP64 bilinear averages; only the device's sin/cos differ from the host's
    scale = np.max(np.abs(ref[written]))
    assert np.max(np.abs(got[written] - ref[written])) <= 1e-12 * scale


@pytest.mark.parametrize("n,s,xc,yc,f", [(512, 256, 0, 0, 0), (600, 384, 37, -51, 1), (1024, 512, 100, 20, 3)])
def test_rphi_device_matches_restatement_large(n, s, xc, yc, f):
    d = image(n, n, n + s)
    ref = postproc.rphi(d, -n // 2, n // 2, -n // 2, n // 2, xc, yc, s, **_flags(f))
    got = cs.rphi_device(torch.from_numpy(d).cuda(), -n // 2, n // 2, -n // 2, n // 2, xc, yc, s,
                         **_flags(f)).cpu().numpy()
    assert np.max(np.abs(got - ref)) <= 1e-12 * np.max(np.abs(ref))


def test_rphi_device_rejects_positive_minimum():
    d = torch.zeros((8, 8), dtype=torch.float64, device="cuda")
    with pytest.raises(cs.CrystalScatterError):
        cs.rphi_device(d, 1, 9, 0, 8, 4, 4, 8)
