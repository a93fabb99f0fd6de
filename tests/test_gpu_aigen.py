"""The training-data generator's loop with the library's GPU calculation and
GPU r-phi transform (aigen.LibraryCalc): the images it writes, and its r-phi
images against the host restatement on the same inputs."""
import numpy as np
import pytest

import crystalscatter_gb300 as cs
from crystalscatter_gb300 import aigen, configs, postproc, tpv

pytestmark = pytest.mark.gpu


class RecordingCalc(aigen.LibraryCalc):
    def __init__(self, params):
        super().__init__(params, mode=cs.CS_MODE_FP64)
        self.seen = []

    def rphi(self, image, x0, x1, y0, y1, bx, by, size, scale, clip, clip40):
        out = super().rphi(image, x0, x1, y0, y1, bx, by, size, scale, clip, clip40)
        self.seen.append((np.array(image), x0, x1, y0, y1, bx, by, size, scale, clip, clip40, np.array(out)))
        return out


def test_generator_on_the_gpu(tmp_path):
    p = cs.params_from_mapping(configs.scaled(configs.SPHERE, 16))
    calc = RecordingCalc(p)
    f = tmp_path / "gen.txt"
    f.write_text(f"PATH|{tmp_path}/o\nCOLTBL|*\nRPHI|24;Scale\nTPV|BS0.2;0.2;0.5;0.5|NO|RP\nrun|#FAC=2|EditRadius=0.1\n")
    tpv.srand(7)
    aigen.generate_ai_files(calc, str(f))
    assert sorted(x.name for x in (tmp_path / "o" / "scat").iterdir()) == ["scat_0.spr", "scat_1.spr"]
    assert sorted(x.name for x in (tmp_path / "o" / "rphi").iterdir()) == ["rphi_0.spr", "rphi_1.spr"]
    assert len(calc.seen) == 2
    for img, x0, x1, y0, y1, bx, by, size, sc, cl, c40, out in calc.seen:
        want = postproc.rphi(img, x0, x1, y0, y1, bx, by, size, sc, cl, c40)
        assert out.shape == (size, size)
        assert np.max(np.abs(out - want)) <= 1e-12 * max(np.max(np.abs(want)), 1e-300)
