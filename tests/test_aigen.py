"""The training-data generator's file loop (crystalscatter_gb300/aigen.py,
generateAIfiles) on the CPU, with a stand-in calculation: settings and TPV
lines, the reference's file names, the text images and the post-processing
(noise, beam stop, detector lines, r-phi) in its order."""
import math

import numpy as np
import pytest

import crystalscatter_gb300 as cs
from crystalscatter_gb300 import aigen, tpv


class FakeCalc(aigen.HostRphi):
    """A smooth image around the beam on a 32 x 32 detector (x, y in -16..16)."""

    def __init__(self):
        self.params = cs.default_params()
        self.params.radius = 10.0
        self.calls = 0

    def update_param(self, key, value):
        field = {"EditRadius": "radius", "EditSigma": "sigma", "Length": "length"}[key]
        setattr(self.params, field, value)

    def beam_pos(self):
        return self.params.beamx, self.params.beamy

    def compute(self):
        self.calls += 1
        xs, ys = np.meshgrid(np.arange(-16, 16), np.arange(-16, 16))
        img = 1.0 + self.params.radius * np.exp(-((xs - 0.5) ** 2 + ys ** 2) / 60.0)
        return img, -16, 16, -16, 16


def read_spr(fn):
    with open(fn) as f:
        lines = f.read().split("\n")
    sx, sy = [int(t) for t in lines[0].split()[:2]]
    assert lines[0] == f"    {sx}    {sy} Start pixel = (       1       1)"
    rows = []
    for y in range(sy):
        body = lines[1 + y]
        assert body.startswith("  ") and (len(body) - 1) == 14 * sx
        rows.append([float(body[1 + 14 * i:1 + 14 * (i + 1)]) for i in range(sx)])
    return np.array(rows)


def test_named_images_and_file_names(tmp_path):
    f = tmp_path / "gen.txt"
    f.write_text(f"PATH|{tmp_path}/out\nCOLTBL|*gray\nsize|EditRadius=10.500|EditSigma=0.100\n"
                 "size|#FN_Length=12.25|EditRadius=7\nsize|#DEF|EditRadius=8\n")
    calc = FakeCalc()
    log = aigen.generate_ai_files(calc, str(f))
    out = tmp_path / "out" / "size"
    names = sorted(p.name for p in out.iterdir())
    # "_EditRadius=10.500_EditSigma=0.100": "Edit" dropped, "0_" -> "_", trailing zeros cut
    assert names == ["Length=12.25.spr", "Radius=10.5_Sigma=0.1.spr", "Radius=8_DEF.spr"], names
    img = read_spr(out / "Radius=10.5_Sigma=0.1.spr")
    xs, ys = np.meshgrid(np.arange(-16, 16), np.arange(-16, 16))
    want = 1.0 + 10.5 * np.exp(-((xs - 0.5) ** 2 + ys ** 2) / 60.0)
    assert np.allclose(img, want, rtol=1e-6, atol=0)
    assert any("PNG output is not built" in s for s in log) is False


def test_tpv_postprocessing_in_the_reference_order(tmp_path):
    f = tmp_path / "gen.txt"
    f.write_text(f"PATH|{tmp_path}/o\nCOLTBL|*\nRPHI|16;Scale\nTPV|BS0.2;0.2;0.5;0.5|LI1;1;2;1|NO|RP|IX\n"
                 "run|#FAC=3|EditRadius=0.1\n")
    calc = FakeCalc()
    tpv.srand(123)
    log = aigen.generate_ai_files(calc, str(f))
    scat = sorted(p.name for p in (tmp_path / "o" / "scat").iterdir())
    assert scat == ["scat_0.spr", "scat_1.spr", "scat_2.spr"]
    assert sorted(p.name for p in (tmp_path / "o" / "rphi").iterdir()) == ["rphi_0.spr", "rphi_1.spr", "rphi_2.spr"]
    assert sorted(p.name for p in (tmp_path / "o" / "scat_org").iterdir()) == scat
    assert sum("TPV: no random values" in s for s in log) == 1  # the last of the #FAC images
    # the draws: randomised radius, then noise per pixel, beam stop (4), lines (1 + 1)
    tpv.srand(123)
    p = cs.default_params()
    p.radius = 10.0
    r = tpv.TpvRandom()
    r.perform(p, ["EditRadius=0.1"])
    xs, ys = np.meshgrid(np.arange(-16, 16), np.arange(-16, 16))
    base = 1.0 + p.radius * np.exp(-((xs - 0.5) ** 2 + ys ** 2) / 60.0)
    assert np.allclose(read_spr(tmp_path / "o" / "scat_org" / "scat_2.spr"), base, rtol=1e-6, atol=0)
    flat = base.reshape(-1).copy()
    for i in range(flat.size):
        flat[i] = flat[i] + tpv.zuf() * math.sqrt(flat[i])
    bx = int(0 * (1 + 0.2 * tpv.zuf()))
    by = int(0 * (1 + 0.2 * tpv.zuf()))
    dx = int(2 * (1 + 0.5 * tpv.zuf()))
    dy = int(2 * (1 + 0.5 * tpv.zuf()))
    img = flat.reshape(32, 32)
    img[by - dy + 16:by + dy + 17, bx - dx + 16:bx + dx + 17] = 0
    xp = int(-16 + abs(tpv.zuf()) * 33)
    img[:, xp + 16:xp + 18] = 0
    yp = int(-16 + abs(tpv.zuf()) * 33)
    img[yp + 16:yp + 17, :] = 0
    got = read_spr(tmp_path / "o" / "scat" / "scat_2.spr")
    assert np.allclose(got, img, rtol=1e-6, atol=1e-12)
    rphi = read_spr(tmp_path / "o" / "rphi" / "rphi_2.spr")
    assert rphi.shape == (16, 16) and np.nanmax(rphi) <= 1.0 + 1e-12


def test_string_form_and_settings():
    calc = FakeCalc()
    log = aigen.generate_ai_files(calc, "@PATH|/nonexistent-dir-for-test@@x")
    assert calc.calls == 0 and log == []


@pytest.mark.parametrize("v,txt", [(1.5, "  1.500000e+00"), (-12.25, " -1.225000e+01"), (float("nan"), "           nan")])
def test_text_number_format(v, txt):
    assert " " + aigen._e13(v) == txt
