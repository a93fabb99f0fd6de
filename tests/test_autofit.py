"""The command-file driven fit (crystalscatter_gb300/autofit.py,
automaticFit) on the CPU with a stand-in calculation and fit: the command
set, the fit loop's stop rule, per-loop logs and per-file results."""
import os

import numpy as np

from crystalscatter_gb300 import autofit


class FakeCalc:
    params = None

    def __init__(self):
        self.v = {k: 1.0 for k in autofit.FIT_KEYS}
        self.v["EditRadius"] = 10.0
        self.saved = []

    def value(self, key):
        return self.v.get(key, 0.0)

    def update_param(self, key, value):
        self.v[key] = value

    def save(self, path):
        with open(path, "w") as f:
            for k in sorted(self.v):
                f.write(f"{k}={self.v[k]!r}\n")
        self.saved.append(path)


def half_way(target):
    calls = []

    def fit(calc, image, table, stp, maxit, tol, border, bstop):
        calls.append((table, stp, maxit, tol, border, bstop, image.data.shape))
        res = {t["key"]: (t["start"] + target) / 2 if t["used"] else t["start"] for t in table}
        return res, {"ms": 1.0, "repetitions": 3, "images": 7}
    return fit, calls


def write_spr(fn, n=12):
    rows = [f"    {n}    {n} Start pixel = (       1       1)"]
    for r in range(n):
        rows.append("  " + " ".join(f"{1.0 + r + c:13.6e}" for c in range(n)))
    fn.write_text("\n".join(rows) + "\n")


def test_command_file_over_a_directory(tmp_path):
    d = tmp_path / "data"
    d.mkdir()
    write_spr(d / "b_img.spr")
    write_spr(d / "a_img.spr")
    (d / "skip.txt").write_text("x")
    par = tmp_path / "start.ini"
    par.write_text("[General]\nEditRadius=10\nEditSigma=0.1\n")
    cmd = tmp_path / "fit.cmd"
    cmd.write_text("\n".join([
        "# autofit test",
        "GlobLog: log",
        f"Param: {par}",
        "DirMask: *.spr",
        f"DirUp: {d}",
        "Limits: EditRadius; 1; 50",
        "Use: EditRadius  # the radius only",
        "Border: 2; 0; 1",
        "Fit: Stp=3.0; Iter=20; Tol=0.001; Diff<5; Kenn=run",
        "EOF",
        "Fit: Iter=99",
    ]) + "\n")
    calc = FakeCalc()
    fit, calls = half_way(12.0)
    out = tmp_path / "out"
    log = autofit.automatic_fit(calc, str(cmd), outdir=str(out), fit=fit)
    # two images in ascending order; the first takes two loops (10 -> 11:
    # 10 %, 11 -> 11.5: 4.5 % < 5 %), the second one (11.5 -> 11.75: 2.2 %)
    assert [os.path.basename(p) for p in calc.saved] == ["a_img_out.ini", "b_img_out.ini"]
    assert len(calls) == 3
    table, stp, maxit, tol, border, bstop, shape = calls[0]
    radius = [t for t in table if t["key"] == "EditRadius"][0]
    assert (radius["min"], radius["max"], radius["used"]) == (1.0, 50.0, True)
    assert sum(t["used"] for t in table) == 1
    assert (stp, maxit, tol, border, bstop, shape) == (0.03, 20, 0.001, 2, -1, (12, 12))
    assert calc.v["EditRadius"] == 11.75 and calc.v["EditSigma"] == 0.1
    assert sorted(os.listdir(out)) == ["a_img_out.ini", "b_img_out.ini", "run-01_calc.log", "run-02_calc.log"]
    assert "MeanDiff=4.54545" in (out / "run-02_calc.log").read_text()
    assert any(s.startswith("Dir (Up) 2 files found.") for s in log)


def test_no_parameter_used(tmp_path):
    cmd = tmp_path / "c.cmd"
    cmd.write_text("Use: NoSuchKey\nFit: Stp=1\n")
    log = autofit.automatic_fit(FakeCalc(), str(cmd), fit=half_way(1.0)[0])
    assert log[-1] == "ERROR no parameter used: Use: NoSuchKey"


def test_single_image_argument(tmp_path):
    img = tmp_path / "one.spr"
    write_spr(img, 8)
    cmd = tmp_path / "c.cmd"
    cmd.write_text("Use: EditRadius, I0\nFit: Diff<100\n")
    calc = FakeCalc()
    fit, calls = half_way(20.0)
    autofit.automatic_fit(calc, str(cmd), imgfile=str(img), outdir=str(tmp_path / "o"), fit=fit)
    # loop 1: 10 -> 15 (50 %), 1 -> 10.5 (950 %); loop 2: 16.7 % and 45 %, mean 31 % < 100 %
    assert len(calls) == 2 and calc.v["EditRadius"] == 17.5 and calc.v["I0"] == 15.25
    assert os.path.exists(tmp_path / "o" / "one_out.ini")
    assert np.isclose(calls[0][1], 0.03)
