"""Fit-target file formats: the program's saved images (.dat/.csv/.txt), the
no-fit rectangles, KWS and EDF detector files and the beam-stop centre
finder, on synthetic files built byte by byte in the formats the reference
reads and writes (Source/widimage.cpp:1480-1500 and :154-166,
Source/sc_readdata.cpp:534-1010 and :1769-2121)."""
import struct

import numpy as np
import pytest

from crystalscatter_gb300 import readers as R


def _image(minX=-4, maxX=5, minY=-3, maxY=3, seed=1):
    rng = np.random.default_rng(seed)
    data = rng.uniform(1e-6, 2.0, size=(maxY - minY, maxX - minX))
    return R.Image(data, minX, maxX, minY, maxY, {"ComboBoxParticle": "sphere {0}", "EditRadius": "10"})


def test_dat_bytes_pinned(tmp_path):
    # header "%4d %4d %4d %4d" (19 bytes), then doubles, y outer, x inner
    vals = [[1.5, -2.25, 3.0], [4.0, 5.5, 6.125]]
    raw = b"  -1    2    0    2" + b"".join(struct.pack("<d", v) for row in vals for v in row)
    fn = tmp_path / "img.dat"
    fn.write_bytes(raw)
    img = R.read_sascrystal_dat(str(fn))
    assert (img.minX, img.maxX, img.minY, img.maxY) == (-1, 2, 0, 2)
    assert np.array_equal(img.data, np.array(vals))
    assert img.get(-1, 1) == 4.0 and img.get(1, 0) == 3.0


def test_dat_bad_sizes(tmp_path):
    fn = tmp_path / "bad.dat"
    fn.write_bytes(b"   0    2    0    2" + struct.pack("<3d", 1, 2, 3))
    with pytest.raises(ValueError):
        R.read_sascrystal_dat(str(fn))
    fn.write_bytes(b"garbage header!!!!!" + struct.pack("<4d", 1, 2, 3, 4))
    with pytest.raises(ValueError):
        R.read_sascrystal_dat(str(fn))


def test_round_trip_dat_csv(tmp_path):
    img = _image()
    base = str(tmp_path / "saved")
    R.write_sascrystal(img, base)
    a = R.read_sascrystal_dat(base + ".dat")
    b = R.read_sascrystal_csv(base + ".csv")
    assert np.array_equal(a.data, img.data)
    assert (a.minX, a.maxX, a.minY, a.maxY) == (img.minX, img.maxX, img.minY, img.maxY)
    # the CSV reader returns extents 0..cols, 0..rows with the values in file order
    assert (b.minX, b.maxX, b.minY, b.maxY) == (0, img.cols, 0, img.rows)
    assert np.array_equal(b.data, img.data)
    assert b.meta["NbRows"] == str(img.rows) and b.meta["NbCols"] == str(img.cols)
    assert b.meta["ComboBoxParticle"] == "sphere {0}" and a.meta["EditRadius"] == "10"


def test_csv_needs_metadata(tmp_path):
    base = str(tmp_path / "x")
    R.write_sascrystal(_image(), base)
    (tmp_path / "x.txt").unlink()
    assert R.read_sascrystal_csv(base + ".csv") is None


def test_csv_six_digit_values(tmp_path):
    # the reference writes six significant digits; short rows and stray lines are skipped
    (tmp_path / "s.csv").write_text("X:;0;3\nY:;0;2\nY=0:;1e-06;2.5;3\nnoise\nY=1:;4;5.25e+02;6\n")
    (tmp_path / "s.txt").write_text("From File\tignored\nEditRadius\t7\n")
    img = R.read_sascrystal_csv(str(tmp_path / "s.csv"))
    assert np.array_equal(img.data, np.array([[1e-6, 2.5, 3.0], [4.0, 525.0, 6.0]]))
    assert img.meta["EditRadius"] == "7" and img.meta["From File"].endswith("s.csv")


def test_nofit(tmp_path):
    fn = str(tmp_path / "img.dat")
    assert R.read_nofit(fn) == [(-1, -1, -1, -1)] * 4
    (tmp_path / "img.dat.nofit").write_text("2 2 10 12\n30 40 50 60\n0 0\n")
    rects = R.read_nofit(fn)
    assert rects == [(2, 2, 10, 12), (30, 40, 50, 60), (0, 0, -1, -1), (-1, -1, -1, -1)]
    # a .csv image takes the .dat.nofit file
    assert R.read_nofit(str(tmp_path / "img.csv")) == rects

    class Rec:
        def __init__(self):
            self.calls = []

        def setNoFitRect(self, *a):
            self.calls.append(a)

    rec = Rec()
    R.apply_nofit(rec, rects)
    assert rec.calls[1] == (1, 30, 40, 50, 60) and len(rec.calls) == 4


def _kws_text(n, wl="lambda= 6.0A", det_rows=("[m]  x  y  z", "1  8.0  0  0"), neg=True):
    counts = np.arange(n * n, dtype=float) % 97
    if neg:
        counts[5] = -3.0
    lines = ["(* Comment *)", f"  sample run {wl}", "(* Detector Discription *)"]
    lines += list(det_rows)
    lines += ["(* Data *)", "$"]
    for i in range(0, n * n, 8):
        lines.append(" ".join(f"{v:g}" for v in counts[i:i + 8]))
    lines.append("")
    return "\n".join(lines), np.maximum(counts, 0).reshape(n, n)


@pytest.mark.parametrize("n,beam", [(128, 64), (144, 72)])
def test_kws(tmp_path, n, beam):
    text, want = _kws_text(n)
    fn = tmp_path / "run.kws"
    fn.write_text(text)
    img = R.read_kws(str(fn))
    assert np.array_equal(img.data, want)
    assert img.meta["wavelength"] == "0.6 nm"
    assert img.meta["SampleDist"] == "8.0 m"
    assert img.meta["BeamPosX"] == str(beam) and img.meta["Pixel_X"] == "5.3"


def test_kws_nm_and_rejects(tmp_path):
    text, _ = _kws_text(128, wl="lambda= 0.45n", det_rows=())
    fn = tmp_path / "a.kws"
    fn.write_text(text)
    img = R.read_kws(str(fn))
    assert img.meta["wavelength"] == "0.45 nm" and img.meta["SampleDist"] == "4.0 m"
    fn.write_text("Data columns: x y\n1 2 3 4 5 6 7 8\n")
    assert R.read_kws(str(fn)) is None  # a 2D-SANS file; not a 2D-SANS extension
    text, _ = _kws_text(128)
    fn.write_text(text.replace("$\n", "$\n1 2 3 4 5 6 7 8\n", 1))
    with pytest.raises(ValueError):
        R.read_kws(str(fn))


def _beamstop_image(cx, cy, hw, hh, n=64):
    data = np.ones((n, n))
    data[cy - hh:cy + hh + 1, cx - hw:cx + hw + 1] = 0.0
    return R.Image(data, 0, n, 0, n)


def test_beam_center_walk_from_inside():
    img = _beamstop_image(30, 20, 4, 3)
    assert R.find_beam_center(img, 31, 21) == (30, 20)


def test_beam_center_search():
    # start outside the shadow: the widest inner runs of each row and column
    img = _beamstop_image(40, 25, 5, 2)
    x, y = R.find_beam_center(img, 5, 5)
    assert (x, y) == (40, 25)
    # a shadow run of at most 2 pixels is not taken: the full extent remains
    img = _beamstop_image(40, 25, 0, 0)
    assert R.find_beam_center(img, 5, 5) == ((0 + 63) // 2, (0 + 63) // 2)


def test_beam_center_negative_extents():
    data = np.ones((9, 11))
    data[3:6, 4:7] = 0.0
    img = R.Image(data, -5, 6, -4, 5)
    # shadow x in -1..1, y in -1..1
    assert R.find_beam_center(img, 0, 0) == (0, 0)


def _edf_bytes(kind, data, dtype, order="LowByteFirst", extra=()):
    n = data.shape[0]
    bo = "<" if order == "LowByteFirst" else ">"
    body = data.astype(bo + dtype).tobytes()
    names = {"f4": "FloatValue", "i4": "SignedInteger", "u2": "UnsignedShort", "f8": "DoubleValue"}
    if kind == "K1":
        hdr = ["EDF_DataBlockID = 0.Image.Psd ;", f"EDF_BinarySize = {len(body)} ;", "EDF_HeaderSize = 1024 ;",
               f"ByteOrder = {order} ;", f"DataType = {names[dtype]} ;", f"Dim_1 = {n} ;", f"Dim_2 = {n} ;",
               "Title = test image ;", "Center_1 = 12.5 ;", "Center_2 = 7 ;", "PSize_1 = 0.000172 ;",
               "PSize_2 = 0.000172 ;", "SampleDistance = 3.2 ;", "WaveLength = 1.54e-10 ;"]
    else:
        hdr = ["HeaderID = EH:000001:000000:000000 ;", f"ByteOrder = {order} ;", f"DataType = {names[dtype]} ;",
               f"Dim_1 = {n} ;", f"Dim_2 = {n} ;", f"Size = {len(body)} ;"]
    hdr += list(extra)
    text = "{\n" + "\n".join(hdr) + "\n"
    text += " " * ((-(len(text) + 2)) % 512) + "}\n"
    return text.encode("latin-1") + body


@pytest.mark.parametrize("dtype", ["f4", "i4", "u2", "f8"])
@pytest.mark.parametrize("order", ["LowByteFirst", "HighByteFirst"])
def test_edf_types_and_layout(tmp_path, dtype, order):
    n = 9
    rng = np.random.default_rng(3)
    filedata = rng.integers(0, 60000, size=(n, n)).astype(np.float64)
    if dtype in ("f4", "f8"):
        filedata = filedata / 7.0
    fn = tmp_path / "a.edf"
    fn.write_bytes(_edf_bytes("K1", filedata, dtype, order))
    img = R.read_edf(str(fn))
    want = filedata.astype(dtype).astype(np.float64)
    if order == "HighByteFirst":
        # the reference reads both byte orders as little-endian (its swap is a no-op)
        want = np.frombuffer(filedata.astype(">" + dtype).tobytes(), "<" + dtype).reshape(n, n).astype(np.float64)
    # file pixel (r, c) lands at x = n-1-r, y = c
    for r, c in [(0, 0), (0, 5), (3, 2), (8, 8)]:
        assert img.get(n - 1 - r, c) == want[r, c]
    assert img.meta["FileType"] == "K1" and img.meta["BeamPosX"] == "12.5" and img.meta["BeamPosY"] == "7"
    assert img.meta["Pixel_x"] == "0.172" and img.meta["SampleDist"] == "3.2"
    assert img.meta["wavelength"] == "0.154" and img.meta["Title"] == "test image"


def test_edf_e1_defaults_and_rejects(tmp_path):
    n = 7
    data = np.arange(n * n, dtype=np.float64).reshape(n, n)
    fn = tmp_path / "b.edf"
    fn.write_bytes(_edf_bytes("E1", data, "f4"))
    img = R.read_edf(str(fn))
    assert img.meta["FileType"] == "E1" and img.meta["BeamPosX"] == "4"  # round(3.5) = 4
    assert img.meta["Pixel_x"] == "0.26" and img.meta["wavelength"] == "0.124"
    assert img.get(n - 1, 0) == 0.0 and img.get(0, n - 1) == data[n - 1, n - 1]
    fn.write_bytes(b"{\nEDF_DataFormatVersion = 2.0 ;\n}\n")
    assert R.read_edf(str(fn)) is None
    bad = _edf_bytes("K1", data, "f4").replace(b"DataType = FloatValue", b"DataType = Complex128  ")
    fn.write_bytes(bad)
    with pytest.raises(ValueError):
        R.read_edf(str(fn))


def test_spreadsheet(tmp_path):
    n = 20
    data = np.ones((n, n)) * 3.0
    data[8:13, 5:10] = 0.0  # beam stop centred at x = 7, y = 10
    lines = [f"    {n}    {n} Start pixel = (       1       1)"]
    for r in range(n):
        lines.append("  " + " ".join(f"{v:13.6e}" for v in data[r]))
    fn = tmp_path / "img.spr"
    fn.write_text("\n".join(lines) + "\n")
    img = R.read_spreadsheet(str(fn))
    assert np.array_equal(img.data, data)
    assert img.get(7, 10) == 0.0
    assert (img.meta["BeamPosX"], img.meta["BeamPosY"]) == ("7", "10")
    fn.write_text("no header\n1 2\n")
    assert R.read_spreadsheet(str(fn)) is None
