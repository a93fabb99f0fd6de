"""Measured and saved 2D images as fit targets.

Host-side readers for the image files the reference loads as fit data, with
the same layout and metadata keys, so that a target can go straight to
``SasCalc_GENERIC_calculation.setFitData``:

* the program's own saved images (``<name>.csv`` with ``<name>.txt``
  metadata, ``Source/sc_readdata.cpp:534-650``; the binary ``<name>.dat``
  written by ``Source/widimage.cpp:1480-1500``);
* the no-fit rectangles saved beside an image (``<image>.nofit``,
  ``Source/widimage.cpp:154-166`` and ``:243-262``);
* KWS detector files (``Source/sc_readdata.cpp:655-876``);
* EDF detector files (``Source/sc_readdata.cpp:1769-2121``);
* SAXSLAB/Pilatus TIFF files (``Source/sc_readdata.cpp:24-520``);
* 2D-SANS (ILL) images, text and XML (``Source/sc_readdata.cpp:1466-1767``);
* spreadsheet text images (``Source/sc_readdata.cpp:2123-2190``);
* the beam-stop centre finder (``SC_ReadData::findBeamCenter``,
  ``Source/sc_readdata.cpp:878-1010``).

Numbers are parsed as Qt's ``QString::toDouble``/``toInt`` parse them (the
whole text, else 0). Every reader is pinned to the reference's own readers,
compiled from ``Source/sc_readdata.cpp`` with Qt stand-ins, on committed
input files (``tests/test_readers_ref.py``).

An image is returned as :class:`Image`: ``data`` has shape (rows, cols) =
(maxY - minY, maxX - minX), row y holds x = minX .. maxX - 1 (the order of
the files and of ``setFitData``), and ``meta`` holds the metadata strings
under the reference's keys.
"""
import math
import os
import re
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Image:
    data: np.ndarray
    minX: int
    maxX: int
    minY: int
    maxY: int
    meta: dict = field(default_factory=dict)

    @property
    def rows(self):
        return self.maxY - self.minY

    @property
    def cols(self):
        return self.maxX - self.minX

    def get(self, x, y):
        """Value at detector coordinates (x, y), like widImage::getData."""
        return self.data[y - self.minY, x - self.minX]


_QT_NUMBER = re.compile(r"[+-]?(\d+\.?\d*|\.\d+)([eE][+-]?\d+)?|[+-]?(inf|nan)")


def _qt_double(text):
    """QString::toDouble: the whole text (white space around it allowed) as a
    number, else 0."""
    t = text.strip()
    return float(t) if _QT_NUMBER.fullmatch(t) else 0.0


def _qt_int(text):
    """QString::toInt: the whole text as a decimal integer, else 0."""
    t = text.strip()
    return int(t) if re.fullmatch(r"[+-]?\d+", t) else 0


def _base(path):
    root, _ = os.path.splitext(path)
    return root


def read_sascrystal_csv(path):
    """A saved image: ``<base>.csv`` and its ``<base>.txt`` metadata.

    The CSV holds ``X:;minX;maxX``, ``Y:;minY;maxY`` and one ``Y=<y>:;v;v;...``
    line per row. As in the reference, the image is returned with extents
    0..cols, 0..rows (the values in file order), its metadata from the
    tab-separated ``.txt`` plus ``From File``, ``NbRows`` and ``NbCols``.
    Returns None when either file is missing, like the reference."""
    base = _base(path)
    fncsv, fntxt = base + ".csv", base + ".txt"
    if not (os.path.exists(fncsv) and os.path.exists(fntxt)):
        return None
    vals = []
    nrows = ncols = 0
    with open(fncsv, "r", errors="replace") as f:
        for line in f:
            sl = [t for t in line.strip().split(";") if t != ""]
            if len(sl) < 2:
                continue
            if sl[0] == "X:":
                ncols = _qt_int(sl[2]) - _qt_int(sl[1])
            elif sl[0] == "Y:":
                nrows = _qt_int(sl[2]) - _qt_int(sl[1])
            elif sl[0].startswith("Y=") and len(sl) > ncols:
                vals.extend(_qt_double(t) for t in sl[1:])
    data = np.asarray(vals, dtype=np.float64)
    if data.size != nrows * ncols:
        raise ValueError(f"{fncsv}: {data.size} values for {nrows} x {ncols}")
    meta = {"From File": fncsv, "NbRows": str(nrows), "NbCols": str(ncols)}
    meta.update(_read_meta(fntxt))
    return Image(data.reshape(nrows, ncols), 0, ncols, 0, nrows, meta)


def _read_meta(fntxt):
    meta = {}
    with open(fntxt, "r", errors="replace") as f:
        for line in f:
            sl = [t for t in line.strip().split("\t") if t != ""]
            if len(sl) < 2 or sl[0] in ("From File", "NbRows", "NbCols"):
                continue
            meta[sl[0]] = sl[1]
    return meta


DAT_HEADER_BYTES = 19  # "%4d %4d %4d %4d" of minX maxX minY maxY


def read_sascrystal_dat(path):
    """The binary image file: a 19-byte text header with minX, maxX, minY,
    maxY (each right-aligned in 4 characters), then the values as native
    little-endian doubles, y outer, x inner. The ``.txt`` beside it, if
    present, supplies the metadata."""
    with open(path, "rb") as f:
        raw = f.read()
    head = raw[:DAT_HEADER_BYTES].decode("ascii", errors="replace").split()
    if len(head) != 4:
        raise ValueError(f"{path}: header {raw[:DAT_HEADER_BYTES]!r} is not four integers")
    minX, maxX, minY, maxY = (int(t) for t in head)
    n = (maxX - minX) * (maxY - minY)
    body = raw[DAT_HEADER_BYTES:]
    if len(body) != 8 * n:
        raise ValueError(f"{path}: {len(body)} bytes of data for {n} doubles")
    data = np.frombuffer(body, dtype="<f8").reshape(maxY - minY, maxX - minX).copy()
    meta = {"From File": path}
    fntxt = _base(path) + ".txt"
    if os.path.exists(fntxt):
        meta.update(_read_meta(fntxt))
    return Image(data, minX, maxX, minY, maxY, meta)


def write_sascrystal(img, base):
    """Writes ``<base>.dat`` and ``<base>.csv`` (and ``<base>.txt`` from
    ``img.meta``) in the formats above, for round trips and for handing a
    computed image to the reference's GUI."""
    with open(base + ".dat", "wb") as f:
        f.write(f"{img.minX:4d} {img.maxX:4d} {img.minY:4d} {img.maxY:4d}".encode("ascii"))
        f.write(np.ascontiguousarray(img.data, dtype="<f8").tobytes())
    with open(base + ".csv", "w") as f:
        f.write(f"X:;{img.minX};{img.maxX}\n")
        f.write(f"Y:;{img.minY};{img.maxY}\n")
        for r in range(img.rows):
            f.write(f"Y={img.minY + r}:" + "".join(";" + repr(float(v)) for v in img.data[r]) + "\n")
    with open(base + ".txt", "w") as f:
        for k, v in img.meta.items():
            f.write(f"{k}\t{v}\n")


def read_nofit(path):
    """The four no-fit rectangles saved beside an image as (left, top, right,
    bottom) tuples; missing numbers read as -1 and a missing file as four
    unused rectangles, as in the reference. For a ``.csv`` image the file is
    ``<base>.dat.nofit``, otherwise ``<image>.nofit``."""
    if path.lower().endswith(".csv"):
        fn = path[:-4] + ".dat.nofit"
    else:
        fn = path + ".nofit"
    rects = [(-1, -1, -1, -1)] * 4
    if not os.path.exists(fn):
        return rects
    with open(fn, "r", errors="replace") as f:
        lines = f.read().split("\n")
    out = []
    for i in range(4):
        sl = lines[i].split() if i < len(lines) else []
        while len(sl) < 4:
            sl.append("-1")
        out.append(tuple(int(t) for t in sl[:4]))
    return out


def apply_nofit(calc, rects):
    """Hands the rectangles to ``setNoFitRect`` (index 0..3)."""
    for i, (x0, y0, x1, y1) in enumerate(rects):
        calc.setNoFitRect(i, x0, y0, x1, y1)


_KWS_SIZES = {128 * 128: (128, 64), 144 * 144: (144, 72), 256 * 256: (256, 128)}


def read_kws(path):
    """A KWS detector file: a header up to the line starting with ``$`` (the
    wavelength from ``lambda=`` after the comment marker, in nm, converted
    from Angstrom when it ends in ``A``; the sample-detector distance from the
    detector description table), then whitespace-separated counts (lines of
    at least 8 numbers; negative counts read as 0). 128², 144² and 256²
    detectors are recognised, with the beam at the centre and 5.3 mm pixels.
    Files whose first 40 lines name ``Data columns`` are 2D-SANS files and go
    to :func:`read_2dsans`."""
    with open(path, "r", errors="replace") as f:
        lines = f.read().split("\n")
    for line in lines[:40]:
        if "Data columns" in line.strip():
            return read_2dsans(path)  # a 2D-SANS file, as the reference decides
    is_hdr = True
    look_lambda = look_det = False
    det_hdr = True
    wavelen, detpos = "0.5 nm", "4.0 m"
    vals = []
    for line in lines:
        line = line.strip()
        if is_hdr:
            if line.startswith("(* Comment *)"):
                look_lambda = True
            elif look_lambda and "lambda=" in line:
                look_lambda = False
                rest = line[line.index("lambda=") + 7:]
                wl = _qt_double(rest[:-1])  # the unit's last letter cut off; "0.45nm" reads as 0
                if rest.endswith("A"):
                    wl = wl / 10
                wavelen = f"{wl:g} nm"
            if line.startswith("(* Detector Discription *)"):
                look_det = True
            elif look_det:
                if line.startswith("(*"):
                    look_det = False
                elif det_hdr and line[:1] == "[":
                    det_hdr = False
                elif not det_hdr:
                    sl = line.split()
                    if len(sl) == 4:
                        detpos = sl[1] + " m"
            if line.startswith("$"):
                is_hdr = False
            continue
        sl = line.split()
        if len(sl) < 8:
            continue
        vals.extend(max(_qt_double(t), 0.0) for t in sl)
    if len(vals) not in _KWS_SIZES:
        raise ValueError(f"{path}: {len(vals)} values, not a 128², 144² or 256² detector")
    n, beam = _KWS_SIZES[len(vals)]
    meta = {"From File": path, "NbRows": str(n), "NbCols": str(n), "BeamPosX": str(beam),
            "BeamPosY": str(beam), "wavelength": wavelen, "EditWAXSangle": "0.0 deg", "SampleDist": detpos,
            "Pixel_X": "5.3", "Pixel_Y": "5.3"}
    return Image(np.asarray(vals, dtype=np.float64).reshape(n, n), 0, n, 0, n, meta)


_EDF_TYPES = {
    ("FloatValue", 4): "f4", ("FloatIEEE32", 4): "f4",
    ("SignedInteger", 4): "i4", ("Signed32", 4): "i4", ("SignedLong", 4): "i4",
    ("UnsignedShort", 2): "u2", ("Unsigned16", 2): "u2",
    ("DoubleValue", 8): "f8", ("DoubleIEEE64", 8): "f8",
}

_EDF_K1_KEYS = ["EDF_BinarySize", "EDF_HeaderSize", "ByteOrder", "DataType", "Dim_1", "Dim_2", "Title",
                "ExposureTime", "Center_1", "Center_2", "PSize_1", "PSize_2", "SampleDistance", "WaveLength",
                "DetectorPosition"]


def _fmt_num(v):
    # QString::number(double): up to 6 significant digits
    return f"{v:.6g}"


def read_edf(path):
    """An EDF detector file with one data block. The header runs from the
    line starting with ``{`` to the line holding ``}``; the data follow that
    line. Two header kinds are read as in the reference:

    * ``EDF_DataBlockID`` first ("K1"): sizes, byte order, type, centre,
      pixel size (m, reported in mm), sample distance (m) and wavelength (m,
      reported in nm) from their keys;
    * ``HeaderID`` first ("E1"): byte order, type, Dim_1/Dim_2 and Size, with
      the beam at the centre, 0.26 mm pixels, 5.005 m and 0.124 nm.

    ``EDF_DataFormatVersion`` headers are not read (None), as in the
    reference. Types: 32-bit float and signed integer, 16-bit unsigned, 64-bit
    float; both byte orders are read as little-endian, as the reference's
    byte swap leaves the bytes as they are. Pixel k of the file (row r = k / Dim_1,
    column c = k % Dim_1) lands at x = rows - 1 - r, y = c, the reference's
    layout, which is defined for square detectors (others raise
    ValueError). Each record is read once; the reference's loops for the types
    other than little-endian float also visit one record past every
    2048-byte block (a stale value that shifts the pixels after it, and a
    write past the image at the end), which is not reproduced."""
    with open(path, "rb") as f:
        raw = f.read()
    pos = 0

    def readline():
        nonlocal pos
        if pos >= len(raw):
            return None
        e = raw.find(b"\n", pos)
        e = len(raw) if e < 0 else e + 1
        line = raw[pos:e]
        pos = e
        return line.decode("latin-1").strip()

    while True:
        line = readline()
        if line is None or line.startswith("{"):
            break
    vals = {"EDF_BinarySize": 0, "EDF_HeaderSize": 0, "ByteOrder": "", "DataType": "", "Dim_1": 0, "Dim_2": 0,
            "Title": "", "ExposureTime": 0.0, "Center_1": 0.0, "Center_2": 0.0, "PSize_1": 0.0, "PSize_2": 0.0,
            "SampleDistance": 0.0, "WaveLength": 0.0, "DetectorPosition": 0.0}
    line = readline() or ""

    def header(keys):
        while True:
            ln = readline()
            if ln is None or "}" in ln:
                return
            tmp = ln.split(" = ")
            if len(tmp) < 2:
                continue
            v = tmp[1]
            if v.endswith(";"):
                v = v[:-1].strip()
            if tmp[0] in keys:
                yield tmp[0], v

    def num(v, conv):
        return _qt_int(v) if conv is int else _qt_double(v)

    if line.startswith("EDF_DataBlockID"):
        file_type = "K1"
        for k, v in header(_EDF_K1_KEYS):
            if k in ("EDF_BinarySize", "EDF_HeaderSize", "Dim_1", "Dim_2"):
                vals[k] = num(v, int)
            elif k in ("ByteOrder", "DataType", "Title"):
                vals[k] = v
            else:
                vals[k] = num(v, float)
        beam_x, beam_y = vals["Center_1"], vals["Center_2"]
        pixel_x, pixel_y = 1e3 * vals["PSize_1"], 1e3 * vals["PSize_2"]
        dist, wavelen = vals["SampleDistance"], 1e9 * vals["WaveLength"]
    elif line.startswith("EDF_DataFormatVersion"):
        return None
    elif line.startswith("HeaderID"):
        file_type = "E1"
        for k, v in header(["ByteOrder", "DataType", "Dim_1", "Dim_2", "Size"]):
            if k == "Size":
                vals["EDF_BinarySize"] = num(v, int)
            elif k in ("Dim_1", "Dim_2"):
                vals[k] = num(v, int)
            else:
                vals[k] = v
        # C round(): halves away from zero
        beam_x = float(math.floor(vals["Dim_1"] / 2.0 + 0.5))
        beam_y = float(math.floor(vals["Dim_2"] / 2.0 + 0.5))
        pixel_x = pixel_y = 0.260
        dist, wavelen = 5.005, 1.24e-1
    else:
        raise ValueError(f"{path}: unknown EDF header kind {line!r}")
    ncols, nrows = vals["Dim_1"], vals["Dim_2"]
    if ncols <= 0 or nrows <= 0:
        raise ValueError(f"{path}: image size {ncols} x {nrows}")
    if ncols != nrows:
        raise ValueError(f"{path}: the EDF pixel layout is defined for square detectors only")
    rec = vals["EDF_BinarySize"] // ncols // nrows
    key = (vals["DataType"], rec)
    if key not in _EDF_TYPES:
        raise ValueError(f"{path}: data type {vals['DataType']} with {rec}-byte records is not supported")
    # the reference's byte swap for HighByteFirst (SC_ReadData::swapBytes)
    # copies the unswapped bytes back over its reversed copy: both orders are
    # read as little-endian
    order = "<"
    n = ncols * nrows
    body = raw[pos:pos + n * rec]
    if len(body) < n * rec:
        raise ValueError(f"{path}: {len(body)} data bytes for {n} records of {rec}")
    flat = np.frombuffer(body, dtype=order + _EDF_TYPES[key]).astype(np.float64)
    # x = rows - 1 - r, y = c  ->  out[c, rows-1-r] = file[r, c]
    data = flat.reshape(nrows, ncols)[::-1].T.copy()
    meta = {"From File": path, "NbRows": str(nrows), "NbCols": str(ncols), "BeamPosX": _fmt_num(beam_x),
            "BeamPosY": _fmt_num(beam_y), "FileType": file_type, "Pixel_x": _fmt_num(pixel_x),
            "Pixel_y": _fmt_num(pixel_y), "SampleDist": _fmt_num(dist), "wavelength": _fmt_num(wavelen),
            "EditWAXSangle": "0.0 deg", "EDF_BinarySize": str(vals["EDF_BinarySize"]),
            "headSize": str(vals["EDF_HeaderSize"]), "ByteOrder": vals["ByteOrder"], "DataType": vals["DataType"],
            "Title": vals["Title"], "ExposureTime": _fmt_num(vals["ExposureTime"]),
            "DetectorPos": _fmt_num(vals["DetectorPosition"]), "@": ""}
    return Image(data, 0, ncols, 0, nrows, meta)


def read_spreadsheet(path):
    """A text image whose first line is ``<rows> <cols> Start pixel = ...``
    followed by one line of values per row (lines with fewer than ``cols``
    values are skipped, and count against the rows). The beam position starts
    at (cols/2, rows/2) and is then placed at the beam-stop centre
    (:func:`find_beam_center`), as the reference does for these files, which
    carry no metadata. Returns None when the first line has no ``Start
    pixel``."""
    with open(path, "r", errors="replace") as f:
        lines = f.read().split("\n")
    first = lines[0].strip() if lines else ""
    pos = first.find("Start pixel")
    if pos < 0:
        return None
    sl = first[:pos].split()
    nrows, ncols = int(sl[0]), int(sl[1])
    vals = []
    for line in lines[1:1 + nrows]:
        sl = line.split()
        if len(sl) < ncols:
            continue
        vals.extend(_qt_double(t) for t in sl)
    if len(vals) != nrows * ncols:
        raise ValueError(f"{path}: {len(vals)} values for {nrows} x {ncols}")
    img = Image(np.asarray(vals, dtype=np.float64).reshape(nrows, ncols), 0, ncols, 0, nrows,
                {"From File": path, "NbRows": str(nrows), "NbCols": str(ncols)})
    bx, by = find_beam_center(img, ncols // 2, nrows // 2)
    img.meta["BeamPosX"] = str(bx)
    img.meta["BeamPosY"] = str(by)
    return img


def _tiff_xml_params(window):
    """The name/value pairs the reference scrapes from the 20000 bytes that
    start at ``<?xml version=``: a double quote opens a name, the next one
    closes it and starts its value, which runs (without ``<`` and ``>``)
    up to the next ``<``. The scan starts at the window's second byte and
    runs over whatever follows the XML (binary data included); a name whose
    first character is NUL (or an empty name) drops every pair collected so
    far and ends the scan. The XML declaration's pair is dropped."""
    names, vals = [], []
    pstart = nstart = False
    for ii in range(1, len(window)):
        c = chr(window[ii])
        if pstart and c != '"':
            names[-1] += c
        if nstart and c != ">" and c != "<":
            vals[-1] += c
        if nstart and c == "<":
            nstart = False
        if c == '"':
            if not pstart:
                pstart = True
                names.append("")
                vals.append("")
            else:
                pstart = False
                nstart = True
                if names[-1][:1] in ("", "\0"):
                    names, vals = [], []
                    break
    if names:
        names.pop(0)
        vals.pop(0)
    return names, vals


def read_tiff(path):
    """A SAXSLAB/Pilatus TIFF image (``Source/sc_readdata.cpp:24-520``): the
    parameters of its XML header (see :func:`_tiff_xml_params`; the file must
    hold 20000 bytes from the header's start, else None), then the TIFF
    directory's width, length, bits per sample, compression (1 only, else
    None), photometric interpretation (0 or 1, else None), strip offset and
    samples per pixel (1 only, else None), each added to the meta information
    as the reference names it. As in the reference, the header's third byte
    must be 42 (``II*`` files; a big-endian ``MM`` file has 0 there and is not
    read), and every number of the directory is read little-endian.

    Pixel values: 8-bit signed characters, 16-bit signed integers (both
    stored transposed, at x = row, y = column, which the reference defines
    for square images only), 32-bit signed integers (little-endian files:
    row r at y = rows-1-r; ``MM*`` files: unswapped, transposed). Where the
    reference's loops would write outside the image (1 and 2 bytes per pixel,
    or a big-endian file, with data following the image in the last 2048-byte
    block) or leave pixels unwritten, ValueError."""
    with open(path, "rb") as f:
        raw = f.read()
    head = raw[:20000]
    anf = 0
    for i in range(5, len(head)):
        if head.startswith(b"<?xml version=", i):
            anf = i
            break
    window = raw[anf:anf + 20000]
    if len(window) != 20000:
        return None
    names, vals = _tiff_xml_params(window)
    if len(raw) < 8 or raw[:2] not in (b"II", b"MM") or raw[2] != 42:
        return None
    little = raw[:2] == b"II"

    def i32(off):
        return int.from_bytes(raw[off:off + 4].ljust(4, b"\0"), "little", signed=True)

    pos = i32(4)
    ntags = int.from_bytes(raw[pos:pos + 2].ljust(2, b"\0"), "little", signed=True)
    pos += 2
    ncols = nrows = bps = strip = 0
    for _ in range(max(ntags, 0)):
        code = int.from_bytes(raw[pos:pos + 2], "little")
        nval, val = i32(pos + 4), i32(pos + 8)
        pos += 12
        if code == 256 and nval == 1:
            ncols = val
            names.append("NbCols")
            vals.append(str(ncols))
        elif code == 257 and nval == 1:
            nrows = val
            names.append("NbRows")
            vals.append(str(nrows))
        elif code == 258 and nval == 1:
            bps = val
            names.append("BitsPerSample")
            vals.append(str(bps))
        elif code == 259 and nval == 1 and val != 1:
            return None
        elif code == 262 and nval == 1:
            if val not in (0, 1):
                return None
            names.append("PhotomInterp")
            vals.append(str(val))
        elif code == 273:
            strip = val if nval == 1 else i32(val)
            names.append("StripOffsets")
            vals.append(str(strip))
        elif code == 277 and nval == 1:
            if val != 1:
                return None
            names.append("SamplesPerPixel")
            vals.append(str(val))
    n = nrows * ncols
    bpp = int(bps / 8)
    if n <= 0 or bpp not in (1, 2, 4):
        raise ValueError(f"{path}: {ncols} x {nrows} pixels of {bps} bits are not read")
    kind = {1: "<i1", 2: "<i2", 4: "<i4"}[bpp]
    body = raw[strip:]
    bounded = bpp == 4 and little
    # the reference reads 2048-byte blocks; unbounded loops finish the block
    nrec = len(body) // bpp if bounded else min(len(body), -(-n * bpp // 2048) * 2048) // bpp
    if nrec < n or (not bounded and (nrec > n or nrows != ncols)):
        raise ValueError(f"{path}: the data do not fill the {ncols} x {nrows} image as the reference reads it")
    v = np.frombuffer(body[:n * bpp], dtype=kind).astype(np.float64).reshape(nrows, ncols)
    # origIma[x + cols*y]: little-endian 32-bit at x = c, y = rows-1-r;
    # the others at x = r, y = c
    data = v[::-1].copy() if bounded else v.T.copy()
    meta = {"From File": path}
    for k, val in zip(names, vals):
        meta[k] = val
    meta["@"] = ""
    return Image(data, 0, ncols, 0, nrows, meta)


def _2dsans_xml(path):
    """The XML (canSAS-like) walk of readImage2dSans: rows = SASdata
    elements, columns = the Idata elements before the second SASdata, values
    = the I elements' text; ID, name, radiation and date texts become meta
    information under the path of the enclosing elements (all but SASroot,
    SASentry and Idata; an end tag removes its name and everything after it
    from the path); Q, Idev and Qdev are skipped. None for a malformed
    document or a value element with child elements (Qt's reader fails
    there)."""
    import xml.etree.ElementTree as ET
    try:
        root = ET.parse(path).getroot()
    except ET.ParseError:
        return None
    loc = lambda t: t.rsplit("}", 1)[-1].split(":")[-1]  # noqa: E731
    state = {"rows": 0, "cols": 0, "first": True, "path": [], "vals": [], "meta": {}, "bad": False}

    def walk(e):
        name = loc(e.tag)
        if name == "SASdata":
            state["rows"] += 1
            if state["rows"] > 1:
                state["first"] = False
        elif name == "Idata" and state["first"]:
            state["cols"] += 1
        elif name in ("I", "ID", "name", "radiation", "date"):
            if len(e):
                state["bad"] = True
                return False
            text = e.text or ""
            if name == "I":
                state["vals"].append(_qt_double(text))
            elif text:
                state["meta"]["/".join(state["path"]) + "/" + name] = text
            return True  # its end tag is consumed with the text
        elif name not in ("Q", "Idev", "Qdev", "Idata", "SASroot", "SASentry"):
            state["path"].append(name)
        for c in e:
            if not walk(c):
                return False
        if name in state["path"]:
            while name in state["path"]:
                state["path"].pop()
        return True

    walk(root)
    if state["bad"]:
        return None
    return state["vals"], state["rows"], state["cols"], state["meta"]


def read_2dsans(path):
    """A 2D-SANS (ILL) image (``Source/sc_readdata.cpp:1466-1767``) in its
    text forms:

    * ``.csv``: the first block of lines (it ends at a line shorter than two
      characters); lines starting with ``A`` are skipped, the rest hold a
      three-character row index and comma-separated values (at least 8;
      ``nan...`` reads as 0); the rows are the last index + 1 (an index that
      does not parse, e.g. one padded with blanks, which the line's trimming
      moves, leaves them at 0: an empty image), the columns the first row's
      count;
    * ``.dat``: a header up to the ``ASCII`` line (``Data columns are A - B -
      I - ...`` names the intensity column, the first starting with ``I``,
      else None; ``key: value`` lines become meta information), then
      whitespace-separated rows whose intensity column is read (0 where it
      does not parse, rows too short skipped); the image is sqrt(n) rows
      (at least 2) of n / rows columns.

    * ``.xml``: see :func:`_2dsans_xml`.

    Rows are stored bottom-up (file row r at y = rows - 1 - r). Other
    extensions give None, as in the reference. Data that do not fill rows x
    columns raise ValueError (the reference reads past its buffer there)."""
    low = path.lower()
    meta = {}
    vals = []
    nrows = ncols = 0
    if low.endswith(".xml"):
        r = _2dsans_xml(path)
        if r is None:
            return None
        vals, nrows, ncols, meta = r
    elif low.endswith(".csv"):
        with open(path, "rb") as f:
            raw = f.read().decode("latin-1")
        for line in raw.split("\n"):
            line = line.strip()
            if len(line) < 2:
                break
            if line.startswith("A"):
                continue
            sl = [t for t in line[3:].split(",") if t != ""]
            if len(sl) < 8:
                continue
            head = line[:3].strip()
            if re.fullmatch(r"[+-]?\d+", head):
                nrows = int(head) + 1
            if ncols == 0:
                ncols = len(sl)
            for t in sl:
                vals.append(0.0 if t.startswith("nan") else _qt_double(t))
    elif low.endswith(".dat"):
        with open(path, "rb") as f:
            raw = f.read().decode("latin-1")
        hdr, index = True, -1
        for line in raw.split("\n"):
            line = line.strip()
            if len(line) < 2:
                continue
            if hdr:
                if line.startswith("Data columns"):
                    cols = line.replace("Data columns ", "").replace("are ", "").split(" - ")
                    for i, c in enumerate(cols):
                        if c.startswith("I"):
                            index = i
                            break
                elif line.startswith("ASCII"):
                    hdr = False
                    if index < 0:
                        return None
                elif ":" in line:
                    pos = line.index(":")
                    meta[line[:pos]] = line[pos + 1:].strip()
            else:
                sl = [t for t in re.split(r"[\t ]", line) if t != ""]
                if index >= len(sl):
                    continue
                vals.append(_qt_double(sl[index]))
        nrows = max(int(math.sqrt(len(vals))), 2)
        ncols = len(vals) // nrows
    else:
        return None
    if nrows * ncols > len(vals) or nrows < 0 or ncols < 0:
        raise ValueError(f"{path}: {len(vals)} values for {nrows} x {ncols}")
    data = np.asarray(vals[:nrows * ncols], dtype=np.float64).reshape(nrows, ncols)[::-1].copy()
    m = {"From File": path, "NbRows": str(nrows), "NbCols": str(ncols)}
    m.update(meta)
    return Image(data, 0, ncols, 0, nrows, m)


def open_meas_file(path):
    """local_OpenMeasFile (``Source/sc_mainCons.cpp:1613-1652``): the reader
    for a measured-data file by its extension; returns (image, is_kws). A
    ``.dat``/``.csv``/``.txt`` with all three files of its base present is the
    program's own saved image; otherwise ``.tif``/``.tiff`` TIFF, ``.dat``/
    ``.data`` KWS, ``.edf`` EDF, ``.spr`` spreadsheet, ``.xml``/``.csv``/
    ``.txt`` 2D-SANS. HDF5 is not built (ValueError)."""
    low = path.lower()
    if low.endswith((".dat", ".csv", ".txt")):
        base = _base(path)
        if all(os.path.exists(base + e) for e in (".csv", ".dat", ".txt")):
            img = read_sascrystal_csv(path)
            if img is not None:
                return img, False
    if low.endswith((".tif", ".tiff")):
        return read_tiff(path), False
    if low.endswith((".dat", ".data")):
        return read_kws(path), True
    if low.endswith(".edf"):
        return read_edf(path), False
    if low.endswith(".spr"):
        return read_spreadsheet(path), False
    if low.endswith((".xml", ".csv", ".txt")):
        return read_2dsans(path), False
    raise ValueError(f"{path}: no reader for this file type here")


def find_beam_center(img, x0, y0):
    """Centre of the beam stop, SC_ReadData::findBeamCenter: pixels at or
    below the reference level (the first pixel's value when that is at most
    0.001, else 0) are shadow. If (x0, y0) is in the shadow, the shadow is
    walked outward from it along its row and column; otherwise every row and
    column is scanned for its widest inner run of shadow pixels (longer than
    2), and the centre of the widest runs is returned. Returns (x, y)."""
    d = img.data
    ref = d.flat[0]
    if ref > 0.001:
        ref = 0.0
    get = img.get
    bsxmin = bsxmax = x0
    bsymin = bsymax = y0
    if get(x0, y0) > ref:
        bsxmin, bsxmax = img.minX, img.maxX - 1
        bsymin, bsymax = img.minY, img.maxY - 1
        maxbsx = maxbsy = 2
        for y in range(img.minY, img.maxY):
            row = d[y - img.minY]
            xx0, xx1 = img.minX, img.maxX - 1
            while xx0 < xx1 and row[xx0 - img.minX] <= ref:
                xx0 += 1
            while xx0 < xx1 and row[xx1 - img.minX] <= ref:
                xx1 -= 1
            inner, tmp = False, 0
            for x in range(xx0, xx1 + 1):
                if row[x - img.minX] <= ref:
                    if not inner:
                        tmp, inner = x, True
                elif inner:
                    if x - tmp > maxbsx:
                        bsxmin, bsxmax, maxbsx = tmp, x - 1, x - tmp
                    inner = False
        for x in range(img.minX, img.maxX):
            col = d[:, x - img.minX]
            yy0, yy1 = img.minY, img.maxY - 1
            while yy0 < yy1 and col[yy0 - img.minY] <= ref:
                yy0 += 1
            while yy0 < yy1 and col[yy1 - img.minY] <= ref:
                yy1 -= 1
            inner, tmp = False, 0
            for y in range(yy0, yy1 + 1):
                if col[y - img.minY] <= ref:
                    if not inner:
                        tmp, inner = y, True
                elif inner:
                    if y - tmp > maxbsy:
                        bsymin, bsymax, maxbsy = tmp, y - 1, y - tmp
                    inner = False
    else:
        while bsxmin >= img.minX and get(bsxmin, y0) <= ref:
            bsxmin -= 1
        while bsxmax < img.maxX and get(bsxmax, y0) <= ref:
            bsxmax += 1
        while bsymin >= img.minY and get(x0, bsymin) <= ref:
            bsymin -= 1
        while bsymax < img.maxY and get(x0, bsymax) <= ref:
            bsymax += 1
    return _cdiv2(bsxmin + bsxmax), _cdiv2(bsymin + bsymax)


def _cdiv2(v):
    """C integer division by 2 (truncation toward zero)."""
    return v // 2 if v >= 0 else -((-v) // 2)
