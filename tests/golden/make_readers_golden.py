"""Golden fixtures for the measured-data readers, from the reference's own
readers (Source/sc_readdata.cpp, built by oracle/build_ref.sh into
oracle/_ref/libscreaders.so with Qt stand-ins).

Writes small synthetic input files in the reference's formats into
tests/golden/readers/ (KWS text, EDF with each data type and byte order,
spreadsheet text, the program's own .csv/.txt pair), runs the reference's
reader on each and stores its image extents, data and meta information in
readers_ref.npz / readers_ref.json, together with the reference's beam-centre
finder on a set of images. Usage (needs the reference build):

    python tests/golden/make_readers_golden.py
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from oracle import refbind  # noqa: E402

IN = os.path.join(HERE, "readers")


def kws_file(name, n, lam, det_rows, tail_short=True, seed=0):
    rng = np.random.default_rng(seed)
    counts = rng.integers(-2, 400, size=n * n)
    lines = ["KWS1_MEASUREMENT KFA-IFF spectrum_data file version V-5.00", name,
             "(* Comment *)", "kws1 | someone", f"test sample {lam}", "(* Collimation discription *)",
             "Coll_Position Wind(1)_Pos Beamwindow_X Beamwindow_Y", "          [m]         [m]         [mm]"]
    lines += ["(* Detector Discription *)", "Li6 Detector is in normal mode."]
    lines += list(det_rows)
    lines += ["(* Sample discription *)", "Sample_Nr Sample_Pos", "(* Detector Data *)", "$"]
    for i in range(0, n * n, 8):
        lines.append("  ".join(f"{v:7d}" for v in counts[i:i + 8]))
    if tail_short:
        lines.append("   1   2   3")
    lines.append("")
    return "\n".join(lines)


def edf_file(kind, n, dtype, order, seed=0, extra=()):
    rng = np.random.default_rng(seed)
    data = rng.integers(0, 60000, size=(n, n)).astype(np.float64)
    if dtype in ("f4", "f8"):
        data = data / 7.0
    bo = "<" if order == "LowByteFirst" else ">"
    body = data.astype(bo + dtype).tobytes()
    names = {"f4": "FloatValue", "i4": "SignedInteger", "u2": "UnsignedShort", "f8": "DoubleValue"}
    if kind == "K1":
        hdr = ["EDF_DataBlockID = 0.Image.Psd ;", f"EDF_BinarySize = {len(body)} ;", "EDF_HeaderSize = 1024 ;",
               f"ByteOrder = {order} ;", f"DataType = {names[dtype]} ;", f"Dim_1 = {n} ;", f"Dim_2 = {n} ;",
               "Title = test image ;", "Center_1 = 12.5 ;", "Center_2 = 7 ;", "PSize_1 = 0.000172 ;",
               "PSize_2 = 0.000172 ;", "SampleDistance = 3.2 ;", "WaveLength = 1.54e-10 ;",
               "ExposureTime = 60 ;", "DetectorPosition = 2.5 ;"]
    else:
        hdr = ["HeaderID = EH:000001:000000:000000 ;", f"ByteOrder = {order} ;", f"DataType = {names[dtype]} ;",
               f"Dim_1 = {n} ;", f"Dim_2 = {n} ;", f"Size = {len(body)} ;"]
    hdr += list(extra)
    text = "{\n" + "\n".join(hdr) + "\n"
    text += " " * ((-(len(text) + 2)) % 512) + "}\n"
    return text.encode("latin-1") + body


def spreadsheet_file(n, seed=0):
    rng = np.random.default_rng(seed)
    data = rng.uniform(0.5, 9.0, size=(n, n))
    data[8:13, 5:10] = 0.0
    lines = [f"    {n}    {n} Start pixel = (       1       1)"]
    for r in range(n):
        lines.append("  " + " ".join(f"{v:13.6e}" for v in data[r]))
    return "\n".join(lines) + "\n"


def sascrystal_files(minX, maxX, minY, maxY, seed=0):
    rng = np.random.default_rng(seed)
    data = rng.uniform(1e-6, 2.0, size=(maxY - minY, maxX - minX))
    csv = [f"X:;{minX};{maxX}", f"Y:;{minY};{maxY}"]
    for j, y in enumerate(range(minY, maxY)):
        csv.append(f"Y={y}:;" + ";".join(f"{v:.6g}" for v in data[j]))
    txt = ["From File\tsomewhere.csv", "NbRows\t1", "ComboBoxParticle\tsphere {0}", "EditRadius\t10",
           "EditSigma\t0.1"]
    return "\n".join(csv) + "\n", "\n".join(txt) + "\n"


SAXSLAB_XML = ('<?xml version="1.0" ?><SAXSLABparameters><param name="det_pixel_size">172e-6 172e-6</param>'
               '<param name="wavelength">1.3414</param><param name="detector_dist">536.7868</param>'
               '<param name="beamcenter_actual">371.94    198.97</param>'
               '<param name="Meas.Description">test sample, 22.27C</param></SAXSLABparameters>')


def tiff_file(n, bps, data_off=20480, magic=b"II*\0", compression=1, strip_table=False, xml_at=256,
              total=None, data=None, seed=0):
    """A TIFF in the SAXSLAB layout: directory at byte 8, the XML header at
    xml_at, the n x n image (bps bits, little-endian) at data_off."""
    rng = np.random.default_rng(seed)
    if data is None:
        hi = {8: 256, 16: 65536, 32: 2 ** 31 - 1}[bps]
        data = rng.integers(0, hi, size=n * n)
    kind = {8: "u1", 16: "<u2", 32: "<i4"}[bps]
    body = np.asarray(data).astype(kind).tobytes()
    tags = [(256, 4, 1, n), (257, 4, 1, n), (258, 3, 1, bps), (259, 3, 1, compression), (262, 3, 1, 1),
            (270, 2, 12, 4000), (277, 3, 1, 1), (34710, 4, 1, 1024)]
    out = bytearray(max(data_off + len(body), total or 0))
    if strip_table:
        tags.append((273, 4, 4, 6000))
        out[6000:6016] = np.array([data_off, data_off + 1, 0, 0], dtype="<i4").tobytes()
    else:
        tags.append((273, 4, 1, data_off))
    out[0:8] = magic + (8).to_bytes(4, "little")
    ifd = len(tags).to_bytes(2, "little") + b"".join(
        c.to_bytes(2, "little") + t.to_bytes(2, "little") + k.to_bytes(4, "little") + v.to_bytes(4, "little")
        for c, t, k, v in tags)
    out[8:8 + len(ifd)] = ifd
    x = SAXSLAB_XML.encode("latin-1")
    out[xml_at:xml_at + len(x)] = x
    out[data_off:data_off + len(body)] = body
    return bytes(out)


def inputs():
    """name -> (reader kind, file name, bytes)"""
    out = {}
    det = ("Offset Z_Position X_Position Y_Position", "  [m]        [m]       [mm]       [mm]",
           " -0.38       1.50      -4.10     9.00", " -0.38       1.50      -4.10     9.00")
    out["kws_128_A"] = ("kws", "kws_128_A.kws", kws_file("kws_128_A", 128, "lambda=6.0A", det).encode())
    out["kws_144_nm"] = ("kws", "kws_144_nm.kws",
                         kws_file("kws_144_nm", 144, "lambda= 0.45nm", (), tail_short=False, seed=1).encode())
    out["kws_128_n"] = ("kws", "kws_128_n.kws", kws_file("kws_128_n", 128, "lambda= 0.45n", det[:2], seed=2).encode())
    out["kws_bad_size"] = ("kws", "kws_bad_size.kws", kws_file("kws_bad", 100, "lambda=5A", det).encode())
    for dtype in ("f4", "i4", "u2", "f8"):
        for order in ("LowByteFirst", "HighByteFirst"):
            nm = f"edf_k1_{dtype}_{'le' if order == 'LowByteFirst' else 'be'}"
            out[nm] = ("edf", nm + ".edf", edf_file("K1", 9, dtype, order, seed=3))
    out["edf_e1_f4"] = ("edf", "edf_e1_f4.edf", edf_file("E1", 7, "f4", "LowByteFirst", seed=4))
    out["edf_version2"] = ("edf", "edf_version2.edf", b"{\nEDF_DataFormatVersion = 2.0 ;\n}\n")
    out["spreadsheet_20"] = ("spreadsheet", "spreadsheet_20.spr", spreadsheet_file(20, seed=5).encode())
    out["tiff_i4"] = ("tiff", "tiff_i4.tif", tiff_file(16, 32, seed=8))
    out["tiff_i2"] = ("tiff", "tiff_i2.tif", tiff_file(16, 16, seed=9))
    out["tiff_u1"] = ("tiff", "tiff_u1.tif", tiff_file(16, 8, seed=10))
    out["tiff_strip_table"] = ("tiff", "tiff_strip_table.tif", tiff_file(16, 32, strip_table=True, seed=11))
    out["tiff_mm"] = ("tiff", "tiff_mm.tif", tiff_file(16, 32, magic=b"MM\0*", seed=12))
    out["tiff_mm_star"] = ("tiff", "tiff_mm_star.tif", tiff_file(16, 32, magic=b"MM*\0", seed=13))
    out["tiff_compressed"] = ("tiff", "tiff_compressed.tif", tiff_file(16, 32, compression=5, seed=14))
    out["tiff_short"] = ("tiff", "tiff_short.tif", tiff_file(16, 32, data_off=4096, seed=15))
    # an image at the end of the XML window holding a quote, a NUL and a
    # quote: the reference drops every XML parameter (the file ends with the
    # image: the 8-bit loop would otherwise run past it)
    q = np.full(16 * 16, 7)
    q[40], q[41], q[60] = 0x22, 0, 0x22
    out["tiff_quote"] = ("tiff", "tiff_quote.tif", tiff_file(16, 8, data_off=256 + 20000 - 256, data=q))
    rng = np.random.default_rng(16)
    for name, fmt in (("2dsans_csv", "{:03d}"), ("2dsans_csv_blanks", "{:3d}")):
        rows = ["A  ," + ",".join(f"{c}" for c in range(10))]
        for r in range(6):
            v = rng.uniform(0.0, 50.0, size=10)
            rows.append(fmt.format(r) + "," + ",".join("nan" if (r, c) == (2, 3) else f"{x:.5f}"
                                                      for c, x in enumerate(v)))
        rows += ["", "000,9,9,9,9,9,9,9,9,9,9"]  # a second block: not read
        out[name] = ("2dsans", name + ".csv", ("\n".join(rows) + "\n").encode())
    hdr = ["Instrument: D22", "Date: 2024-03-01 12:00:00", "Data columns are Qx - Qy - I(Qx,Qy) - Err", "ASCII data"]
    body = [f"{0.01 * i:.4f} {0.02 * i:.4f}\t{rng.uniform(1, 9):.6f} 0.1" for i in range(30)]
    body.insert(5, "0.5 0.5")  # too short: skipped
    body.insert(9, "0.5 0.5 x7 0.1")  # the intensity does not parse: 0
    out["2dsans_dat"] = ("2dsans", "sans_ill.dat", ("\n".join(hdr + body) + "\n").encode())
    out["2dsans_dat_no_i"] = ("2dsans", "sans_noi.dat", b"Data columns are Qx - Qy - Err\nASCII data\n1 2 3\n")
    out["kws_to_2dsans"] = ("kws", "sans_via_kws.dat", ("\n".join(hdr + body) + "\n").encode())
    x = ['<?xml version="1.0"?>', '<!-- canSAS-like 2D data -->',
         '<SASroot xmlns="urn:cansas1d:1.1"><SASentry><Title>run 7</Title>',
         '<SASsample><ID>sample A &amp; B</ID><name></name></SASsample>',
         '<SASinstrument><SASsource><radiation>neutron</radiation></SASsource></SASinstrument>']
    for r in range(4):
        x.append("<SASdata>")
        for c in range(5):
            x.append(f"<Idata><Q>0.{r}{c}</Q><I> {rng.uniform(1, 9):.6f} </I><Idev>0.1</Idev></Idata>")
        x.append("</SASdata>")
    x.append("<SASnote><date>2024-03-01</date></SASnote></SASentry></SASroot>")
    out["2dsans_xml"] = ("2dsans", "sans_cansas.xml", ("\n".join(x) + "\n").encode())
    out["2dsans_xml_nested"] = ("2dsans", "sans_nested.xml",
                                b"<SASroot><SASdata><Idata><I><v>1</v></I></Idata></SASdata></SASroot>\n")
    csv, txt = sascrystal_files(-4, 5, -3, 3, seed=6)
    out["sascrystal"] = ("sascrystal", "sascrystal.csv", csv.encode())
    out["sascrystal_txt"] = (None, "sascrystal.txt", txt.encode())
    return out


def beam_images():
    """name -> (data rows y, minX, maxX, minY, maxY, start x, start y)"""
    out = {}
    d = np.ones((64, 64))
    d[17:24, 26:35] = 0.0
    out["walk_inside"] = (d, 0, 64, 0, 64, 31, 21)
    out["search_outside"] = (d, 0, 64, 0, 64, 5, 5)
    d2 = np.ones((64, 64))
    d2[25, 40] = 0.0
    out["narrow_shadow"] = (d2, 0, 64, 0, 64, 5, 5)
    d3 = np.ones((9, 11))
    d3[3:6, 4:7] = 0.0
    out["negative_extents"] = (d3, -5, 6, -4, 5, 0, 0)
    rng = np.random.default_rng(7)
    d4 = rng.uniform(0.5, 3.0, size=(48, 40))
    d4[10:30, 12:20] = 0.0
    d4[0, 0] = 0.0005
    out["noisy_offcentre"] = (d4, 0, 40, 0, 48, 20, 24)
    return out


def main():
    if not refbind.readers_available():
        sys.exit("oracle/_ref/libscreaders.so not built (oracle/build_ref.sh)")
    os.makedirs(IN, exist_ok=True)
    files = inputs()
    for _, (kind, fn, raw) in files.items():
        with open(os.path.join(IN, fn), "wb") as f:
            f.write(raw)
    arrays, meta = {}, {"images": {}, "beam_center": {}}
    for name, (kind, fn, _) in files.items():
        if kind is None:
            continue
        r = refbind.read_image(kind, os.path.join(IN, fn))
        if r is None:
            meta["images"][name] = {"kind": kind, "file": fn, "image": None}
            print(name, "no image")
            continue
        arrays[name] = r["data"]
        kv = [(k, os.path.basename(v) if k == "From File" else v) for k, v in r["meta"]]
        meta["images"][name] = {"kind": kind, "file": fn, "dims": r["dims"], "meta": kv, "title": r["title"]}
        print(name, r["dims"], len(kv), "meta entries")
    for name, (d, x0, x1, y0, y1, sx, sy) in beam_images().items():
        arrays["beam_" + name] = d
        c = refbind.find_beam_center(d, x0, x1, y0, y1, sx, sy)
        meta["beam_center"][name] = {"dims": [x0, x1, y0, y1], "start": [sx, sy], "center": list(c)}
        print("beam", name, c)
    np.savez_compressed(os.path.join(HERE, "readers_ref.npz"), **arrays)
    with open(os.path.join(HERE, "readers_ref.json"), "w") as f:
        json.dump(meta, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main()
