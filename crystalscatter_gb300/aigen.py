"""The training-data generator's file loop: ``generateAIfiles``
(``Source/sc_mainCons.cpp:916-1468``) with its text output
(``saveAIfile``, ``:1469-1517``).

A generator file holds ``|``-separated lines:

* ``PATH|<dir>``, ``COLTBL|<table>``, ``RPHI|<size>;<Scale,Clip1,Clip4>``,
  ``FFT|...`` (two fields): settings;
* ``TPV|BS<x0>;<y0>;<xs>;<ys>|LI<nx>;<ny>[;<wx>;<wy>]|NO|CO|RP|IX|GP|SC``:
  the training-pattern variation mode (random beam stop, detector lines,
  noise, r-phi output, the unmodified image, PNG output, [0, 1] scaling);
* image lines. With TPV: ``<name>|<key>=<rel. deviation>|...`` (or
  ``#FAC=<n>`` for n images of the same line), the parameters randomised as
  ``tpvPerformRandom`` does (:mod:`tpv`); without: ``<category>|<key>=<value>
  |...`` (``#DEF``, ``#FN_<key>=<value>``, ``#Calc=<n>``), the values set and
  the file name built from them as the reference builds it.

Each image is calculated by the library (:class:`LibraryCalc`: the C-ABI
calculation on the GPU, the r-phi transform on the GPU), post-processed in
the reference's order with the reference's random draws (``zuf``, the C
library's ``rand``: noise ``z * sqrt(I)`` per pixel, the beam-stop position
and size, the detector lines), and written as the reference's text image
(``<name>.spr``: ``sx sy Start pixel = (1 1)`` then rows of ``%13.6e``) when
the colour table starts with ``*``. Not built: PNG output (no image encoder
here; logged), the FFT image (``calculateIFFT``, FFTW; logged), the
convolution (a no-op in the reference as well).

The calculation is injected: any object with ``params`` (a ``CsParams``),
``update_param(key, value)``, ``compute()`` -> (image rows y, minX, maxX,
minY, maxY), ``beam_pos()`` -> (BeamPosX, BeamPosY) and ``rphi(image, minX,
maxX, minY, maxY, bx, by, size, scale, clip, clip40)`` can drive the loop.
"""
import math
import os

import numpy as np

from . import postproc, tpv


def _qt_double(text):
    try:
        return float(text.strip())
    except ValueError:
        return 0.0


def _qt_int(text):
    t = text.strip()
    try:
        return int(t)
    except ValueError:
        return 0


def _e13(v):
    """QString("%1").arg(v, 13, 'e', 6)"""
    if math.isnan(v):
        return f"{'nan':>13}"
    if math.isinf(v):
        return f"{'inf' if v > 0 else '-inf':>13}"
    return f"{v:13.6e}"


def save_ai_file(fn, src, sx, sy, linflg, coltbl, log):
    """saveAIfile: the text image when the colour table starts with ``*``
    (r-phi and FFT images into the ``rphi``/``fft`` trees, the unmodified
    image into ``scat_org``); PNG output is not built."""
    if coltbl.startswith("*"):
        if linflg in (1, 11):
            fn = fn.replace("scat", "rphi")
        elif linflg in (2, 12):
            fn = fn.replace("scat", "fft")
        elif linflg in (3, 13):
            fn = fn.replace("scat/", "scat_org/")
        a = np.asarray(src, dtype=np.float64).reshape(sy, sx)
        try:
            with open(fn + ".spr", "w") as fo:
                fo.write(f"    {sx}    {sy} Start pixel = (       1       1)\n")
                for y in range(sy):
                    fo.write(" " + "".join(" " + _e13(float(v)) for v in a[y]) + "\n")
            log.append(f"Save {fn}")
        except OSError as e:
            log.append(f"ERROR {e} ({fn}.spr)")
        if linflg < 10:
            return
    log.append(f"PNG output is not built: {fn}.png not written")


def scale_intensity_lin(img):
    """scaleIntensity(true) (Source/sc_calc_generic_cpu.cpp:11195-11236), the
    linear branch: (v - min) / (max - min) with the reference's running
    minimum and maximum (a value that lowers the minimum is not compared with
    the maximum), widened when they are within 1e-6."""
    flat = img.reshape(-1)
    vmin, vmax = 1e20, 1e-20
    for v in flat:
        if v < vmin:
            vmin = v
        elif v > vmax:
            vmax = v
    if abs(vmin - vmax) < 1e-6:
        vmin *= 0.998
        vmax *= 1.002
        if vmax == 0:
            vmax = 0.2
    flat[:] = (flat - vmin) / (vmax - vmin)


def log_scale(values, mask=None):
    """The log scaling of the FFT/r-phi inputs and of scaleAndClipData's log
    option: (log10 v - min) / (max - min) over the positive values (those in
    mask, when given, set min and max), 0 elsewhere; a value that lowers the
    minimum is not compared with the maximum."""
    flat = np.asarray(values, dtype=np.float64).reshape(-1)
    vmin, vmax = 1e26, 0.0
    for i, v in enumerate(flat):
        if (mask is None or mask[i]) and v > 0:
            lv = math.log10(v)
            if lv < vmin:
                vmin = lv
            elif lv > vmax:
                vmax = lv
    out = np.zeros_like(flat)
    pos = flat > 0
    with np.errstate(divide="ignore", invalid="ignore"):
        out[pos] = (np.log10(flat[pos]) - vmin) / (vmax - vmin)
    return out


class LibraryCalc:
    """The library's calculation for the generator: the single-image C-ABI
    call on the GPU (mixed or FP64) and the GPU r-phi transform."""

    def __init__(self, params=None, mode=None):
        import crystalscatter_gb300 as cs
        self.cs = cs
        self.mode = cs.CS_MODE_MIXED if mode is None else mode
        self.params = params if params is not None else cs.default_params()

    def update_param(self, key, value):
        c = self.cs.SasCalc_GENERIC_calculation()
        c.set_params(self.params)
        c.setParam(key, value)
        self.params = c.params()
        c.cleanup()

    def beam_pos(self):
        return self.params.beamx, self.params.beamy

    def compute(self):
        c = self.cs.SasCalc_GENERIC_calculation()
        c.set_params(self.params)
        c.doCalculation(0, False, False, mode=self.mode)
        img = np.array(c.data(), dtype=np.float64)
        dims = c.minX(), c.maxX(), c.minY(), c.maxY()
        c.cleanup()
        return (img,) + tuple(dims)

    def rphi(self, image, x0, x1, y0, y1, bx, by, size, scale, clip, clip40):
        import torch
        d = torch.as_tensor(np.ascontiguousarray(image), device="cuda")
        out = self.cs.rphi_device(d, x0, x1, y0, y1, bx, by, size, scale, clip, clip40)
        torch.cuda.synchronize()
        return out.cpu().numpy()


def generate_ai_files(calc, aifile, nofft=False, log=None):
    """Runs a generator file (or, when ``aifile`` starts with ``@``, the
    ``@``-separated lines of the string) through ``calc``; returns the log
    lines. Random draws come from :func:`tpv.zuf` (seed with
    :func:`tpv.srand` for the reference's sequence)."""
    log = [] if log is None else log
    if aifile.startswith("@"):
        lines = aifile.split("@")
        from_string = True
    else:
        with open(aifile, "r", errors="replace") as f:
            lines = f.read().split("\n")
        if lines and lines[-1] == "":
            lines.pop()
        from_string = False
    path = ""
    coltbl = ""
    fft_input_lin = False
    rphi_size = 0
    rphi_scale = rphi_clip = rphi_clip40 = False
    fft_out_size = 0
    use_tpv = False
    bs = [-1.0, -1.0, -1.0, -1.0]
    lines_x = lines_y = 0
    lines_xw = lines_yw = 1
    add_noise = add_rphi = save_extra = gen_png = scale_scat = False
    factor_in_line = False
    factor_count = 0
    rnd = tpv.TpvRandom()
    sl = []
    img_count = 0
    while True:
        if factor_in_line and factor_count == 0:
            break
        if not (factor_in_line and factor_count > 0) and not lines:
            break
        if not factor_in_line:
            dbg = lines.pop(0)
            if not from_string:
                dbg = dbg.strip()
            sl = [t for t in dbg.split("|") if t != ""]
            if len(sl) < 2:
                continue
            if len(sl) == 2:
                if sl[0] == "PATH":
                    path = sl[1]
                    if not path.endswith("/"):
                        path += "/"
                    continue
                if sl[0] == "COLTBL":
                    coltbl = sl[1]
                    continue
                if sl[0] == "FFT" and not nofft:
                    fft = sl[1].split(";") + ["0"] * 9
                    fft_input_lin = fft[0] == "InLin"
                    rphi_size = _qt_int(fft[1])
                    rphi_scale, rphi_clip, rphi_clip40 = ("Scale" in fft[2], "Clip1" in fft[2], "Clip4" in fft[2])
                    fft_out_size = _qt_int(fft[3])
                    continue
                if sl[0] == "RPHI":
                    fft = sl[1].split(";") + ["0"] * 2
                    rphi_size = _qt_int(fft[0])
                    rphi_scale, rphi_clip, rphi_clip40 = ("Scale" in fft[1], "Clip1" in fft[1], "Clip4" in fft[1])
                    continue
            if sl[0] == "TPV":
                use_tpv = True
                for t in sl[1:]:
                    if t.startswith("BS"):
                        val = t[2:].split(";")
                        if len(val) != 4:
                            continue
                        bs = [_qt_double(v) for v in val]
                    elif t.startswith("LI"):
                        val = t[2:].split(";")
                        if len(val) >= 2:
                            lines_x, lines_y = _qt_int(val[0]), _qt_int(val[1])
                        if len(val) >= 4:
                            lines_xw, lines_yw = _qt_int(val[2]), _qt_int(val[3])
                    elif t.startswith("NO"):
                        add_noise = True
                    elif t.startswith("RP"):
                        add_rphi = True
                    elif t.startswith("IX"):
                        save_extra = True
                    elif t.startswith("GP"):
                        gen_png = True
                    elif t.startswith("SC"):
                        scale_scat = True
                continue
            if scale_scat:
                fft_input_lin = True
        is_def = False
        if use_tpv:
            fn = "_scat_" + (str(factor_count - 1) if factor_in_line else sl[0])
            category = "scat"
            entries = []
            for t in sl[1:]:
                if not factor_in_line and t.startswith("#FAC"):
                    factor_in_line = True
                    factor_count = _qt_int(t.split("=")[1])
                    fn = "_scat_" + str(factor_count - 1)
                    log.append(f"TPV Factor {factor_count}")
                if t.startswith("#"):
                    continue
                entries.append(t)
        else:
            rnd.perform(calc.params, [])  # forget the saved values
            category = sl[0]
            fn = ""
            fixed = False
            for t in sl[1:]:
                vv = t.split("=")
                if t.startswith("#Calc") or t.startswith("#DEF"):
                    is_def = is_def or t.startswith("#DEF")
                elif t.startswith("#FN_"):
                    fixed = True
                    fn = vv[0][3:] + f"={_qt_double(vv[1]):.3f}"
                else:
                    calc.update_param(vv[0], _qt_double(vv[1]))
                    if not fixed:
                        fn += f"_{vv[0]}={_qt_double(vv[1]):.3f}"
            low = fn.lower()
            while "edit" in low:
                i = low.index("edit")
                fn = fn[:i] + fn[i + 4:]
                low = fn.lower()
            while "0_" in fn:
                fn = fn.replace("0_", "_")
            fn = fn.replace("._", "_")
            while fn.endswith("0"):
                fn = fn[:-1]
            if fn.endswith("."):
                fn = fn[:-1]
            if is_def:
                fn += "_DEF"
        fnpng = path + category + "/" + fn[1:]
        if not os.path.isdir(path + category):
            os.makedirs(path + category, exist_ok=True)
            if use_tpv:
                if add_rphi:
                    os.makedirs(path + "rphi", exist_ok=True)
                if save_extra:
                    os.makedirs(path + "scat_org", exist_ok=True)
        if use_tpv:
            if (factor_in_line and factor_count > 1) or not factor_in_line:
                log.append("\n" + rnd.perform(calc.params, entries))
            else:
                log.append("\nTPV: no random values for this image.")
        src, x0, x1, y0, y1 = calc.compute()
        src = np.array(src, dtype=np.float64).reshape(y1 - y0, x1 - x0)
        sx, sy = x1 - x0, y1 - y0
        n = sx * sy
        bpx, bpy = calc.beam_pos()
        bsx0, bsy0 = int(bpx), int(bpy)
        bsdx = bsdy = 2
        flat = src.reshape(-1)
        if use_tpv:
            msg = ""
            if scale_scat:
                scale_intensity_lin(src)
            if save_extra:
                save_ai_file(fnpng, flat, sx, sy, 13 if gen_png else 3, coltbl, log)
            if add_noise:
                minz, maxz = 200.0, -200.0
                for i in range(n):
                    z = tpv.zuf()
                    minz, maxz = min(minz, z), max(maxz, z)
                    d = flat[i]
                    root = math.sqrt(d) if d >= 0 else math.nan
                    flat[i] = d + (z / 100.0 if scale_scat else z) * root
                msg += f"AddNoise [{minz:g},{maxz:g}]\n"
            if bs[0] > 0:
                bsx0 = int(bsx0 * (1.0 + bs[0] * tpv.zuf()))
                bsy0 = int(bsy0 * (1.0 + bs[1] * tpv.zuf()))
                bsdx = int(bsdx * (1.0 + bs[2] * tpv.zuf()))
                bsdy = int(bsdy * (1.0 + bs[3] * tpv.zuf()))
                for x in range(x0, x1):
                    if bsx0 - bsdx <= x <= bsx0 + bsdx:
                        for y in range(y0, y1):
                            if bsy0 - bsdy <= y <= bsy0 + bsdy:
                                flat[(x - x0) + sx * (y - y0)] = 0
                msg += f"AddBeamstop Pos=({bsx0},{bsy0}) Size=({bsdx},{bsdy})\n"
            if lines_x > 0:
                xc = (x1 - x0 + 1) // lines_x
                msg += "AddLinesX at"
                for i in range(lines_x):
                    xp = int(x0 + i * xc + abs(tpv.zuf()) * xc)
                    msg += f" {xp}"
                    for x in range(xp, xp + lines_xw):
                        for y in range(y0, y1):
                            ii = (x - x0) + sx * (y - y0)
                            if 0 <= ii < n:
                                flat[ii] = 0
                msg += "\n"
            if lines_y > 0:
                yc = (y1 - y0 + 1) // lines_y
                msg += "AddLinesY at"
                for i in range(lines_y):
                    yp = int(y0 + i * yc + abs(tpv.zuf()) * yc)
                    msg += f" {yp}"
                    for y in range(yp, yp + lines_yw):
                        for x in range(x0, x1):
                            ii = (x - x0) + sx * (y - y0)
                            if 0 <= ii < n:
                                flat[ii] = 0
                msg += "\n"
            log.append(msg)
        save_ai_file(fnpng, flat, sx, sy, 10 if gen_png else 0, coltbl, log)
        if (fft_out_size > 0 and not nofft) or rphi_size > 0:
            data = None
            if not fft_input_lin:
                xs, ys = np.meshgrid(np.arange(x0, x1), np.arange(y0, y1))
                mask = (((x0 < 0) & (xs != 0) & (ys != 0)) | (x0 == 0)).reshape(-1)
                data = log_scale(flat, mask)
            if rphi_size > 0:
                inp = (flat if data is None else data).reshape(sy, sx)
                r = np.asarray(calc.rphi(inp, x0, x1, y0, y1, bsx0, bsy0, rphi_size, rphi_scale, rphi_clip,
                                         rphi_clip40), dtype=np.float64).reshape(-1)
                r = log_scale(r)
                save_ai_file(fnpng, r, rphi_size, rphi_size, 11 if gen_png else 1, coltbl, log)
            if fft_out_size > 0:
                log.append(f"FFT output is not built: {fnpng} (fft) not written")
        img_count += 1
        if use_tpv and factor_in_line:
            factor_count -= 1
            if factor_count <= 0:
                break
    return log


class HostRphi:
    """r-phi on the host (:func:`postproc.rphi`), for drivers without a GPU
    (tests); the library's calculation uses the GPU kernel."""

    @staticmethod
    def rphi(image, x0, x1, y0, y1, bx, by, size, scale, clip, clip40):
        return postproc.rphi(image, x0, x1, y0, y1, bx, by, size, scale, clip, clip40)
