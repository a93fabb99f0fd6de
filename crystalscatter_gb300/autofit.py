"""The automatic fit driven by a command file: ``automaticFit``
(``Source/sc_mainCons.cpp:1830-2519``) with ``doFitStart`` (``:1653-1742``).

Command lines (``#`` starts a comment, ``EOF`` ends the file):

* read on the first pass only: ``Param: <file>`` (parameters as
  ``key=value`` lines, ``[section]`` lines ignored), ``DirMask: <glob>``,
  ``DirUp: <dir>`` / ``DirDown: <dir>`` (the directory's files in ascending /
  descending case-insensitive name order), ``File: <path>``, ``Limits:
  <text>; <min>; <max>`` (the first fit parameter whose name the text
  contains, case-insensitive; the reference takes the first in its hash
  order, here the first in name order), ``GlobLog:`` (a start line in the
  log);
* on every pass: ``Info: <text>``, ``Use: <key>, <key>, ...`` (the fitted
  parameters; their start values are the current ones), ``Border: <border>;
  <beam stop>; <corner>`` and ``Fit: Stp=..; Iter=..; Tol=..; Diff<..;
  Kenn=..``: up to 20 simplex fits (step Stp/100, Iter iterations, tolerance
  Tol) until the mean relative change of the fitted parameters falls below
  Diff percent; each loop logs to ``<Kenn><NN>_calc.log``.

Without an image argument the files named by ``File``/``DirUp``/``DirDown``
are fitted one after another, the command file read again for each; after
each file the fitted parameters are saved as ``<name>_out.ini``. KWS images
get their beam centre from the beam-stop finder first, as in the reference.
The fit parameters and their limits are the reference's fittable parameters
(``FIT_LIMITS``) and Editdom1..3 (0..1000). Not built: the LaTeX report, PNG
images, the GUI's saved fit limits.

The calculation and the fit are injected: ``calc`` holds ``params`` (a
``CsParams``) and offers ``value(key)``, ``update_param(key, value)`` and
``save(path)``; ``fit(calc, image, table, stp, maxit, tol, border, bstop)``
runs one simplex fit over ``table`` (dicts with key, min, max, start, used)
and returns ({key: result}, report). :func:`library_fit` is the library's
(``simplex_fit``, on the GPU).
"""
import fnmatch
import os

from . import readers

# The reference's fittable parameters and their input limits (the GUI
# definitions of Source/sc_calc_generic.cpp, "NF;key;frac|min|max|unit;...").
FIT_LIMITS = {
    "uca": (0.01, 1000.0), "ucb": (0.01, 1000.0), "ucc": (0.01, 1000.0), "ucalpha": (0.0, 360.0),
    "ucbeta": (0.0, 360.0), "ucgamma": (0.0, 360.0), "EditCeff": (0.0, 1.0), "EditCeffcyl": (0.0, 999.0),
    "reff": (-10000.0, 10000.0), "acpl": (0.0, 1.0), "bcpl": (0.0, 1.0), "ifluc": (0.0, 1000.0),
    "rfluc": (0.0, 1000.0), "EditRadius": (0.0, 1000.0), "EditRadiusi": (0.0, 1000.0),
    "EditSigma": (-10000.0, 10000.0), "EditDbeta": (0.0, 360.0), "Length": (0.0, 1000.0),
    "SigmaL": (-10000.0, 10000.0), "Alpha": (-10000.0, 10000.0), "EditRho": (-10000.0, 10000.0),
    "RotAlpha": (-10000.0, 10000.0), "EditPeakPar": (0.0, 1000000.0), "EditDebyeWaller": (0.0, 100.0),
    "EditAzi": (-10000.0, 10000.0), "EditDomainSize": (0.0, 5000.0), "SigX": (0.01, 9999.0),
    "SigY": (0.01, 9999.0), "SigZ": (0.01, 9999.0), "ucpsi": (0.0, 360.0), "ucn1": (-10000.0, 10000.0),
    "ucn2": (-10000.0, 10000.0), "ucn3": (-10000.0, 10000.0), "theta": (0.0, 360.0), "phi": (0.0, 360.0),
    "rotTheta": (0.0, 360.0), "rotPhi": (0.0, 360.0), "EditPixelNoX": (-10000.0, 10000.0),
    "EditPixelNoY": (-10000.0, 10000.0), "EditPixelX": (-10000.0, 10000.0), "EditPixelY": (-10000.0, 10000.0),
    "EditDet": (-10000.0, 10000.0), "EditWavelength": (-10000.0, 10000.0), "BeamPosX": (-10000.0, 10000.0),
    "BeamPosY": (-10000.0, 10000.0), "iso": (-10000.0, 10000.0), "I0": (0.0, 100000.0),
    "Base": (-10000.0, 10000.0),
}
# paramsForMethod(fit): the fittable parameters and Editdom1..3, sorted
FIT_KEYS = sorted(list(FIT_LIMITS) + ["Editdom1", "Editdom2", "Editdom3"])


def _qt_double(text):
    try:
        return float(text.strip())
    except ValueError:
        return 0.0


def _qt_int(text):
    try:
        return int(text.strip())
    except ValueError:
        return 0


def library_fit(calc, image, table, stp, maxit, tol, border, bstop):
    """One simplex fit with the library (``simplex_fit``: the reference's
    simplex, images on the GPU in FP64)."""
    import crystalscatter_gb300 as cs
    return cs.simplex_fit(calc.params, image.data, table, stp=stp, maxit=maxit, ftol=tol, border=border, bstop=bstop)


class LibraryFitCalc:
    """The calculation side for :func:`automatic_fit` with the library: the
    parameters as a key/value mapping of the reference's keys (unset keys
    read as 0), turned into a ``CsParams`` for each fit, saved as
    ``key=value`` lines."""

    def __init__(self, mapping):
        self.values = dict(mapping)

    @property
    def params(self):
        import crystalscatter_gb300 as cs
        return cs.params_from_mapping(self.values)

    def value(self, key):
        return float(self.values.get(key, 0.0))

    def update_param(self, key, value):
        self.values[key] = value

    def save(self, path):
        with open(path, "w") as f:
            f.write("[Parameter]\n")
            for k in sorted(self.values):
                f.write(f"{k}={self.values[k]!r}\n")


class _Limit:
    def __init__(self, start, lo, hi):
        self.orgval = self.fitstart = self.fitres = start
        self.min, self.max = lo, hi
        self.used = False


def _fit_start(calc, img, p2f, fit, stp, tol, maxit, border, bstop, log):
    """doFitStart with one repetition: the simplex from the current start
    values, then the mean relative change of the fitted parameters (in
    percent; absolute where the original value is 0)."""
    table = [{"key": k, "min": f.min, "max": f.max, "start": f.fitstart, "used": f.used} for k, f in p2f.items()]
    res, rep = fit(calc, img, table, stp * 0.01, maxit, tol, border, bstop)
    total, n = 0.0, 0
    for k, f in p2f.items():
        if not f.used:
            continue
        f.fitres = res.get(k, f.fitstart)
        tmp = abs(f.orgval - f.fitres) if f.orgval == 0 else abs(f.orgval - f.fitres) * 100.0 / f.orgval
        log.append(f"{k}: {f.orgval:g} -> {f.fitres:g} ({tmp:g}%)")
        total += tmp
        n += 1
        f.fitstart = f.orgval = f.fitres
        calc.update_param(k, f.fitres)
    mean = total / n if n else float("nan")
    log.append(f"Overall: {rep.get('ms', 0):g} ms / {rep.get('repetitions', 0)} loops / {rep.get('images', 0)} img"
               f" / MeanDif {mean:g}%")
    return mean


def _load_params(calc, path):
    with open(path, "r", errors="replace") as f:
        for line in f:
            line = line.strip()
            if not line or line.startswith(("[", "#", ";")) or "=" not in line:
                continue
            k, _, v = line.partition("=")
            calc.update_param(k.strip(), _qt_double(v))


def _dir_files(d, mask, reverse):
    names = [n for n in os.listdir(d) if os.path.isfile(os.path.join(d, n)) and fnmatch.fnmatch(n, mask)]
    names.sort(key=str.lower, reverse=reverse)
    return [os.path.abspath(os.path.join(d, n)) for n in names]


def automatic_fit(calc, autofit, imgfile="", outdir="", fit=library_fit):
    """Runs a command file; returns the global log lines. Outputs go to
    ``outdir`` (default: the command file's directory)."""
    glog = []
    base = (outdir or os.path.dirname(os.path.abspath(autofit))) + "/"
    os.makedirs(base, exist_ok=True)
    img = None
    if imgfile:
        img, iskws = readers.open_meas_file(imgfile)
        if iskws:
            _beam_from_kws(calc, img, glog)
    p2f = {}
    for k in FIT_KEYS:
        lo, hi = FIT_LIMITS.get(k, (0.0, 1000.0))
        p2f[k] = _Limit(calc.value(k), lo, hi)
    kenn = "-autofit-"
    first = True
    dir_mask = "*"
    used_images = []
    border = bstop = 0
    param2values = {}
    with open(autofit, "r", errors="replace") as f:
        cmd_lines = f.read().split("\n")
    while True:
        cur_img = ""
        for raw in cmd_lines:
            line = raw.strip()
            pos = line.find("#")
            if pos >= 0:
                line = line[:pos].strip()
            if not line:
                continue
            if first:
                glog.append("Autofit: " + line)
            if line.startswith("EOF"):
                break
            if first:
                if line.startswith("GlobLog:"):
                    glog.append("Start")
                    continue
                if line.startswith("Param:"):
                    glog.append("Load Paramfile " + line[6:].strip())
                    _load_params(calc, line[6:].strip())
                    continue
                if line.startswith("DirMask:"):
                    dir_mask = line[8:].strip()
                    glog.append("Set directory mask to " + dir_mask)
                    continue
                if line.startswith("DirUp:") or line.startswith("DirDown:"):
                    down = line.startswith("DirDown:")
                    files = _dir_files(line[8 if down else 6:].strip(), dir_mask, down)
                    used_images += files
                    glog.append(f"Dir ({'Down' if down else 'Up'}) {len(files)} files found.")
                    continue
                if line.startswith("File:"):
                    used_images.append(line[5:].strip())
                    glog.append("File added " + line[5:].strip())
                    continue
                if line.startswith("Limits:"):
                    names = [t.strip() for t in line[7:].strip().split(";")]
                    for k, fl in p2f.items():
                        if k.lower() in names[0].lower():
                            if len(names) >= 2:
                                fl.min = _qt_double(names[1])
                            if len(names) >= 3:
                                fl.max = _qt_double(names[2])
                            break
                    continue
            if line.startswith("Info:"):
                if not first:
                    glog.append("Autofit: " + line)
                continue
            if line.startswith("Use:"):
                names = [t.strip().lower() for t in line[4:].strip().split(",")]
                one = False
                for k, fl in p2f.items():
                    fl.used = k.lower() in names
                    fl.orgval = fl.fitstart = calc.value(k)
                    one |= fl.used
                    if k not in param2values and fl.used:
                        param2values[k] = [fl.orgval, fl.orgval]
                if not one:
                    glog.append("ERROR no parameter used: " + line)
                    return glog
                continue
            if line.startswith("Border:"):
                cmd = [t.strip() for t in line[7:].strip().split(";")] + ["0", "0", "0"]
                border, bstop = _qt_int(cmd[0]), _qt_int(cmd[1])
                if _qt_int(cmd[2]) != 0:
                    bstop = -1
                continue
            if line.startswith("Fit:"):
                max_dif, stp, tol, maxit = 100.0, 3.0, 0.001, 10
                for t in (s.strip() for s in line[4:].strip().split(";")):
                    if t.startswith("Stp="):
                        stp = _qt_double(t[4:])
                    elif t.startswith("Iter="):
                        maxit = _qt_int(t[5:])
                    elif t.startswith("Tol="):
                        tol = _qt_double(t[4:])
                    elif t.startswith("Diff<"):
                        max_dif = _qt_double(t[5:])
                    elif t.startswith("Kenn="):
                        kenn = t[5:]
                        if used_images:
                            kenn = kenn.replace("@F", os.path.splitext(os.path.basename(used_images[0]))[0])
                        else:
                            kenn = kenn.replace("@F", "")
                        if not kenn.endswith("-"):
                            kenn += "-"
                if not imgfile and used_images and cur_img != used_images[0]:
                    img, iskws = readers.open_meas_file(used_images[0])
                    cur_img = used_images[0]
                    glog.append("Imgfile " + cur_img)
                    if iskws:
                        _beam_from_kws(calc, img, glog)
                if img is None:
                    glog.append("ERROR no image to fit")
                    return glog
                for loop in range(20):
                    llog = []
                    mean = _fit_start(calc, img, p2f, fit, stp, tol, maxit, border, bstop, llog)
                    llog.append(f"\nAutoFit: loop={loop + 1}, MeanDiff={mean:g}, MaxDiff={max_dif:g}\n")
                    name = base + kenn + f"{loop + 1:02d}" + "_calc.log"
                    with open(name, "w") as lf:
                        lf.write("\n".join(llog) + "\n")
                    glog.append("Logfile " + name)
                    if mean < 0:
                        glog.append("Autofit MeanChangePercent < 0")
                        return glog
                    if mean < max_dif:
                        for k, fl in p2f.items():
                            if fl.used:
                                param2values[k][1] = fl.fitres
                        break
                continue
        if not imgfile and used_images:
            out = base + os.path.splitext(os.path.basename(used_images[0]))[0] + "_out"
            calc.save(out + ".ini")
            glog.append("Save params to " + out + ".ini (PNG output is not built)")
            param2values = {}
            first = False
            used_images.pop(0)
            if not used_images:
                break
        else:
            break
    if imgfile:
        calc.save(os.path.splitext(base + os.path.basename(imgfile))[0] + "_out.ini")
    return glog


def _beam_from_kws(calc, img, glog):
    """A KWS image's beam centre from the beam-stop finder, started at the
    detector centre (BeamPosX/Y in the file), as the reference does; the
    calculation's beam position relative to the image centre."""
    x0 = int(_qt_double(img.meta.get("BeamPosX", "0")))
    y0 = int(_qt_double(img.meta.get("BeamPosY", "0")))
    bx, by = readers.find_beam_center(img, x0, y0)
    img.meta["BeamPosX"], img.meta["BeamPosY"] = str(bx), str(by)
    calc.update_param("BeamPosX", bx - img.cols / 2.0)
    calc.update_param("BeamPosY", by - img.rows / 2.0)
    glog.append(f"AutoBeamstop: in data ({bx} / {by}), in calc ({bx - img.cols / 2.0:g} / {by - img.rows / 2.0:g})")
