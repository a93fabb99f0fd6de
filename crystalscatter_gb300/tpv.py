"""Parameter randomisation of the training-data generator (TPV).

``TpvRandom.perform`` restates ``SasCalc_GENERIC_calculation::
tpvPerformRandom`` (``Source/sc_calc_generic_cpu.cpp:1028-1143``) on a
``CsParams``: each ``key=value`` entry scales the parameter's value from the
first call after ``clear()`` by ``1 + value * zuf``, with ``zuf`` uniform in
[-1, 1] from the C library's ``rand()`` (the reference's generator, so a
seed given to ``srand`` reproduces its draws):

* relative: I0, EditRadius, EditSigma, Length, SigmaL, uca, ucpsi,
  EditDbeta, Base, EditRho, and EditDomainSize (the width factor,
  ``tpv_domain_dev``);
* ucb, ucc: set to the current uca;
* phi: an absolute draw in [2, 88] degrees;
* EditDebyeWaller: the factor d^2/3 scaled (``tpv_dw_dev``);
* EditAzi: draws a number, without effect (the reference changes phiwidth,
  which its preparation recomputes from the unchanged azimuth width).

Afterwards core/shell particles and vesicles get length += radius when
length <= radius, and disks length += 2 radius when length <= 2 radius. The
returned text lists ``key = value`` per entry as the reference's log does.
"""
import ctypes
import ctypes.util

_libc = ctypes.CDLL(ctypes.util.find_library("c") or None)
_libc.rand.restype = ctypes.c_int
_libc.srand.argtypes = [ctypes.c_uint]
RAND_MAX = 2147483647  # glibc

# key -> (cs_params field, kind)
_KEYS = {
    "I0": ("izero", "norm"), "EditRadius": ("radius", "norm"), "EditSigma": ("sigma", "norm"),
    "Length": ("length", "norm"), "SigmaL": ("sigmal", "norm"), "uca": ("uca", "norm"),
    "ucb": ("ucb", "uca"), "ucc": ("ucc", "uca"), "ucpsi": ("ucpsi", "norm"),
    "EditDbeta": ("dbeta", "norm"), "EditDomainSize": ("tpv_domain_dev", "width"),
    "EditAzi": (None, "azi"), "EditDebyeWaller": ("tpv_dw_dev", "dw"), "phi": ("phi", "phi"),
    "Base": ("base", "norm"), "EditRho": ("rho", "norm"),
}


def srand(seed):
    _libc.srand(seed)


def zuf():
    """((rand()/RAND_MAX * 200) - 100) / 100, in [-1, 1]."""
    return ((float(_libc.rand()) / RAND_MAX * 200.0) - 100.0) / 100.0


def _stod(text):
    """std::stod in the C locale: the longest leading decimal number."""
    t = text.lstrip()
    best = None
    for n in range(len(t), 0, -1):
        try:
            best = float(t[:n])
            break
        except ValueError:
            continue
    if best is None:
        raise ValueError(f"no number in {text!r}")
    return best


def _to_string(v):
    return f"{v:.6f}"  # std::to_string(double)


class TpvRandom:
    def __init__(self):
        self.old = None

    def clear(self):
        """The call with an empty list: forget the saved values."""
        self.old = None

    def perform(self, p, ids, particle=None, interior=None):
        """Randomises the CsParams ``p`` in place for the entries ``ids``
        ("key=value"); ``particle``/``interior`` are the combobox indices
        (default: from ``p``). Returns the log text."""
        if not ids:
            self.clear()
            p.tpv_domain_dev = 0.0
            # the reference's next parameter load overwrites its randomised
            # dwfactor; here the draw is a separate factor, reset with the rest
            p.tpv_dw_dev = 0.0
            return "TPV: clear"
        if self.old is None:
            self.old = {f: getattr(p, f) for f, _ in _KEYS.values() if f and not f.startswith("tpv_")}
            self.old["tpv_domain_dev"] = 1.0  # width factor at the first call
            # the azimuthal width and the displacement are restored from their
            # values at the first call before every draw (hlp->oldval)
            self.old["azi"] = p.azi
            self.old["debyewaller"] = p.debyewaller
        out = ""
        for entry in ids:
            key, _, val = entry.partition("=")
            dval = _stod(val)
            if dval < 0.00001 and len(val) > 2:
                # the reference swaps the decimal separator and parses again
                pk = val.find(".")
                if pk >= 0:
                    val = val[:pk] + "," + val[pk + 1:]
                else:
                    pk = val.find(",")
                    val = val[:pk] + "." + val[pk + 1:]
                dval = _stod(val)
            if key not in _KEYS:
                continue
            field, kind = _KEYS[key]
            if kind == "norm":
                v = self.old[field] * (1 + dval * zuf())
                setattr(p, field, v)
            elif kind == "width":
                z = zuf()
                v = 1.0 * (1 + dval * z)
                p.tpv_domain_dev = dval * z
            elif kind == "uca":
                v = p.uca
                setattr(p, field, v)
            elif kind == "phi":
                v = 2.0 + (zuf() + 1) * 43.0
                p.phi = v
            elif kind == "azi":
                # phiwidth = 4/aziwidth * (1 + dval*zuf), recomputed by the preparation
                p.azi = self.old["azi"]
                v = 4.0 / p.azi * (1 + dval * zuf())
            else:  # dw
                p.debyewaller = self.old["debyewaller"]
                z = zuf()
                v = p.debyewaller * p.debyewaller / 3.0 * (1 + dval * z)
                p.tpv_dw_dev = dval * z
            out += key + " = " + _to_string(v) + "\n"
        part = p.particle if particle is None else particle
        inter = p.interior if interior is None else interior
        if (inter == 1 or part == 3) and p.length <= p.radius:
            p.length = p.radius + p.length
        if part == 2 and p.length <= 2.0 * p.radius:
            p.length = 2.0 * p.radius + p.length
        return out
