"""ctypes binding of oracle/_ref/libscref.so — the reference's own FP64 CPU
path compiled from its sources by oracle/build_ref.sh.

TEST INFRASTRUCTURE ONLY: used by tests/ and tests/golden/make_golden.py to
pin the oracle and to generate golden fixtures. Nothing in the product imports
it. The library exists only where the reference sources were available at
build time.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_ref", "libscref.so")
PROBE = os.path.join(HERE, "_ref", "libscref_probe.so")

_lib = None
_probe = None


def available():
    return os.path.exists(LIB)


def load(probe=False):
    """The reference library; probe=True: its one-ulp probe build."""
    global _lib, _probe
    if probe:
        if _probe is None:
            _probe = _bind(ctypes.CDLL(PROBE))
            _probe.ref_set_probe.argtypes = [ctypes.c_int]
        return _probe
    if _lib is None:
        _lib = _bind(ctypes.CDLL(LIB))
    return _lib


def _bind(lib):
    V = ctypes.c_void_p
    lib.ref_create.restype = V
    lib.ref_destroy.argtypes = [V]
    lib.ref_set.argtypes = [V, ctypes.c_char_p, ctypes.c_double]
    lib.ref_clear.argtypes = [V]
    lib.ref_run.argtypes = [V, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.ref_error.restype = ctypes.c_char_p
    lib.ref_error.argtypes = [V]
    lib.ref_dims.argtypes = [V] + [ctypes.POINTER(ctypes.c_int)] * 4
    lib.ref_image.argtypes = [V, ctypes.c_void_p, ctypes.c_long]
    lib.ref_image.restype = ctypes.c_long
    lib.ref_timer.argtypes = [V, ctypes.c_int]
    lib.ref_timer.restype = ctypes.c_double
    lib.ref_get_array.argtypes = [V, ctypes.c_char_p, ctypes.c_void_p]
    lib.ref_get_scalar.argtypes = [V, ctypes.c_char_p]
    lib.ref_get_scalar.restype = ctypes.c_double
    lib.ref_get_latpar.argtypes = [V, ctypes.c_int, ctypes.c_void_p]
    lib.ref_set_fit_data.argtypes = [V, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    lib.ref_set_nofit_rect.argtypes = [V] + [ctypes.c_int] * 5
    if hasattr(lib, "ref_tpv_run"):
        lib.ref_tpv_run.argtypes = [V, ctypes.c_char_p, ctypes.c_uint, ctypes.c_int, ctypes.c_int, ctypes.c_char_p,
                                    ctypes.c_size_t]
    lib.ref_fit.argtypes = [V, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_long),
                            ctypes.POINTER(ctypes.c_long)]
    lib.ref_fit.restype = ctypes.c_double
    lib.ref_fit_fqs.argtypes = [V, ctypes.c_void_p, ctypes.c_long]
    lib.ref_fit_fqs.restype = ctypes.c_long
    return lib


class RefCalc:
    """One reference calculation: parameters by reference key, then run()."""

    def __init__(self, params=None, probe=False):
        self.lib = load(probe)
        self.h = self.lib.ref_create()
        if params:
            self.set(params)

    def close(self):
        if self.h:
            self.lib.ref_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set(self, params):
        for k, v in params.items():
            self.lib.ref_set(self.h, k.encode(), float(v))

    def run(self, nthreads=1, ign_new_switch=False, ign_cbs=False):
        rc = self.lib.ref_run(self.h, int(nthreads), int(ign_new_switch), int(ign_cbs))
        return rc, self.lib.ref_error(self.h).decode()

    def tpv_run(self, ids, seed, nthreads=1, ign_cbs=False):
        """(status, log text) of tpvPerformRandom(ids) after srand(seed), then
        the calculation (oracle/ref_driver.cpp ref_tpv_run)."""
        buf = ctypes.create_string_buffer(4096)
        rc = self.lib.ref_tpv_run(self.h, "\n".join(ids).encode(), int(seed), int(nthreads), int(ign_cbs), buf,
                                  len(buf))
        return rc, buf.value.decode()

    def dims(self):
        d = [ctypes.c_int() for _ in range(4)]
        self.lib.ref_dims(self.h, *[ctypes.byref(x) for x in d])
        return [x.value for x in d]

    def image(self):
        x0, x1, y0, y1 = self.dims()
        n = (x1 - x0) * (y1 - y0)
        out = np.zeros(max(n, 1), dtype=np.float64)
        if n > 0:
            self.lib.ref_image(self.h, out.ctypes.data, n)
        return out[:n].reshape(y1 - y0, x1 - x0) if n > 0 else out[:0]

    def array(self, name):
        n = 131 * 131 if name.startswith("carr11") or name.startswith("carr22") else 151
        out = np.zeros(n, dtype=np.float64)
        self.lib.ref_get_array(self.h, name.encode(), out.ctypes.data)
        return out

    def scalar(self, name):
        return self.lib.ref_get_scalar(self.h, name.encode())

    def latpar(self, which):
        if which == 3:
            out = np.zeros(2500 * 17, dtype=np.float32)
        else:
            out = np.zeros(2500 * 6, dtype=np.int32)
        self.lib.ref_get_latpar(self.h, which, out.ctypes.data)
        return out.reshape(2500, -1)

    def timer(self, which):
        return self.lib.ref_timer(self.h, which)

    def fit(self, data, nthreads=1, bstop=0, border=0, nofit=()):
        data = np.ascontiguousarray(data, dtype=np.float64)
        h, w = data.shape
        self.lib.ref_set_fit_data(self.h, w, h, data.ctypes.data)
        for i in range(4):
            r = nofit[i] if i < len(nofit) else (-1, -1, -1, -1)
            self.lib.ref_set_nofit_rect(self.h, i, *r)
        cnt = ctypes.c_long()
        nan = ctypes.c_long()
        chi2 = self.lib.ref_fit(self.h, int(nthreads), int(bstop), int(border), ctypes.byref(cnt), ctypes.byref(nan))
        fqs = np.zeros(w * h, dtype=np.float64)
        self.lib.ref_fit_fqs(self.h, fqs.ctypes.data, w * h)
        return chi2, cnt.value, nan.value, fqs.reshape(h, w)


PROBE_MODES = (0x1FF, 0x100, 0x155, 0x0AA)


def condition(params, ign_new_switch=0, ign_cbs=0, nthreads=8, modes=PROBE_MODES):
    """Per-pixel sensitivity of the reference's own result to one-ulp changes
    of its math library: max over probe modes of |I_mode - I| / max(|I|, tau),
    I the unperturbed image of the probe build; non-finite disagreements are
    inf."""
    lib = load(probe=True)
    imgs = []
    for m in (-1,) + tuple(modes):
        lib.ref_set_probe(int(m))
        r = RefCalc(params, probe=True)
        rc, err = r.run(nthreads=nthreads, ign_new_switch=ign_new_switch, ign_cbs=ign_cbs)
        assert rc == 0, err
        imgs.append(r.image())
        r.close()
    lib.ref_set_probe(-1)
    base = imgs[0]
    fin = np.isfinite(base)
    tau = 1e-30 * (np.max(np.abs(base[fin])) if fin.any() else 1.0)
    cond = np.zeros(base.shape)
    for out in imgs[1:]:
        with np.errstate(invalid="ignore", over="ignore"):
            d = np.abs(out - base) / np.maximum(np.abs(base), tau)
        same_nf = (~np.isfinite(base)) & ((np.isnan(base) & np.isnan(out)) | (base == out))
        d[same_nf] = 0.0
        d[~np.isfinite(d)] = np.inf
        cond = np.maximum(cond, d)
    return cond


def prepared_block(params, ign_new_switch=0, ign_cbs=0):
    """The reference's own host preparation of a parameter set, exported into
    the prepared-block layout the CPU oracle evaluates (ref_prepare +
    ref_export_prepared in oracle/ref_driver.cpp). Returns (bytes, error):
    error is the reference's message when it rejects the set, else ""."""
    lib = load()
    if not hasattr(lib.ref_prepare, "_bound"):
        lib.ref_prepare.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        lib.ref_export_prepared.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
        lib.ref_export_prepared.restype = ctypes.c_long
        lib.ref_prepare._bound = True
    r = RefCalc(params)
    try:
        if lib.ref_prepare(r.h, int(ign_new_switch), int(ign_cbs)) != 0:
            return None, lib.ref_error(r.h).decode()
        size = 1 << 20
        buf = ctypes.create_string_buffer(size)
        n = lib.ref_export_prepared(r.h, buf, size)
        assert n > 0
        return buf.raw[:n], ""
    finally:
        r.close()


# ----------------------------------------------------------------- readers
READERS = os.path.join(HERE, "_ref", "libscreaders.so")
_readers = None


def readers_available():
    return os.path.exists(READERS)


def _readers_lib():
    global _readers
    if _readers is None:
        lib = ctypes.CDLL(READERS)
        lib.ref_read_image.restype = ctypes.c_void_p
        lib.ref_read_image.argtypes = [ctypes.c_char_p, ctypes.c_char_p]
        lib.ref_image_dims.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
        lib.ref_image_data.restype = ctypes.c_long
        lib.ref_image_data.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_long]
        lib.ref_image_meta_count.argtypes = [ctypes.c_void_p]
        for f in (lib.ref_image_meta_key, lib.ref_image_meta_value):
            f.restype = ctypes.c_char_p
            f.argtypes = [ctypes.c_void_p, ctypes.c_int]
        lib.ref_image_title.restype = ctypes.c_char_p
        lib.ref_image_title.argtypes = [ctypes.c_void_p]
        lib.ref_image_from_data.restype = ctypes.c_void_p
        lib.ref_image_from_data.argtypes = [ctypes.c_int] * 4 + [ctypes.c_void_p]
        lib.ref_find_beam_center.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                             ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_int)]
        lib.ref_image_free.argtypes = [ctypes.c_void_p]
        _readers = lib
    return _readers


def read_image(kind, path):
    """The reference's reader `kind` ("kws", "edf", "spreadsheet",
    "sascrystal") on a file: {"dims": [minX, maxX, minY, maxY], "data": rows
    y, columns x, "meta": [(key, value), ...] in reading order, "title"}, or
    None where the reader returns no image."""
    lib = _readers_lib()
    h = lib.ref_read_image(kind.encode(), os.fsencode(path))
    if not h:
        return None
    try:
        d = (ctypes.c_int * 4)()
        lib.ref_image_dims(h, d)
        dims = list(d)
        n = (dims[1] - dims[0]) * (dims[3] - dims[2])
        data = np.zeros(max(n, 0))
        got = lib.ref_image_data(h, data.ctypes.data, data.size)
        assert got == n, (got, n)
        meta = [(lib.ref_image_meta_key(h, i).decode("latin-1"), lib.ref_image_meta_value(h, i).decode("latin-1"))
                for i in range(lib.ref_image_meta_count(h))]
        return {"dims": dims, "data": data.reshape(dims[3] - dims[2], dims[1] - dims[0]), "meta": meta,
                "title": lib.ref_image_title(h).decode("latin-1")}
    finally:
        lib.ref_image_free(h)


def find_beam_center(data, minX, maxX, minY, maxY, x0, y0):
    """The reference's findBeamCenter on an image (rows y, columns x) from the
    start point (x0, y0)."""
    lib = _readers_lib()
    a = np.ascontiguousarray(data, dtype=np.float64)
    h = lib.ref_image_from_data(minX, maxX, minY, maxY, a.ctypes.data)
    try:
        xe, ye = ctypes.c_int(0), ctypes.c_int(0)
        lib.ref_find_beam_center(h, x0, y0, ctypes.byref(xe), ctypes.byref(ye))
        return xe.value, ye.value
    finally:
        lib.ref_image_free(h)
