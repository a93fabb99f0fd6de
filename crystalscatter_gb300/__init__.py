"""Python host binding of the GB300 CrystalScatter pixel calculation.

The native library (``_lib/libcrystalscatter.so``, C ABI in
``include/crystalscatter.h``) does all preparation and computing. This module
loads it with ctypes and mirrors the public methods of the reference class
``SasCalc_GENERIC_calculation`` (Source/sc_calc_generic_gpu.h:77-598) with the
same names and argument meaning, plus the console's key/value entry
(``--mcpval``). There is no CPU fallback: without the native library or
without a GPU every calculation raises.
"""
import ctypes
import os

import numpy as np

__all__ = [
    "CsParams", "SasCalc_GENERIC_calculation", "SasCalcBatch", "CrystalScatterError", "load_library",
    "library_path", "params_from_mapping", "simplex_fit", "simplex_minimize", "CS_MODE_FP64", "CS_MODE_MIXED", "CS_SCHED_PLAIN",
    "CS_SCHED_PERSISTENT", "CS_FIT_SEQUENTIAL", "CS_FIT_BATCHED",
]

CS_OK = 0
CS_ERR_PARAM = 1
CS_ERR_CUDA = 2
CS_ERR_TIMEOUT = 3
CS_ERR_UNSUPPORTED = 4
CS_ERR_ALLOC = 5
CS_ERR_STATE = 6
CS_ERR_SIZE = 7
CS_MODE_FP64 = 0
CS_MODE_MIXED = 1
CS_SCHED_PLAIN = 0
CS_SCHED_PERSISTENT = 1
CS_FIT_SEQUENTIAL = 0
CS_FIT_BATCHED = 1

_HERE = os.path.dirname(os.path.abspath(__file__))


def library_path():
    return os.path.join(_HERE, "_lib", "libcrystalscatter.so")


class CrystalScatterError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code
        self.msg = msg


_D3 = ctypes.c_double * 3


class CsParams(ctypes.Structure):
    """Mirror of ``cs_params`` (include/crystalscatter.h)."""
    _fields_ = [
        ("ltype", ctypes.c_int),
        ("uca", ctypes.c_double), ("ucb", ctypes.c_double), ("ucc", ctypes.c_double),
        ("ucalpha", ctypes.c_double), ("ucbeta", ctypes.c_double), ("ucgamma", ctypes.c_double),
        ("ceff", ctypes.c_double),
        ("twinned", ctypes.c_int),
        ("ceffcyl", ctypes.c_double), ("reff", ctypes.c_double), ("acpl", ctypes.c_double),
        ("bcpl", ctypes.c_double), ("ifluc", ctypes.c_double), ("rfluc", ctypes.c_double),
        ("particle", ctypes.c_int), ("ordis", ctypes.c_int), ("interior", ctypes.c_int),
        ("radius", ctypes.c_double), ("radiusi", ctypes.c_double), ("sigma", ctypes.c_double),
        ("dbeta", ctypes.c_double), ("length", ctypes.c_double), ("sigmal", ctypes.c_double),
        ("alphash", ctypes.c_double), ("rho", ctypes.c_double), ("alpha", ctypes.c_double),
        ("peak", ctypes.c_int),
        ("peakpar", ctypes.c_double), ("debyewaller", ctypes.c_double), ("azi", ctypes.c_double),
        ("domainsize", ctypes.c_double),
        ("debyescherrer", ctypes.c_int), ("para", ctypes.c_int),
        ("ax1", _D3), ("ax2", _D3), ("ax3", _D3), ("sigxyz", _D3),
        ("ucpsi", ctypes.c_double), ("ucn1", ctypes.c_double), ("ucn2", ctypes.c_double),
        ("ucn3", ctypes.c_double), ("theta", ctypes.c_double), ("phi", ctypes.c_double),
        ("rottheta", ctypes.c_double), ("rotphi", ctypes.c_double),
        ("gridpoints", ctypes.c_int), ("hklmax", ctypes.c_int),
        ("qmax", ctypes.c_double), ("qmin", ctypes.c_double),
        ("radq1", ctypes.c_int), ("radq2", ctypes.c_int), ("radq4", ctypes.c_int),
        ("expand", ctypes.c_int), ("use1d", ctypes.c_int),
        ("pixnox", ctypes.c_double), ("pixnoy", ctypes.c_double), ("pixx_mm", ctypes.c_double),
        ("pixy_mm", ctypes.c_double), ("det", ctypes.c_double), ("wavelength", ctypes.c_double),
        ("beamx", ctypes.c_double), ("beamy", ctypes.c_double),
        ("usebeamstop", ctypes.c_int),
        ("bfactor", ctypes.c_double),
        ("waxs", ctypes.c_int),
        ("p1", ctypes.c_double),
        ("iso", ctypes.c_double), ("izero", ctypes.c_double), ("base", ctypes.c_double),
        ("tpv_domain_dev", ctypes.c_double), ("tpv_dw_dev", ctypes.c_double),
    ]


_lib = None


class CsFitParam(ctypes.Structure):
    """cs_fit_param (include/crystalscatter.h)"""
    _fields_ = [("key", ctypes.c_char * 48), ("min", ctypes.c_double), ("max", ctypes.c_double),
                ("fitstart", ctypes.c_double), ("fitres", ctypes.c_double), ("used", ctypes.c_int),
                ("fitvalid", ctypes.c_int)]


class CsFitReport(ctypes.Structure):
    """cs_fit_report (include/crystalscatter.h)"""
    _fields_ = [("repetitions", ctypes.c_int), ("aborted", ctypes.c_int), ("images", ctypes.c_long),
                ("chi2", ctypes.c_double), ("ms", ctypes.c_double), ("info", ctypes.c_char * 256)]


_OBJECTIVE = ctypes.CFUNCTYPE(None, ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_int,
                              ctypes.POINTER(ctypes.c_double), ctypes.c_void_p)


def _sig(lib):
    H = ctypes.c_void_p
    P = ctypes.POINTER
    lib.cs_version.restype = ctypes.c_char_p
    lib.cs_gpu_available.restype = ctypes.c_int
    lib.cs_measure_pipe_peaks.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    lib.cs_measure_pipe_peaks.restype = ctypes.c_int
    lib.cs_create.restype = H
    lib.cs_destroy.argtypes = [H]
    lib.cs_default_params.argtypes = [P(CsParams)]
    lib.cs_set_params.argtypes = [H, P(CsParams)]
    lib.cs_get_params.argtypes = [H, P(CsParams)]
    lib.cs_set_param.argtypes = [H, ctypes.c_char_p, ctypes.c_double]
    lib.cs_set_param_text.argtypes = [H, ctypes.c_char_p, ctypes.c_char_p]
    lib.cs_set_kv.argtypes = [H, ctypes.c_char_p]
    lib.cs_calc_image.argtypes = [H, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.cs_image_dims.argtypes = [H] + [P(ctypes.c_int)] * 4
    lib.cs_data.restype = P(ctypes.c_double)
    lib.cs_data.argtypes = [H]
    lib.cs_copy_image.argtypes = [H, ctypes.c_void_p, ctypes.c_size_t]
    lib.cs_timer_ms.restype = ctypes.c_double
    lib.cs_timer_ms.argtypes = [H, ctypes.c_int]
    lib.cs_new_switch_used.argtypes = [H]
    lib.cs_calc_image_device.argtypes = [H, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_int,
                                         ctypes.c_int, ctypes.c_int]
    lib.cs_launch_prepared.argtypes = [H, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_int]
    lib.cs_prepared_pixels.argtypes = [H, P(ctypes.c_long)]
    lib.cs_set_fit_data.argtypes = [H, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
    lib.cs_set_nofit_rect.argtypes = [H, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.cs_fit_chi2.argtypes = [H, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, P(ctypes.c_double),
                                P(ctypes.c_long), P(ctypes.c_long)]
    lib.cs_mixed_redo_pixels.argtypes = [H, P(ctypes.c_long)]
    lib.cs_last_error.restype = ctypes.c_char_p
    lib.cs_last_error.argtypes = [H]
    lib.cs_prepared_size.restype = ctypes.c_size_t
    lib.cs_prepare_params.argtypes = [P(CsParams), ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t,
                                      ctypes.c_char_p, ctypes.c_size_t]
    B = ctypes.c_void_p
    lib.cs_batch_create.restype = B
    lib.cs_batch_destroy.argtypes = [B]
    lib.cs_batch_last_error.restype = ctypes.c_char_p
    lib.cs_batch_last_error.argtypes = [B]
    lib.cs_batch_prepare.argtypes = [B, P(CsParams), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    lib.cs_batch_info.argtypes = [B, P(ctypes.c_size_t), P(ctypes.c_long), P(ctypes.c_int)]
    lib.cs_batch_upload_bytes.argtypes = [B, P(ctypes.c_size_t)]
    lib.cs_batch_set_schedule.argtypes = [B, ctypes.c_int, ctypes.c_int]
    lib.cs_batch_schedule.argtypes = [B, ctypes.c_int, P(ctypes.c_int), P(ctypes.c_int), P(ctypes.c_int),
                                      P(ctypes.c_double), P(ctypes.c_int)]
    lib.cs_batch_layout.argtypes = [B, ctypes.c_int, P(ctypes.c_size_t)] + [P(ctypes.c_int)] * 4
    lib.cs_batch_launch.argtypes = [B, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
    lib.cs_batch_profile.argtypes = [B, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_int,
                                     ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]
    lib.cs_batch_capture.argtypes = [B, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int]
    lib.cs_batch_replay.argtypes = [B, ctypes.c_void_p]
    lib.cs_batch_graph_nodes.argtypes = [B, P(ctypes.c_size_t)]
    lib.cs_batch_redo_pixels.argtypes = [B, ctypes.c_void_p, P(ctypes.c_long), P(ctypes.c_long)]
    lib.cs_batch_set_redo_capacity.argtypes = [B, ctypes.c_long]
    lib.cs_batch_timer_ms.restype = ctypes.c_double
    lib.cs_batch_timer_ms.argtypes = [B]
    lib.cs_batch_run_host.argtypes = [B, ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t]
    lib.cs_batch_set_fit.argtypes = [B, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_void_p]
    lib.cs_batch_fit_chi2.argtypes = [B, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    lib.cs_simplex_fit.argtypes = [P(CsParams), ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p,
                                   P(CsFitParam), ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double,
                                   ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_double,
                                   P(CsFitReport)]
    lib.cs_launch_prepared_mixed_noalloc.argtypes = [H, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
    M = ctypes.c_void_p
    lib.cs_mlp_create.restype = M
    lib.cs_mlp_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_ulonglong]
    lib.cs_mlp_destroy.argtypes = [M]
    lib.cs_mlp_last_error.restype = ctypes.c_char_p
    lib.cs_mlp_last_error.argtypes = [M]
    lib.cs_mlp_forward.argtypes = [M, ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.cs_mlp_gradients.argtypes = [M, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, P(ctypes.c_float),
                                     ctypes.c_void_p]
    lib.cs_mlp_train_step.argtypes = [M, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int, ctypes.c_float,
                                      P(ctypes.c_float), ctypes.c_void_p]
    lib.cs_mlp_layer_dims.argtypes = [M, ctypes.c_int, P(ctypes.c_int), P(ctypes.c_int)]
    lib.cs_mlp_get_layer.argtypes = [M, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                     ctypes.c_void_p]
    lib.cs_mlp_set_layer.argtypes = [M, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    lib.cs_upsample_bilinear.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_void_p, ctypes.c_void_p]
    lib.cs_rphi_device.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 8 + [ctypes.c_void_p, ctypes.c_void_p]
    lib.cs_simplex_minimize.argtypes = [_OBJECTIVE, ctypes.c_void_p, P(CsFitParam), ctypes.c_int, ctypes.c_double,
                                        ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.c_double, P(CsFitReport)]
    lib.cs_calc_batch.argtypes = [B, P(CsParams), ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_void_p, ctypes.c_size_t]
    return lib


def load_library(path=None):
    """Load the native library (built by ``crystalscatter_gb300.build``); raises if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or library_path()
    if not os.path.exists(p):
        raise CrystalScatterError(CS_ERR_CUDA, f"native library not built: {p} (run __graft_entry__.build())")
    lib = _sig(ctypes.CDLL(p))
    if path is None:
        _lib = lib
    return lib


def measure_pipe_peaks(stream=None):
    """Measured FMA rates (TFLOP/s: FP32, packed FP32 pairs, FP64) and the
    special-function unit's ex2 rate (Tops/s) of the current device
    (cs_measure_pipe_peaks)."""
    out = (ctypes.c_double * 4)()
    rc = load_library().cs_measure_pipe_peaks(_torch_stream(stream), out, 4)
    if rc != 0:
        raise CrystalScatterError(rc, "cs_measure_pipe_peaks failed")
    return {"fp32_tflops": out[0], "fp32x2_tflops": out[1], "fp64_tflops": out[2], "mufu_tops": out[3]}


def default_params():
    p = CsParams()
    load_library().cs_default_params(ctypes.byref(p))
    return p


def prepare_params(params, ign_new_switch=0, ign_cbs=0):
    """Host preparation only: returns (status, raw prepared block bytes, message)."""
    lib = load_library()
    n = lib.cs_prepared_size()
    buf = ctypes.create_string_buffer(n)
    err = ctypes.create_string_buffer(512)
    rc = lib.cs_prepare_params(ctypes.byref(params), ign_new_switch, ign_cbs, buf, n, err, 512)
    return rc, buf, err.value.decode()


class SasCalc_GENERIC_calculation:
    """Drop-in for the reference class: setters by group, doCalculation,
    doFitCalculation, setFitData, setNoFitRect, data()/minX()... ."""

    def __init__(self):
        self._lib = load_library()
        self._h = self._lib.cs_create()
        if not self._h:
            raise CrystalScatterError(CS_ERR_ALLOC, "cs_create failed")
        self.higResTimerElapsedPrep = 0.0
        self.higResTimerElapsedCalc = 0.0

    def __del__(self):
        self.cleanup()

    def cleanup(self):
        if getattr(self, "_h", None):
            self._lib.cs_destroy(self._h)
            self._h = None

    def _check(self, rc):
        if rc != CS_OK:
            raise CrystalScatterError(rc, self._lib.cs_last_error(self._h).decode())
        return rc

    # ---------------------------------------------------------------- params
    def params(self):
        p = CsParams()
        self._lib.cs_get_params(self._h, ctypes.byref(p))
        return p

    def set_params(self, p):
        self._check(self._lib.cs_set_params(self._h, ctypes.byref(p)))

    def setParam(self, key, value):
        """Reference key (e.g. 'EditRadius', 'ComboBoxParticle') -> number or combobox text."""
        if isinstance(value, str):
            return self._check(self._lib.cs_set_param_text(self._h, key.encode(), value.encode()))
        return self._check(self._lib.cs_set_param(self._h, key.encode(), float(value)))

    def setParams(self, mapping):
        for k, v in mapping.items():
            self.setParam(k, v)

    def setKeyValues(self, kv):
        """The console's ``--mcpval`` string ``"radius=10;cbparticle=sphere;..."``."""
        self._check(self._lib.cs_set_kv(self._h, kv.encode()))

    # the reference's individual setters (sc_calc_generic_gpu.h:108-353)
    def setLType(self, v): self.setParam("LType", v)
    def setUCA(self, v): self.setParam("uca", v)
    def setUCB(self, v): self.setParam("ucb", v)
    def setUCC(self, v): self.setParam("ucc", v)
    def setComboBoxParticle(self, v): self.setParam("ComboBoxParticle", v)
    def setOrdis(self, v): self.setParam("Ordis", v)
    def setComboBoxInterior(self, v): self.setParam("ComboBoxInterior", v)
    def setRadiusF(self, v): self.setParam("EditRadius", v)
    def setRadiusI(self, v): self.setParam("EditRadiusi", v)
    def setSigmaF(self, v): self.setParam("EditSigma", v)
    def setDBetaF(self, v): self.setParam("EditDbeta", v)
    def setLength(self, v): self.setParam("Length", v)
    def setSigmaL(self, v): self.setParam("SigmaL", v)
    def setComboBoxPeak(self, v): self.setParam("ComboBoxPeak", v)
    def setDisplacement(self, v): self.setParam("EditDebyeWaller", v)
    def setAzi(self, v): self.setParam("EditAzi", v)
    def setDomainsize(self, v): self.setParam("EditDomainSize", v)
    def setRadioButtonDebyeScherrer(self, f): self.setParam("RadButDebyeScherrer", 1 if f else 0)
    def setPolTheta(self, v): self.setParam("theta", v)
    def setPolPhi(self, v): self.setParam("phi", v)
    def setHKLmax(self, v): self.setParam("HKLmax", v)
    def setGridPoints(self, v, d1=False): self.setParam("GridPoints", v)
    def setpixnox(self, v): self.setParam("EditPixelNoX", v)
    def setpixnoy(self, v): self.setParam("EditPixelNoY", v)
    def setpixx(self, v): self.setParam("EditPixelX", v)
    def setpixy(self, v): self.setParam("EditPixelY", v)
    def setdet(self, v): self.setParam("EditDet", v)
    def setwave(self, v): self.setParam("EditWavelength", v)
    def setBeamStop(self, x, y):
        self.setParam("BeamPosX", x)
        self.setParam("BeamPosY", y)
    def setUseBeamStop(self, f): self.setParam("CenterBeam", 1 if f else 0)
    def setIso(self, v): self.setParam("iso", v)
    def setIZero(self, v): self.setParam("I0", v)
    def setBase(self, v): self.setParam("Base", v)

    # ------------------------------------------------------------ calculation
    def doCalculation(self, numThreads=0, bIgnoreNewSwitch=False, bIgnoreCbs=False, mode=CS_MODE_FP64):
        self._check(self._lib.cs_calc_image(self._h, int(numThreads), int(bool(bIgnoreNewSwitch)),
                                            int(bool(bIgnoreCbs)), int(mode)))
        self.higResTimerElapsedPrep = self._lib.cs_timer_ms(self._h, 0)
        self.higResTimerElapsedCalc = self._lib.cs_timer_ms(self._h, 1)

    def _dims(self):
        d = [ctypes.c_int() for _ in range(4)]
        self._lib.cs_image_dims(self._h, *[ctypes.byref(x) for x in d])
        return [x.value for x in d]

    def minX(self): return self._dims()[0]
    def maxX(self): return self._dims()[1]
    def minY(self): return self._dims()[2]
    def maxY(self): return self._dims()[3]

    def data(self):
        """The image as a (maxY-minY, maxX-minX) float64 array (copy)."""
        x0, x1, y0, y1 = self._dims()
        n = (x1 - x0) * (y1 - y0)
        out = np.empty(max(n, 0), dtype=np.float64)
        if n > 0:
            self._check(self._lib.cs_copy_image(self._h, out.ctypes.data, n))
        return out.reshape((y1 - y0, x1 - x0)) if n > 0 else out

    def xyIntensity(self, x, y):
        x0, x1, y0, y1 = self._dims()
        return float(self.data()[y - y0, x - x0])

    def newSwitchUsed(self):
        return bool(self._lib.cs_new_switch_used(self._h))

    def getLastErrorMessage(self):
        return self._lib.cs_last_error(self._h).decode()

    @staticmethod
    def gpuAvailable():
        return bool(load_library().cs_gpu_available())

    # -------------------------------------------------------------------- fit
    def setFitData(self, sx, sy, data):
        a = np.ascontiguousarray(data, dtype=np.float64).reshape(-1)
        if a.size != sx * sy:
            raise CrystalScatterError(CS_ERR_SIZE, "fit data size mismatch")
        self._check(self._lib.cs_set_fit_data(self._h, int(sx), int(sy), a.ctypes.data))
        return True

    def setNoFitRect(self, i, x0, y0, x1, y1):
        self._lib.cs_set_nofit_rect(self._h, i, x0, y0, x1, y1)

    def doFitCalculation(self, numThreads=0, bstop=0, border=0, mode=CS_MODE_FP64):
        """Returns (chi2, cnt, nancnt); chi2 is 1e20 on failure like the reference."""
        chi2 = ctypes.c_double()
        cnt = ctypes.c_long()
        nan = ctypes.c_long()
        rc = self._lib.cs_fit_chi2(self._h, int(numThreads), int(bstop), int(border), int(mode),
                                   ctypes.byref(chi2), ctypes.byref(cnt), ctypes.byref(nan))
        self._check(rc)
        return chi2.value, cnt.value, nan.value

    # --------------------------------------------------------- device-resident
    def calc_device(self, d_out_ptr, n_doubles, stream_ptr=0, bIgnoreNewSwitch=False, bIgnoreCbs=False,
                    mode=CS_MODE_FP64):
        self._check(self._lib.cs_calc_image_device(self._h, ctypes.c_void_p(d_out_ptr), n_doubles,
                                                   ctypes.c_void_p(stream_ptr), int(bool(bIgnoreNewSwitch)),
                                                   int(bool(bIgnoreCbs)), int(mode)))

    def launch_prepared(self, d_out_ptr, n_doubles, stream_ptr=0, mode=CS_MODE_FP64):
        self._check(self._lib.cs_launch_prepared(self._h, ctypes.c_void_p(d_out_ptr), n_doubles,
                                                 ctypes.c_void_p(stream_ptr), int(mode)))

    def mixed_redo_pixels(self):
        n = ctypes.c_long()
        self._check(self._lib.cs_mixed_redo_pixels(self._h, ctypes.byref(n)))
        return n.value

    def prepared_pixels(self):
        n = ctypes.c_long()
        self._check(self._lib.cs_prepared_pixels(self._h, ctypes.byref(n)))
        return n.value


def params_from_mapping(mapping):
    """A cs_params from reference keys, applied to the console defaults."""
    c = SasCalc_GENERIC_calculation()
    try:
        c.setParams(mapping)
        return c.params()
    finally:
        c.cleanup()


class SasCalcBatch:
    """Many parameter sets per launch (cs_batch_* of the C ABI).

    ``prepare(sets)`` takes reference-key dictionaries or CsParams; the images
    of all sets then lie in one float64 buffer (``info()``, ``layout(k)``).
    ``launch`` / ``capture`` + ``replay`` enqueue all images into a device
    buffer; ``calc`` is the host-buffer form returning one 2D array per set."""

    def __init__(self):
        self._lib = load_library()
        self._b = self._lib.cs_batch_create()
        if not self._b:
            raise CrystalScatterError(CS_ERR_ALLOC, "cs_batch_create failed")
        self.n = 0

    def __del__(self):
        self.cleanup()

    def cleanup(self):
        if getattr(self, "_b", None):
            self._lib.cs_batch_destroy(self._b)
            self._b = None

    def _check(self, rc):
        if rc != CS_OK:
            raise CrystalScatterError(rc, self._lib.cs_batch_last_error(self._b).decode())
        return rc

    @staticmethod
    def _array(sets):
        arr = (CsParams * len(sets))()
        for i, s in enumerate(sets):
            arr[i] = s if isinstance(s, CsParams) else params_from_mapping(s)
        return arr

    def prepare(self, sets, bIgnoreNewSwitch=False, bIgnoreCbs=False, host_threads=0):
        arr = self._array(sets)
        self._check(self._lib.cs_batch_prepare(self._b, arr, len(sets), int(bool(bIgnoreNewSwitch)),
                                               int(bool(bIgnoreCbs)), int(host_threads)))
        self.n = len(sets)
        return self

    def prep_ms(self):
        return self._lib.cs_batch_timer_ms(self._b)

    def info(self):
        """(total doubles of the image buffer, calculated pixels, key groups)"""
        d, p, g = ctypes.c_size_t(), ctypes.c_long(), ctypes.c_int()
        self._check(self._lib.cs_batch_info(self._b, ctypes.byref(d), ctypes.byref(p), ctypes.byref(g)))
        return d.value, p.value, g.value

    def set_schedule(self, chunk=-1, blocks_per_sm=0):
        """Force the mixed persistent kernel's work unit (0 = block tiles,
        32..256 = warp chunk) and resident blocks per SM; chunk -1 = autotune."""
        self._check(self._lib.cs_batch_set_schedule(self._b, int(chunk), int(blocks_per_sm)))

    def schedule(self, group=0):
        """The schedule in use for a key group: dict(key, chunk, blocks_per_sm,
        ns_per_pixel, tuned)."""
        k, c, b, t = ctypes.c_int(), ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        ns = ctypes.c_double()
        self._check(self._lib.cs_batch_schedule(self._b, int(group), ctypes.byref(k), ctypes.byref(c), ctypes.byref(b),
                                                ctypes.byref(ns), ctypes.byref(t)))
        return {"key": hex(k.value), "chunk": c.value, "blocks_per_sm": b.value, "ns_per_pixel": ns.value,
                "tuned": bool(t.value)}

    def upload_bytes(self):
        """host-to-device bytes of the last prepare"""
        n = ctypes.c_size_t()
        self._check(self._lib.cs_batch_upload_bytes(self._b, ctypes.byref(n)))
        return n.value

    def layout(self, k):
        """(offset, xmin, xmax, ymin, ymax) of set k's image in the buffer"""
        o = ctypes.c_size_t()
        d = [ctypes.c_int() for _ in range(4)]
        self._check(self._lib.cs_batch_layout(self._b, int(k), ctypes.byref(o), *[ctypes.byref(x) for x in d]))
        return (o.value,) + tuple(x.value for x in d)

    def launch(self, d_out_ptr, n_doubles, stream_ptr=0, mode=CS_MODE_FP64, schedule=CS_SCHED_PERSISTENT):
        self._check(self._lib.cs_batch_launch(self._b, ctypes.c_void_p(d_out_ptr), int(n_doubles),
                                              ctypes.c_void_p(stream_ptr), int(mode), int(schedule)))

    def profile(self, d_out_ptr, n_doubles, stream_ptr=0, mode=CS_MODE_MIXED):
        """One persistent run with CUDA events around the main and redo kernels:
        (main_ms, redo_ms)."""
        a, r = ctypes.c_double(), ctypes.c_double()
        self._check(self._lib.cs_batch_profile(self._b, ctypes.c_void_p(d_out_ptr), int(n_doubles),
                                               ctypes.c_void_p(stream_ptr), int(mode), ctypes.byref(a),
                                               ctypes.byref(r)))
        return a.value, r.value

    def capture(self, d_out_ptr, n_doubles, mode=CS_MODE_FP64, schedule=CS_SCHED_PERSISTENT):
        self._check(self._lib.cs_batch_capture(self._b, ctypes.c_void_p(d_out_ptr), int(n_doubles), int(mode),
                                               int(schedule)))

    def replay(self, stream_ptr=0):
        self._check(self._lib.cs_batch_replay(self._b, ctypes.c_void_p(stream_ptr)))

    def graph_nodes(self):
        n = ctypes.c_size_t()
        self._check(self._lib.cs_batch_graph_nodes(self._b, ctypes.byref(n)))
        return n.value

    def redo_pixels(self, stream_ptr=0):
        """(guarded pixels of the last mixed persistent run, list capacity per group)"""
        n, cap = ctypes.c_long(), ctypes.c_long()
        self._check(self._lib.cs_batch_redo_pixels(self._b, ctypes.c_void_p(stream_ptr), ctypes.byref(n),
                                                   ctypes.byref(cap)))
        return n.value, cap.value

    def set_redo_capacity(self, entries_per_group):
        self._check(self._lib.cs_batch_set_redo_capacity(self._b, int(entries_per_group)))

    def split(self, flat):
        """Per-set 2D views of a flat image buffer laid out by this batch."""
        out = []
        for k in range(self.n):
            o, x0, x1, y0, y1 = self.layout(k)
            out.append(flat[o:o + (x1 - x0) * (y1 - y0)].reshape(y1 - y0, x1 - x0))
        return out

    def set_fit(self, data, bstop=0, border=0, nofit=None):
        """Target image (2D, the image's size) and masks of doFitCalculation;
        nofit: up to 4 rectangles (x0, y0, x1, y1). Prepare the batch after it."""
        a = np.ascontiguousarray(data, dtype=np.float64)
        h, w = a.shape
        nf = np.full(16, -1, dtype=np.int32)
        for i, r in enumerate(nofit or []):
            nf[4 * i:4 * i + 4] = r
        self._check(self._lib.cs_batch_set_fit(self._b, int(w), int(h), a.ctypes.data, int(bstop), int(border),
                                               nf.ctypes.data))

    def fit_chi2(self, mode=CS_MODE_FP64):
        """(chi2, cnt, nancnt) arrays over the prepared sets."""
        chi2 = np.empty(self.n, dtype=np.float64)
        cnt = np.empty(self.n, dtype=np.int64)
        nan = np.empty(self.n, dtype=np.int64)
        self._check(self._lib.cs_batch_fit_chi2(self._b, int(mode), chi2.ctypes.data, cnt.ctypes.data,
                                                nan.ctypes.data))
        return chi2, cnt, nan

    def run_host(self, mode=CS_MODE_FP64, out=None):
        """Computes the prepared sets (persistent schedule) into a host buffer
        (flat float64, allocated when not given) and returns it."""
        total = self.info()[0]
        if out is None:
            out = np.empty(total, dtype=np.float64)
        self._check(self._lib.cs_batch_run_host(self._b, int(mode), out.ctypes.data, out.size))
        return out

    def calc(self, sets, bIgnoreNewSwitch=False, bIgnoreCbs=False, mode=CS_MODE_FP64):
        """Host in, host out: prepares and computes all sets and returns one
        image per set."""
        self.prepare(sets, bIgnoreNewSwitch, bIgnoreCbs)
        return [a.copy() for a in self.split(self.run_host(mode))]


def _fit_table(fit_params):
    arr = (CsFitParam * len(fit_params))()
    for i, fp in enumerate(fit_params):
        arr[i].key = fp["key"].encode()
        arr[i].min = float(fp["min"])
        arr[i].max = float(fp["max"])
        arr[i].fitstart = float(fp["start"])
        arr[i].used = 1 if fp.get("used", True) else 0
    return arr


def _report(rep):
    return {"repetitions": rep.repetitions, "aborted": rep.aborted, "images": rep.images, "chi2": rep.chi2,
            "ms": rep.ms}


def simplex_minimize(fn, fit_params, stp=0.1, maxit=100, ftol=1e-4, schedule=CS_FIT_SEQUENTIAL, chi2_stop=0.0):
    """The library's simplex (cs_simplex_minimize) over a Python objective:
    fn(points) with points an (n, nparams) array in the simplex's table order
    (fitted keys sorted, then fixed keys sorted) returns n values."""
    lib = load_library()

    def cb(points, n, m, values, ctx):
        pts = np.ctypeslib.as_array(points, shape=(n, m)).copy()
        v = np.asarray(fn(pts), dtype=np.float64)
        for i in range(n):
            values[i] = float(v[i])

    cfn = _OBJECTIVE(cb)
    arr = _fit_table(fit_params)
    rep = CsFitReport()
    rc = lib.cs_simplex_minimize(cfn, None, arr, len(fit_params), float(stp), int(maxit), float(ftol), int(schedule),
                                 float(chi2_stop), ctypes.byref(rep))
    if rc != CS_OK:
        raise CrystalScatterError(rc, rep.info.decode() or "simplex failed")
    return {arr[i].key.decode(): arr[i].fitres for i in range(len(fit_params))}, _report(rep)


def simplex_fit(base, data, fit_params, stp=0.1, maxit=100, ftol=1e-4, border=0, bstop=0, nofit=None,
                mode=CS_MODE_FP64, schedule=CS_FIT_SEQUENTIAL, chi2_stop=0.0):
    """SasCalc_SimplexFit2D::doSimplexFit2D on the GPU (cs_simplex_fit).

    base: reference-key dict or CsParams; data: 2D target of the image's size;
    fit_params: list of dicts {key, min, max, start, used}. Returns
    ({key: fitres}, report dict)."""
    lib = load_library()
    p = base if isinstance(base, CsParams) else params_from_mapping(base)
    a = np.ascontiguousarray(data, dtype=np.float64)
    h, w = a.shape
    nf = np.full(16, -1, dtype=np.int32)
    for i, r in enumerate(nofit or []):
        nf[4 * i:4 * i + 4] = r
    arr = _fit_table(fit_params)
    rep = CsFitReport()
    rc = lib.cs_simplex_fit(ctypes.byref(p), a.ctypes.data, int(w), int(h), nf.ctypes.data, arr, len(fit_params),
                            float(stp), int(maxit), float(ftol), int(border), int(bstop), int(mode), int(schedule),
                            float(chi2_stop), ctypes.byref(rep))
    if rc != CS_OK:
        raise CrystalScatterError(rc, rep.info.decode() or "simplex fit failed")
    res = {arr[i].key.decode(): arr[i].fitres for i in range(len(fit_params))}
    return res, _report(rep)


def _torch_stream(stream):
    """The stream handle for the cs_mlp calls: the caller's, else torch's
    current stream, so that the network's kernels are ordered after the torch
    operations that produced their inputs (0 = the legacy default stream, for
    which the library uses the network's own stream, synchronous with it)."""
    if stream is not None:
        return int(stream)
    import torch
    return int(torch.cuda.current_stream().cuda_stream)


class SurrogateMLP:
    """The surrogate network of the library (cs_mlp_*): n_in -> hidden x3 ->
    n_out with GELU, BF16 tensor-core GEMMs with FP32 accumulation, Adam on
    the device. Inputs and outputs are CUDA float32 tensors (torch is used for
    device memory only)."""

    def __init__(self, n_in, hidden=512, n_out=4096, seed=0):
        self._lib = load_library()
        self._m = self._lib.cs_mlp_create(int(n_in), int(hidden), int(n_out), int(seed))
        if not self._m:
            raise CrystalScatterError(CS_ERR_CUDA, "cs_mlp_create failed (no GPU or unsupported sizes)")
        self.n_in, self.hidden, self.n_out = n_in, hidden, n_out

    def __del__(self):
        self.cleanup()

    def cleanup(self):
        if getattr(self, "_m", None):
            self._lib.cs_mlp_destroy(self._m)
            self._m = None

    def _check(self, rc):
        if rc != CS_OK:
            raise CrystalScatterError(rc, self._lib.cs_mlp_last_error(self._m).decode())

    def forward(self, x, stream=None):
        import torch
        stream = _torch_stream(stream)
        x = x.contiguous().float()
        y = torch.empty((x.shape[0], self.n_out), dtype=torch.float32, device=x.device)
        self._check(self._lib.cs_mlp_forward(self._m, x.data_ptr(), x.shape[0], y.data_ptr(), ctypes.c_void_p(stream)))
        return y

    def gradients(self, x, t, stream=None):
        stream = _torch_stream(stream)
        loss = ctypes.c_float()
        x = x.contiguous().float()
        t = t.contiguous().float()
        self._check(self._lib.cs_mlp_gradients(self._m, x.data_ptr(), t.data_ptr(), x.shape[0], ctypes.byref(loss),
                                               ctypes.c_void_p(stream)))
        return loss.value

    def train_step(self, x, t, lr, stream=None, want_loss=True):
        stream = _torch_stream(stream)
        loss = ctypes.c_float()
        self._check(self._lib.cs_mlp_train_step(self._m, x.data_ptr(), t.data_ptr(), x.shape[0], float(lr),
                                                ctypes.byref(loss) if want_loss else None, ctypes.c_void_p(stream)))
        return loss.value if want_loss else None

    def layer(self, l):
        r, c = ctypes.c_int(), ctypes.c_int()
        self._lib.cs_mlp_layer_dims(self._m, l, ctypes.byref(r), ctypes.byref(c))
        w = np.empty((r.value, c.value), np.float32)
        b = np.empty(r.value, np.float32)
        gw = np.empty_like(w)
        gb = np.empty_like(b)
        self._check(self._lib.cs_mlp_get_layer(self._m, l, w.ctypes.data, b.ctypes.data, gw.ctypes.data,
                                               gb.ctypes.data))
        return {"w": w, "b": b, "gw": gw, "gb": gb}

    def set_layer(self, l, w, b):
        w = np.ascontiguousarray(w, np.float32)
        b = np.ascontiguousarray(b, np.float32)
        self._check(self._lib.cs_mlp_set_layer(self._m, l, w.ctypes.data, b.ctypes.data))


def upsample_bilinear(x, factor, stream=None):
    """(n, s, s) CUDA float32 -> (n, s*factor, s*factor), cs_upsample_bilinear"""
    import torch
    stream = _torch_stream(stream)
    x = x.contiguous().float()
    n, s = x.shape[0], x.shape[1]
    out = torch.empty((n, s * factor, s * factor), dtype=torch.float32, device=x.device)
    rc = load_library().cs_upsample_bilinear(x.data_ptr(), n, s, int(factor), out.data_ptr(), ctypes.c_void_p(stream))
    if rc != CS_OK:
        raise CrystalScatterError(rc, "upsample failed")
    return out


CS_RPHI_SCALE, CS_RPHI_CLIP, CS_RPHI_CLIP40 = 1, 2, 4


def rphi_device(img, x0, x1, y0, y1, xcenter, ycenter, s, scale=False, clip=False, clip40=False, stream=None):
    """The r-phi image (s x s CUDA float64) of a CUDA image (rows y0..y1-1,
    columns x0..x1-1) around the beam centre, cs_rphi_device; the GPU form of
    ``postproc.rphi`` (SasCalc_PostProc::generateRphi)."""
    import torch
    img = img.contiguous().to(torch.float64)
    if img.numel() != (y1 - y0) * (x1 - x0):
        raise ValueError("image size does not match its coordinate ranges")
    out = torch.empty((s, s), dtype=torch.float64, device=img.device)
    flags = (CS_RPHI_SCALE if scale else 0) | (CS_RPHI_CLIP if clip else 0) | (CS_RPHI_CLIP40 if clip40 else 0)
    rc = load_library().cs_rphi_device(img.data_ptr(), x0, x1, y0, y1, xcenter, ycenter, s, flags,
                                       out.data_ptr(), _torch_stream(stream))
    if rc != CS_OK:
        raise CrystalScatterError(rc, "r-phi transform rejected its arguments" if rc == CS_ERR_PARAM
                                  else "r-phi transform failed")
    return out
