"""ctypes mirror of the prepared constant block ``cs_prepared``
(crystalscatter_gb300/csrc/cs_prepared.h), for inspecting the host
preparation from Python (known-answer tests, diagnostics)."""
import ctypes

_I = ctypes.c_int
_D = ctypes.c_double


class CsPrepared(ctypes.Structure):
    _fields_ = (
        [(n, _I) for n in ("key ign_switch particle shp ltype ordis cs part cdim partdim orcase "
                           "lattice twin debyescherrer para use1d usebeamstop zmax zzmin zzmax iimin iimax "
                           "xmin xmax ymin ymax calc_quadrants expand").split()]
        + [(n, _D) for n in ("qmax qmin pixnox pixnoy pixx_m pixy_m beamx0 beamy0 det wave base izero iso ifluc "
                             "rfluc radius radiusi sigma sigmal length p1 rho alphash1 alpha poltheta polphi dbeta "
                             "norm por order").split()]
        + [("limq", _D * 10), ("limqf", _D * 10)]
        + [(n, _D) for n in "cosphic sinphic cosphi sinphi costheta sintheta".split()]
        + [("sig", _D * 3), ("ax1", _D * 3), ("ax2", _D * 3), ("ax3", _D * 3), ("gamma_ratio", _D * 2),
           ("romb_delta_b", _D), ("romb_chi_b", _D), ("romb_dbeta", _D), ("romb_p", _D * 9),
           ("peakmax1", _I), ("peakmax2", _I), ("latpar", _D * 4)]
        + [(n, _D) for n in "dwfactor uca ucb domainsize width_zuf reldis dist phiwidth ceff".split()]
        + [("carrp", (_D * 151) * 9), ("carrf", (_D * 151) * 9), ("carr11pm", (_D * 131) * 131),
           ("latpar1", (_I * 6) * 2500), ("latpar2", (_I * 6) * 2500), ("latpar3", (ctypes.c_float * 17) * 2500)]
        + [("nofit_x0", _I * 4), ("nofit_x1", _I * 4), ("nofit_y0", _I * 4), ("nofit_y1", _I * 4)]
        + [(n, _I) for n in "fit_width fit_height fit_bstop fit_border".split()]
        + [(n, _D) for n in "pk_c1 pk_c2 pk_c3 pk_c4 pk_eta pk_beta pk_gbeta pk_gbeta_h".split()]
    )


def prepare(params, ign_new_switch=0, ign_cbs=0):
    """(status, CsPrepared, message) for a cs_params."""
    from . import load_library
    lib = load_library()
    assert lib.cs_prepared_size() == ctypes.sizeof(CsPrepared), "cs_prepared layout mismatch"
    out = CsPrepared()
    err = ctypes.create_string_buffer(512)
    rc = lib.cs_prepare_params(ctypes.byref(params), ign_new_switch, ign_cbs, ctypes.byref(out),
                               ctypes.sizeof(out), err, 512)
    return rc, out, err.value.decode()
