"""Image post-processing of the training-data generator: the r-phi transform.

``rphi`` resamples a detector image onto a polar grid around the beam
centre (rows: angle, columns: radius), as ``SasCalc_PostProc::generateRphi``
(``Source/sc_postproc.cpp:53-334``) does for the AI/TPV data sets, with its
scaling and clipping options (``scaleAndClipData``, ``:764-823``).

The grid follows the reference step by step:

* radius k runs over ``ir = 0, irstp, 2 irstp, ...`` while ``ir <= irmax``,
  accumulated in single precision (``irstp = float(irmax)/float(s-1)``,
  ``irmax`` the farthest corner distance rounded, corners taken at 1 and
  size-1); the output column is ``int(float(i*s) + ir/irstp)``, so a float
  step that lands just below an integer writes the column before it;
* angle row i = 0..s averages ``umf = max(ceil(phiber*rad), 1)`` samples at
  ``phi = (i-1.5)*phiber + (j-0.5)*phiber/umf`` (row s falls outside the
  array), each bilinear over the four neighbours inside the image with
  weights from ``int()`` truncation (toward zero), the average clamped at 0.

Entries no radius step writes are 0 here; the reference leaves whatever its
reused array held. Images are given with minimum coordinates at most 0 (the
reference shifts those to 0; a positive minimum makes its pixel lookup read
the wrong rows, which is not reproduced: ValueError).
"""
import math

import numpy as np

F32 = np.float32


def scale_and_clip(a, scale=False, clip=False, clip40=False):
    """scaleAndClipData without the log option, in place; returns a."""
    if scale:
        # the reference's running maximum from 0 (NaN entries never win)
        m = float(np.nanmax(a, initial=0.0)) if a.size else 0.0
        with np.errstate(divide="ignore", invalid="ignore"):
            a /= m
    if clip:
        with np.errstate(divide="ignore"):
            a[:] = ((np.log(np.abs(a) / 1e-20) / math.log(10)) + 6.0) / 6.0
        a[a < 0] = 0.0
    if clip40:
        a[:] = 1.0 - (1.0 - a) / (1.0 - 0.4)
        a[a < 0] = 0.0
    return a


def rphi(data, x0, x1, y0, y1, xcenter, ycenter, s, scale=False, clip=False, clip40=False):
    """The r-phi image (s x s, row = angle index, column = radius index) of
    ``data`` (rows y0..y1-1, columns x0..x1-1, row-major) around the beam
    centre (xcenter, ycenter) in the same coordinates."""
    if s < 2:
        raise ValueError("output size must be at least 2")
    d = np.asarray(data, dtype=np.float64).reshape(y1 - y0, x1 - x0)
    if x0 < 0:
        x1 -= x0
        xcenter -= x0
        x0 = 0
    if y0 < 0:
        y1 -= y0
        ycenter -= y0
        y0 = 0
    if x0 > 0 or y0 > 0:
        raise ValueError("r-phi transform: image minimum coordinates must be at most 0")
    srcsx, srcsy = x1 - x0, y1 - y0
    out = np.zeros(s * s)
    phisteps = s
    phiber = 2.0 * math.pi / phisteps
    sq = lambda v: v * v  # noqa: E731
    rmax = math.sqrt(sq(1.0 - xcenter) + sq(1.0 - ycenter))
    rmax = max(rmax, math.sqrt(sq((srcsx - 1.0) - xcenter) + sq(1.0 - ycenter)))
    rmax = max(rmax, math.sqrt(sq((srcsx - 1.0) - xcenter) + sq((srcsy - 1.0) - ycenter)))
    rmax = max(rmax, math.sqrt(sq(1.0 - xcenter) + sq((srcsy - 1.0) - ycenter)))
    irmax = int(rmax + 0.5)
    irstp = F32(F32(irmax) / F32(s - 1))
    rows = np.arange(phisteps + 1, dtype=np.float64)
    flat = d.reshape(-1)
    ir = F32(0.0)
    while ir <= F32(irmax):
        rad = float(ir)
        umf = max(1024 - int(1024.0 - phiber * rad), 1)
        j = np.arange(1, umf + 1, dtype=np.float64)
        phi = (rows[:, None] - 1.5) * phiber + (j[None, :] - 0.5) * phiber / umf
        xs = xcenter + rad * np.cos(phi)
        ys = ycenter + rad * np.sin(phi)
        ix1 = np.trunc(xs).astype(np.int64)
        iy1 = np.trunc(ys).astype(np.int64)
        rex = xs - ix1
        rey = ys - iy1
        twt = np.zeros(phisteps + 1)
        avg = np.zeros(phisteps + 1)
        for dx, dy, w in ((0, 0, (1.0 - rex) * (1.0 - rey)), (1, 0, rex * (1.0 - rey)),
                          (0, 1, (1.0 - rex) * rey), (1, 1, rex * rey)):
            ix, iy = ix1 + dx, iy1 + dy
            ok = (ix >= 0) & (ix < srcsx) & (iy >= 0) & (iy < srcsy)
            vals = np.where(ok, flat[np.where(ok, ix + srcsx * iy, 0)], 0.0)
            twt += np.where(ok, w, 0.0).sum(axis=1)
            avg += np.where(ok, w * vals, 0.0).sum(axis=1)
        pos = twt > 0.0
        avg[pos] = avg[pos] / twt[pos]
        col = F32(ir / irstp)
        for i in range(phisteps + 1):
            idx = int(F32(F32(i * s) + col))
            if idx < s * s:
                out[idx] = 0.0 if avg[i] < 0 else avg[i]
        ir = F32(ir + irstp)
    return scale_and_clip(out, scale, clip, clip40).reshape(s, s)
