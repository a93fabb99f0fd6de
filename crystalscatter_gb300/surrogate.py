"""Surrogate-seeded 2D fits: a small network, trained on patterns the
simulator itself computes, proposes the simplex's start point; the exact
calculation refines and judges every fit (the reference's fit,
Source/sc_simplexfit2d.cpp, starts wherever the user puts it).

Families (parameters uniform within +-30 % of the nominal values):
  "2"   cylinders, Gaussian orientation, axis in the detector plane at
        azimuth 30 deg (the benchmark's config 2) with its 8 free parameters
        radius, sigma, length, sigma_L, orientation width, theta, phi, I0;
  "2x"  the same at azimuth 0 (axis along x), whose orientation average runs
        the full nested Romberg; theta and phi stay at 90 / 0, because any
        other value selects the reference's general-orientation case, whose
        orientation integral is zero (6 free parameters).

Network: parameters (scaled to [-1, 1]) -> 512 -> 512 -> 512 -> 64 x 64
log10 intensity (GELU, BF16 tensor-core GEMMs, FP32 accumulation; the
library's cs_mlp kernels), bilinearly upsampled to the 256 x 256 fit grid.

Training patterns are computed on a 128 x 128 detector with the fit image's
q-range and averaged over 2 x 2 pixels; targets carry Poisson noise (a peak of
`counts` counts) on the 256 x 256 fit grid.
"""
import math
import time

import numpy as np

import crystalscatter_gb300 as cs
from crystalscatter_gb300 import configs as C

SPREAD = 0.30
# start vectors stay inside +-START_BOX: the reference's initial simplex moves
# every parameter up by a fraction of its step, so a start at a fit limit
# puts every vertex outside the limits (chi^2 1e20) and the fit cannot move
START_BOX = 0.8
FLOOR = 1e-9  # intensity floor of the log10 targets (zero pixels of the degenerate family)
FAMILIES = {
    "2": (C.CYL_GAUSS, ["EditRadius", "EditSigma", "Length", "SigmaL", "EditDbeta", "theta", "phi", "I0"]),
    "2x": (C.CYL_GAUSS_X, ["EditRadius", "EditSigma", "Length", "SigmaL", "EditDbeta", "I0"]),
}
# first key in the fit table: the reference's initialisation zeroes the first
# parameter (sorted by key) of every initial vertex; EditAzi sorts first, is not
# used by these families and its limits 0..360 are not checked
PAD_KEY = {"key": "EditAzi", "min": 0.0, "max": 360.0, "start": 5.0, "used": True}


class Family:
    """train_grid: GridPoints of the training patterns (half their edge), which
    are averaged down to the network's 64 x 64 grid: 256 gives the benchmark's
    own 512 x 512 detector (8 x 8 pixels per coarse pixel, i.e. 2 x 2 to the
    256 x 256 fit grid, then 4 x 4); 64 gives 128 x 128 patterns (2 x 2)."""

    def __init__(self, name, fit_grid=128, train_grid=64):
        base, keys = FAMILIES[name]
        self.name = name
        self.keys = keys
        self.nominal = {k: float(base.get(k, 1.0 if k == "I0" else 0.0)) for k in keys}
        self.fit_base = C.scaled(base, fit_grid)  # 256 x 256 fit image, the detector's q-range
        self.train_grid = train_grid
        self.train_base = C.scaled(base, train_grid)

    def params(self, u, base):
        p = dict(base)
        for k, v in zip(self.keys, u):
            p[k] = self.nominal[k] * (1.0 + SPREAD * float(v))
        return p

    def limits(self, k):
        a, b = self.nominal[k] * (1 - SPREAD), self.nominal[k] * (1 + SPREAD)
        return min(a, b), max(a, b)

    def u_of(self, res):
        return np.array([(res[k] / self.nominal[k] - 1.0) / SPREAD for k in self.keys])


def bin2(img):
    h, w = img.shape[-2:]
    return img.reshape(img.shape[:-2] + (h // 2, 2, w // 2, 2)).mean(axis=(-1, -3))


def simulate(fam, U, base, mode=cs.CS_MODE_MIXED, chunk=1024):
    """images of the parameter vectors U (n x k) on `base`'s detector"""
    out = []
    b = cs.SasCalcBatch()
    for s in range(0, len(U), chunk):
        sets = [fam.params(u, base) for u in U[s:s + chunk]]
        out.extend(b.calc(sets, mode=mode))
    b.cleanup()
    return np.stack(out)


def training_set(fam, n, seed=0, mode=cs.CS_MODE_MIXED):
    """(U, Y): n parameter vectors in [-1, 1]^k and 64 x 64 log10 targets"""
    rng = np.random.default_rng(seed)
    U = rng.uniform(-1, 1, (n, len(fam.keys)))
    imgs = simulate(fam, U, fam.train_base, mode)
    binned = bin2(np.where(np.isfinite(imgs), imgs, 0.0))  # the reference's non-finite pixels count as empty
    Y = np.log10(np.maximum(binned, FLOOR)).reshape(n, -1).astype(np.float32)
    return U.astype(np.float32), Y


def training_set_device(fam, n, seed=0, mode=cs.CS_MODE_MIXED, chunk=1024):
    """(U, Y) as CUDA tensors: n parameter vectors in [-1, 1]^k and their 64 x 64
    log10 targets, the patterns computed on fam.train_base's detector into a
    device buffer (batched persistent launches) and averaged to 64 x 64 there;
    only the coarse targets stay (n x 4096 float32). Returns also the seconds
    spent in host preparation."""
    import torch
    rng = np.random.default_rng(seed)
    U = rng.uniform(-1, 1, (n, len(fam.keys)))
    edge = 2 * fam.train_grid
    f = edge // 64
    Y = torch.empty((n, 64 * 64), dtype=torch.float32, device="cuda")
    b = cs.SasCalcBatch()
    buf = None
    t_prep = 0.0
    # a created stream: handle 0 (torch's default stream) would select the
    # batch's own stream, unordered with the torch operations around the launch
    ts = torch.cuda.Stream()
    ts.wait_stream(torch.cuda.current_stream())
    try:
        with torch.cuda.stream(ts):
            for s0 in range(0, n, chunk):
                sets = [fam.params(u, fam.train_base) for u in U[s0:s0 + chunk]]
                t0 = time.perf_counter()
                b.prepare(sets)
                t_prep += time.perf_counter() - t0
                total = b.info()[0]
                m = len(sets)
                # the sets' images (equal sizes) at their offsets in the buffer
                offs = []
                for k in range(m):
                    o, x0, x1, y0, y1 = b.layout(k)
                    assert (x1 - x0, y1 - y0) == (edge, edge)
                    offs.append(o)
                if buf is None or buf.numel() < total:
                    buf = torch.empty(total, dtype=torch.float64, device="cuda")
                b.launch(buf.data_ptr(), total, ts.cuda_stream, mode=mode)
                idx = torch.tensor(offs, dtype=torch.int64, device="cuda")[:, None] + \
                    torch.arange(edge * edge, dtype=torch.int64, device="cuda")[None, :]
                img = buf[idx].view(m, edge, edge)
                # the reference's non-finite pixels count as empty
                img = torch.where(torch.isfinite(img), img, torch.zeros_like(img))
                coarse = img.view(m, 64, f, 64, f).mean(dim=(2, 4))
                Y[s0:s0 + m] = torch.log10(coarse.clamp_min(FLOOR)).view(m, -1).float()
                # the next prepare rewrites the prepared blocks these kernels read
                ts.synchronize()
        torch.cuda.synchronize()
    finally:
        b.cleanup()
    return torch.from_numpy(U.astype(np.float32)).cuda(), Y, t_prep


class Surrogate:
    """the trained network with its input/output scaling"""

    def __init__(self, fam, hidden=512, seed=0):
        self.fam = fam
        self.net = cs.SurrogateMLP(len(fam.keys), hidden, 64 * 64, seed=seed)
        self.mean, self.std = 0.0, 1.0  # per-pixel tensors after training

    def train(self, U, Y, epochs=200, batch=512, lr=1e-3, seed=0, pixel_norm=False):
        """U, Y: numpy arrays or CUDA tensors (rows: parameter vectors and
        their 64 x 64 log10 targets)."""
        import torch
        if not isinstance(Y, torch.Tensor):
            Y = torch.from_numpy(np.ascontiguousarray(Y, dtype=np.float32)).cuda()
        if not isinstance(U, torch.Tensor):
            U = torch.from_numpy(np.ascontiguousarray(U, dtype=np.float32)).cuda()
        # per-pixel standardisation: the network learns each q's deviation from
        # its mean over the family (floor: 5 % of the overall spread); or one
        # mean and spread for all pixels
        Yd = Y.double()
        if pixel_norm:
            mean = Yd.mean(dim=0)
            std = torch.clamp(Yd.std(dim=0), min=0.05 * float(Yd.std()) + 1e-6)
        else:
            mean = torch.full((Y.shape[1],), float(Yd.mean()), dtype=torch.float64, device="cuda")
            std = torch.full((Y.shape[1],), float(Yd.std()) or 1.0, dtype=torch.float64, device="cuda")
        self.mean = mean.float()
        self.std = std.float()
        x = U.contiguous()
        y = ((Yd - mean) / std).float().contiguous()
        del Yd
        n = len(U)
        g = torch.Generator(device="cpu").manual_seed(seed)
        steps = epochs * max(1, n // batch)
        losses = []
        k = 0
        t0 = time.perf_counter()
        for ep in range(epochs):
            perm = torch.randperm(n, generator=g).cuda()
            for s in range(0, n - batch + 1, batch):
                idx = perm[s:s + batch]
                rate = lr * 0.5 * (1 + math.cos(math.pi * k / steps))
                want = s + 2 * batch > n
                loss = self.net.train_step(x[idx].contiguous(), y[idx].contiguous(), rate, want_loss=want)
                if want:
                    losses.append(loss)
                k += 1
        torch.cuda.synchronize()
        return {"epochs": epochs, "steps": k, "seconds": time.perf_counter() - t0, "loss_per_epoch": losses}

    def predict(self, U):
        """64 x 64 log10 intensities of the rows of U (CUDA tensor)"""
        return self.net.forward(U) * self.std + self.mean

    def propose(self, target, rounds=3, candidates=4096, keep=16, seed=0, shortlist=8, spacing=0.15):
        """Candidate search on the network's prediction: (best start vector u in
        [-1, 1]^k by the FQSVERGL distance of the upsampled prediction to the
        target (256 x 256, pixels <= 0 ignored), its distance, shortlist). Each
        round samples around the mean of the previous round's best `keep`; the
        shortlist holds up to `shortlist` mutually distant (max-norm >= spacing)
        candidates, best first, drawn from all rounds, for an exact check."""
        import torch
        rng = np.random.default_rng(seed)
        t = torch.from_numpy(np.log10(np.where(target > 0, target, 1.0))).float().cuda()
        mask = torch.from_numpy(target > 0).cuda()
        k = len(self.fam.keys)
        centre, width = np.zeros(k), 1.0
        pool_u, pool_c = [], []
        for r in range(rounds):
            U = np.clip(centre + width * rng.uniform(-1, 1, (candidates, k)), -1, 1).astype(np.float32)
            cost = []
            for s in range(0, candidates, 512):
                pred = self.predict(torch.from_numpy(U[s:s + 512]).cuda()).reshape(-1, 64, 64)
                up = cs.upsample_bilinear(pred, target.shape[0] // 64)
                d = torch.where(mask, up - t, torch.zeros_like(up))
                cost.append((d * d).sum(dim=(1, 2)).cpu().numpy())
            cost = np.concatenate(cost)
            order = np.argsort(cost)
            pool_u.append(U[order[:4 * shortlist]])
            pool_c.append(cost[order[:4 * shortlist]])
            centre = U[order[:keep]].mean(axis=0)
            width *= 0.35
        pu, pc = np.concatenate(pool_u), np.concatenate(pool_c)
        picks = []
        for i in np.argsort(pc):
            if all(np.abs(pu[i] - pu[j]).max() >= spacing for j in picks):
                picks.append(i)
            if len(picks) == shortlist:
                break
        return pu[picks[0]].copy(), float(pc[picks[0]]), pu[picks].copy()


def exact_pick(fam, target, U, mode=cs.CS_MODE_MIXED):
    """The row of U whose image has the lowest exact chi^2 (doFitCalculation
    without masks) against the 256 x 256 target: one batched evaluation."""
    b = cs.SasCalcBatch()
    try:
        b.set_fit(target)
        b.prepare([fam.params(u, fam.fit_base) for u in U])
        chi2, _, _ = b.fit_chi2(mode)
    finally:
        b.cleanup()
    chi2 = np.where(np.isfinite(chi2), chi2, np.inf)
    i = int(np.argmin(chi2))
    return U[i].copy(), float(chi2[i])


def noisy_target(fam, u, counts=1e4, seed=0):
    """the 512 x 512 image of parameters u, averaged to 256 x 256, with Poisson
    noise scaled to `counts` counts at the peak (zero-count pixels are 0)"""
    img = simulate(fam, np.array([u]), C.scaled(FAMILIES[fam.name][0], 256), mode=cs.CS_MODE_FP64)[0]
    img = bin2(np.where(np.isfinite(img), img, 0.0))
    rng = np.random.default_rng(seed)
    peak = float(np.max(img))
    scale = counts / peak if peak > 0 else 1.0
    return rng.poisson(np.maximum(img, 0) * scale) / scale


def fit_table(fam, u_start):
    table = [dict(PAD_KEY)]
    for k, v in zip(fam.keys, u_start):
        lo, hi = fam.limits(k)
        table.append({"key": k, "min": lo, "max": hi, "start": fam.nominal[k] * (1 + SPREAD * float(v)), "used": True})
    return table


def seeded_fit(fam, target, u0, chi2_stop, maxit, ftol, stp, schedule, restarts=3):
    """Mixed-precision simplex fits from u0 until chi2 <= chi2_stop: when a
    simplex has contracted (ftol) above it, a fresh simplex of size stp starts
    at the best vertex, up to `restarts` times and maxit iterations in all.
    Returns (fitres of the best fit, report with summed images/repetitions)."""
    u = np.asarray(u0, dtype=np.float64)
    best_res, best = None, None
    images = reps = 0
    for r in range(restarts + 1):
        res, rep = cs.simplex_fit(fam.fit_base, target, fit_table(fam, u), stp=stp, maxit=maxit - reps, ftol=ftol,
                                  mode=cs.CS_MODE_MIXED, schedule=schedule, chi2_stop=chi2_stop)
        images += rep["images"]
        reps += rep["repetitions"]
        if best is None or rep["chi2"] < best["chi2"]:
            best_res, best = res, dict(rep)
        if best["chi2"] <= chi2_stop or reps >= maxit:
            break
        u = np.clip(fam.u_of(best_res), -START_BOX, START_BOX)
    best.update({"images": images, "repetitions": reps, "restarts": r})
    return best_res, best


def compare_fits(fam, sur, n_targets=8, seed=0, maxit=300, ftol=1e-5, stp=0.1, stp_seeded=0.05,
                 schedule_seeded=cs.CS_FIT_BATCHED, shortlist=8, restarts=3):
    """Plain fits (FP64, sequential, random start, initial simplex stp)
    against surrogate-seeded fits (mixed precision; the start is the shortlist
    candidate with the lowest exact chi^2, the initial simplex the tighter
    stp_seeded), which stop once they reach the plain fit's chi^2 and restart
    from their best vertex when the simplex contracts (ftol) before that.
    A third arm runs that same mixed batched simplex with restarts from the
    plain fit's random start (initial simplex stp): the network's own gain is
    its time over the seeded fit's."""
    rng = np.random.default_rng(seed)
    rows = []
    for i in range(n_targets):
        u_true = rng.uniform(-0.8, 0.8, len(fam.keys))
        target = noisy_target(fam, u_true, seed=seed + i)
        u_rand = rng.uniform(-1, 1, len(fam.keys))
        t0 = time.perf_counter()
        res_p, rep_p = cs.simplex_fit(fam.fit_base, target, fit_table(fam, u_rand), stp=stp, maxit=maxit, ftol=ftol,
                                      mode=cs.CS_MODE_FP64, schedule=cs.CS_FIT_SEQUENTIAL)
        t_plain = time.perf_counter() - t0
        t0 = time.perf_counter()
        u_s, _, short = sur.propose(target, seed=seed + i, shortlist=shortlist)
        chi2_start = float("nan")
        if shortlist > 1:
            u_s, chi2_start = exact_pick(fam, target, short)
        t_prop = time.perf_counter() - t0
        res_s, rep_s = seeded_fit(fam, target, np.clip(u_s, -START_BOX, START_BOX), rep_p["chi2"] * (1 + 1e-3),
                                  maxit, ftol, stp_seeded, schedule_seeded, restarts)
        t_seeded = time.perf_counter() - t0  # proposal + fit
        t0 = time.perf_counter()
        res_r, rep_r = seeded_fit(fam, target, np.clip(u_rand, -START_BOX, START_BOX), rep_p["chi2"] * (1 + 1e-3),
                                  maxit, ftol, stp, schedule_seeded, restarts)
        t_random = time.perf_counter() - t0
        rows.append({"target": i, "chi2_plain": rep_p["chi2"], "chi2_seeded": rep_s["chi2"], "chi2_start": chi2_start,
                     "restarts": rep_s["restarts"],
                     "reached": bool(rep_s["chi2"] <= rep_p["chi2"] * (1 + 1e-3)),
                     "t_plain_s": t_plain, "t_seeded_s": t_seeded, "t_propose_s": t_prop,
                     "t_batched_random_s": t_random, "chi2_batched_random": rep_r["chi2"],
                     "reached_batched_random": bool(rep_r["chi2"] <= rep_p["chi2"] * (1 + 1e-3)),
                     "images_plain": rep_p["images"], "images_seeded": rep_s["images"],
                     "iters_plain": rep_p["repetitions"], "iters_seeded": rep_s["repetitions"],
                     "u_err_plain": float(np.abs(fam.u_of(res_p) - u_true).max()),
                     "u_err_seeded": float(np.abs(fam.u_of(res_s) - u_true).max()),
                     "u_err_start": float(np.abs(u_s - u_true).max())})
    sp = [r["t_plain_s"] / r["t_seeded_s"] for r in rows]
    sn = [r["t_batched_random_s"] / r["t_seeded_s"] for r in rows]
    return {"family": fam.name, "targets": n_targets, "median_speedup": float(np.median(sp)),
            "median_speedup_over_batched_random_start": float(np.median(sn)),
            "reached_fraction": float(np.mean([r["reached"] for r in rows])),
            "reached_fraction_batched_random": float(np.mean([r["reached_batched_random"] for r in rows])),
            "rows": rows}
