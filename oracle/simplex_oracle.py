"""The reference's 2D simplex fit restated in plain Python (TEST INFRASTRUCTURE).

Follows SasCalc_SimplexFit2D::doSimplexFit2D, amotry and the limit check of
fehlerquadratsumme (Source/sc_simplexfit2d.cpp:19-611) statement by statement,
over an arbitrary objective f(params) instead of the image chi^2, including the
reference's two trajectory-changing behaviours: the initialisation loop of
:375-380 (inner loop over `i` that sets p[i][0] = 0 for i < map) and amotry's
centroid factor over all listed parameters. The checker for the library's
cs_simplex_minimize / cs_simplex_fit.
"""
import math

NAP = 31
MAP = 30


def plain_sum(it):
    """Left-to-right double sum as the reference's loops (Python's sum() of
    floats is compensated since 3.12)."""
    s = 0.0
    for v in it:
        s += v
    return s


def simplex(f, table, stp, maxit, ftol):
    """table: list of dicts {key, min, max, start, used}. Returns
    (fitres by key, repetitions, y[ilo], evaluations)."""
    keys = sorted(t["key"] for t in table)
    by = {t["key"]: t for t in table}
    ind = [k for k in keys if by[k]["used"]] + [k for k in keys if not by[k]["used"]]
    numfit = sum(1 for k in keys if by[k]["used"])
    mmax = len(ind)
    enabled = [by[k]["used"] for k in ind]
    values = [0.0] * NAP
    minv = [0.0] * NAP
    maxv = [0.0] * NAP
    for i, k in enumerate(ind):
        values[i] = float(by[k]["start"])
        minv[i] = float(by[k]["min"])
        maxv[i] = float(by[k]["max"])
    evals = [0]

    def fqs(par):
        for j in range(numfit):
            if enabled[j]:
                if minv[j] == 0.0 and maxv[j] == 360.0:
                    continue
                if par[j] < minv[j] or par[j] > maxv[j]:
                    return 1e20
        evals[0] += 1
        return f(list(par[:mmax]))

    alfa, beta, gamma = 1.0, 0.5, 2.0
    y = [0.0] * NAP
    pp = [0.0] * MAP
    q = [0.0] * MAP
    step = [0.0] * MAP
    psum = [0.0] * MAP
    p = [[0.0] * MAP for _ in range(NAP)]
    nmax = mmax + 1.0
    ndim = mmax
    mpts = numfit + 1
    rootn1 = math.sqrt(nmax) - 1.0
    mroot2 = 1.0 / (mmax * math.sqrt(2.0))
    for i in range(mmax):
        psum[i] = values[i]
        p[0][i] = values[i]
        if i < numfit:
            if values[i] == 0:
                step[i] = stp if minv[i] == 0 else minv[i] * stp
            else:
                step[i] = values[i] * stp
        else:
            step[i] = 0.0
        pp[i] = step[i] * (rootn1 + mmax) * mroot2
        q[i] = step[i] * rootn1 * mroot2
    # for (i=0; i<nap; i++) { y[i]=0; for (j=0; i<map; i++) p[i][j]=0; }
    i = 0
    while i < NAP:
        y[i] = 0.0
        j = 0
        while i < MAP:
            p[i][j] = 0.0
            i += 1
        i += 1
    y[0] = fqs(values)
    i = 1
    while i < nmax:
        for j in range(mmax):
            p[i][j] = p[0][j] + q[j]
        p[i][i - 1] = p[i][i - 1] + pp[i - 1]
        i += 1
    i = 1
    while i < nmax:
        for j in range(numfit):
            values[j] = p[i][j]
        y[i] = y[numfit + 1] if i > numfit + 1 else fqs(values)
        i += 1
    for j in range(ndim):
        psum[j] = plain_sum(p[i][j] for i in range(mpts))

    def amotry(ihi, fac):
        ptry = [0.0] * MAP
        for j in range(mmax):
            ptry[j] = psum[j]
        fac1 = (1.0 - fac) / mmax
        fac2 = fac1 - fac
        for j in range(numfit):
            ptry[j] = psum[j] * fac1 - p[ihi][j] * fac2
        ytry = fqs(ptry)
        if ytry < y[ihi]:
            y[ihi] = ytry
            for j in range(numfit):
                psum[j] += ptry[j] - p[ihi][j]
                p[ihi][j] = ptry[j]
        return ytry

    ilo = 0
    rep = 0
    while rep < maxit:
        ilo = 0
        if y[0] > y[1]:
            ihi, inhi = 0, 1
        else:
            ihi, inhi = 1, 0
        for i in range(mpts):
            if y[i] < y[ilo]:
                ilo = i
            if y[i] > y[ihi]:
                inhi = ihi
                ihi = i
            elif y[i] > y[inhi]:
                if i != ihi:
                    inhi = i
        if math.isnan(y[ihi]) or math.isnan(y[ilo]) or abs(y[ihi]) + abs(y[ilo]) == 0:
            break
        rtol = 2.0 * abs(y[ihi] - y[ilo]) / (abs(y[ihi]) + abs(y[ilo]))
        if rtol <= ftol:
            break
        ytry = amotry(ihi, -alfa)
        if ytry <= y[ilo]:
            amotry(ihi, gamma)
        elif ytry >= y[inhi]:
            ysave = y[ihi]
            ytry = amotry(ihi, beta)
            if ytry >= ysave:
                for i in range(mpts):
                    if i != ilo:
                        for j in range(ndim):
                            psum[j] = 0.5 * (p[i][j] + p[ilo][j])
                            p[i][j] = psum[j]
                        y[i] = fqs(psum)
                for j in range(ndim):
                    psum[j] = plain_sum(p[i][j] for i in range(mpts))
        rep += 1
    return {k: p[ilo][i] for i, k in enumerate(ind)}, rep, y[ilo], evals[0]
