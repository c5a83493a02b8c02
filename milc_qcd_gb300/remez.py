"""Rational approximations for the RHMC (host side; numpy + scipy).

Replaces the reference's remez-milc generator (ks_imp_rhmc/remez-milc/,
which needs GMP).  For f(x) = prod_k (x + 4 m_k^2)^(y_k/z_k) on [lo, hi] it
finds a type-(n, n) rational function with small maximum relative error
|r/f - 1| and writes it as MILC stores and applies it
(load_rhmc_params.c, ks_ratinv.c):

    r(x) = res[0] + sum_{k=1..n} res[k] / (x + pole[k]).

Method, in two stages.  (1) A near-minimax start by AAA-Lawson
(Nakatsukasa & Trefethen, "An algorithm for real and complex rational
minimax approximation", SIAM J. Sci. Comput. 42 (2020) A3157).  AAA
(Nakatsukasa, Sete & Trefethen, SIAM J. Sci. Comput. 40 (2018) A1494)
picks n+1 support points greedily; then, with r = N/D,
N = sum a_j/(x - z_j), D = sum b_j/(x - z_j), iteratively reweighted
linearised least squares on |(f D - N)/f|, weights multiplied by the
current error each step, drives the error towards equioscillation.  Poles
are the roots of D (a generalised eigenproblem); the residues and res[0]
are refitted for those poles by Lawson's iteration on the (linear) relative
error problem.  This lands within 0.1-9 % of the minimax error.  (2) The
Remez exchange algorithm (remez_polish) from there to the equioscillating,
i.e. minimax, approximation -- the one the reference's alg_remez computes.
On MILC's own sample rational functions (degrees 7-11 on [1e-15, 90]) the
maximum error equals the reference's to about six digits
(tests/test_remez.py).
"""
import numpy as np

from .rhmc import RationalFunction


def target(y, z, m):
    """f(x) = prod (x + 4 m_k^2)^(y_k / z_k) (terms with y_k = 0 drop out)."""
    terms = [(4.0 * mk * mk, yk / zk) for yk, zk, mk in zip(y, z, m) if yk != 0]

    def f(x):
        x = np.asarray(x, dtype=np.float64)
        out = np.ones_like(x)
        for s, e in terms:
            out = out * (x + s) ** e
        return out
    return f


def _grid(lo, hi, knee, nsample):
    # far below the smallest 4 m^2 the function is flat: sample it sparsely
    # (a few points per decade) and densely above
    start = max(lo, knee * 1e-4) if knee else lo
    g = np.geomspace(start, hi, nsample)
    ndec = int(np.ceil(np.log10(start / lo))) if start > lo else 0
    flat = np.geomspace(lo, start, 4 * ndec + 2) if ndec else np.array([lo])
    return np.unique(np.concatenate([flat, g]))


def aaa_lawson(f, lo, hi, n, knee=None, nsample=4000, iters=300):
    """(max relative error on the sample grid, poles, residues, res0)."""
    import scipy.linalg
    Z = _grid(lo, hi, knee, nsample)
    F = f(Z)
    W = 1.0 / np.abs(F)
    mask = np.ones(len(Z), dtype=bool)
    zj = []
    R = np.full(len(Z), F.mean())
    for _ in range(n + 1):
        j = int(np.argmax(np.abs(F - R) * W * mask))
        zj.append(Z[j])
        mask[j] = False
        zs = np.array(zj)
        fs = f(zs)
        C = 1.0 / (Z[mask, None] - zs[None, :])
        A = (F[mask, None] * C - C * fs[None, :]) * W[mask, None]
        w = np.linalg.svd(A, full_matrices=False)[2][-1]
        R = F.copy()
        R[mask] = (C @ (w * fs)) / (C @ w)
    zs = np.array(zj)
    keep = ~np.isin(Z, zs)
    Zm, Fm = Z[keep], F[keep]
    C = 1.0 / (Zm[:, None] - zs[None, :])
    base = np.hstack([-C, Fm[:, None] * C]) / np.abs(Fm)[:, None]
    wt = np.full(len(Zm), 1.0 / len(Zm))
    best = None
    for _ in range(iters):
        v = np.linalg.svd(base * np.sqrt(wt)[:, None], full_matrices=False)[2][-1]
        a, b = v[:n + 1], v[n + 1:]
        e = np.abs((C @ a) / (C @ b) / Fm - 1.0)
        emax = e.max()
        if best is None or emax < best[0]:
            best = (emax, a.copy(), b.copy())
        wt = wt * e
        wt /= wt.sum()
    emax, a, b = best
    m1 = n + 1
    B = np.eye(m1 + 1)
    B[0, 0] = 0.0
    E = np.zeros((m1 + 1, m1 + 1))
    E[0, 1:] = b
    E[1:, 0] = 1.0
    E[1:, 1:] = np.diag(zs)
    ev = scipy.linalg.eigvals(E, B)
    ev = ev[np.isfinite(ev)]
    with np.errstate(divide="ignore", invalid="ignore"):
        res = np.array([np.sum(a / (p - zs)) / (-np.sum(b / (p - zs) ** 2)) for p in ev])
    return emax, ev, res, a.sum() / b.sum()


def rational_function(y, z, m, lo, hi, order, pole0=99.9, iters=300, polish=True):
    """RationalFunction for prod (x + 4 m_k^2)^(y_k/z_k) on [lo, hi] with
    `order` poles: the AAA-Lawson start, then (polish=True) the Remez
    exchange to the minimax approximation (remez_polish).  Raises if a pole
    comes out complex or outside the cut x <= -lo (the function is then not
    representable as MILC uses it)."""
    rf = _aaa_rational_function(y, z, m, lo, hi, order, pole0, iters)
    if polish:
        pol, emax, _ = remez_polish(rf, lo, hi)
        if emax <= rf.error * (1.0 + 1e-6) and all(p > 0 for p in pol.pole[1:]):
            rf = pol
    return rf


def _aaa_rational_function(y, z, m, lo, hi, order, pole0, iters):
    f = target(y, z, m)
    knee = min((4.0 * mk * mk for yk, mk in zip(y, m) if yk != 0), default=None)
    emax, poles, res, c0 = aaa_lawson(f, lo, hi, order, knee=knee, iters=iters)
    if len(poles) != order or np.abs(poles.imag).max() > 1e-8 * np.abs(poles).max() or (poles.real >= 0).any():
        raise ValueError("rational approximation has poles off the negative real axis")
    pole = np.sort(-poles.real)[::-1]
    # the residues from the barycentric form lose digits in the conversion:
    # refit them (and res[0]) for the fixed poles by Lawson's iteration on the
    # linear problem min max |(res0 + sum res_k/(x + p_k))/f - 1|
    x = _grid(lo, hi, knee, 20000)
    fx = f(x)
    A = np.hstack([np.ones((len(x), 1)), 1.0 / (x[:, None] + pole[None, :])]) / fx[:, None]
    wt = np.full(len(x), 1.0 / len(x))
    best = None
    for _ in range(iters):
        sw = np.sqrt(wt)
        c = np.linalg.lstsq(A * sw[:, None], sw, rcond=None)[0]
        e = np.abs(A @ c - 1.0)
        if best is None or e.max() < best[0]:
            best = (e.max(), c)
        wt = wt * e
        wt /= wt.sum()
    emax, c = best
    rf = RationalFunction(y, z, m, order, [float(v) for v in c], [pole0] + [float(p) for p in pole])
    rf.error = float(emax)
    return rf


def _eval_pf(x, c0, res, pole):
    return c0 + np.sum(res[None, :] / (x[:, None] + pole[None, :]), axis=1)


def _local_extrema(t, e):
    """Indices of the local extrema of e(t) on the grid, ends included."""
    d = np.diff(e)
    idx = [0]
    for i in range(1, len(e) - 1):
        if (d[i - 1] > 0 and d[i] <= 0) or (d[i - 1] < 0 and d[i] >= 0):
            idx.append(i)
    idx.append(len(e) - 1)
    return np.array(sorted(set(idx)))


def _alternant(t, e, npts):
    """npts points of alternating error sign, chosen among the local extrema
    of e so that every same-sign run keeps its largest |e| and, while too
    many remain, the smaller end of the sequence is dropped."""
    idx = _local_extrema(t, e)
    idx = idx[np.abs(e[idx]) > 0]
    merged = []
    for i in idx:
        if merged and np.sign(e[i]) == np.sign(e[merged[-1]]):
            if abs(e[i]) > abs(e[merged[-1]]):
                merged[-1] = i
        else:
            merged.append(i)
    while len(merged) > npts:
        if abs(e[merged[0]]) < abs(e[merged[-1]]):
            merged.pop(0)
        else:
            merged.pop()
    return np.array(merged)


def _refine_extremum(fun, t0, h, iters=60):
    """Golden-section search for the extremum of |fun| near log-abscissa t0."""
    a, b = t0 - h, t0 + h
    g = 0.5 * (np.sqrt(5.0) - 1.0)
    s = np.sign(fun(np.array([t0]))[0]) or 1.0
    c, d = b - g * (b - a), a + g * (b - a)
    fc, fd = s * fun(np.array([c]))[0], s * fun(np.array([d]))[0]
    for _ in range(iters):
        if fc > fd:
            b, d, fd = d, c, fc
            c = b - g * (b - a)
            fc = s * fun(np.array([c]))[0]
        else:
            a, c, fc = c, d, fd
            d = a + g * (b - a)
            fd = s * fun(np.array([d]))[0]
    return 0.5 * (a + b)


def remez_polish(rf, lo, hi, iters=40, nsample=40000, tol=1e-9):
    """Polish a near-minimax rational function rf (type (n, n) in MILC's
    partial-fraction form) into the minimax one by the Remez exchange
    algorithm for the relative error e(x) = r(x)/f(x) - 1 on [lo, hi]:

    1. take 2n+2 abscissae where e alternates in sign (the extrema of the
       current error, refined by golden-section search in log x);
    2. solve e(x_i) = (-1)^i E for the 2n+1 coefficients (res0, res_k and
       the poles p_k = exp(q_k)) and the level E by Newton's method;
    3. repeat until the largest |e| on a fine grid equals |E| to `tol`.

    This is the exchange algorithm the reference's alg_remez applies (there
    to the coefficients of numerator and denominator polynomials in GMP
    multiple precision); here the unknowns are the partial-fraction
    coefficients with the poles in log scale, which keeps the Newton systems
    well conditioned in FP64.  The equioscillating function is the unique
    best approximation, so its maximum error is the reference's.  Returns
    (RationalFunction, max |e|, |E|)."""
    f = target(rf.y, rf.z, rf.m)
    n = rf.order
    c0 = float(rf.res[0])
    res = np.array(rf.res[1:], dtype=np.float64)
    q = np.log(np.array(rf.pole[1:], dtype=np.float64))
    t = np.linspace(np.log(lo), np.log(hi), nsample)
    X = np.exp(t)
    FX = f(X)

    def err(tt, c0, res, q):
        x = np.exp(tt)
        return _eval_pf(x, c0, res, np.exp(q)) / f(x) - 1.0

    best = None
    h = t[1] - t[0]
    for _ in range(iters):
        e = _eval_pf(X, c0, res, np.exp(q)) / FX - 1.0
        emax = float(np.abs(e).max())
        ref = _alternant(t, e, 2 * n + 2)
        if len(ref) < 2 * n + 2:
            break
        tr = np.array([_refine_extremum(lambda u: err(u, c0, res, q), t[i], h) if 0 < i < len(t) - 1 else t[i]
                       for i in ref])
        E = float(np.mean(np.abs(err(tr, c0, res, q))))
        if best is None or emax < best[1]:
            best = ((c0, res.copy(), q.copy()), emax, E)
        if abs(emax - E) <= tol * emax:
            break
        sgn = np.sign(err(tr, c0, res, q))
        # Newton on F(u) = e(x_i; u) - sgn_i E = 0, u = (c0, res, q, E)
        u = np.concatenate([[c0], res, q, [E]])
        xr, fr = np.exp(tr), f(np.exp(tr))
        for _newton in range(30):
            c0u, ru, qu, Eu = u[0], u[1:n + 1], u[n + 1:2 * n + 1], u[-1]
            p = np.exp(qu)
            den = xr[:, None] + p[None, :]
            val = (c0u + np.sum(ru[None, :] / den, axis=1)) / fr - 1.0 - sgn * Eu
            J = np.empty((2 * n + 2, 2 * n + 2))
            J[:, 0] = 1.0 / fr
            J[:, 1:n + 1] = 1.0 / den / fr[:, None]
            J[:, n + 1:2 * n + 1] = -ru[None, :] * p[None, :] / den ** 2 / fr[:, None]
            J[:, -1] = -sgn
            scale = np.abs(J).max(axis=0)
            scale[scale == 0] = 1.0
            du = np.linalg.solve(J / scale[None, :], -val) / scale
            u = u + du
            if np.abs(val).max() < 1e-15 * max(1.0, abs(Eu)) or np.abs(du[n + 1:2 * n + 1]).max() < 1e-14:
                break
        c0, res, q = float(u[0]), u[1:n + 1].copy(), u[n + 1:2 * n + 1].copy()
    if best is None:
        # no alternant of 2n+2 points on the grid (an error near the FP64
        # rounding level): keep the start
        return rf, float(getattr(rf, "error", np.nan)), float("nan")
    (c0, res, q), emax, E = best
    # the finest check: the largest error of the best iterate on a denser grid
    tt = np.linspace(np.log(lo), np.log(hi), 4 * nsample)
    emax = float(np.abs(err(tt, c0, res, q)).max())
    from .rhmc import RationalFunction
    pole = np.exp(q)
    order = np.argsort(-pole)
    out = RationalFunction(rf.y, rf.z, rf.m, n, [c0] + [float(v) for v in res[order]],
                           [rf.pole[0]] + [float(v) for v in pole[order]])
    out.error = emax
    return out, emax, abs(E)


def max_rel_error(rf, lo, hi, nsample=20000):
    """max |r(x)/f(x) - 1| on a geometric grid of [lo, hi]."""
    x = np.geomspace(lo, hi, nsample)
    f = target(rf.y, rf.z, rf.m)(x)
    r = rf.res[0] + sum(rk / (x + pk) for rk, pk in zip(rf.res[1:], rf.pole[1:]))
    return float(np.abs(r / f - 1.0).max())


def eps_naik(am):
    """Tree-level HISQ Naik-term correction for a quark of mass am (Follana
    et al., Phys. Rev. D 75 (2007) 054502, eq. 24): the series the
    reference's calc_eps_naik script evaluates."""
    m2 = am * am
    return -27.0 / 40.0 * m2 + 327.0 / 1120.0 * m2 ** 2 - 15607.0 / 268800.0 * m2 ** 3 - 73697.0 / 3942400.0 * m2 ** 4


def format_rhmc_params(fields):
    """MILC's rational-function file text for a list of
    (naik_term_epsilon, MD, GR, FA) with RationalFunction entries."""
    out = ["n_pseudo %d" % len(fields), ""]
    for eps, md, gr, fa in fields:
        out += ["naik_term_epsilon %.10g" % eps, ""]
        for tag, f in (("MD", md), ("GR", gr), ("FA", fa)):
            out += ["# Rational function for %s, max relative error %.3e" % (tag, getattr(f, "error", float("nan"))),
                    "y_%s %s" % (tag, " ".join(str(v) for v in f.y)),
                    "z_%s %s" % (tag, " ".join(str(v) for v in f.z)),
                    "m_%s %s" % (tag, " ".join("%.6f" % v for v in f.m)),
                    "order_%s %d" % (tag, f.order), ""]
            out += ["res_%s %.16e" % (tag, r) for r in f.res] + [""]
            out += ["pole_%s %.16e" % (tag, p) for p in f.pole] + [""]
    return "\n".join(out)
