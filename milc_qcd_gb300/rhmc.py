"""Rational-function parameters for the RHMC (host side).

``load_rhmc_params`` reads MILC's rational-function file, the format
ks_imp_rhmc/load_rhmc_params.c:96-174 reads (written by the reference's
remez-milc generator): ``n_pseudo N``, then per pseudofermion field
``naik_term_epsilon e`` and three rational functions tagged MD (molecular
dynamics force), GR (heat-bath source) and FA (action), each as

    y_TAG  4 ints      z_TAG 4 ints      m_TAG 4 masses
    order_TAG n
    res_TAG  (n+1 lines; res[0] is the constant term)
    pole_TAG (n+1 lines; pole[0] is unused)

The approximated function is prod_k (x + 4 m_k^2)^(y_k/z_k).  Lines
starting with '#' are comments.  ``ks_ratinv`` / ``ks_rateval`` in the
package apply them (ks_imp_rhmc/ks_ratinv.c:29-137).
"""


class RationalFunction:
    def __init__(self, y, z, m, order, res, pole):
        self.y, self.z, self.m = list(y), list(z), list(m)
        self.order = int(order)
        self.res = [float(r) for r in res]
        self.pole = [float(p) for p in pole]
        if len(self.res) != self.order + 1 or len(self.pole) != self.order + 1:
            raise ValueError("rational function of order %d needs %d residues and poles"
                             % (self.order, self.order + 1))

    def __call__(self, x):
        """res[0] + sum_k res[k] / (x + pole[k])."""
        return self.res[0] + sum(r / (x + p) for r, p in zip(self.res[1:], self.pole[1:]))

    def exact(self, x):
        out = 1.0
        for y, z, m in zip(self.y, self.z, self.m):
            out *= (x + 4.0 * m * m) ** (y / z)
        return out


class PseudofermionParams:
    def __init__(self, naik_term_epsilon, MD, GR, FA):
        self.naik_term_epsilon = float(naik_term_epsilon)
        self.MD, self.GR, self.FA = MD, GR, FA


def _tokens(text):
    for line in text.splitlines():
        line = line.split("#", 1)[0].strip()
        if line:
            yield line.split()


def parse_rhmc_params(text, n_pseudo=None):
    toks = list(_tokens(text))
    pos = 0

    def take(key, nvals=1, conv=float):
        nonlocal pos
        if pos >= len(toks) or toks[pos][0] != key:
            got = toks[pos][0] if pos < len(toks) else "end of file"
            raise ValueError("expected '%s', found '%s'" % (key, got))
        vals = [conv(v) for v in toks[pos][1:1 + nvals]]
        if len(vals) != nvals:
            raise ValueError("'%s' needs %d values" % (key, nvals))
        pos += 1
        return vals if nvals > 1 else vals[0]

    n = take("n_pseudo", 1, int)
    if n_pseudo is not None and n != n_pseudo:
        raise ValueError("wrong value of n_pseudo: file has %d, expected %d" % (n, n_pseudo))
    out = []
    for _ in range(n):
        eps = take("naik_term_epsilon")
        fns = {}
        for tag in ("MD", "GR", "FA"):
            y = take("y_" + tag, 4, lambda v: int(float(v)))
            z = take("z_" + tag, 4, lambda v: int(float(v)))
            m = take("m_" + tag, 4)
            order = take("order_" + tag, 1, int)
            res = [take("res_" + tag) for _ in range(order + 1)]
            pole = [take("pole_" + tag) for _ in range(order + 1)]
            fns[tag] = RationalFunction(y, z, m, order, res, pole)
        out.append(PseudofermionParams(eps, fns["MD"], fns["GR"], fns["FA"]))
    return out


def load_rhmc_params(path, n_pseudo=None):
    with open(path) as f:
        return parse_rhmc_params(f.read(), n_pseudo)


# ---- one trajectory on the GPU (mks_rhmc_trajectory) ----
INTEGRATORS = {"leapfrog": 0, "omelyan": 1, "2G1F": 2, "3G1F": 3}


def update(pseudofermions, beta, u0, nflavors, epsilon, steps, int_alg="3G1F", resid_md=None, resid_fa=None,
           resid_gr=None, max_cg=2500, prec_md=2, prec_fa=2, prec_gr=2, nrestart=5, refresh=True,
           prec_force=2):
    """MILC's update() (ks_imp_rhmc/update_rhmc.c) on the resident links and
    momenta.  pseudofermions: list of PseudofermionParams (or dicts with
    'MD'/'GR'/'FA' -> (res, pole) and 'naik_term_epsilon'); resid_*: one
    residual per field (cgresid_md_fa_gr, not squared).  Returns a dict of
    the action terms, delta_s, plaquettes, counters and timings."""
    import ctypes
    import numpy as np
    from . import _lib, init, check

    n = len(pseudofermions)
    keep = []

    def ratf(fn):
        if isinstance(fn, RationalFunction):
            res, pole = fn.res, fn.pole
        else:
            res, pole = fn
        res = np.ascontiguousarray(res, dtype=np.float64)
        pole = np.ascontiguousarray(pole, dtype=np.float64)
        keep.extend([res, pole])
        return _lib.RatFunc(len(res) - 1, res.ctypes.data_as(_lib.DP), pole.ctypes.data_as(_lib.DP))

    arr = (_lib.Pseudofermion * n)()
    for i, pf in enumerate(pseudofermions):
        if isinstance(pf, PseudofermionParams):
            eps, md, gr, fa = pf.naik_term_epsilon, pf.MD, pf.GR, pf.FA
        else:
            eps, md, gr, fa = pf.get("naik_term_epsilon", 0.0), pf["MD"], pf["GR"], pf["FA"]
        arr[i] = _lib.Pseudofermion(float(eps), ratf(md), ratf(gr), ratf(fa), resid_md[i], resid_fa[i],
                                    resid_gr[i], int(max_cg))
    p = _lib.RhmcParams(beta, u0, int(nflavors), epsilon, int(steps), INTEGRATORS[int_alg], n,
                        ctypes.cast(arr, ctypes.POINTER(_lib.Pseudofermion)), prec_md, prec_fa, prec_gr,
                        int(nrestart), 1 if refresh else 0, int(prec_force))
    r = _lib.RhmcResult()
    check(init().mks_rhmc_trajectory(ctypes.byref(p), ctypes.byref(r)), "mks_rhmc_trajectory")
    out = {f: getattr(r, f) for f, _ in _lib.RhmcResult._fields_ if f != "grsource_sum"}
    out["grsource_sum"] = [r.grsource_sum[i] for i in range(n)]
    out["start"] = (r.g0, r.h0, r.f0)
    out["end"] = (r.g1, r.h1, r.f1)
    return out
