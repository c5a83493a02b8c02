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
