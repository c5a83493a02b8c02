"""One RHMC trajectory composed from the oracle's pieces (test infrastructure).

Restates ks_imp_rhmc/update_rhmc.c:update() for the HISQ action:
refresh the momenta (ranmom), heat-bath pseudofermion sources
(grsource_rhmc.c), the action (d_action_rhmc.c), the 3G1F Omelyan
integrator (update_rhmc.c:361-473) over update_u (update_u.c), the gauge
force (gauge_force_imp.c) and the fermion force from multi-shift solves
(update_h_rhmc.c:40-105), with reunitarization after every double step
(reunitarize_ks.c).  Every numerical piece is the C oracle's
(milc_oracle*.c); this file only sequences them like MILC does.

Links are kept without phases (MILC keeps them in and takes them out for
the gauge action and force; the phases are +-1 per link, so update_u and
the reunitarization give the same links either way once the phases are
handled as reunitarize_ks does).
"""
import numpy as np

from .oracle import EVEN, ODD, GaugeOracle, Oracle


class OracleRHMC:
    def __init__(self, dims, U, beta, u0, nflavors, rational, naik_eps, resid_md, resid_fa, resid_gr,
                 max_cg=2500, nrestart=5, iseed=None):
        import milc_qcd_gb300 as m
        self.m = m
        self.dims = tuple(dims)
        self.orc = Oracle(self.dims)
        self.G = GaugeOracle(self.orc)
        self.V = self.orc.V
        self.Vh = self.V // 2
        self.U = np.ascontiguousarray(U, dtype=np.float64).copy()
        self.beta, self.u0, self.nf = beta, u0, nflavors
        self.rational = rational
        self.naik_eps = list(naik_eps)
        self.eps_distinct = []
        for e in self.naik_eps:
            if e not in self.eps_distinct:
                self.eps_distinct.append(e)
        self.inaik = [self.eps_distinct.index(e) for e in self.naik_eps]
        self.resid = {"MD": resid_md, "FA": resid_fa, "GR": resid_gr}
        self.max_cg, self.nrestart = max_cg, nrestart
        self.mom = np.zeros((self.V, 4, 10))
        self.phi = [None] * len(rational)
        self._links = None
        self.iters = 0
        self.grsource_sums = []
        if iseed is not None:
            self.G.seed(iseed)

    # ---- links ----
    def phased(self):
        return self.m.apply_phases(self.dims, self.U)

    def links(self):
        if self._links is None:
            self._links = self.orc.hisq_links(self.phased(), tuple(self.eps_distinct))
        return self._links

    # ---- rational functions (ks_ratinv.c:29-137) ----
    def ratinv(self, src, ipf, tag):
        res, pole = self.rational[ipf][tag]
        L = self.links()
        g = self.inaik[ipf]
        it, psim, _ = self.orc.multicg_offset(L["fat"][g], L["lng"][g], src, np.asarray(pole[1:]), EVEN,
                                              self.resid[tag][ipf], self.max_cg, self.nrestart)
        self.iters += it
        return psim

    def rateval(self, src, psim, ipf, tag):
        res = self.rational[ipf][tag][0]
        out = np.zeros_like(src)
        out[:self.Vh] = res[0] * src[:self.Vh]
        for j in range(len(psim)):
            out[:self.Vh] += res[j + 1] * psim[j][:self.Vh]
        return out

    # ---- pieces of update() ----
    def ranmom(self):
        self.mom = self.G.ranmom()

    def grsource(self):
        self.grsource_sums = []
        for ipf in range(len(self.rational)):
            g = self.G.gaussian_vector(EVEN)
            self.grsource_sums.append(float((g[:self.Vh] ** 2).sum()))
            self.phi[ipf] = self.rateval(g, self.ratinv(g, ipf, "GR"), ipf, "GR")

    def action(self):
        g = self.G.action(self.U, self.beta, self.u0, self.nf)
        h = self.G.hmom_action(self.mom)
        f = 0.0
        for ipf in range(len(self.rational)):
            s = self.rateval(self.phi[ipf], self.ratinv(self.phi[ipf], ipf, "FA"), ipf, "FA")
            f += float((s[:self.Vh] ** 2).sum())
        return g, h, f

    def update_u(self, eps):
        self.U = self.G.update_u(self.U, self.mom, eps)
        self._links = None

    def update_h_gauge(self, eps):
        self.mom = self.G.force(self.U, eps, self.beta, self.u0, self.nf, self.mom)

    def update_h_fermion(self, eps):
        L = self.links()
        xxx, allres, orders = [], [], [0] * len(self.eps_distinct)
        for g in range(len(self.eps_distinct)):
            for ipf in range(len(self.rational)):
                if self.inaik[ipf] != g:
                    continue
                psim = self.ratinv(self.phi[ipf], ipf, "MD")
                for j in range(len(psim)):
                    x = psim[j].copy()
                    x[self.Vh:] = self.orc.dslash(L["fat"][g], L["lng"][g], x, ODD)[self.Vh:]
                    xxx.append(x)
                    allres.append(self.rational[ipf]["MD"][0][j + 1])
                orders[g] += len(psim)
        self.mom = self.orc.fermion_force_hisq(self.phased(), eps, allres, np.stack(xxx), orders=orders,
                                               eps_naik=tuple(self.eps_distinct), mom=self.mom)

    def reunitarize(self):
        self.U = self.G.reunitarize(self.U)
        self._links = None

    # ---- update() with INT_3G1F (update_rhmc.c:361-473) ----
    def integrate_3g1f(self, epsilon, steps, alpha=0.1, beta=0.1):
        for _ in range(2, steps + 1, 2):
            t = [1.0 / 6.0 - alpha / 3.0, 0.5 - beta, 3.0 / 6.0 + alpha / 3.0, 5.0 / 6.0 - alpha / 3.0,
                 7.0 / 6.0 + alpha / 3.0, 9.0 / 6.0 - alpha / 3.0, 1.5 + beta, 11.0 / 6.0 + alpha / 3.0, 2.0]
            kick = ["G", "F", "G", "G", "G", "G", "F", "G", None]
            prev = 0.0
            for tk, k in zip(t, kick):
                self.update_u(epsilon * (tk - prev))
                prev = tk
                if k == "G":
                    self.update_h_gauge(epsilon / 3.0)
                elif k == "F":
                    self.update_h_fermion(epsilon)
            self.reunitarize()

    def trajectory(self, epsilon, steps):
        self.ranmom()
        self.grsource()
        start = self.action()
        self.integrate_3g1f(epsilon, steps)
        end = self.action()
        return dict(start=start, end=end, delta_s=sum(end) - sum(start), plaq=self.G.plaquette(self.U),
                    grsource_sums=self.grsource_sums, iters=self.iters)
