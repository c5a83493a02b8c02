"""GB300-native improved-staggered (HISQ/asqtad) Dirac hot path.

Python mirror of MILC's generic_ks call surface over the C ABI of
libmilc_ks_gb300.so.  Field arrays are numpy float64 in MILC's layout
(su3_vector[V] -> shape (V, 6); su3_matrix[4*i+dir] -> shape (V, 4, 18);
anti_hermitmat[4*i+dir] -> shape (V, 4, 10)), even sites first.

The functions keep MILC's names and argument meaning:

=============================  ==============================================
this module                    MILC (generic_ks)
=============================  ==============================================
``dslash_fn_field``            dslash_fn.c:348 / dslash_fn_dblstore.c:285
``ks_congrad_parity``          d_congrad5_fn_milc.c:61 (ks_congrad_parity_gpu)
``ks_congrad_field``           d_congrad5.c:334
``ks_congrad_block_parity``    d_congrad5_fn_gpu.c:167
``mat_invert_uml_field``       mat_invert.c:328
``mat_invert_block_uml``       mat_invert.c:409
``ks_multicg_offset_field``    ks_multicg_offset.c:63
``load_hisq_links``            fermion_links_hisq_load_milc.c:547-640
``eo_fermion_force_multi``     fermion_force_hisq_multi.c:170
=============================  ==============================================
"""
import ctypes
import numpy as np

from . import _lib
from ._lib import (MKS_EVEN as EVEN, MKS_ODD as ODD, MKS_EVENANDODD as EVENANDODD,
                   MKS_PREC_HALF as PREC_HALF, MKS_PREC_SINGLE as PREC_SINGLE,
                   MKS_PREC_DOUBLE as PREC_DOUBLE, InvertArg, InvertResult, check, MksError)

__all__ = ["EVEN", "ODD", "EVENANDODD", "PREC_HALF", "PREC_SINGLE", "PREC_DOUBLE", "QuarkInvertControl",
           "init", "set_lattice", "load_fn_links", "get_fn_links", "dslash_fn_field", "ks_congrad_parity",
           "ks_congrad_field",
           "ks_congrad_block_parity", "mat_invert_uml_field", "mat_invert_block_uml",
           "ks_multicg_offset_field", "ks_ratinv", "ks_rateval", "load_hisq_links", "load_asqtad_links", "get_hisq_aux",
           "eo_fermion_force_multi", "fermion_force_adjoint", "gauge_load", "gauge_get", "mom_load", "mom_get",
           "rng_seed", "ranmom", "gaussian_vector", "gauge_force", "gauge_action", "update_u", "mom_action",
           "reunitarize", "plaquette", "rebuild_links", "md_precision", "gen_thin_links", "apply_phases", "gen_vector", "gen_momenta",
           "MksError"]


def _dp(a):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], "float64 C-contiguous array expected"
    return a.ctypes.data_as(_lib.DP)


def _dims(dims):
    return (ctypes.c_int * 4)(*[int(d) for d in dims])


class QuarkInvertControl:
    """MILC's quark_invert_control (include/generic_quark_types.h:167-190)."""

    def __init__(self, resid=1e-8, relresid=0.0, max=1000, nrestart=5, parity=EVEN, prec=PREC_DOUBLE,
                 delta=0.1):
        self.resid, self.relresid, self.max, self.nrestart = resid, relresid, max, nrestart
        self.parity, self.prec, self.delta = parity, prec, delta
        self.final_rsq = self.final_relrsq = self.size_r = self.size_relr = 0.0
        self.final_iters = self.final_restart = self.converged = self.reliable_updates = 0

    def arg(self):
        return InvertArg(self.max, self.nrestart, self.parity, self.prec, self.resid, self.relresid, self.delta)

    def take(self, r):
        self.final_rsq, self.final_relrsq = r.final_rsq, r.final_relrsq
        self.size_r, self.size_relr = r.size_r, r.size_relr
        self.final_iters, self.final_restart = r.final_iters, r.final_restart
        self.converged, self.reliable_updates = r.converged, r.reliable_updates
        return self


_state = {"init": False, "dims": None}


def init(device=0):
    lib = _lib.load()
    if not _state["init"]:
        check(lib.mks_init(device), "mks_init")
        _state["init"] = True
    return lib


def set_lattice(dims):
    lib = init()
    check(lib.mks_set_lattice(_dims(dims)), "mks_set_lattice")
    _state["dims"] = tuple(int(d) for d in dims)


def load_fn_links(fat, lng, eps_naik=0.0, slot=0):
    check(init().mks_load_fn_links(slot, _dp(fat), _dp(lng), eps_naik), "mks_load_fn_links")


def get_fn_links(slot=0):
    V = int(np.prod(_state["dims"]))
    fat = np.zeros((V, 4, 18)); lng = np.zeros((V, 4, 18))
    check(init().mks_get_fn_links(slot, _dp(fat), _dp(lng)), "mks_get_fn_links")
    return fat, lng


def dslash_fn_field(src, dest, parity, fn=0):
    """dest[parity sites] = D src (dest modified in place, like MILC)."""
    check(init().mks_dslash_fn_field(_dp(src), _dp(dest), parity, fn), "mks_dslash_fn_field")
    return dest


def ks_congrad_parity(src, dest, qic, mass, fn=0):
    r = InvertResult()
    a = qic.arg()
    it = check(init().mks_ks_congrad_parity(_dp(src), _dp(dest), mass, fn, ctypes.byref(a), ctypes.byref(r)),
               "mks_ks_congrad_parity")
    qic.take(r)
    return it


def _pp(arrs):
    return (_lib.DP * len(arrs))(*[_dp(a) for a in arrs])


def ks_congrad_field(src, dest, qic, mass, fn=0):
    """generic_ks/d_congrad5.c:334-364: qic.parity EVEN, ODD or EVENANDODD
    (the even solve, then the odd one); returns the summed iterations."""
    parity = qic.parity
    iters = 0
    for par in (EVEN, ODD):
        if parity == par or parity == EVENANDODD:
            qic.parity = par
            try:
                iters += ks_congrad_parity(src, dest, qic, mass, fn)
            finally:
                qic.parity = parity
    return iters


def ks_congrad_block_parity(src, dest, qic, mass, fn=0):
    """src, dest: lists of (V,6) arrays.  Returns (max iterations, per-source results)."""
    n = len(src)
    res = (InvertResult * n)()
    a = qic.arg()
    it = check(init().mks_ks_congrad_block_parity(n, _pp(src), _pp(dest), mass, fn, ctypes.byref(a), res),
               "mks_ks_congrad_block_parity")
    qic.take(res[0])
    return it, [QuarkInvertControl().take(res[i]) for i in range(n)]


def mat_invert_uml_field(src, dest, qic, mass, fn=0):
    r = InvertResult()
    a = qic.arg()
    it = check(init().mks_mat_invert_uml_field(_dp(src), _dp(dest), mass, fn, ctypes.byref(a), ctypes.byref(r)),
               "mks_mat_invert_uml_field")
    qic.take(r)
    return it


def mat_invert_block_uml(src, dest, qic, mass, fn=0):
    n = len(src)
    res = (InvertResult * n)()
    a = qic.arg()
    it = check(init().mks_mat_invert_block_uml(n, _pp(src), _pp(dest), mass, fn, ctypes.byref(a), res),
               "mks_mat_invert_block_uml")
    qic.take(res[0])
    return it


def ks_multicg_offset_field(src, psim, offsets, qic, fn=0):
    """psim: list of (V,6) arrays overwritten with (offset_j - D_eo D_oe)^-1 src."""
    n = len(offsets)
    res = (InvertResult * n)()
    offs = np.ascontiguousarray(offsets, dtype=np.float64)
    a = qic.arg()
    it = check(init().mks_ks_multicg_offset_field(_dp(src), _pp(psim), _dp(offs), n, fn, ctypes.byref(a), res),
               "mks_ks_multicg_offset_field")
    qic.take(res[0])
    return it, [QuarkInvertControl().take(res[i]) for i in range(n)]


def ks_ratinv(src, roots, residues, qic, fn=0):
    """Rational-function inversion, ks_imp_rhmc/ks_ratinv.c:29-112: one
    multi-shift solve with offsets roots[1..order] (roots[0] is the constant
    term's slot).  Returns (iterations, psim list)."""
    order = len(roots) - 1
    psim = [np.zeros_like(src) for _ in range(order)]
    it, _ = ks_multicg_offset_field(src, psim, np.asarray(roots[1:], dtype=np.float64), qic, fn)
    return it, psim


def ks_rateval(src, psim, residues, parity):
    """dest = residues[0] src + sum_j residues[j+1] psim[j] on `parity`
    (ks_imp_rhmc/ks_ratinv.c:116-137); other sites are zero."""
    V = src.shape[0]
    lo, hi = (0, V // 2) if parity == EVEN else ((V // 2, V) if parity == ODD else (0, V))
    dest = np.zeros_like(src)
    dest[lo:hi] = residues[0] * src[lo:hi]
    for j, p in enumerate(psim):
        dest[lo:hi] += residues[j + 1] * p[lo:hi]
    return dest


def load_hisq_links(thin_phased, eps_naik=(0.0,)):
    eps = np.ascontiguousarray(eps_naik, dtype=np.float64)
    check(init().mks_load_links_from_thin(_lib.MKS_ACTION_HISQ, _dp(thin_phased), len(eps), _dp(eps), 1.0),
          "mks_load_links_from_thin")


def load_asqtad_links(thin_phased, u0=1.0):
    eps = np.zeros(1)
    check(init().mks_load_links_from_thin(_lib.MKS_ACTION_ASQTAD, _dp(thin_phased), 1, _dp(eps), u0),
          "mks_load_links_from_thin")


def get_hisq_aux():
    V = int(np.prod(_state["dims"]))
    Vl = np.zeros((V, 4, 18)); W = np.zeros((V, 4, 18))
    check(init().mks_get_hisq_aux(_dp(Vl), _dp(W)), "mks_get_hisq_aux")
    return Vl, W


def eo_fermion_force_multi(eps, residues, xxx, mom, n_orders_naik=None, n_naiks=1, action="hisq"):
    """mom updated in place.  action "hisq": fermion_force_hisq_multi.c:170;
    "asqtad": fermion_force_multi.c:29 (FNMAT, fermion_force_fn_multi.c:80),
    which needs links loaded with load_asqtad_links."""
    res = np.ascontiguousarray(residues, dtype=np.float64)
    if action == "asqtad":
        check(init().mks_fermion_force_multi_asqtad(eps, _dp(res), _pp(list(xxx)), len(res), _dp(mom)),
              "mks_fermion_force_multi_asqtad")
        return mom
    n = len(res)
    if n_orders_naik is None:
        n_orders_naik = [n] + [0] * (n_naiks - 1)
    ords = (ctypes.c_int * len(n_orders_naik))(*n_orders_naik)
    check(init().mks_fermion_force_multi_hisq(eps, _dp(res), _pp(list(xxx)), n, ords, n_naiks, _dp(mom)),
          "mks_fermion_force_multi_hisq")
    return mom


def fermion_force_adjoint(residues, xxx, n_orders_naik=None, n_naiks=1):
    """K_U (V, 4, 18) with dS = 2 Re sum tr(K_U dU) for the fermion bilinear
    S = 2 Re sum_j residues[j] X_j^dag D_eo Y_j (X_j, Y_j the even / odd parts
    of xxx[j]) through the links of the last load (mks_fermion_force_adjoint)."""
    res = np.ascontiguousarray(residues, dtype=np.float64)
    V = int(np.prod(_state["dims"]))
    ku = np.zeros((V, 4, 18))
    ords = None if n_orders_naik is None else (ctypes.c_int * len(n_orders_naik))(*n_orders_naik)
    check(init().mks_fermion_force_adjoint(_dp(res), _pp(list(xxx)), len(res), ords, n_naiks, _dp(ku)),
          "mks_fermion_force_adjoint")
    return ku


# ---- gauge side of the RHMC: resident thin links and momenta ----
def gauge_load(thin_unphased):
    """Resident thin links from MILC's host layout without phases."""
    check(init().mks_gauge_load(_dp(np.ascontiguousarray(thin_unphased, dtype=np.float64))), "mks_gauge_load")


def gauge_get():
    V = int(np.prod(_state["dims"]))
    U = np.zeros((V, 4, 18))
    check(init().mks_gauge_get(_dp(U)), "mks_gauge_get")
    return U


def mom_load(mom):
    check(init().mks_mom_load(_dp(np.ascontiguousarray(mom, dtype=np.float64))), "mks_mom_load")


def mom_get():
    V = int(np.prod(_state["dims"]))
    mom = np.zeros((V, 4, 10))
    check(init().mks_mom_get(_dp(mom)), "mks_mom_get")
    return mom


def rng_seed(iseed):
    check(init().mks_rng_seed(int(iseed)), "mks_rng_seed")


def ranmom():
    check(init().mks_ranmom(), "mks_ranmom")


def gaussian_vector(parity, v=None):
    V = int(np.prod(_state["dims"]))
    v = np.zeros((V, 6)) if v is None else v
    check(init().mks_gaussian_vector(parity, _dp(v)), "mks_gaussian_vector")
    return v


def gauge_force(eps, beta, u0, nflavors, prec=PREC_DOUBLE):
    check(init().mks_gauge_force_prec(eps, beta, u0, nflavors, prec), "mks_gauge_force_prec")


def gauge_action(beta, u0, nflavors):
    a = ctypes.c_double()
    check(init().mks_gauge_action(beta, u0, nflavors, ctypes.byref(a)), "mks_gauge_action")
    return a.value


def update_u(eps):
    check(init().mks_update_u(eps), "mks_update_u")


def mom_action():
    h = ctypes.c_double()
    check(init().mks_mom_action(ctypes.byref(h)), "mks_mom_action")
    return h.value


def reunitarize():
    check(init().mks_reunitarize(), "mks_reunitarize")


def plaquette():
    ss, st = ctypes.c_double(), ctypes.c_double()
    check(init().mks_plaquette(ctypes.byref(ss), ctypes.byref(st)), "mks_plaquette")
    return ss.value, st.value


def md_precision(prec):
    check(init().mks_md_precision(prec), "mks_md_precision")


def rebuild_links(action="hisq", eps_naik=(0.0,), u0=1.0):
    eps = np.ascontiguousarray(eps_naik, dtype=np.float64)
    act = _lib.MKS_ACTION_HISQ if action == "hisq" else _lib.MKS_ACTION_ASQTAD
    check(init().mks_rebuild_links(act, len(eps), _dp(eps), u0), "mks_rebuild_links")


# ---- host-side synthetic inputs (no device work) ----
def gen_thin_links(dims, seed, a=0.3):
    V = int(np.prod(dims))
    U = np.zeros((V, 4, 18))
    check(_lib.load().mks_gen_thin_links(_dims(dims), seed, a, _dp(U)), "mks_gen_thin_links")
    return U


def apply_phases(dims, links):
    out = np.ascontiguousarray(links, dtype=np.float64).copy()
    check(_lib.load().mks_apply_phases(_dims(dims), _dp(out), 1), "mks_apply_phases")
    return out


def gen_vector(dims, seed, parity=EVEN):
    V = int(np.prod(dims))
    v = np.zeros((V, 6))
    check(_lib.load().mks_gen_vector(_dims(dims), seed, parity, _dp(v)), "mks_gen_vector")
    return v


def gen_momenta(dims, seed):
    V = int(np.prod(dims))
    m = np.zeros((V, 4, 10))
    check(_lib.load().mks_gen_momenta(_dims(dims), seed, _dp(m)), "mks_gen_momenta")
    return m
