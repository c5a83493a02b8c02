"""ctypes bindings for the CPU oracle (test infrastructure only).

Two checkers live here:

* ``Oracle`` -- the C restatement in ``milc_oracle.c`` (``liborc.so``),
  built anywhere a C compiler exists (also on the GPU host).
* ``MilcRef`` -- MILC's own CPU code compiled from the reference sources by
  ``oracle/ref/Makefile`` into ``oracle/_ref/libmilc_ref_<action>.so``.  It
  exists only where the reference tree was available at build time.  MILC
  keeps one global lattice per process, so each ``MilcRef`` should run in its
  own process (see ``run_ref_in_subprocess``).

Arrays are numpy float64 in MILC's field layout (see include/milc_ks_gb300.h).
Only tests, the smoke check and the benchmark's CPU-baseline leg import this
module.
"""
import ctypes
import os
import subprocess
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
EVEN, ODD, EVENANDODD = 0x02, 0x01, 0x03

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


def _ptr(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def build_oracle():
    subprocess.run(["make", "-s", "-f", os.path.join(HERE, "Makefile")], check=True)


def build_ref(ref_root=None, jobs=8):
    """Compile MILC's CPU sources into oracle/_ref with the recipe
    oracle/ref/Makefile.  ref_root: the reference source tree; by default
    $MILC_REFERENCE_DIR, else the recipe's own default location.  Where no
    reference tree exists nothing is built and False is returned."""
    ref_root = ref_root or os.environ.get("MILC_REFERENCE_DIR")
    cmd = ["make", "-s", "-j%d" % jobs, "-f", os.path.join(HERE, "ref", "Makefile"), "OUT=%s" % REF_DIR]
    if ref_root:
        cmd.append("REF=%s" % ref_root)
    subprocess.run(cmd, check=True)
    return ref_available("hisq")


def reference_tree():
    """The reference source tree: $MILC_REFERENCE_DIR, else the tree that
    oracle/_ref was built from (the recipe records it in oracle/_ref/source_dir),
    else None (as on hosts without the reference)."""
    p = os.environ.get("MILC_REFERENCE_DIR")
    if not p:
        try:
            with open(os.path.join(REF_DIR, "source_dir")) as f:
                p = f.read().strip()
        except OSError:
            return None
    return p if p and os.path.isdir(p) else None


# ---- the seeded synthetic inputs (mks_synth.h, compiled into liborc.so) ----
def _orc_lib():
    path = os.path.join(HERE, "liborc.so")
    if not os.path.exists(path):
        build_oracle()
    return ctypes.CDLL(path)


def _dims_arr(dims):
    return (ctypes.c_int * 4)(*[int(d) for d in dims])


def gen_thin_links(dims, seed, a=0.3):
    """Unphased thin links U[V][4][18] = exp(i a H); identical to the
    product library's mks_gen_thin_links (same source)."""
    U = np.zeros((int(np.prod(dims)), 4, 18))
    if _orc_lib().orc_gen_thin_links(_dims_arr(dims), ctypes.c_uint64(seed), ctypes.c_double(a), _ptr(U)) != 0:
        raise ValueError("orc_gen_thin_links: bad dims")
    return U


def gen_vector(dims, seed, parity=EVEN):
    v = np.zeros((int(np.prod(dims)), 6))
    if _orc_lib().orc_gen_vector(_dims_arr(dims), ctypes.c_uint64(seed), ctypes.c_int(parity), _ptr(v)) != 0:
        raise ValueError("orc_gen_vector: bad dims")
    return v


def gen_momenta(dims, seed):
    m = np.zeros((int(np.prod(dims)), 4, 10))
    if _orc_lib().orc_gen_momenta(_dims_arr(dims), ctypes.c_uint64(seed), _ptr(m)) != 0:
        raise ValueError("orc_gen_momenta: bad dims")
    return m


def ref_available(action="hisq"):
    return os.path.exists(os.path.join(REF_DIR, "libmilc_ref_%s.so" % action))


class _Lat(ctypes.Structure):
    _fields_ = [("dims", ctypes.c_int * 4), ("V", ctypes.c_size_t), ("Vh", ctypes.c_size_t),
                ("coord", _ip), ("nb", ctypes.POINTER(ctypes.c_size_t))]


class Oracle:
    """The C restatement, one lattice geometry per instance."""

    def __init__(self, dims):
        path = os.path.join(HERE, "liborc.so")
        if not os.path.exists(path):
            build_oracle()
        lib = ctypes.CDLL(path)
        self.lib = lib
        lib.orc_lat_create.restype = ctypes.POINTER(_Lat)
        lib.orc_lat_create.argtypes = [ctypes.c_int] * 4
        lib.orc_congrad.restype = ctypes.c_int
        lib.orc_mat_invert_uml.restype = ctypes.c_int
        lib.orc_multicg_offset.restype = ctypes.c_int
        lib.orc_hisq_links.restype = ctypes.c_int
        lib.orc_u3_unitarize.restype = ctypes.c_int
        if hasattr(lib, "orc_force_action"):
            lib.orc_force_action.restype = ctypes.c_double
        self.dims = tuple(int(d) for d in dims)
        self.L = lib.orc_lat_create(*self.dims)
        self.V = int(np.prod(self.dims))

    def __del__(self):
        try:
            self.lib.orc_lat_free(self.L)
        except Exception:
            pass

    def rephase(self, links):
        out = np.ascontiguousarray(links, dtype=np.float64).copy()
        self.lib.orc_rephase(self.L, _ptr(out))
        return out

    def dslash(self, fat, lng, src, parity, dst=None):
        dst = np.zeros_like(src) if dst is None else dst.copy()
        self.lib.orc_dslash(self.L, _ptr(fat), _ptr(lng), _ptr(src), _ptr(dst), ctypes.c_int(parity))
        return dst

    def congrad(self, fat, lng, src, dst, mass, parity, resid, relresid=0.0, max_iter=1000,
                nrestart=5):
        dst = dst.copy()
        out = np.zeros(7)
        it = self.lib.orc_congrad(self.L, _ptr(fat), _ptr(lng), _ptr(src), _ptr(dst),
                                  ctypes.c_double(mass), ctypes.c_int(parity),
                                  ctypes.c_double(resid), ctypes.c_double(relresid),
                                  ctypes.c_int(max_iter), ctypes.c_int(nrestart), _ptr(out))
        return it, dst, out

    def congrad_multi(self, fat, lng, srcs, dsts, mass, parity, resid, relresid=0.0, max_iter=1000,
                      nrestart=5):
        """Independent CG solves of several sources in lockstep (the links are
        read once per D for all of them); each result equals congrad's."""
        n = len(srcs)
        srcs = [np.ascontiguousarray(s, dtype=np.float64) for s in srcs]
        dsts = [np.ascontiguousarray(d, dtype=np.float64).copy() for d in dsts]
        out = np.zeros((n, 7))
        PA = _dp * n
        it = self.lib.orc_congrad_multi(self.L, _ptr(fat), _ptr(lng), ctypes.c_int(n), PA(*[_ptr(s) for s in srcs]),
                                        PA(*[_ptr(d) for d in dsts]), ctypes.c_double(mass), ctypes.c_int(parity),
                                        ctypes.c_double(resid), ctypes.c_double(relresid),
                                        ctypes.c_int(max_iter), ctypes.c_int(nrestart), _ptr(out))
        return it, dsts, out

    def mat_invert_uml(self, fat, lng, src, dst, mass, resid, max_iter=1000, nrestart=5):
        dst = dst.copy()
        out = np.zeros(7)
        it = self.lib.orc_mat_invert_uml(self.L, _ptr(fat), _ptr(lng), _ptr(src), _ptr(dst),
                                         ctypes.c_double(mass), ctypes.c_double(resid),
                                         ctypes.c_int(max_iter), ctypes.c_int(nrestart), _ptr(out))
        return it, dst, out

    def multicg_offset(self, fat, lng, src, offsets, parity, resid, max_iter=1000, nrestart=5):
        offsets = np.ascontiguousarray(offsets, dtype=np.float64)
        n = len(offsets)
        psim = np.zeros((n,) + src.shape)
        frsq = np.zeros(n)
        it = self.lib.orc_multicg_offset(self.L, _ptr(fat), _ptr(lng), _ptr(src), _ptr(psim),
                                         _ptr(offsets), ctypes.c_int(n), ctypes.c_int(parity),
                                         ctypes.c_double(resid), ctypes.c_int(max_iter),
                                         ctypes.c_int(nrestart), _ptr(frsq))
        return it, psim, frsq

    def asqtad_links(self, U, u0=1.0):
        fat = np.zeros_like(U)
        lng = np.zeros_like(U)
        self.lib.orc_asqtad_links(self.L, _ptr(U), ctypes.c_double(u0), _ptr(fat), _ptr(lng))
        return fat, lng

    def hisq_links(self, U, eps_naik=(0.0,)):
        eps = np.ascontiguousarray(eps_naik, dtype=np.float64)
        n = len(eps)
        Vl = np.zeros_like(U)
        W = np.zeros_like(U)
        fat = np.zeros((n,) + U.shape)
        lng = np.zeros((n,) + U.shape)
        nsvd = self.lib.orc_hisq_links(self.L, _ptr(U), ctypes.c_int(n), _ptr(eps), _ptr(Vl), _ptr(W),
                                       _ptr(fat), _ptr(lng))
        return dict(V=Vl, W=W, fat=fat, lng=lng, nsvd=nsvd)

    def u3_unitarize(self, Vm):
        Vm = np.ascontiguousarray(Vm, dtype=np.float64)
        W = np.zeros(18)
        svd = self.lib.orc_u3_unitarize(_ptr(Vm), _ptr(W))
        return W, svd

    def fermion_force_hisq(self, U, eps, residues, xxx, orders=None, eps_naik=(0.0,), mom=None):
        eps_arr = np.ascontiguousarray(eps_naik, dtype=np.float64)
        res = np.ascontiguousarray(residues, dtype=np.float64)
        xxx = np.ascontiguousarray(xxx, dtype=np.float64)
        nterms = len(res)
        if orders is None:
            orders = [nterms] + [0] * (len(eps_arr) - 1)
        ords = np.ascontiguousarray(orders, dtype=np.int32)
        mom = np.zeros((self.V, 4, 10)) if mom is None else mom.copy()
        self.lib.orc_fermion_force_hisq(self.L, _ptr(U), ctypes.c_int(len(eps_arr)), _ptr(eps_arr),
                                        ctypes.c_double(eps), _ptr(res), _ptr(xxx),
                                        ctypes.c_int(nterms), ords.ctypes.data_as(_ip), _ptr(mom))
        return mom

    def fermion_force_asqtad(self, U, u0, eps, residues, xxx, mom=None):
        res = np.ascontiguousarray(residues, dtype=np.float64)
        xxx = np.ascontiguousarray(xxx, dtype=np.float64)
        mom = np.zeros((self.V, 4, 10)) if mom is None else mom.copy()
        self.lib.orc_fermion_force_asqtad(self.L, _ptr(U), ctypes.c_double(u0), ctypes.c_double(eps),
                                          _ptr(res), _ptr(xxx), ctypes.c_int(len(res)), _ptr(mom))
        return mom

    def force_action(self, U, residues, xxx, orders=None, eps_naik=(0.0,)):
        eps_arr = np.ascontiguousarray(eps_naik, dtype=np.float64)
        res = np.ascontiguousarray(residues, dtype=np.float64)
        xxx = np.ascontiguousarray(xxx, dtype=np.float64)
        nterms = len(res)
        if orders is None:
            orders = [nterms] + [0] * (len(eps_arr) - 1)
        ords = np.ascontiguousarray(orders, dtype=np.int32)
        return self.lib.orc_force_action(self.L, _ptr(U), ctypes.c_int(len(eps_arr)), _ptr(eps_arr),
                                         _ptr(res), _ptr(xxx), ctypes.c_int(nterms),
                                         ords.ctypes.data_as(_ip))


class _Prn(ctypes.Structure):
    _fields_ = [("r", ctypes.c_uint32 * 7), ("multiplier", ctypes.c_uint64), ("addend", ctypes.c_uint64),
                ("ic_state", ctypes.c_uint64)]


class _Loops(ctypes.Structure):
    _fields_ = [("nloop", ctypes.c_int), ("length", ctypes.c_int * 3), ("num", ctypes.c_int * 3),
                ("dirs", ((ctypes.c_int * 6) * 16) * 3), ("coeff", ctypes.c_double * 3)]


class GaugeOracle:
    """Gauge side of the RHMC (milc_oracle_gauge.c) on one Oracle's geometry.
    Links are unphased, momenta (V, 4, 10); the site random generators are
    held here (MILC's SITERAND streams)."""

    def __init__(self, orc):
        self.orc, self.lib, self.L, self.V = orc, orc.lib, orc.L, orc.V
        lib = self.lib
        lib.orc_gauge_action.restype = ctypes.c_double
        lib.orc_hmom_action.restype = ctypes.c_double
        lib.orc_myrand.restype = ctypes.c_double
        lib.orc_gaussian.restype = ctypes.c_double
        self.prn = None

    def loop_table(self, nflavors, u0):
        T = _Loops()
        self.lib.orc_loop_table(ctypes.c_int(nflavors), ctypes.c_double(u0), ctypes.byref(T))
        return T

    def action(self, U, beta, u0, nflavors):
        return self.lib.orc_gauge_action(self.L, _ptr(U), ctypes.c_double(beta), ctypes.c_double(u0),
                                         ctypes.c_int(nflavors))

    def force(self, U, eps, beta, u0, nflavors, mom):
        mom = mom.copy()
        self.lib.orc_gauge_force(self.L, _ptr(U), ctypes.c_double(eps), ctypes.c_double(beta),
                                 ctypes.c_double(u0), ctypes.c_int(nflavors), _ptr(mom))
        return mom

    def update_u(self, U, mom, eps):
        U = U.copy()
        self.lib.orc_update_u(self.L, _ptr(U), _ptr(mom), ctypes.c_double(eps))
        return U

    def hmom_action(self, mom):
        return self.lib.orc_hmom_action(self.L, _ptr(mom))

    def reunitarize(self, U):
        U = U.copy()
        self.lib.orc_reunitarize(self.L, _ptr(U))
        return U

    def plaquette(self, U):
        ss, st = ctypes.c_double(), ctypes.c_double()
        self.lib.orc_plaquette(self.L, _ptr(U), ctypes.byref(ss), ctypes.byref(st))
        return ss.value, st.value

    def seed(self, iseed):
        self.prn = (_Prn * self.V)()
        self.lib.orc_site_prn_init(self.L, ctypes.c_int(iseed), self.prn)

    def ranmom(self):
        mom = np.zeros((self.V, 4, 10))
        self.lib.orc_ranmom(self.L, self.prn, _ptr(mom))
        return mom

    def gaussian_vector(self, parity):
        v = np.zeros((self.V, 6))
        self.lib.orc_gaussian_vector(self.L, self.prn, ctypes.c_int(parity), _ptr(v))
        return v


class MilcRef:
    """MILC's own CPU implementation (single lattice per process)."""

    def __init__(self, dims, action="hisq", eps_naik=(0.0,)):
        path = os.path.join(REF_DIR, "libmilc_ref_%s.so" % action)
        lib = ctypes.CDLL(path, mode=ctypes.RTLD_LOCAL)
        self.lib = lib
        self.action = action
        lib.ref_sites.restype = ctypes.c_size_t
        lib.ref_congrad.restype = ctypes.c_int
        lib.ref_mat_invert_uml.restype = ctypes.c_int
        lib.ref_multicg_offset.restype = ctypes.c_int
        self.dims = tuple(int(d) for d in dims)
        eps = np.ascontiguousarray(eps_naik, dtype=np.float64)
        self.n_naiks = len(eps)
        rc = lib.ref_init(*[ctypes.c_int(d) for d in self.dims], ctypes.c_int(len(eps)), _ptr(eps))
        if rc != 0:
            raise RuntimeError("MILC reference lattice already initialised in this process")
        self.V = int(lib.ref_sites())

    def coords(self):
        c = np.zeros((self.V, 4), dtype=np.int32)
        self.lib.ref_coords(c.ctypes.data_as(_ip))
        return c

    def set_u0(self, u0):
        self.lib.ref_set_u0(ctypes.c_double(u0))

    def set_thin_links(self, U_unphased):
        self.lib.ref_set_thin_links(_ptr(np.ascontiguousarray(U_unphased)))

    def thin_links_phased(self):
        U = np.zeros((self.V, 4, 18))
        self.lib.ref_get_thin_links_phased(_ptr(U))
        return U

    def build_links(self):
        self.lib.ref_build_links()

    def fn_links(self, inaik=0):
        fat = np.zeros((self.V, 4, 18))
        lng = np.zeros((self.V, 4, 18))
        self.lib.ref_get_fn_links(ctypes.c_int(inaik), _ptr(fat), _ptr(lng))
        return fat, lng

    def hisq_aux(self):
        U = np.zeros((self.V, 4, 18)); Vl = np.zeros_like(U); W = np.zeros_like(U)
        self.lib.ref_get_hisq_aux(_ptr(U), _ptr(Vl), _ptr(W))
        return U, Vl, W

    def dslash(self, src, parity, inaik=0, dst=None):
        dst = np.zeros_like(src) if dst is None else dst.copy()
        self.lib.ref_dslash(_ptr(src), _ptr(dst), ctypes.c_int(parity), ctypes.c_int(inaik))
        return dst

    def congrad(self, src, dst, mass, parity, resid, relresid=0.0, max_iter=1000, nrestart=5, inaik=0):
        dst = dst.copy()
        out = np.zeros(7)
        it = self.lib.ref_congrad(_ptr(src), _ptr(dst), ctypes.c_double(mass), ctypes.c_int(parity),
                                  ctypes.c_double(resid), ctypes.c_double(relresid),
                                  ctypes.c_int(max_iter), ctypes.c_int(nrestart), ctypes.c_int(inaik),
                                  _ptr(out))
        return it, dst, out

    def mat_invert_uml(self, src, dst, mass, resid, max_iter=1000, nrestart=5, inaik=0):
        dst = dst.copy()
        out = np.zeros(7)
        it = self.lib.ref_mat_invert_uml(_ptr(src), _ptr(dst), ctypes.c_double(mass),
                                         ctypes.c_double(resid), ctypes.c_int(max_iter),
                                         ctypes.c_int(nrestart), ctypes.c_int(inaik), _ptr(out))
        return it, dst, out

    def multicg_offset(self, src, offsets, parity, resid, max_iter=1000, nrestart=5, inaik=0):
        offsets = np.ascontiguousarray(offsets, dtype=np.float64)
        n = len(offsets)
        psim = np.zeros((n,) + src.shape)
        frsq = np.zeros(n)
        it = self.lib.ref_multicg_offset(_ptr(src), _ptr(psim), _ptr(offsets), ctypes.c_int(n),
                                         ctypes.c_int(parity), ctypes.c_double(resid),
                                         ctypes.c_int(max_iter), ctypes.c_int(nrestart),
                                         ctypes.c_int(inaik), _ptr(frsq))
        return it, psim, frsq

    # ---- gauge side of the RHMC (MILC's own routines) ----
    def set_gauge_params(self, beta, u0, dyn_flavors):
        fl = (ctypes.c_int * len(dyn_flavors))(*dyn_flavors)
        self.lib.ref_set_gauge_params(ctypes.c_double(beta), ctypes.c_double(u0), ctypes.c_int(len(dyn_flavors)), fl)

    def gauge_action(self):
        self.lib.ref_gauge_action.restype = ctypes.c_double
        return self.lib.ref_gauge_action()

    def gauge_force(self, eps, mom):
        mom = np.ascontiguousarray(mom, dtype=np.float64).copy()
        self.lib.ref_gauge_force(ctypes.c_double(eps), _ptr(mom))
        return mom

    def update_u(self, eps, mom):
        self.lib.ref_update_u(ctypes.c_double(eps), _ptr(np.ascontiguousarray(mom, dtype=np.float64)))

    def hmom_action(self, mom):
        self.lib.ref_hmom_action.restype = ctypes.c_double
        return self.lib.ref_hmom_action(_ptr(np.ascontiguousarray(mom, dtype=np.float64)))

    def seed(self, iseed):
        self.lib.ref_seed(ctypes.c_int(iseed))

    def ranmom(self):
        mom = np.zeros((self.V, 4, 10))
        self.lib.ref_ranmom(_ptr(mom))
        return mom

    def gaussian_vector(self, parity):
        v = np.zeros((self.V, 6))
        self.lib.ref_gaussian_vector(ctypes.c_int(parity), _ptr(v))
        return v

    def reunitarize(self):
        self.lib.ref_reunitarize()

    def plaquette(self):
        ss, st = ctypes.c_double(), ctypes.c_double()
        self.lib.ref_plaquette(ctypes.byref(ss), ctypes.byref(st))
        return ss.value, st.value

    def fermion_force(self, eps, residues, xxx, orders=None, mom=None):
        res = np.ascontiguousarray(residues, dtype=np.float64)
        xxx = np.ascontiguousarray(xxx, dtype=np.float64)
        nterms = len(res)
        if orders is None:
            orders = [nterms] + [0] * (self.n_naiks - 1)
        ords = np.ascontiguousarray(orders, dtype=np.int32)
        mom = np.zeros((self.V, 4, 10)) if mom is None else mom.copy()
        self.lib.ref_fermion_force(ctypes.c_double(eps), _ptr(res), _ptr(xxx), ctypes.c_int(nterms),
                                   ords.ctypes.data_as(_ip), _ptr(mom))
        return mom


def run_ref_in_subprocess(func, *args, **kwargs):
    """Run func(*args) in a fresh 'spawn' process (MILC keeps global state)."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Pool(1) as pool:
        return pool.apply(func, args, kwargs)
