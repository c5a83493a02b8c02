"""MILC's shipped asqtad test vectors (8^4, u0 = 0.502, mass 0.1) and the
host-side steps MILC applies to them before its checks.

The fixture tests/golden/milc_sample_l8.npz is made from the reference's
binary_samples by tests/golden/make_milc_samples.py.  The golden scalars
below are the ones MILC prints for the same run in
ks_imp_utilities/test/check_ks_invert.1.sample-out (the .errtol files next
to it give the tolerances: iterations +-10).
"""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "milc_sample_l8.npz")

DIMS = (8, 8, 8, 8)
U0 = 0.502
MASS = 0.1
RESID_MDAGM = 1e-9     # check_ks_invert.1.sample-in: error_for_propagator (invert MdaggerM)
RESID_M = 1e-10        # check_ks_invert.2.sample-in: error_for_propagator (invert M)
PLAQ = (2.6203978710714737e+00, 2.6214473754080179e+00)          # sample-out:41 CHECK PLAQ
LINKTR = (2.8951765559213527e+00, -2.0951840825345069e-06)       # sample-out:42 CHECK LINKTR
ITERS_MDAGM = 61       # sample-out:81 (per parity)
FINAL_RSQ_MDAGM = 7.8e-19
ITERS_M = (64, 13)     # sample-out:136-137 (even solve, odd clean-up)
FINAL_RSQ_M = (8.4e-21, 5.9e-21)
ITER_TOL = 10          # check_ks_invert.1.errtol: "iters= 10"
FORCE_TOL = 1e-5       # check_fermion_force.c: per-link |diff| <= tol |mom| (double build)


def load():
    d = np.load(FIXTURE)
    return {k: d[k] for k in d.files}


def cmat(a):
    return (a[..., 0::2] + 1j * a[..., 1::2]).reshape(a.shape[:-1] + (3, 3))


def real18(m):
    out = np.zeros(m.shape[:-2] + (18,))
    out[..., 0::2] = m.real.reshape(m.shape[:-2] + (9,))
    out[..., 1::2] = m.imag.reshape(m.shape[:-2] + (9,))
    return out


def reunitarize(a):
    """generic/reunitarize2.c:112-216 (reunit_su3), as MILC applies it to a
    lattice read in single precision (generic/io_helpers.c:212): normalise
    row 0, orthogonalise and normalise row 1, row 2 = (row0 x row1)^*."""
    M = cmat(np.asarray(a, dtype=np.float64))
    r0 = M[..., 0, :] / np.sqrt((np.abs(M[..., 0, :]) ** 2).sum(-1))[..., None]
    r1 = M[..., 1, :] - (np.conj(r0) * M[..., 1, :]).sum(-1)[..., None] * r0
    r1 = r1 / np.sqrt((np.abs(r1) ** 2).sum(-1))[..., None]
    r2 = np.conj(np.cross(r0, r1))
    return real18(np.stack([r0, r1, r2], axis=-2))


def uncompress(mom):
    """anti_hermitmat (V, 4, 10) -> (V, 4, 18) (libraries/uncmp_ahmat.c)."""
    A = np.zeros(mom.shape[:-1] + (3, 3), complex)
    A[..., 0, 1] = mom[..., 0] + 1j * mom[..., 1]
    A[..., 0, 2] = mom[..., 2] + 1j * mom[..., 3]
    A[..., 1, 2] = mom[..., 4] + 1j * mom[..., 5]
    A[..., 1, 0] = -np.conj(A[..., 0, 1])
    A[..., 2, 0] = -np.conj(A[..., 0, 2])
    A[..., 2, 1] = -np.conj(A[..., 1, 2])
    A[..., 0, 0] = 1j * mom[..., 6]
    A[..., 1, 1] = 1j * mom[..., 7]
    A[..., 2, 2] = 1j * mom[..., 8]
    return real18(A)


def plaquettes(U, coords, dims=DIMS):
    """MILC's d_plaquette (generic/d_plaq4.c): mean Re tr of the
    space-space and space-time plaquettes; U (V, 4, 18) unphased, MILC order,
    coords (V, 4) the site coordinates."""
    Uc = cmat(U)
    L = np.array(dims)
    lex = coords[:, 0] + L[0] * (coords[:, 1] + L[1] * (coords[:, 2] + L[2] * coords[:, 3]))
    where = np.empty(len(lex), dtype=np.int64)
    where[lex] = np.arange(len(lex))

    def up(mu):
        c = coords.copy()
        c[:, mu] = (c[:, mu] + 1) % L[mu]
        return where[c[:, 0] + L[0] * (c[:, 1] + L[1] * (c[:, 2] + L[2] * c[:, 3]))]

    def plaq(mu, nu):
        P = Uc[:, mu] @ Uc[up(mu), nu] @ np.conj(np.swapaxes(Uc[up(nu), mu], -1, -2)) \
            @ np.conj(np.swapaxes(Uc[:, nu], -1, -2))
        return np.trace(P, axis1=-2, axis2=-1).real.mean()

    ss = np.mean([plaq(0, 1), plaq(0, 2), plaq(1, 2)])
    st = np.mean([plaq(0, 3), plaq(1, 3), plaq(2, 3)])
    return ss, st


def link_trace(U):
    t = np.trace(cmat(U), axis1=-2, axis2=-1).mean()
    return t.real, t.imag


def force_errors(mom, golden_sub, sub):
    """MILC's check (check_fermion_force.c:101-134) on the fixture's sites:
    per-link |diff| and |mom| (Frobenius), uncompressed."""
    M = uncompress(mom)[sub]
    G = golden_sub.astype(np.float64)
    diff = np.sqrt(((M - G) ** 2).sum(-1))
    norm = np.sqrt((M ** 2).sum(-1))
    return diff, norm


def site_coords(dims=DIMS):
    """(V, 4) coordinates of every MILC index (package host geometry)."""
    import ctypes
    from milc_qcd_gb300 import _lib
    lib = _lib.load()
    d4 = (ctypes.c_int * 4)(*dims)
    V = int(np.prod(dims))
    out = np.zeros((V, 4), dtype=np.int64)
    c = (ctypes.c_int * 4)()
    for i in range(V):
        lib.mks_site_coords(d4, i, c)
        out[i] = list(c)
    return out


def ref_run(Ur, src):
    """MILC's own CPU code (oracle/_ref, asqtad build) on the sample:
    fat/long links, (M^dag M)^-1 on both parities, M^-1, and the force.
    Runs in a fresh process (MILC keeps one global lattice)."""
    from oracle.oracle import MilcRef
    ref = MilcRef(DIMS, "asqtad")
    ref.set_u0(U0)
    ref.set_thin_links(Ur)
    ref.build_links()
    fat, lng = ref.fn_links()
    x = np.zeros_like(src)
    its = []
    for par in (0x02, 0x01):
        it, x, out = ref.congrad(src, x, MASS, par, RESID_MDAGM, 0.0, 300, 5)
        its.append(it)
    it_m, xm, _ = ref.mat_invert_uml(src, np.zeros_like(src), MASS, RESID_M, 300, 5)
    mom = ref.fermion_force(1.0, [1.0], src[None])
    return dict(fat=fat, lng=lng, x=x, iters=its, xm=xm, iters_m=it_m, mom=mom)
