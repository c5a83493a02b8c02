"""Multi-shift CG on the GPU against the oracle (MILC's ks_multicg_offset_field)."""
import numpy as np
import pytest

from conftest import hisq_setup, rel

pytestmark = pytest.mark.gpu
DIMS = (8, 8, 8, 8)


def test_multishift_fp64_matches_oracle(gpu, oracle_cls):
    m = gpu
    U, orc, L = hisq_setup(m, oracle_cls, DIMS)
    fat, lng = L["fat"][0], L["lng"][0]
    m.set_lattice(DIMS)
    m.load_fn_links(fat, lng)
    b = m.gen_vector(DIMS, 51, m.EVEN)
    offs = 4 * 0.02 ** 2 + np.logspace(-4, 0, 11)
    psim = [np.zeros_like(b) for _ in offs]
    qic = m.QuarkInvertControl(resid=1e-10, max=1000, nrestart=5, parity=m.EVEN, prec=m.PREC_DOUBLE)
    it, per = m.ks_multicg_offset_field(b, psim, offs, qic)
    it_o, po, fo = orc.multicg_offset(fat, lng, b, offs, m.EVEN, 1e-10)
    assert abs(it - it_o) <= 1
    for j in range(len(offs)):
        assert rel(psim[j], po[j]) < 1e-9, (j, rel(psim[j], po[j]))
        assert per[j].converged == 1


@pytest.mark.parametrize("prec", ["PREC_SINGLE", "PREC_HALF"])
def test_multishift_mixed_refined(gpu, oracle_cls, prec):
    m = gpu
    U, orc, L = hisq_setup(m, oracle_cls, DIMS)
    fat, lng = L["fat"][0], L["lng"][0]
    m.set_lattice(DIMS)
    m.load_fn_links(fat, lng)
    b = m.gen_vector(DIMS, 52, m.EVEN)
    offs = np.logspace(-3, 0, 6)
    psim = [np.zeros_like(b) for _ in offs]
    qic = m.QuarkInvertControl(resid=1e-10, max=2000, nrestart=5, parity=m.EVEN, prec=getattr(m, prec))
    it, per = m.ks_multicg_offset_field(b, psim, offs, qic)
    for j, s in enumerate(offs):
        # exact FP64 residual of each shifted system through the oracle
        Dx = orc.dslash(fat, lng, orc.dslash(fat, lng, psim[j], m.ODD), m.EVEN)
        r = b - (s * psim[j] - Dx)
        V2 = b.shape[0] // 2
        assert np.linalg.norm(r[:V2]) / np.linalg.norm(b[:V2]) < 1.01e-10, j
        assert per[j].converged == 1


def test_multishift_rejects_nonpositive_offset(gpu, oracle_cls):
    m = gpu
    U, orc, L = hisq_setup(m, oracle_cls, DIMS)
    m.set_lattice(DIMS)
    m.load_fn_links(L["fat"][0], L["lng"][0])
    b = m.gen_vector(DIMS, 53, m.EVEN)
    qic = m.QuarkInvertControl(resid=1e-8, parity=m.EVEN)
    with pytest.raises(m.MksError):
        m.ks_multicg_offset_field(b, [np.zeros_like(b)] * 2, [0.1, 0.0], qic)


def test_ratinv_rateval_against_single_solves(gpu, oracle_cls):
    """R(A) b = a0 b + sum_j a_j (A + sigma_j)^-1 b, A = -D_eo D_oe, through the
    multi-shift solve (ks_ratinv) and the linear combination (ks_rateval)."""
    m = gpu
    U, orc, L = hisq_setup(m, oracle_cls, DIMS)
    fat, lng = L["fat"][0], L["lng"][0]
    m.set_lattice(DIMS)
    m.load_fn_links(fat, lng)
    b = m.gen_vector(DIMS, 54, m.EVEN)
    roots = [0.0, 0.002, 0.03, 0.4]
    residues = [0.7, 0.05, 0.2, 0.9]
    qic = m.QuarkInvertControl(resid=1e-11, max=2000, nrestart=5, parity=m.EVEN, prec=m.PREC_DOUBLE)
    it, psim = m.ks_ratinv(b, roots, residues, qic)
    dest = m.ks_rateval(b, psim, residues, m.EVEN)
    ref = residues[0] * b
    for j, s in enumerate(roots[1:]):
        _, x, _ = orc.congrad(fat, lng, b, np.zeros_like(b), np.sqrt(s) / 2, m.EVEN, 1e-13, 0.0, 2000, 5)
        ref = ref + residues[j + 1] * x
    V2 = b.shape[0] // 2
    assert rel(dest[:V2], ref[:V2]) < 1e-9


@pytest.mark.parametrize("resid", [1e-10, 1e-6])
def test_multishift_several_fields(gpu, oracle_cls, resid):
    """Three fields with their own offsets solved in one batched FP32 multi-
    shift (mks_ks_multicg_offset_multi_dev): every shifted system of every
    field meets the residual in FP64, checked through the oracle."""
    import ctypes
    torch = pytest.importorskip("torch")
    m = gpu
    U, orc, L = hisq_setup(m, oracle_cls, DIMS)
    fat, lng = L["fat"][0], L["lng"][0]
    m.set_lattice(DIMS)
    m.load_fn_links(fat, lng)
    lib = m._lib.load()
    bs = [m.gen_vector(DIMS, 60 + f, m.EVEN) for f in range(3)]
    offs = [np.logspace(-3, 0, 6), np.logspace(-2, 0.5, 4), 4 * 0.3 ** 2 + np.logspace(-1, 1, 5)]
    nsh = [len(o) for o in offs]
    d_src = [torch.from_numpy(b).cuda() for b in bs]
    d_psim = [torch.zeros_like(d_src[f]) for f in range(3) for _ in offs[f]]
    flat = np.ascontiguousarray(np.concatenate(offs), dtype=np.float64)
    res = (m._lib.InvertResult * len(flat))()
    arg = m._lib.InvertArg(2000, 5, m.EVEN, m.PREC_SINGLE, resid, 0.0, 0.1)
    it = lib.mks_ks_multicg_offset_multi_dev(
        3, (ctypes.c_void_p * 3)(*[t.data_ptr() for t in d_src]), (ctypes.c_int * 3)(*nsh),
        flat.ctypes.data_as(m._lib.DP), (ctypes.c_void_p * len(d_psim))(*[t.data_ptr() for t in d_psim]), 0,
        ctypes.byref(arg), res)
    m.check(it, "mks_ks_multicg_offset_multi_dev")
    V2 = bs[0].shape[0] // 2
    k = 0
    for f in range(3):
        for s in offs[f]:
            x = d_psim[k].cpu().numpy()
            Dx = orc.dslash(fat, lng, orc.dslash(fat, lng, x, m.ODD), m.EVEN)
            r = bs[f] - (s * x - Dx)
            assert np.linalg.norm(r[:V2]) / np.linalg.norm(bs[f][:V2]) < 1.01 * resid, (f, s)
            assert res[k].converged == 1
            k += 1


def test_multishift_page_locked_host_arrays(gpu, oracle_cls):
    """Page-locked source and solution arrays are used in place by the layout
    kernels: the solutions equal those of pageable arrays bit for bit and the
    other parity's half of each solution array is not written."""
    torch = pytest.importorskip("torch")
    m = gpu
    U, orc, L = hisq_setup(m, oracle_cls, DIMS)
    m.set_lattice(DIMS)
    m.load_fn_links(L["fat"][0], L["lng"][0])
    b = m.gen_vector(DIMS, 61, m.EVEN)
    offs = np.logspace(-3, 0, 5)
    qic = m.QuarkInvertControl(resid=1e-8, max=2000, nrestart=5, parity=m.EVEN, prec=m.PREC_SINGLE)
    ref = [np.full_like(b, 0.25) for _ in offs]
    m.ks_multicg_offset_field(b, ref, offs, qic)
    pb = torch.from_numpy(b.copy()).pin_memory().numpy()
    pp = [torch.from_numpy(np.full_like(b, 0.25)).pin_memory().numpy() for _ in offs]
    it, per = m.ks_multicg_offset_field(pb, pp, offs, qic)
    V2 = b.shape[0] // 2
    for j in range(len(offs)):
        assert per[j].converged == 1
        assert np.array_equal(pp[j], ref[j]), j
        assert np.all(pp[j][V2:] == 0.25)


def test_multishift_counts_bound_the_update_work(gpu, oracle_cls):
    """mks_multishift_counts reports the iteration phase's iterations and
    shift updates: every iteration advances the lowest shift and at most all
    of them; in mixed precision, shifts converged a decade below the target
    stop being advanced before the end."""
    import ctypes
    m = gpu
    U, orc, L = hisq_setup(m, oracle_cls, DIMS)
    m.set_lattice(DIMS)
    m.load_fn_links(L["fat"][0], L["lng"][0])
    b = m.gen_vector(DIMS, 57, m.EVEN)
    offs = 4 * 0.02 ** 2 + np.logspace(-4, 0, 11)
    lib = m._lib.load()
    n_it, n_upd = ctypes.c_longlong(), ctypes.c_longlong()
    psim = [np.zeros_like(b) for _ in offs]
    qic = m.QuarkInvertControl(resid=1e-10, max=1000, nrestart=5, parity=m.EVEN, prec=m.PREC_DOUBLE)
    it, _ = m.ks_multicg_offset_field(b, psim, offs, qic)
    m.check(lib.mks_multishift_counts(ctypes.byref(n_it), ctypes.byref(n_upd)), "counts")
    assert n_it.value == it
    assert n_it.value <= n_upd.value <= len(offs) * n_it.value
    psim = [np.zeros_like(b) for _ in offs]
    qic = m.QuarkInvertControl(resid=1e-10, max=1000, nrestart=5, parity=m.EVEN, prec=m.PREC_SINGLE)
    it, _ = m.ks_multicg_offset_field(b, psim, offs, qic)
    m.check(lib.mks_multishift_counts(ctypes.byref(n_it), ctypes.byref(n_upd)), "counts")
    assert 0 < n_it.value <= it  # `it` also counts the refinement iterations
    assert n_it.value <= n_upd.value < len(offs) * n_it.value
