"""D_eo on the GPU against the oracle (FP64: 1e-13 relative, MILC's dslash_fn_field)."""
import numpy as np
import pytest

from conftest import hisq_setup, rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims", [(8, 8, 8, 8), (6, 8, 10, 12), (16, 8, 8, 16)])
def test_dslash_f64_matches_oracle(gpu, oracle_cls, dims):
    m = gpu
    U, orc, L = hisq_setup(m, oracle_cls, dims)
    fat, lng = L["fat"][0], L["lng"][0]
    m.set_lattice(dims)
    m.load_fn_links(fat, lng)
    src = m.gen_vector(dims, 3, m.EVENANDODD)
    for par in (m.EVEN, m.ODD, m.EVENANDODD):
        out = np.zeros_like(src)
        m.dslash_fn_field(src, out, par)
        ref = orc.dslash(fat, lng, src, par)
        assert rel(out, ref) < 1e-13, (par, rel(out, ref))
    # the parity not written keeps its input values (MILC writes only `parity`)
    out = np.full_like(src, 7.0)
    m.dslash_fn_field(src, out, m.EVEN)
    V = src.shape[0]
    assert np.all(out[V // 2:] == 7.0)


def test_fn_links_roundtrip(gpu, oracle_cls):
    m = gpu
    dims = (8, 8, 8, 8)
    U, orc, L = hisq_setup(m, oracle_cls, dims)
    m.set_lattice(dims)
    m.load_fn_links(L["fat"][0], L["lng"][0], slot=3)
    f, l = m.get_fn_links(slot=3)
    assert np.array_equal(f, L["fat"][0]) and np.array_equal(l, L["lng"][0])


def test_bench_dslash_runs(gpu, oracle_cls):
    import ctypes
    m = gpu
    dims = (8, 8, 8, 8)
    U, orc, L = hisq_setup(m, oracle_cls, dims)
    m.set_lattice(dims)
    m.load_fn_links(L["fat"][0], L["lng"][0])
    lib = m._lib.load()
    for prec in (0, 1, 2):
        for nsrc in (1, 4):
            ms = ctypes.c_double()
            m.check(lib.mks_bench_dslash(prec, nsrc, m.EVEN, 0, 3, 0, ctypes.byref(ms)), "bench")
            assert ms.value > 0
