"""HISQ / asqtad link construction on the GPU against the oracle
(MILC's load_hisq_aux_links + load_hisq_fn_links / load_fatlinks)."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("dims", [(8, 8, 8, 8), (6, 8, 10, 12)])
def test_hisq_links_match_oracle(gpu, oracle_cls, dims):
    m = gpu
    U = m.apply_phases(dims, m.gen_thin_links(dims, 17, 0.3))
    orc = oracle_cls(dims)
    eps = (0.0, -0.1, 0.05)
    L = orc.hisq_links(U, eps)
    m.set_lattice(dims)
    m.load_hisq_links(U, eps)
    assert m._lib.load().mks_hisq_reunit_svd_count() == 0 and L["nsvd"] == 0
    Vg, Wg = m.get_hisq_aux()
    assert rel(Vg, L["V"]) < 1e-13
    assert rel(Wg, L["W"]) < 1e-12
    # W is unitary
    Wc = Wg.reshape(-1, 3, 3, 2)
    Wc = Wc[..., 0] + 1j * Wc[..., 1]
    assert np.abs(np.einsum("nij,nkj->nik", Wc, Wc.conj()) - np.eye(3)).max() < 1e-12
    for i in range(len(eps)):
        f, l = m.get_fn_links(slot=i)
        assert rel(f, L["fat"][i]) < 1e-12 and rel(l, L["lng"][i]) < 1e-12, i


def test_asqtad_links_match_oracle(gpu, oracle_cls):
    m = gpu
    dims = (8, 8, 8, 8)
    U = m.apply_phases(dims, m.gen_thin_links(dims, 19, 0.3))
    orc = oracle_cls(dims)
    for u0 in (1.0, 0.87):
        fat_o, lng_o = orc.asqtad_links(U, u0)
        m.set_lattice(dims)
        m.load_asqtad_links(U, u0)
        f, l = m.get_fn_links(slot=0)
        assert rel(f, fat_o) < 1e-13 and rel(l, lng_o) < 1e-13


def test_hisq_links_then_dslash(gpu, oracle_cls):
    m = gpu
    dims = (8, 8, 8, 8)
    U = m.apply_phases(dims, m.gen_thin_links(dims, 23, 0.3))
    orc = oracle_cls(dims)
    L = orc.hisq_links(U)
    m.set_lattice(dims)
    m.load_hisq_links(U)
    src = m.gen_vector(dims, 2, m.EVENANDODD)
    out = np.zeros_like(src)
    m.dslash_fn_field(src, out, m.EVENANDODD)
    assert rel(out, orc.dslash(L["fat"][0], L["lng"][0], src, m.EVENANDODD)) < 1e-12
