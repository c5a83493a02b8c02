"""The C oracle against golden outputs of MILC itself (tests/golden/*.npz,
produced by tests/golden/make_golden.py from MILC's compiled CPU code).
This pins the oracle on machines without the reference tree."""
import os

import numpy as np
import pytest

from conftest import ROOT, rel

G = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def hisq():
    return dict(np.load(os.path.join(G, "hisq_4x4x4x8.npz")))


@pytest.fixture(scope="module")
def asqtad():
    return dict(np.load(os.path.join(G, "asqtad_4x4x4x8.npz")))


def test_generator_reproduces_fixture_inputs(lib, hisq):
    dims = tuple(hisq["dims"])
    assert np.array_equal(lib.gen_thin_links(dims, 101, 0.3), hisq["thin"])
    assert np.array_equal(lib.apply_phases(dims, hisq["thin"]), hisq["thin_phased"])


def test_oracle_phases(oracle_cls, hisq):
    orc = oracle_cls(tuple(hisq["dims"]))
    assert np.array_equal(orc.rephase(hisq["thin"]), hisq["thin_phased"])


def test_oracle_hisq_links(oracle_cls, hisq):
    orc = oracle_cls(tuple(hisq["dims"]))
    L = orc.hisq_links(hisq["thin_phased"], tuple(hisq["eps_naik"]))
    assert L["nsvd"] == 0
    assert rel(L["V"], hisq["V"]) < 1e-14
    assert rel(L["W"], hisq["W"]) < 1e-13
    for g in range(len(hisq["eps_naik"])):
        assert rel(L["fat"][g], hisq["fat%d" % g]) < 1e-13
        assert rel(L["lng"][g], hisq["lng%d" % g]) < 1e-13


def test_oracle_dslash(oracle_cls, hisq):
    orc = oracle_cls(tuple(hisq["dims"]))
    for name, par in (("even", 2), ("odd", 1), ("both", 3)):
        out = orc.dslash(hisq["fat0"], hisq["lng0"], hisq["src"], par)
        assert rel(out, hisq["dslash_" + name]) < 1e-14


def test_oracle_cg_same_iterations(oracle_cls, hisq):
    orc = oracle_cls(tuple(hisq["dims"]))
    b = hisq["cg_src"]
    it, x, q = orc.congrad(hisq["fat0"], hisq["lng0"], b, np.zeros_like(b), float(hisq["mass"]), 2, 1e-9, 0.0, 40, 10)
    assert it == int(hisq["cg_iters"])
    assert rel(x, hisq["cg_x"]) < 1e-13
    assert np.allclose(q, hisq["cg_qic"], rtol=1e-6, atol=1e-30)


def test_oracle_multishift(oracle_cls, hisq):
    orc = oracle_cls(tuple(hisq["dims"]))
    b = hisq["cg_src"]
    it, psim, _ = orc.multicg_offset(hisq["fat0"], hisq["lng0"], b, hisq["ms_offsets"], 2, 1e-10)
    assert it == int(hisq["ms_iters"])
    assert rel(psim, hisq["ms_psim"]) < 1e-13


def test_oracle_mat_invert(oracle_cls, hisq):
    orc = oracle_cls(tuple(hisq["dims"]))
    src = hisq["src"]
    it, x, _ = orc.mat_invert_uml(hisq["fat0"], hisq["lng0"], src, np.zeros_like(src), float(hisq["mass"]), 1e-10)
    assert it == int(hisq["mi_iters"])
    assert rel(x, hisq["mi_x"]) < 1e-12


def test_oracle_force_matches_milc(oracle_cls, hisq):
    orc = oracle_cls(tuple(hisq["dims"]))
    mom = orc.fermion_force_hisq(hisq["thin_phased"], float(hisq["ff_eps"]), hisq["ff_res"], hisq["ff_xxx"],
                                 orders=list(hisq["ff_orders"]), eps_naik=tuple(hisq["eps_naik"]),
                                 mom=hisq["ff_mom0"])
    d, dr = mom - hisq["ff_mom0"], hisq["ff_mom"] - hisq["ff_mom0"]
    assert rel(d[..., :9], dr[..., :9]) < 1e-12  # forces are required to agree within 1e-10


def test_oracle_asqtad(oracle_cls, asqtad):
    orc = oracle_cls(tuple(asqtad["dims"]))
    fat, lng = orc.asqtad_links(asqtad["thin_phased"], 1.0)
    assert rel(fat, asqtad["fat"]) < 1e-14 and rel(lng, asqtad["lng"]) < 1e-14
    assert rel(orc.dslash(fat, lng, asqtad["src"], 3), asqtad["dslash_both"]) < 1e-14
    b = asqtad["cg_src"]
    it, x, _ = orc.congrad(fat, lng, b, np.zeros_like(b), float(asqtad["mass"]), 2, 1e-9, 0.0, 40, 10)
    assert it == int(asqtad["cg_iters"]) and rel(x, asqtad["cg_x"]) < 1e-13


def test_oracle_lockstep_cg_equals_single_source(oracle_cls, hisq):
    """The lockstep multi-source oracle CG (used to check the benchmark's block
    solves at full size) gives each source exactly what the single-source CG
    gives: solutions bit for bit, same iterations, restarts and residuals.
    Sources converge at different iterations, one is zero, and the restart
    length is short so that restarts interleave with the iterations."""
    from oracle import oracle as O
    dims = tuple(hisq["dims"])
    orc = oracle_cls(dims)
    fat, lng, mass = hisq["fat0"], hisq["lng0"], float(hisq["mass"])
    srcs = [O.gen_vector(dims, 800 + k, 2) * (1.0 + k) for k in range(3)] + [np.zeros_like(hisq["cg_src"])]
    srcs[1][::7] *= 30.0  # a differently conditioned right-hand side
    x0 = [np.zeros_like(s) for s in srcs]
    x0[2] = O.gen_vector(dims, 900, 2) * 0.1
    it, xs, out = orc.congrad_multi(fat, lng, srcs, x0, mass, 2, 1e-9, 0.0, 15, 20)
    its = []
    for k in range(len(srcs)):
        itk, xk, ok = orc.congrad(fat, lng, srcs[k], x0[k], mass, 2, 1e-9, 0.0, 15, 20)
        its.append(itk)
        assert np.array_equal(xs[k], xk), k
        assert np.array_equal(out[k], ok), k
    assert it == max(its) and len(set(its[:3])) > 1
