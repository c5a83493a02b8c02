"""The GPU path against MILC's own shipped test vectors (asqtad, 8^4,
u0 = 0.502, mass 0.1; see milc_samples.py): link construction, the
(M^dag M)^-1 and M^-1 solves on both parities and the asqtad fermion force,
each compared with the stored MILC answer (float32 files) and with the
oracle on the same inputs."""
import numpy as np
import pytest

import milc_samples as S
from conftest import rel

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def sample(gpu, oracle_cls):
    d = S.load()
    Up = gpu.apply_phases(S.DIMS, S.reunitarize(d["lat"]))
    orc = oracle_cls(S.DIMS)
    fat, lng = orc.asqtad_links(Up, S.U0)
    gpu.set_lattice(S.DIMS)
    gpu.load_asqtad_links(Up, S.U0)
    return dict(d=d, Up=Up, orc=orc, fat=fat, lng=lng, src=d["src"].astype(np.float64))


def test_links(gpu, sample):
    fat, lng = gpu.get_fn_links()
    assert rel(fat, sample["fat"]) < 1e-14 and rel(lng, sample["lng"]) < 1e-14
    sub = sample["d"]["sub"]
    assert rel(fat[sub], sample["d"]["fat_sub"]) < 2e-7
    assert rel(lng[sub], sample["d"]["long_sub"]) < 2e-7


@pytest.mark.parametrize("prec", ["double", "single", "half"])
def test_mdagm_inverse(gpu, sample, prec):
    gpu.set_lattice(S.DIMS)
    gpu.load_asqtad_links(sample["Up"], S.U0)
    p = {"double": gpu.PREC_DOUBLE, "single": gpu.PREC_SINGLE, "half": gpu.PREC_HALF}[prec]
    qic = gpu.QuarkInvertControl(resid=S.RESID_MDAGM, max=300, nrestart=5, parity=gpu.EVENANDODD, prec=p)
    x = np.zeros_like(sample["src"])
    iters = gpu.ks_congrad_field(sample["src"], x, qic, S.MASS)
    assert qic.converged and qic.final_rsq < S.RESID_MDAGM ** 2
    assert rel(x, sample["d"]["ans_mdagm"]) < 5e-7
    if prec == "double":
        assert abs(iters - 2 * S.ITERS_MDAGM) <= 2 * S.ITER_TOL
        assert f"{qic.final_rsq:.1e}" == f"{S.FINAL_RSQ_MDAGM:.1e}"


def test_m_inverse(gpu, sample):
    gpu.set_lattice(S.DIMS)
    gpu.load_asqtad_links(sample["Up"], S.U0)
    qic = gpu.QuarkInvertControl(resid=S.RESID_M, max=300, nrestart=5, parity=gpu.EVENANDODD,
                                 prec=gpu.PREC_DOUBLE)
    x = np.zeros_like(sample["src"])
    iters = gpu.mat_invert_uml_field(sample["src"], x, qic, S.MASS)
    assert abs(iters - sum(S.ITERS_M)) <= 2 * S.ITER_TOL
    assert rel(x, sample["d"]["ans_m"]) < 5e-7


def test_asqtad_force(gpu, sample):
    gpu.set_lattice(S.DIMS)
    gpu.load_asqtad_links(sample["Up"], S.U0)
    src = sample["src"]
    mom = np.zeros((src.shape[0], 4, 10))
    gpu.eo_fermion_force_multi(1.0, [1.0], [src], mom, action="asqtad")
    diff, norm = S.force_errors(mom, sample["d"]["mom_sub"], sample["d"]["sub"])
    assert (diff <= S.FORCE_TOL * norm).all()
    assert diff.max() / norm.max() < 2e-7
    ref = sample["orc"].fermion_force_asqtad(sample["Up"], S.U0, 1.0, [1.0], src[None])
    assert np.abs(mom - ref).max() < 1e-12 * np.abs(ref).max()


def test_asqtad_force_needs_asqtad_links(gpu, sample):
    from milc_qcd_gb300 import MksError
    gpu.set_lattice(S.DIMS)
    gpu.load_hisq_links(sample["Up"])
    mom = np.zeros((sample["src"].shape[0], 4, 10))
    with pytest.raises(MksError):
        gpu.eo_fermion_force_multi(1.0, [1.0], [sample["src"]], mom, action="asqtad")
