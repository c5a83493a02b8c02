"""One HISQ RHMC trajectory on the GPU (mks_rhmc_trajectory) against
MILC's own regression, ks_imp_rhmc/test/su3_rhmc_hisq.2.sample-out (double
precision; 6^4, 2+1 flavours, 4 pseudofermion fields, 3G1F, 10 steps):
the heat-bath source sums, the action terms before and after, Delta S and
the final plaquette, with FP64 multi-shift solves; and with mixed-precision
solves against the same numbers within MILC's own tolerance file."""
import numpy as np
import pytest

import milc_samples as S
import rhmc_sample as R

pytestmark = pytest.mark.gpu


def _run(m, prec):
    from milc_qcd_gb300.rhmc import update
    d = R.load()
    m.set_lattice(R.DIMS)
    m.gauge_load(S.reunitarize(d["lat"]))
    m.mom_load(np.zeros((int(np.prod(R.DIMS)), 4, 10)))
    m.rng_seed(R.ISEED)
    pfs = [dict(d["rational"][i], naik_term_epsilon=float(d["naik_eps"][i])) for i in range(R.N_PSEUDO)]
    return update(pfs, R.BETA, R.U0, R.nflavors(), R.EPSILON, R.STEPS, R.INT_ALG, R.RESID_MD, R.RESID_FA,
                  R.RESID_GR, R.MAX_CG, prec, prec, prec, R.NRESTART, True, prec_force=prec)


def test_trajectory_fp64_reproduces_milc_sample(gpu):
    out = _run(gpu, gpu.PREC_DOUBLE)
    for got, want in zip(out["grsource_sum"], R.GRSOURCE_SUMS):
        assert abs(got - want) < 1e-10 * want
    for got, want in zip(out["start"], R.ACTION_START):
        assert abs(got - want) < 1e-11 * abs(want)
    for got, want in zip(out["end"], R.ACTION_END):
        assert abs(got - want) < 1e-10 * abs(want)
    assert abs(out["delta_s"] - R.DELTA_S) < 1e-7
    assert abs(out["plaq_ss"] - R.PLAQ_END[0]) < 1e-11 and abs(out["plaq_st"] - R.PLAQ_END[1]) < 1e-11
    assert out["unconverged"] == 0
    assert out["n_fermion_force"] == 10 and out["n_gauge_force"] == 30


@pytest.mark.parametrize("prec", ["PREC_SINGLE"])
def test_trajectory_mixed_precision_within_milc_tolerance(gpu, prec):
    out = _run(gpu, getattr(gpu, prec))
    assert abs(out["delta_s"] - R.DELTA_S) < R.DELTA_S_TOL
    assert abs(out["plaq_ss"] - R.PLAQ_END[0]) < R.PLAQ_END_TOL[0]
    assert abs(out["plaq_st"] - R.PLAQ_END[1]) < R.PLAQ_END_TOL[1]
    assert out["unconverged"] == 0
