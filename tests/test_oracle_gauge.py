"""The gauge side of the RHMC in the oracle (milc_oracle_gauge.c) against
MILC itself (oracle/_ref, when present), and the composed oracle trajectory
against MILC's own HISQ RHMC regression output (su3_rhmc_hisq.2.sample-out,
double precision build): heat-bath source sums, start and end action
terms, the trajectory's Delta S and the final plaquette."""
import numpy as np
import pytest

import milc_samples as S
import rhmc_sample as R
from conftest import rel

DIMS = (4, 4, 4, 6)


def _ref_gauge(U, mom):
    from oracle.oracle import MilcRef, EVEN
    r = MilcRef(DIMS, "hisq")
    r.set_gauge_params(7.4, 0.89, [2, 1])
    r.set_thin_links(U)
    out = dict(plaq=r.plaquette(), g=r.gauge_action(), force=r.gauge_force(0.02, mom), h=r.hmom_action(mom))
    r.update_u(0.013, mom)
    out["U1"] = r.thin_links_phased()
    r.seed(86658)
    out["mom_rand"] = r.ranmom()
    out["g_rand"] = r.gaussian_vector(EVEN)
    r.reunitarize()
    out["U2"] = r.thin_links_phased()
    return out


def test_loop_table(oracle_cls):
    from oracle.oracle import GaugeOracle
    T = GaugeOracle(oracle_cls(DIMS)).loop_table(3, 0.89)
    assert list(T.num) == [6, 12, 16]          # G_LOOP counts of the sample output
    assert T.coeff[0] == 1.0
    lu = np.log(0.89)
    assert abs(T.coeff[1] - (-1.0 / (20 * 0.89 ** 2) * (1 - (0.6264 - 1.1746 * 3) * lu))) < 1e-15
    assert abs(T.coeff[2] - (1.0 / 0.89 ** 2 * (0.0433 - 0.0156 * 3) * lu)) < 1e-15


def test_gauge_oracle_matches_milc(lib, oracle_cls):
    from oracle.oracle import GaugeOracle, ref_available, run_ref_in_subprocess, EVEN
    if not ref_available("hisq"):
        pytest.skip("MILC reference build not present")
    U = lib.gen_thin_links(DIMS, 5, 0.3)
    mom = lib.gen_momenta(DIMS, 6)
    Rr = run_ref_in_subprocess(_ref_gauge, U, mom)
    G = GaugeOracle(oracle_cls(DIMS))
    ss, st = G.plaquette(U)
    assert abs(ss + Rr["plaq"][0]) < 1e-13 and abs(st + Rr["plaq"][1]) < 1e-13   # MILC's has phases in
    assert abs(G.action(U, 7.4, 0.89, 3) - Rr["g"]) < 1e-12 * abs(Rr["g"])
    assert rel(G.force(U, 0.02, 7.4, 0.89, 3, mom), Rr["force"]) < 1e-15
    assert abs(G.hmom_action(mom) - Rr["h"]) < 1e-12
    U1 = G.update_u(lib.apply_phases(DIMS, U), mom, 0.013)
    assert rel(U1, Rr["U1"]) < 1e-15
    G.seed(86658)
    assert np.array_equal(G.ranmom(), Rr["mom_rand"])
    assert np.array_equal(G.gaussian_vector(EVEN), Rr["g_rand"])
    U2 = lib.apply_phases(DIMS, G.reunitarize(lib.apply_phases(DIMS, U1)))
    assert rel(U2, Rr["U2"]) < 1e-15


def test_gauge_force_is_minus_gradient(lib, oracle_cls):
    """dS_g/dt along U -> exp(t A) U equals -Re tr(A F) summed, with F the
    momentum change per unit eps (central differences, h = 1e-5)."""
    from oracle.oracle import GaugeOracle
    G = GaugeOracle(oracle_cls(DIMS))
    U = lib.gen_thin_links(DIMS, 15, 0.3)
    A = lib.gen_momenta(DIMS, 16)            # random su(3) direction per link
    F = G.force(U, 1.0, 7.4, 0.89, 3, np.zeros_like(A))   # mom after one unit kick from zero
    h = 1e-5
    Sp = G.action(G.update_u(U, A, h), 7.4, 0.89, 3)
    Sm = G.action(G.update_u(U, A, -h), 7.4, 0.89, 3)
    fd = (Sp - Sm) / (2 * h)
    # dS/dt = -<A, F>, <A, F> = -Re tr(A F) for anti-Hermitian A, F; in
    # MILC's compressed form the off-diagonal 2(re re + im im) + diagonal im im
    dot = 2 * (A[..., :6] * F[..., :6]).sum() + (A[..., 6:9] * F[..., 6:9]).sum()
    assert abs(fd + dot) < 1e-6 * abs(fd)


@pytest.fixture(scope="module")
def rhmc():
    d = R.load()
    return d, S.reunitarize(d["lat"])


def test_rhmc_sample_plaquette(rhmc, oracle_cls):
    from oracle.oracle import GaugeOracle
    d, U = rhmc
    ss, st = GaugeOracle(oracle_cls(R.DIMS)).plaquette(d["lat"].astype(np.float64))
    assert abs(ss - R.PLAQ_START[0]) < 1e-14 and abs(st - R.PLAQ_START[1]) < 1e-14


def test_oracle_trajectory_reproduces_milc_sample(rhmc):
    from oracle.rhmc_oracle import OracleRHMC
    d, U = rhmc
    o = OracleRHMC(R.DIMS, U, R.BETA, R.U0, R.nflavors(), d["rational"], d["naik_eps"], R.RESID_MD,
                   R.RESID_FA, R.RESID_GR, R.MAX_CG, R.NRESTART, R.ISEED)
    out = o.trajectory(R.EPSILON, R.STEPS)
    for got, want in zip(out["grsource_sums"], R.GRSOURCE_SUMS):
        assert abs(got - want) < 1e-10 * want
    for got, want in zip(out["start"], R.ACTION_START):
        assert abs(got - want) < 1e-12 * abs(want)
    for got, want in zip(out["end"], R.ACTION_END):
        assert abs(got - want) < 1e-11 * abs(want)
    assert abs(out["delta_s"] - R.DELTA_S) < 1e-8
    assert abs(out["plaq"][0] - R.PLAQ_END[0]) < 1e-12 and abs(out["plaq"][1] - R.PLAQ_END[1]) < 1e-12
