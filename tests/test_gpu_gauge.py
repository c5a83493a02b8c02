"""Gauge side of the RHMC on the GPU against the oracle (which is pinned to
MILC in test_oracle_gauge.py): resident links round trip, plaquette, gauge
action and force, link update, momentum action, reunitarization, MILC's
site random generators, and fermion links rebuilt from updated links."""
import numpy as np
import pytest

from conftest import rel

pytestmark = pytest.mark.gpu

DIMS = (4, 4, 6, 8)
BETA, U0, NF = 7.4, 0.89, 3


@pytest.fixture(scope="module")
def setup(gpu, oracle_cls):
    from oracle.oracle import GaugeOracle
    m = gpu
    m.set_lattice(DIMS)
    U = m.gen_thin_links(DIMS, 41, 0.3)
    mom = m.gen_momenta(DIMS, 42)
    orc = oracle_cls(DIMS)
    return m, U, mom, orc, GaugeOracle(orc)


def _load(m, U, mom):
    m.set_lattice(DIMS)
    m.gauge_load(U)
    m.mom_load(mom)


def test_gauge_round_trip(setup):
    m, U, mom, orc, G = setup
    _load(m, U, mom)
    assert np.array_equal(m.gauge_get(), U)
    assert np.array_equal(m.mom_get(), mom)


def test_plaquette_and_action(setup):
    m, U, mom, orc, G = setup
    _load(m, U, mom)
    ss, st = m.plaquette()
    oss, ost = G.plaquette(U)
    assert abs(ss - oss) < 1e-13 and abs(st - ost) < 1e-13
    a = m.gauge_action(BETA, U0, NF)
    assert abs(a - G.action(U, BETA, U0, NF)) < 1e-12 * abs(a)
    assert abs(m.mom_action() - G.hmom_action(mom)) < 1e-10


def test_gauge_force(setup):
    m, U, mom, orc, G = setup
    _load(m, U, mom)
    m.gauge_force(0.017, BETA, U0, NF)
    assert rel(m.mom_get(), G.force(U, 0.017, BETA, U0, NF, mom)) < 1e-14


def test_gauge_force_fp32(setup):
    m, U, mom, orc, G = setup
    _load(m, U, mom)
    m.gauge_force(0.017, BETA, U0, NF, m.PREC_SINGLE)
    want = G.force(U, 0.017, BETA, U0, NF, mom)
    assert rel(m.mom_get() - mom, want - mom) < 1e-5


def test_update_u_and_reunitarize(setup):
    m, U, mom, orc, G = setup
    _load(m, U, mom)
    m.update_u(0.023)
    U1 = G.update_u(U, mom, 0.023)
    assert rel(m.gauge_get(), U1) < 1e-15
    m.reunitarize()
    assert rel(m.gauge_get(), G.reunitarize(U1)) < 1e-14


def test_random_generators(setup):
    from oracle.oracle import EVEN
    m, U, mom, orc, G = setup
    _load(m, U, mom)
    m.rng_seed(86658)
    G.seed(86658)
    m.ranmom()
    # CUDA's log may differ from the host's in the last bit
    assert np.abs(m.mom_get() - G.ranmom()).max() < 1e-13
    v = m.gaussian_vector(m.EVEN)
    assert np.abs(v - G.gaussian_vector(EVEN)).max() < 1e-13
    Vh = v.shape[0] // 2
    assert not v[Vh:].any()


def test_links_rebuilt_from_updated_links(setup):
    m, U, mom, orc, G = setup
    _load(m, U, mom)
    m.update_u(0.05)
    with pytest.raises(m.MksError):           # fermion links were invalidated
        m.dslash_fn_field(m.gen_vector(DIMS, 1, m.ODD), np.zeros((U.shape[0], 6)), m.EVEN)
    m.rebuild_links("hisq", (0.0, -0.05))
    U1p = m.apply_phases(DIMS, G.update_u(U, mom, 0.05))
    L = orc.hisq_links(U1p, (0.0, -0.05))
    for g in range(2):
        fat, lng = m.get_fn_links(g)
        assert rel(fat, L["fat"][g]) < 1e-13 and rel(lng, L["lng"][g]) < 1e-13
